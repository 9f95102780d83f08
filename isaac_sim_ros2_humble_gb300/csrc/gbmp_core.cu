// gbmp_core.cu -- robot / environment handles, FK, state checks and edge
// validation kernels of libgbmp, and their C-ABI entry points.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>

#include "gbmp_groups.h"
#include "gbmp_internal.h"
#include "gbmp_order.h"

namespace gbmp {

static thread_local std::string g_err;

void set_error(const char *fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
}

// ---------------------------------------------------------------------------------
// Launch helpers.
// ---------------------------------------------------------------------------------
static size_t block_smem(const DevRobot &R, int nwords) {
    return smem_tables_bytes(R, nwords) + smem_warp_bytes(R) * kWarpsPerBlock;
}

static DeviceKernelSet g_smem_optin;

gbmp_status ensure_smem_optin(const void *fn) {
    int dev = 0;
    GBMP_CUDA(cudaGetDevice(&dev));
    if (g_smem_optin.contains(dev, fn)) return GBMP_OK;
    // the dynamic limit is what the device allows a block minus the kernel's static shared
    // memory (the staging mbarrier and flags)
    cudaFuncAttributes fa;
    GBMP_CUDA(cudaFuncGetAttributes(&fa, fn));
    int optin = 0;
    GBMP_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    GBMP_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes));
    GBMP_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared));
    g_smem_optin.insert(dev, fn);
    return GBMP_OK;
}

template <typename K>
static gbmp_status persistent_grid(K kernel, size_t smem, int num_sms, int *grid) {
    gbmp_status st = ensure_smem_optin((const void *)kernel);
    if (st) return st;
    int per_sm = 0;
    GBMP_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kWarpsPerBlock * kWarp, smem));
    if (per_sm < 1) {
        set_error("kernel does not fit on an SM (%zu bytes of shared memory)", smem);
        return GBMP_ERR_CAPACITY;
    }
    *grid = per_sm * num_sms;
    return GBMP_OK;
}

// ---------------------------------------------------------------------------------
// Kernels.
// ---------------------------------------------------------------------------------

// FK (+ sphere centres) of n states; one warp per state.
__global__ void __launch_bounds__(kWarpsPerBlock *kWarp)
    k_fk(DevRobot R, const float *__restrict__ q, long long n, float *__restrict__ poses,
         float *__restrict__ centers) {
    extern __shared__ __align__(16) unsigned char smem[];
    DevEnv E{0, 0, 0, nullptr};
    SmemTables t = carve_tables(smem, R, 0);
    if (!stage_tables(R, E, t, 0)) return;
    WarpScratch w = carve_warp(smem + smem_tables_bytes(R, 0), R, threadIdx.x / kWarp);
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const long long nw = (long long)gridDim.x * kWarpsPerBlock;
    for (long long s = blockIdx.x * (long long)kWarpsPerBlock + threadIdx.x / kWarp; s < n; s += nw) {
        for (int j = lane; j < R.L; j += kWarp) w.q[j] = q[s * R.L + j];
        __syncwarp();
        warp_fk(t, R.L, w, lane);
        store_fk(t, R, w, s, poses, centers, lane);
        __syncwarp();
    }
}

// Collision check of n states; one warp per state.  With poses / centers non-null the
// FK of each state is also written out (the reference's update() and checkStates() from
// one FK).  Four blocks per SM (64 registers): 4,096 states then take one round of the
// resident warps (4,864) instead of two of 3,648 (measured 16.3 against 18.4 us on the
// plain 4,096-configuration workload).
template <bool COST, int SPL>
__global__ void __launch_bounds__(kWarpsPerBlock *kWarp, 4)
    k_check_states(DevRobot R, DevEnv E, const float *__restrict__ q, long long n,
                   unsigned char *__restrict__ verdict, float *__restrict__ costs, float *__restrict__ total,
                   float *__restrict__ poses, float *__restrict__ centers) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int nwords = env_words(E.ns, E.nb, E.nc);
    SmemTables t = carve_tables(smem, R, nwords);
    if (!stage_tables(R, E, t, nwords)) return;
    WarpScratch w = carve_warp(smem + smem_tables_bytes(R, nwords), R, threadIdx.x / kWarp);
    __syncthreads();
    const int lane = threadIdx.x & 31;
    const long long nw = (long long)gridDim.x * kWarpsPerBlock;
    for (long long s = blockIdx.x * (long long)kWarpsPerBlock + threadIdx.x / kWarp; s < n; s += nw)
        check_state<COST, SPL>(t, R, E, w, q, s, n, verdict, costs, total, poses, centers, lane);
}

// Edge set-up: step count, direction, L2 length (KernelGenerator.h:433-465); one thread per
// edge.  Also counts the edges per length bucket (hist, longest bucket first) for the
// longest-first processing order.  An edge of more than kMaxEdgeStates states gets
// kMaxEdgeStates + 1 and is not validated.
__global__ void k_edge_setup(const float *__restrict__ from, const float *__restrict__ to, long long E, int L,
                             float res, int rule, int *__restrict__ nsteps, float *__restrict__ dir,
                             int *__restrict__ hist, float *__restrict__ length_out, int *__restrict__ nsteps_out) {
    const long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (k >= E) return;
    const float *f = from + k * L, *t = to + k * L;
    float d2 = 0.f, dinf = 0.f;
    for (int j = 0; j < L; ++j) {
        const float d = __fadd_rn(f[j], -t[j]);
        d2 = __fmaf_rn(d, d, d2);
        dinf = fmaxf(dinf, fabsf(d));
    }
    const float len = __fsqrt_rn(d2);
    // checkMotions: n = floor(metric / res) + 1 states, dir = (to - from) / n; the count
    // rule (pRRTC's granularity G = res): n = G + 1 states at k / G, dir = (to - from) / G
    const bool count = rule == GBMP_STEP_COUNT;
    const float metric = rule == GBMP_STEP_LINF ? dinf : len;
    const float ratio = count ? res : __fdiv_rn(metric, res);
    const int n = ratio < (float)kMaxEdgeStates ? (int)ratio + 1 : kMaxEdgeStates + 1;
    const float fn = count ? (float)(n - 1) : (float)n;
    for (int j = 0; j < L; ++j) dir[k * L + j] = __fdiv_rn(__fadd_rn(t[j], -f[j]), fn);
    nsteps[k] = n;
    atomicAdd(hist + edge_bucket(n), 1);
    if (length_out) length_out[k] = len;
    if (nsteps_out) nsteps_out[k] = n;
}

// Processing order of the edges, longest bucket first: order[slot] = edge, the slots of a
// bucket following the counts of the longer buckets (hist) in arrival order (cursor).
__global__ void k_edge_order(const int *__restrict__ nsteps, long long E, const int *__restrict__ hist,
                             int *__restrict__ cursor, int *__restrict__ order) {
    __shared__ int base[kEdgeBuckets];
    if (threadIdx.x == 0) {
        int acc = 0;
        for (int b = 0; b < kEdgeBuckets; ++b) { base[b] = acc; acc += hist[b]; }
    }
    __syncthreads();
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < E; k += (long long)gridDim.x * blockDim.x) {
        const int b = edge_bucket(nsteps[k]);
        order[base[b] + atomicAdd(cursor + b, 1)] = (int)k;
    }
}

// Edge validation state by state (robots with more than 32 sphere groups, and the
// per-state form of the others): a warp takes the next edge of `order` (a shared
// counter), walks its states -- in order when the first hit is asked for, else coarse to
// fine (verdict_order_state, gbmp_order.h) -- and stops at a colliding state.
template <int SPL, bool CULL>
__global__ void __launch_bounds__(kWarpsPerBlock *kWarp, CULL ? 3 : 1)
    k_edge_states(DevRobot R, DevEnv E, const float *__restrict__ from, const float *__restrict__ to,
                  const int *__restrict__ nsteps, const float *__restrict__ dir, const int *__restrict__ order,
                  long long n_edges, int *__restrict__ next, unsigned char *__restrict__ ok_out,
                  int *__restrict__ first_hit_out) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int nwords = env_words(E.ns, E.nb, E.nc);
    SmemTables t = carve_tables(smem, R, nwords);
    if (!stage_tables(R, E, t, nwords)) return;
    WarpScratch w = carve_warp(smem + smem_tables_bytes(R, nwords), R, threadIdx.x / kWarp);
    const int lane = threadIdx.x & 31;
    for (;;) {
        int i = 0;
        if (lane == 0) i = atomicAdd(next, 1);
        i = __shfl_sync(kFull, i, 0);
        if (i >= n_edges) break;
        const int e = order[i];
        const int n = nsteps[e];
        int hit = -1;
        if (n > kMaxEdgeStates) {
            hit = -2;   // too long to validate
        } else {
            const long long off = (long long)e * R.L;
            const bool any = first_hit_out == nullptr;
            for (int c = 0; c < n; ++c) {
                const int s = any ? verdict_order_state(c, n) : c;
                for (int j = lane; j < R.L; j += kWarp)
                    w.q[j] = (s == n - 1) ? to[off + j] : __fmaf_rn(dir[off + j], (float)s, from[off + j]);
                __syncwarp();
                warp_fk(t, R.L, w, lane);
                const bool h = CULL ? warp_collide_culled<SPL>(t, R, E, w, lane)
                                    : warp_collide<SPL, false>(t, R, E, w, lane, nullptr);
                __syncwarp();
                if (h) { hit = s; break; }
            }
        }
        if (lane == 0) {
            if (ok_out) ok_out[e] = hit == -1;
            if (first_hit_out) first_hit_out[e] = hit;
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------------
// Host helpers.
// ---------------------------------------------------------------------------------
static void host_unit_axis(const float *a, float *n) {
    const float len = sqrtf(fmaf(a[2], a[2], fmaf(a[1], a[1], a[0] * a[0])));
    const float valid = (len >= 1e-12f) ? 1.f : 0.f;
    const float inv = 1.f / fmaxf(len, 1e-12f);
    n[0] = a[0] * inv * valid;
    n[1] = a[1] * inv * valid;
    n[2] = a[2] * inv * valid;
    n[3] = valid;
}

// Inverse pose [R^T | -R^T t] (EnvConstraintCuboid.cu:13-34, EnvConstraintCylinder.cu:17-45).
static void host_inverse_pose(const float *pos, const float *rot, float4 *rows) {
    const float t00 = rot[0], t01 = rot[3], t02 = rot[6];
    const float t10 = rot[1], t11 = rot[4], t12 = rot[7];
    const float t20 = rot[2], t21 = rot[5], t22 = rot[8];
    rows[0] = make_float4(t00, t01, t02, -(t00 * pos[0] + t01 * pos[1] + t02 * pos[2]));
    rows[1] = make_float4(t10, t11, t12, -(t10 * pos[0] + t11 * pos[1] + t12 * pos[2]));
    rows[2] = make_float4(t20, t21, t22, -(t20 * pos[0] + t21 * pos[1] + t22 * pos[2]));
}

static int current_device_sms(int *dev) {
    int d = 0, sms = 0;
    if (cudaGetDevice(&d) != cudaSuccess) return 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, d) != cudaSuccess) return 0;
    *dev = d;
    return sms;
}

// Host-side dispatch on spheres per lane (each instantiation gets its own register
// allocation).
#define GBMP_SPL_SWITCH(spl, ...)                          \
    switch (spl) {                                         \
    case 1: { constexpr int SPL = 1; __VA_ARGS__; } break; \
    case 2: { constexpr int SPL = 2; __VA_ARGS__; } break; \
    case 3: { constexpr int SPL = 3; __VA_ARGS__; } break; \
    case 4: { constexpr int SPL = 4; __VA_ARGS__; } break; \
    case 5: { constexpr int SPL = 5; __VA_ARGS__; } break; \
    case 6: { constexpr int SPL = 6; __VA_ARGS__; } break; \
    case 7: { constexpr int SPL = 7; __VA_ARGS__; } break; \
    default: { constexpr int SPL = 8; __VA_ARGS__; } break; \
    }

}  // namespace gbmp

using namespace gbmp;

// ---------------------------------------------------------------------------------
// C-ABI.
// ---------------------------------------------------------------------------------
extern "C" {

const char *gbmp_last_error(void) { return g_err.c_str(); }

const char *gbmp_status_string(gbmp_status s) {
    switch (s) {
    case GBMP_OK: return "ok";
    case GBMP_ERR_INVALID_ARGUMENT: return "invalid argument";
    case GBMP_ERR_OUT_OF_MEMORY: return "out of device memory";
    case GBMP_ERR_CUDA: return "CUDA error";
    case GBMP_ERR_CODEGEN: return "code generation failed";
    case GBMP_ERR_CAPACITY: return "capacity exceeded";
    case GBMP_ERR_TIMEOUT: return "timed out";
    case GBMP_ERR_NOT_SOLVED: return "not solved";
    case GBMP_ERR_UNSUPPORTED: return "unsupported";
    default: return "unknown status";
    }
}

gbmp_status gbmp_get_limits(gbmp_limits *out) {
    GBMP_CHECK_ARG(out, "out is NULL");
    out->max_links = kMaxLinks;
    out->max_spheres = kMaxSpheres;
    out->max_self_pairs = kMaxSelfPairs;
    out->max_env_words = kMaxEnvWords;
    return GBMP_OK;
}

gbmp_status gbmp_device_count(int32_t *count) {
    GBMP_CHECK_ARG(count, "count is NULL");
    int c = 0;
    cudaError_t e = cudaGetDeviceCount(&c);
    if (e != cudaSuccess) {
        cudaGetLastError();
        c = 0;
    }
    *count = c;
    return GBMP_OK;
}

}  // extern "C"

namespace gbmp {
constexpr int kGroupPiece = 8;   // smallest piece of a link's spheres in the chunk kernels' groups
}  // namespace gbmp

// The robot's device tables, packed and uploaded as one block (*block) with the sphere
// groups of `piece` (see below), and their device view D.
static gbmp_status pack_tables(gbmp_robot_s *r, int piece, void **block, DevRobot &D) {
    const int L = r->L, S = r->S;
    std::vector<unsigned char> blob;
    auto put = [&](const void *src, size_t bytes) {
        size_t off = align16(blob.size());
        blob.resize(off + align16(bytes), 0);
        if (bytes) memcpy(blob.data() + off, src, bytes);
        return off;
    };
    std::vector<float> jl(12 * L), axn(4 * L), axr(4 * L), sph(4 * (S ? S : 1));
    for (int i = 0; i < L; ++i) {
        for (int k = 0; k < 12; ++k) jl[12 * i + k] = r->pose16[16 * i + k];
        host_unit_axis(&r->axis[3 * i], &axn[4 * i]);
        axr[4 * i] = r->axis[3 * i]; axr[4 * i + 1] = r->axis[3 * i + 1]; axr[4 * i + 2] = r->axis[3 * i + 2];
        axr[4 * i + 3] = 0.f;
    }
    for (int k = 0; k < S; ++k) {
        sph[4 * k] = r->sph_pos[3 * k]; sph[4 * k + 1] = r->sph_pos[3 * k + 1];
        sph[4 * k + 2] = r->sph_pos[3 * k + 2]; sph[4 * k + 3] = r->sph_r[k];
    }
    r->h_jl = jl;
    r->h_axn = axn;
    r->h_axr = axr;
    // Sphere groups (gbmp_groups.h) and their bounding spheres.  Pieces of links stay
    // within min(kMaxGroups, 3 L) groups: the chunk kernels keep K x G group centres where
    // the chunk's K x L pose rows were.
    std::vector<int> glink, sgrp;
    split_sphere_groups(L, S, r->slink.data(), r->sph_pos.data(), piece, piece > 0 ? std::min(kMaxGroups, 3 * L) : 0,
                        glink, sgrp);
    const int G = (int)glink.size();
    std::vector<float> grp(4 * (G ? G : 1), 0.f);
    for (int g = 0; g < G; ++g) {
        double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
        for (int k = 0; k < S; ++k)
            if (sgrp[k] == g)
                for (int a = 0; a < 3; ++a) {
                    lo[a] = std::min(lo[a], (double)r->sph_pos[3 * k + a] - r->sph_r[k]);
                    hi[a] = std::max(hi[a], (double)r->sph_pos[3 * k + a] + r->sph_r[k]);
                }
        double c[3] = {0.5 * (lo[0] + hi[0]), 0.5 * (lo[1] + hi[1]), 0.5 * (lo[2] + hi[2])}, rad = 0.0;
        for (int k = 0; k < S; ++k)
            if (sgrp[k] == g) {
                double d2 = 0.0;
                for (int a = 0; a < 3; ++a) d2 += (r->sph_pos[3 * k + a] - c[a]) * (r->sph_pos[3 * k + a] - c[a]);
                rad = std::max(rad, std::sqrt(d2) + r->sph_r[k]);
            }
        for (int a = 0; a < 3; ++a) grp[4 * g + a] = (float)c[a];
        grp[4 * g + 3] = nextafterf((float)(rad + kBroadMargin), 1e30f);
    }
    // Device pair list sorted by group pair; each enabled group pair owns a range.
    std::vector<int> order(r->P);
    for (int p = 0; p < r->P; ++p) order[p] = p;
    auto key = [&](int p) {
        const int a = sgrp[r->pairs[2 * p]], b = sgrp[r->pairs[2 * p + 1]];
        return std::make_pair(std::min(a, b), std::max(a, b));
    };
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return key(x) < key(y); });
    std::vector<unsigned> packed(r->P);
    std::vector<float> thr_sorted(r->P);
    std::vector<int> lpair;
    for (int q = 0; q < r->P; ++q) {
        const int p = order[q];
        packed[q] = (unsigned)r->pairs[2 * p] | ((unsigned)r->pairs[2 * p + 1] << 16);
        thr_sorted[q] = r->thr[p];
        if (q == 0 || key(p) != key(order[q - 1])) {
            lpair.insert(lpair.end(), {key(p).first, key(p).second, q, q});
        }
        lpair.back() = q + 1;
    }
    const int NPL = (int)lpair.size() / 4;
    std::vector<int> gso(G + 1, 0), gsl(S ? S : 1, 0);   // spheres of each group, index order
    for (int k = 0; k < S; ++k) gso[sgrp[k] + 1]++;
    for (int g = 0; g < G; ++g) gso[g + 1] += gso[g];
    {
        std::vector<int> fill(gso.begin(), gso.end() - 1);
        for (int k = 0; k < S; ++k) gsl[fill[sgrp[k]]++] = k;
    }
    // The tables the kernels stage in shared memory come first, segment for segment in
    // the order and 16-byte alignment of carve_tables, so that one bulk copy of
    // smem_tables_bytes(R, 0) bytes stages them; the tables read from global memory follow.
    size_t o_jl = put(jl.data(), jl.size() * 4), o_axn = put(axn.data(), axn.size() * 4);
    size_t o_axr = put(axr.data(), axr.size() * 4), o_sph = put(sph.data(), 4 * 4 * (size_t)S);
    size_t o_type = put(r->type.data(), 4 * L), o_par = put(r->parent.data(), 4 * L);
    size_t o_sl = put(r->slink.data(), 4 * (size_t)S);
    size_t o_grp = put(grp.data(), 4 * 4 * (size_t)G), o_glink = put(glink.data(), 4 * (size_t)G);
    size_t o_sgrp = put(sgrp.data(), 4 * (size_t)S), o_lpair = put(lpair.data(), 4 * lpair.size());
    size_t o_gso = put(gso.data(), 4 * (size_t)(G + 1)), o_gsl = put(gsl.data(), 4 * (size_t)S);
    const size_t staged_bytes = align16(blob.size());
    size_t o_pairs = put(packed.data(), 4 * (size_t)r->P), o_thr = put(thr_sorted.data(), 4 * (size_t)r->P);
    size_t o_lo = put(r->lower.data(), 4 * L), o_up = put(r->upper.data(), 4 * L);
    size_t o_def = put(r->defv.data(), 4 * L), o_act = put(r->active.data(), L);
    const unsigned zero = 0;
    size_t o_fault = put(&zero, sizeof zero);

    cudaError_t e = cudaMalloc(block, blob.size());
    if (e == cudaSuccess) e = cudaMemcpy(*block, blob.data(), blob.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        set_error("uploading robot tables failed: %s", cudaGetErrorString(e));
        return e == cudaErrorMemoryAllocation ? GBMP_ERR_OUT_OF_MEMORY : GBMP_ERR_CUDA;
    }
    auto *b = static_cast<unsigned char *>(*block);
    D = DevRobot{};
    D.L = L; D.S = S; D.P = r->P; D.spl = S ? (S + kWarp - 1) / kWarp : 1;
    D.jl = (const float *)(b + o_jl); D.axn = (const float *)(b + o_axn); D.axr = (const float *)(b + o_axr);
    D.sph = (const float *)(b + o_sph); D.type = (const int *)(b + o_type); D.parent = (const int *)(b + o_par);
    D.slink = (const int *)(b + o_sl); D.pairs = (const unsigned *)(b + o_pairs); D.thr = (const float *)(b + o_thr);
    D.lower = (const float *)(b + o_lo); D.upper = (const float *)(b + o_up); D.defv = (const float *)(b + o_def);
    D.active = (const unsigned char *)(b + o_act);
    D.G = G; D.NPL = NPL; D.cull = (G <= kMaxGroups) ? 1 : 0;
    D.work = nullptr;
    {
        long long fk = 0;
        for (int i = 1; i < L; ++i) fk += r->type[i] == 1 ? 151 : (r->type[i] == 2 ? 129 : (r->type[i] == 5 ? 63 : 0));
        D.base_flops = fk + 24LL * S + 24LL * G;   // FK, sphere + group transforms (18) and A terms (6)
    }
    D.grp = (const float *)(b + o_grp); D.glink = (const int *)(b + o_glink);
    D.sgrp = (const int *)(b + o_sgrp); D.lpair = (const int4 *)(b + o_lpair);
    D.gso = (const int *)(b + o_gso); D.gsl = (const int *)(b + o_gsl);
    D.stage = b;
    D.stage_bytes = (unsigned)staged_bytes;
    D.fault = (unsigned *)(b + o_fault);
    D.stage_polls = kStageWaitPolls;
    if (staged_bytes != smem_tables_bytes(D, 0)) {   // the layouts must agree byte for byte
        set_error("internal: staged table block of %zu bytes, shared-memory layout of %zu", staged_bytes,
                  smem_tables_bytes(D, 0));
        return GBMP_ERR_CUDA;
    }
    return GBMP_OK;
}

extern "C" {

gbmp_status gbmp_robot_create(const gbmp_robot_desc *d, int32_t flags, gbmp_robot *out) {
    GBMP_CHECK_ARG(d && out, "desc/out is NULL");
    *out = nullptr;
    const int L = d->num_links, S = d->num_spheres;
    GBMP_CHECK_ARG(L >= 1 && L <= kMaxLinks, "num_links %d outside [1, %d]", L, kMaxLinks);
    GBMP_CHECK_ARG(S >= 0 && S <= kMaxSpheres, "num_spheres %d outside [0, %d]", S, kMaxSpheres);
    GBMP_CHECK_ARG(d->joint_types && d->joint_poses && d->joint_axes && d->parent, "kinematic table is NULL");
    GBMP_CHECK_ARG(d->active_joints && d->lower && d->upper && d->default_values, "joint table is NULL");
    GBMP_CHECK_ARG(S == 0 || (d->sphere_link && d->sphere_pos && d->sphere_radius), "sphere table is NULL");
    GBMP_CHECK_ARG(d->resolution > 0.f && std::isfinite(d->resolution), "resolution must be > 0");
    // SingleArmSpace.cu:63-69: every parent index must be smaller than its link index.
    for (int i = 0; i < L; ++i) {
        GBMP_CHECK_ARG(d->parent[i] < i, "Link parent link map is not valid at index %d. Value: %d", i, d->parent[i]);
        GBMP_CHECK_ARG(i == 0 || d->parent[i] >= 0, "link %d has no parent", i);
    }
    for (int k = 0; k < S; ++k)
        GBMP_CHECK_ARG(d->sphere_link[k] >= 0 && d->sphere_link[k] < L, "sphere %d attached to link %d", k,
                       d->sphere_link[k]);

    auto *r = new gbmp_robot_s();
    r->L = L;
    r->S = S;
    r->resolution = d->resolution;
    r->type.assign(d->joint_types, d->joint_types + L);
    r->parent.assign(d->parent, d->parent + L);
    r->pose16.assign(d->joint_poses, d->joint_poses + 16 * L);
    r->axis.assign(d->joint_axes, d->joint_axes + 3 * L);
    r->active.assign(d->active_joints, d->active_joints + L);
    r->lower.assign(d->lower, d->lower + L);
    r->upper.assign(d->upper, d->upper + L);
    r->defv.assign(d->default_values, d->default_values + L);
    if (S) {
        r->slink.assign(d->sphere_link, d->sphere_link + S);
        r->sph_pos.assign(d->sphere_pos, d->sphere_pos + 3 * S);
        r->sph_r.assign(d->sphere_radius, d->sphere_radius + S);
    }
    if (d->self_enables) r->enables.assign(d->self_enables, d->self_enables + L * L);
    r->dim = 0;
    for (int i = 0; i < L; ++i) r->dim += r->active[i] != 0;
    // Self-collision pair list, SelfCollisionConstraint.cu:28-38.
    for (int i = 0; i < S; ++i)
        for (int j = i + 1; j < S; ++j) {
            const int li = r->slink[i], lj = r->slink[j];
            if (li == lj) continue;
            if (!r->enables.empty() && !r->enables[li * L + lj]) continue;
            r->pairs.push_back(i);
            r->pairs.push_back(j);
            const float s = r->sph_r[i] + r->sph_r[j];
            r->thr.push_back(s * s);
        }
    r->P = (int)r->thr.size();
    if (r->P > kMaxSelfPairs) {
        delete r;
        set_error("%d self-collision pairs exceed the limit %d", (int)r->thr.size(), kMaxSelfPairs);
        return GBMP_ERR_CAPACITY;
    }

    int dev = 0;
    r->num_sms = current_device_sms(&dev);
    r->device = dev;
    if (r->num_sms <= 0) {
        delete r;
        set_error("no CUDA device available");
        return GBMP_ERR_CUDA;
    }
    // Two views of the tables: sphere groups by link for the per-state kernels, and links
    // cut into pieces of kGroupPiece or more spheres for the chunk kernels, whose broad
    // phase and self-pair tests run once per chunk and gain from tighter groups (the
    // per-state kernels test every obstacle against every group and lose).  Both views
    // share one device-status word.
    gbmp_status pst = pack_tables(r, 0, &r->d_block, r->dev);
    if (!pst) pst = pack_tables(r, kGroupPiece, &r->d_block_chunk, r->dev_chunk);
    if (pst) {
        gbmp_robot_destroy(r);
        return pst;
    }
    r->dev_chunk.fault = r->dev.fault;
    if (flags & GBMP_ROBOT_CODEGEN) {
        gbmp_status st = codegen_build(r);
        if (st) {
            const std::string why = g_err;
            gbmp_robot_destroy(r);
            g_err = why;
            return st;
        }
        r->use_cg = true;
    }
    *out = r;
    return GBMP_OK;
}

gbmp_status gbmp_robot_destroy(gbmp_robot r) {
    if (!r) return GBMP_OK;
    if (r->d_block) cudaFree(r->d_block);
    if (r->d_block_chunk) cudaFree(r->d_block_chunk);
    codegen_free(r->cg);
    delete r;
    return GBMP_OK;
}

gbmp_status gbmp_robot_info(gbmp_robot r, int32_t *L, int32_t *S, int32_t *P, int32_t *dim, int32_t *cg) {
    GBMP_CHECK_ARG(r, "robot is NULL");
    if (L) *L = r->L;
    if (S) *S = r->S;
    if (P) *P = r->P;
    if (dim) *dim = r->dim;
    if (cg) *cg = r->use_cg ? 1 : 0;
    return GBMP_OK;
}

gbmp_status gbmp_robot_self_pairs(gbmp_robot r, int32_t *h_pairs, float *h_thr, int32_t cap) {
    GBMP_CHECK_ARG(r, "robot is NULL");
    GBMP_CHECK_ARG(cap >= r->P, "capacity %d < %d pairs", cap, r->P);
    if (h_pairs) memcpy(h_pairs, r->pairs.data(), sizeof(int32_t) * 2 * r->P);
    if (h_thr) memcpy(h_thr, r->thr.data(), sizeof(float) * r->P);
    return GBMP_OK;
}

gbmp_status gbmp_robot_joints(gbmp_robot r, uint8_t *h_active, float *h_default, float *h_lower, float *h_upper) {
    GBMP_CHECK_ARG(r, "robot is NULL");
    const size_t L = (size_t)r->L;
    if (h_active) memcpy(h_active, r->active.data(), L);
    if (h_default) memcpy(h_default, r->defv.data(), sizeof(float) * L);
    if (h_lower) memcpy(h_lower, r->lower.data(), sizeof(float) * L);
    if (h_upper) memcpy(h_upper, r->upper.data(), sizeof(float) * L);
    return GBMP_OK;
}

gbmp_status gbmp_robot_device_status(gbmp_robot r, int32_t *status) {
    GBMP_CHECK_ARG(r && status, "robot/status is NULL");
    unsigned f = 0;
    GBMP_CUDA(cudaMemcpy(&f, r->dev.fault, sizeof f, cudaMemcpyDeviceToHost));
    *status = f ? GBMP_ERR_TIMEOUT : GBMP_OK;
    return GBMP_OK;
}

gbmp_status gbmp_robot_use_codegen(gbmp_robot r, int32_t enable) {
    GBMP_CHECK_ARG(r, "robot is NULL");
    if (enable && !r->cg) {
        set_error("robot was created without GBMP_ROBOT_CODEGEN");
        return GBMP_ERR_UNSUPPORTED;
    }
    r->use_cg = enable != 0;
    return GBMP_OK;
}

// Obstacle order of a scene: a k-d split of the bounding-sphere centres (longest axis,
// left part a multiple of 32 points) so that every run of 32 consecutive obstacles of a
// type is spatially compact.  Ties break on the input index, so the order is the same
// on every host.
static void cluster_order(const std::vector<double> &c, std::vector<int> &idx, int lo, int hi) {
    if (hi - lo <= 32) return;
    double mn[3] = {1e300, 1e300, 1e300}, mx[3] = {-1e300, -1e300, -1e300};
    for (int k = lo; k < hi; ++k)
        for (int a = 0; a < 3; ++a) {
            mn[a] = std::min(mn[a], c[3 * idx[k] + a]);
            mx[a] = std::max(mx[a], c[3 * idx[k] + a]);
        }
    int ax = 0;
    for (int a = 1; a < 3; ++a)
        if (mx[a] - mn[a] > mx[ax] - mn[ax]) ax = a;
    const int mid = lo + ((hi - lo + 63) / 64) * 32;
    std::nth_element(idx.begin() + lo, idx.begin() + mid, idx.begin() + hi, [&](int a, int b) {
        const double va = c[3 * a + ax], vb = c[3 * b + ax];
        return va < vb || (va == vb && a < b);
    });
    cluster_order(c, idx, lo, mid);
    cluster_order(c, idx, mid, hi);
}

// Bounding sphere of each run of 32 obstacles (bounding-sphere centres c and radii r
// of the obstacles, idx in run order), rounded outwards.
static void cluster_spheres(const std::vector<double> &c, const std::vector<double> &r, const std::vector<int> &idx,
                            float4 *out) {
    const int n = (int)idx.size();
    for (int b = 0; b * 32 < n; ++b) {
        const int lo = 32 * b, hi = std::min(n, lo + 32);
        double mn[3] = {1e300, 1e300, 1e300}, mx[3] = {-1e300, -1e300, -1e300};
        for (int k = lo; k < hi; ++k)
            for (int a = 0; a < 3; ++a) {
                mn[a] = std::min(mn[a], c[3 * idx[k] + a]);
                mx[a] = std::max(mx[a], c[3 * idx[k] + a]);
            }
        const double cx = 0.5 * (mn[0] + mx[0]), cy = 0.5 * (mn[1] + mx[1]), cz = 0.5 * (mn[2] + mx[2]);
        double rad = 0.0;
        for (int k = lo; k < hi; ++k) {
            const int i = idx[k];
            const double dx = c[3 * i] - cx, dy = c[3 * i + 1] - cy, dz = c[3 * i + 2] - cz;
            rad = std::max(rad, std::sqrt(dx * dx + dy * dy + dz * dz) + r[i]);
        }
        out[b] = make_float4((float)cx, (float)cy, (float)cz, (float)(rad * (1.0 + 1e-6) + 1e-5));
    }
}

gbmp_status gbmp_env_create(int32_t ns, const float *sp, const float *sr, int32_t nb, const float *bp,
                            const float *brot, const float *bmin, const float *bmax, int32_t nc, const float *cp,
                            const float *crot, const float *crad, const float *chei, gbmp_env *out) {
    GBMP_CHECK_ARG(out, "out is NULL");
    *out = nullptr;
    GBMP_CHECK_ARG(ns >= 0 && nb >= 0 && nc >= 0, "negative obstacle count");
    GBMP_CHECK_ARG(ns == 0 || (sp && sr), "sphere arrays are NULL");
    GBMP_CHECK_ARG(nb == 0 || (bp && brot && bmin && bmax), "cuboid arrays are NULL");
    GBMP_CHECK_ARG(nc == 0 || (cp && crot && crad && chei), "cylinder arrays are NULL");
    const long long words = 2LL * ns + (ns + 3) / 4 + 5LL * nb + 4LL * nc + env_clusters(ns) + env_clusters(nb) +
                            env_clusters(nc);
    if (words > kMaxEnvWords) {
        set_error("environment needs %lld float4 words, limit %d", words, kMaxEnvWords);
        return GBMP_ERR_CAPACITY;
    }
    // bounding sphere of every obstacle, then the run order of each type
    std::vector<double> sc(3 * (size_t)ns), srd(ns), bc(3 * (size_t)nb), brd(nb), cc(3 * (size_t)nc), crd(nc);
    for (int i = 0; i < ns; ++i) {
        for (int a = 0; a < 3; ++a) sc[3 * i + a] = sp[3 * i + a];
        srd[i] = sr[i];
    }
    for (int i = 0; i < nb; ++i) {   // box: centre pos + R (min + max) / 2, radius half the diagonal
        const float *R = brot + 9 * i;
        double l[3], h2 = 0.0;
        for (int a = 0; a < 3; ++a) {
            l[a] = 0.5 * ((double)bmin[3 * i + a] + bmax[3 * i + a]);
            const double h = 0.5 * ((double)bmax[3 * i + a] - bmin[3 * i + a]);
            h2 += h * h;
        }
        for (int a = 0; a < 3; ++a)
            bc[3 * i + a] = bp[3 * i + a] + R[3 * a] * l[0] + R[3 * a + 1] * l[1] + R[3 * a + 2] * l[2];
        brd[i] = std::sqrt(h2);
    }
    for (int i = 0; i < nc; ++i) {   // cylinder: centre pos, radius sqrt(r^2 + (h/2)^2)
        for (int a = 0; a < 3; ++a) cc[3 * i + a] = cp[3 * i + a];
        crd[i] = std::sqrt((double)crad[i] * crad[i] + 0.25 * (double)chei[i] * chei[i]);
    }
    std::vector<int> os(ns), ob(nb), oc(nc);
    for (int i = 0; i < ns; ++i) os[i] = i;
    for (int i = 0; i < nb; ++i) ob[i] = i;
    for (int i = 0; i < nc; ++i) oc[i] = i;
    cluster_order(sc, os, 0, ns);
    cluster_order(bc, ob, 0, nb);
    cluster_order(cc, oc, 0, nc);

    auto *e = new gbmp_env_s();
    e->ns = ns; e->nb = nb; e->nc = nc;
    e->h_words.resize(words ? words : 1);
    float4 *w = e->h_words.data();
    for (int k = 0; k < ns; ++k) {
        const int i = os[k];
        w[k] = make_float4(sp[3 * i], sp[3 * i + 1], sp[3 * i + 2], sr[i]);
    }
    w += ns;
    for (int k = 0; k < nb; ++k) {
        const int i = ob[k];
        host_inverse_pose(bp + 3 * i, brot + 9 * i, w + 5 * k);
        w[5 * k + 3] = make_float4(bmin[3 * i], bmin[3 * i + 1], bmin[3 * i + 2], 0.f);
        w[5 * k + 4] = make_float4(bmax[3 * i], bmax[3 * i + 1], bmax[3 * i + 2], 0.f);
    }
    w += 5 * nb;
    for (int k = 0; k < nc; ++k) {
        const int i = oc[k];
        host_inverse_pose(cp + 3 * i, crot + 9 * i, w + 4 * k);
        w[4 * k + 3] = make_float4(crad[i], chei[i] * 0.5f, 0.f, 0.f);
    }
    w += 4 * nc;
    float *nbv = reinterpret_cast<float *>(w + ns);
    for (int k = 0; k < ns; ++k) {
        const int i = os[k];
        const double x = sp[3 * i], y = sp[3 * i + 1], z = sp[3 * i + 2], rr = sr[i];
        w[k] = make_float4(2.f * sp[3 * i], 2.f * sp[3 * i + 1], 2.f * sp[3 * i + 2], 2.f * sr[i]);
        nbv[k] = (float)(-(x * x + y * y + z * z - rr * rr));
    }
    float4 *runs = e->h_words.data() + env_cluster_base(ns, nb, nc);
    cluster_spheres(sc, srd, os, runs);
    cluster_spheres(bc, brd, ob, runs + env_clusters(ns));
    cluster_spheres(cc, crd, oc, runs + env_clusters(ns) + env_clusters(nb));
    cudaError_t err = cudaMalloc(&e->d_words, sizeof(float4) * e->h_words.size());
    if (err == cudaSuccess)
        err = cudaMemcpy(e->d_words, e->h_words.data(), sizeof(float4) * e->h_words.size(), cudaMemcpyHostToDevice);
    if (err != cudaSuccess) {
        set_error("uploading environment failed: %s", cudaGetErrorString(err));
        gbmp_env_destroy(e);
        return err == cudaErrorMemoryAllocation ? GBMP_ERR_OUT_OF_MEMORY : GBMP_ERR_CUDA;
    }
    *out = e;
    return GBMP_OK;
}

gbmp_status gbmp_env_destroy(gbmp_env e) {
    if (!e) return GBMP_OK;
    if (e->d_words) cudaFree(e->d_words);
    delete e;
    return GBMP_OK;
}

gbmp_status gbmp_env_counts(gbmp_env e, int32_t *ns, int32_t *nb, int32_t *nc) {
    GBMP_CHECK_ARG(e, "env is NULL");
    if (ns) *ns = e->ns;
    if (nb) *nb = e->nb;
    if (nc) *nc = e->nc;
    return GBMP_OK;
}

gbmp_status gbmp_fk(gbmp_robot r, const float *d_q, int64_t n, float *d_poses, float *d_centers, void *stream) {
    GBMP_CHECK_ARG(r, "robot is NULL");
    GBMP_CHECK_ARG(n >= 0, "n < 0");
    if (n == 0) return GBMP_OK;
    GBMP_CHECK_ARG(d_q, "q is NULL");
    if (r->use_cg) return codegen_fk(r, d_q, n, d_poses, d_centers, (cudaStream_t)stream);
    if (r->dev.L <= 16) {
        ProfScope ps(GBMP_PROF_FK, (cudaStream_t)stream);
        return fk_chunk_launch(r->dev, r->num_sms, d_q, n, d_poses, d_centers, (cudaStream_t)stream);
    }
    const size_t smem = smem_tables_bytes(r->dev, 0) + smem_warp_bytes(r->dev) * kWarpsPerBlock;
    int grid = 0;
    gbmp_status st = persistent_grid(k_fk, smem, r->num_sms, &grid);
    if (st) return st;
    const long long need = (n + kWarpsPerBlock - 1) / kWarpsPerBlock;
    if (need < grid) grid = (int)need;
    ProfScope ps(GBMP_PROF_FK, (cudaStream_t)stream);
    k_fk<<<grid, kWarpsPerBlock * kWarp, smem, (cudaStream_t)stream>>>(r->dev, d_q, n, d_poses, d_centers);
    GBMP_CUDA(cudaGetLastError());
    return GBMP_OK;
}

gbmp_status gbmp_check_states_fk(gbmp_robot r, gbmp_env env, const float *d_q, int64_t n, int32_t mode,
                                 uint8_t *d_verdict, float *d_costs, float *d_total, float *d_poses,
                                 float *d_centers, void *stream) {
    GBMP_CHECK_ARG(r && env, "robot/env is NULL");
    GBMP_CHECK_ARG(n >= 0, "n < 0");
    GBMP_CHECK_ARG(mode == GBMP_CHECK_VERDICT || mode == GBMP_CHECK_COST, "unknown mode %d", mode);
    if (n == 0) return GBMP_OK;
    GBMP_CHECK_ARG(d_q, "q is NULL");
    const DevEnv E = env->dev();
    DevRobot D = r->dev;
    D.work = work_counter();
    const size_t smem = block_smem(D, env_words(E.ns, E.nb, E.nc));
    const long long need = (n + kWarpsPerBlock - 1) / kWarpsPerBlock;
    gbmp_status st = GBMP_OK;
    cudaStream_t s = (cudaStream_t)stream;
    GBMP_SPL_SWITCH(r->dev.spl, {
        int grid = 0;
        if (mode == GBMP_CHECK_COST) {
            st = persistent_grid(k_check_states<true, SPL>, smem, r->num_sms, &grid);
            if (st) return st;
            if (need < grid) grid = (int)need;
            ProfScope ps(GBMP_PROF_CHECK_STATES, s);
            k_check_states<true, SPL><<<grid, kWarpsPerBlock * kWarp, smem, s>>>(D, E, d_q, n, d_verdict, d_costs,
                                                                                 d_total, d_poses, d_centers);
        } else {
            st = persistent_grid(k_check_states<false, SPL>, smem, r->num_sms, &grid);
            if (st) return st;
            if (need < grid) grid = (int)need;
            ProfScope ps(GBMP_PROF_CHECK_STATES, s);
            k_check_states<false, SPL><<<grid, kWarpsPerBlock * kWarp, smem, s>>>(D, E, d_q, n, d_verdict, nullptr,
                                                                                  nullptr, d_poses, d_centers);
        }
    });
    GBMP_CUDA(cudaGetLastError());
    return GBMP_OK;
}

gbmp_status gbmp_check_states(gbmp_robot r, gbmp_env env, const float *d_q, int64_t n, int32_t mode,
                              uint8_t *d_verdict, float *d_costs, float *d_total, void *stream) {
    return gbmp_check_states_fk(r, env, d_q, n, mode, d_verdict, d_costs, d_total, nullptr, nullptr, stream);
}

gbmp_status gbmp_robot_set_stage_wait(gbmp_robot r, int32_t polls) {
    GBMP_CHECK_ARG(r, "robot is NULL");
    GBMP_CHECK_ARG(polls >= -1, "polls %d < -1", polls);
    r->dev.stage_polls = r->dev_chunk.stage_polls = polls < 0 ? kStageWaitPolls : polls;
    return GBMP_OK;
}

gbmp_status gbmp_robot_set_edge_form(gbmp_robot r, int32_t form) {
    GBMP_CHECK_ARG(r, "robot is NULL");
    GBMP_CHECK_ARG(form == 0 || form == 1 || form == 4 || form == 10, "edge form %d is not 0, 1, 4 or 10", form);
    r->edge_form = form;
    return GBMP_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------------
// Edge validation (replaces SingleArmSpace::checkMotions, SingleArmSpace.cu:628-848).
// Both entry points run the same kernels; they differ only in where the working memory
// comes from: gbmp_check_edges grows a buffer owned by the robot handle, and
// gbmp_check_edges_noalloc uses one fixed array that the library holds on each device.
// Three launches, no host round trip:
//   k_edge_setup   step count, direction and length per edge, length histogram;
//   k_edge_order   the edges in longest-first order (counting sort by buckets);
//   validation     a warp takes the next edge of that order (shared counter), walks its
//                  states in order (chunks of consecutive states, or state by state) and
//                  stops at the first colliding state; it writes the edge's outputs.
// Working memory of E edges of L links:
//   nsteps[E], order[E]   int
//   dir[E*L]              float
//   ctr[kEdgeCtrInts]     int    MUST START AT ZERO (hist[64], cursor[64], next):
//                                zeroed on the stream by every call
// ---------------------------------------------------------------------------------
namespace gbmp {

constexpr int kEdgeCtrInts = 2 * kEdgeBuckets + 32;

struct EdgeScratch {
    int *nsteps, *order;
    float *dir;
    int *ctr;
};

// Argument checks shared by the edge entry points; on success *res is the step to use.
static gbmp_status edge_args(gbmp_robot r, gbmp_env env, long long E, float *res, int rule) {
    GBMP_CHECK_ARG(r && env, "robot/env is NULL");
    GBMP_CHECK_ARG(E >= 0 && E < INT_MAX, "edge count %lld outside [0, 2^31)", E);
    GBMP_CHECK_ARG(rule == GBMP_STEP_L2 || rule == GBMP_STEP_LINF || rule == GBMP_STEP_COUNT, "unknown step rule %d",
                   rule);
    GBMP_CHECK_ARG(rule != GBMP_STEP_COUNT || (*res >= 1.f && *res <= 1e6f), "step count %g outside [1, 1e6]", *res);
    if (rule == GBMP_STEP_COUNT) *res = floorf(*res);
    if (!(*res > 0.f)) *res = r->resolution;
    GBMP_CHECK_ARG(std::isfinite(*res), "resolution is not finite");
    return GBMP_OK;
}

static gbmp_status edge_validate(gbmp_robot r, gbmp_env env, const float *d_from, const float *d_to, long long E,
                                 float res, int rule, uint8_t *d_ok, int32_t *d_first_hit, float *d_length,
                                 int32_t *d_num_steps, cudaStream_t s, const EdgeScratch &sc) {
    int *nsteps = sc.nsteps, *order = sc.order, *ctr = sc.ctr;
    int *hist = ctr, *cursor = ctr + kEdgeBuckets, *next = ctr + 2 * kEdgeBuckets;
    float *dir = sc.dir;
    const int L = r->L;
    GBMP_CUDA(cudaMemsetAsync(ctr, 0, kEdgeCtrInts * sizeof(int), s));
    const int tb = 256;
    const unsigned blocks = (unsigned)((E + tb - 1) / tb);
    gbmp_status st = GBMP_OK;
    if (r->use_cg && rule != GBMP_STEP_COUNT) {   // the generated set-up knows the checkMotions rules
        st = codegen_edge_setup(r, d_from, d_to, E, res, rule, nsteps, dir, hist, d_length, d_num_steps, s);
        if (st) return st;
    } else {
        ProfScope ps(GBMP_PROF_OTHER, s);
        k_edge_setup<<<blocks, tb, 0, s>>>(d_from, d_to, E, L, res, rule, nsteps, dir, hist, d_length, d_num_steps);
    }
    GBMP_CUDA(cudaGetLastError());
    {
        ProfScope ps(GBMP_PROF_OTHER, s);
        k_edge_order<<<(unsigned)std::min<long long>(blocks, 4LL * r->num_sms), tb, 0, s>>>(nsteps, E, hist, cursor,
                                                                                            order);
    }
    GBMP_CUDA(cudaGetLastError());

    const DevEnv Ev = env->dev();
    DevRobot D = r->dev;
    D.work = work_counter();
    size_t smem = block_smem(D, env_words(Ev.ns, Ev.nb, Ev.nc));
    int grid = 0;
    const bool cull = r->dev.cull != 0;
    // the chunk kernel reads the tables grouped by pieces of links
    DevRobot Dc = r->dev_chunk;
    Dc.work = D.work;
    int K = edge_chunk_states(D, r->edge_form);
    if (K) {
        st = edge_chunk_prepare(Dc, Ev, r->num_sms, K, &smem, &grid);
        if (st == GBMP_ERR_CAPACITY) {   // chunk scratch does not fit next to a large scene
            K = 0;
            st = GBMP_OK;
            smem = block_smem(D, env_words(Ev.ns, Ev.nb, Ev.nc));
        }
    }
    if (!K) {
        GBMP_SPL_SWITCH(r->dev.spl, {
            st = cull ? persistent_grid(k_edge_states<SPL, true>, smem, r->num_sms, &grid)
                      : persistent_grid(k_edge_states<SPL, false>, smem, r->num_sms, &grid);
        });
    }
    if (st) return st;
    const long long need = (E + kWarpsPerBlock - 1) / kWarpsPerBlock;   // one warp per edge at most
    if (need < grid) grid = (int)need;
    {
        ProfScope ps(GBMP_PROF_EDGE_WAVE, s);
        if (K) {
            st = edge_chunk_launch(Dc, Ev, K, grid, smem, s, d_from, d_to, nsteps, dir, order, E, next, d_ok,
                                   d_first_hit);
            if (st) return st;
        } else {
            GBMP_SPL_SWITCH(r->dev.spl, {
                if (cull)
                    k_edge_states<SPL, true><<<grid, kWarpsPerBlock * kWarp, smem, s>>>(
                        D, Ev, d_from, d_to, nsteps, dir, order, E, next, d_ok, d_first_hit);
                else
                    k_edge_states<SPL, false><<<grid, kWarpsPerBlock * kWarp, smem, s>>>(
                        D, Ev, d_from, d_to, nsteps, dir, order, E, next, d_ok, d_first_hit);
            });
        }
    }
    GBMP_CUDA(cudaGetLastError());
    return GBMP_OK;
}

// ---------------------------------------------------------------------------------
// The fixed working memory of gbmp_check_edges_noalloc: one file-scope device array,
// laid out as EdgeScratch for up to kNoAllocMaxEdges edges and kNoAllocMaxDirFloats
// edges x links:
//   [0, 4 Ei)            nsteps[E]
//   [4 Ei, 8 Ei)         order[E]
//   [8 Ei, +4 D)         dir[E*L]
//   [.., +4 C)           ctr[C]     zeroed on the stream at the start of every call
// with Ei = kNoAllocMaxEdges, D = kNoAllocMaxDirFloats, C = kEdgeCtrInts.  Every call on a
// device shares the array, so calls that overlap on the device race.
// ---------------------------------------------------------------------------------
constexpr long long kNoAllocMaxEdges = 65536;
constexpr long long kNoAllocMaxDirFloats = 1LL << 20;   // n_edges * links
constexpr size_t kNoAllocEdgeInts = sizeof(int) * kNoAllocMaxEdges;
constexpr size_t kNoAllocDirOffset = 2 * kNoAllocEdgeInts;
constexpr size_t kNoAllocCtrOffset = kNoAllocDirOffset + sizeof(float) * kNoAllocMaxDirFloats;
constexpr size_t kNoAllocBytes = (kNoAllocCtrOffset + sizeof(int) * kEdgeCtrInts + 255) & ~size_t(255);
static_assert(kNoAllocDirOffset % 256 == 0 && kNoAllocCtrOffset % 256 == 0, "scratch regions stay aligned");

static __device__ __align__(256) unsigned char g_edge_scratch[kNoAllocBytes];

constexpr int kNoAllocMaxDevices = 64;

// Device address of g_edge_scratch on the current device, looked up once per device with
// that device current (the host-side name g_edge_scratch is not a device address).  The
// address belongs to the device's context: it is not valid after cudaDeviceReset.
static gbmp_status noalloc_scratch(unsigned char **out) {
    static std::mutex mu;
    static unsigned char *addr[kNoAllocMaxDevices] = {};
    int dev = 0;
    GBMP_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kNoAllocMaxDevices) {
        set_error("device %d is beyond the %d devices the allocation-free scratch is tracked for", dev,
                  kNoAllocMaxDevices);
        return GBMP_ERR_UNSUPPORTED;
    }
    std::lock_guard<std::mutex> lock(mu);
    if (!addr[dev]) {
        void *p = nullptr;
        GBMP_CUDA(cudaGetSymbolAddress(&p, g_edge_scratch));
        if (!p) {
            set_error("cudaGetSymbolAddress gave no address for the edge scratch on device %d", dev);
            return GBMP_ERR_CUDA;
        }
        addr[dev] = static_cast<unsigned char *>(p);
    }
    *out = addr[dev];
    return GBMP_OK;
}

}  // namespace gbmp

extern "C" {

gbmp_status gbmp_check_edges(gbmp_robot r, gbmp_env env, const float *d_from, const float *d_to, int64_t E,
                             float res, int32_t rule, uint8_t *d_ok, int32_t *d_first_hit, float *d_length,
                             int32_t *d_num_steps, void *stream) {
    gbmp_status st = edge_args(r, env, E, &res, rule);
    if (st) return st;
    if (E == 0) return GBMP_OK;
    GBMP_CHECK_ARG(d_from && d_to, "from/to is NULL");
    cudaStream_t s = (cudaStream_t)stream;
    // the working memory is the handle's: calls with the same robot are ordered on the host
    // (the lock is held while the launches are queued, not while they run; calls on
    // different streams with the same robot must be ordered by the caller)
    std::lock_guard<std::mutex> lock(r->scratch_mu);
    const size_t eb = align16(sizeof(int) * (size_t)E);
    const size_t db = align16(sizeof(float) * (size_t)E * r->L);
    st = r->scratch.reserve(2 * eb + db + kEdgeCtrInts * sizeof(int));
    if (st) return st;
    auto *base = static_cast<unsigned char *>(r->scratch.ptr);
    EdgeScratch sc{(int *)base, (int *)(base + eb), (float *)(base + 2 * eb), (int *)(base + 2 * eb + db)};
    return edge_validate(r, env, d_from, d_to, E, res, rule, d_ok, d_first_hit, d_length, d_num_steps, s, sc);
}

gbmp_status gbmp_check_edges_noalloc(gbmp_robot r, gbmp_env env, const float *d_from, const float *d_to,
                                     int64_t E, float res, int32_t rule, uint8_t *d_ok, int32_t *d_first_hit,
                                     float *d_length, int32_t *d_num_steps, void *stream) {
    gbmp_status st = edge_args(r, env, E, &res, rule);
    if (st) return st;
    if (E > kNoAllocMaxEdges || E * (long long)r->L > kNoAllocMaxDirFloats) {
        set_error("%lld edges x %d links exceed the allocation-free scratch (at most %lld edges and %lld "
                  "edges x links); use gbmp_check_edges or split the call",
                  (long long)E, r->L, kNoAllocMaxEdges, kNoAllocMaxDirFloats);
        return GBMP_ERR_CAPACITY;
    }
    unsigned char *base = nullptr;
    st = noalloc_scratch(&base);   // also the per-device set-up when E == 0
    if (st) return st;
    if (E == 0) return GBMP_OK;
    GBMP_CHECK_ARG(d_from && d_to, "from/to is NULL");
    EdgeScratch sc{(int *)base, (int *)(base + kNoAllocEdgeInts), (float *)(base + kNoAllocDirOffset),
                   (int *)(base + kNoAllocCtrOffset)};
    return edge_validate(r, env, d_from, d_to, E, res, rule, d_ok, d_first_hit, d_length, d_num_steps,
                         (cudaStream_t)stream, sc);
}

}  // extern "C"
