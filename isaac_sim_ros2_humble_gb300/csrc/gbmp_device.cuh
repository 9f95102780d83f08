// gbmp_device.cuh -- device-side data layout and the warp-per-state FK + collision
// routine shared by every kernel of libgbmp.
//
// Execution model: one warp validates one joint state.
//   * FK: lanes 0..11 each own one element of the 3x4 pose of the current link and
//     walk the chain link by link (KernelGenerator.h:369-400); the poses stay in the
//     warp's shared-memory scratch, never in HBM unless the caller asks for them.
//   * Collision: lane l owns robot spheres l, l+32, ... (registers); obstacles are
//     staged once per block in shared memory and read as broadcasts; self pairs are
//     strided over the lanes.  Any-hit early exit uses __any_sync.
// Arithmetic that decides parity with the CPU oracle (matrix products, sphere
// centres, interpolation) is written with explicit __fmul_rn/__fmaf_rn/__fadd_rn so
// that FMA contraction cannot change it.
#pragma once

#include <cstdint>

namespace gbmp {

constexpr int kMaxLinks = 64;
constexpr int kMaxSpheres = 256;          // 8 spheres per lane
constexpr int kWarp = 32;
constexpr unsigned kFull = 0xffffffffu;
constexpr float kFar = 1.0e15f;           // parking spot for unused sphere slots

// ---------------------------------------------------------------------------------
// Device tables (global memory).  Robot block layout, all 16-byte aligned:
//   jl    [L*12]  joint origin pose, 3x4 row-major (rows 0..2 of the 4x4)
//   axn   [L*4]   normalised axis (nx, ny, nz, valid)  (KernelGenerator.h:295-304)
//   axr   [L*4]   raw axis (prismatic translation uses it unnormalised, :349-354)
//   sph   [S*4]   sphere (x, y, z, r) in its link frame
//   type  [L], parent [L], slink [S] (int32)
//   pairs [P] packed (i | j << 16), thr [P] squared distance thresholds, sorted by
//         link pair so that each enabled link pair owns a contiguous range
//   grp   [G*4]  per sphere-carrying link ("group"): bounding sphere (x, y, z, R) in the
//         link frame enclosing all its spheres, inflated by kBroadMargin
//   glink [G], sgrp [S] (group of each sphere), lpair [NPL*4] (ga, gb, p0, p1)
//   gso [G+1], gsl [S]: the spheres of group g are gsl[gso[g] .. gso[g+1]) in index order
// Environment words (float4):
//   spheres  [ns]     (x, y, z, r)
//   cuboids  [nb*5]   inverse pose rows 0..2, (min xyz, 0), (max xyz, 0)
//   cylinders[nc*4]   inverse pose rows 0..2, (radius, half height, 0, 0)
//   spheres  [ns]     expanded form (2x, 2y, 2z, 2r)
//   spheres  [ceil(ns/4)] -(|o|^2 - r^2), four per word
//   runs     [ceil(ns/32) + ceil(nb/32) + ceil(nc/32)]  (x, y, z, R): obstacles of each
//            type are stored in spatially compact runs of 32; word c of a type bounds
//            every obstacle of its run c (obstacles 32c .. 32c + 31)
// ---------------------------------------------------------------------------------
struct DevRobot {
    int L, S, P, spl;                 // spl = spheres per lane = ceil(S/32)
    int G, NPL;                       // sphere groups, enabled group pairs
    int cull;                         // 1: groups fit a 32-bit mask, broad phase available
    const float *jl, *axn, *axr, *sph;
    const int *type, *parent, *slink;
    const unsigned *pairs;
    const float *thr;
    const float *lower, *upper, *defv;
    const unsigned char *active;
    const float *grp;
    const int *glink, *sgrp;
    const int4 *lpair;
    const int *gso, *gsl;
    // Executed-work accounting (only when `work` is non-null): work[0] += flops executed,
    // work[1] += states evaluated.  base_flops = per-state FK + sphere + group transforms.
    unsigned long long *work;
    long long base_flops;
    // The staged tables (jl .. gsl above) as one block laid out exactly as carve_tables
    // lays them out in shared memory: `stage_bytes` bytes at `stage` (16-byte aligned), so
    // that one bulk copy stages them.  `fault`: device word a kernel sets (bit 0) when a
    // bounded device-side wait gave up.  `stage_polls`: polls of the staging wait before it
    // gives up (kStageWaitPolls; a test sets 0 to see the give-up path report).
    const void *stage;
    unsigned stage_bytes;
    unsigned *fault;
    int stage_polls;
};

// Flop weights of the executed tests (multiply/add/compare = 1, FMA = 2).
constexpr int kFlSphereX = 9;     // expanded sphere-sphere test: 4 FMA + compare
constexpr int kFlCuboid = 33;     // 3x4 transform + clamp + squared distance + compare
constexpr int kFlCylinder = 34;   // 3x4 transform + finite-cylinder distance + compare
constexpr int kFlSelf = 9;        // 3 sub, 1 mul + 2 FMA, compare
constexpr int kFlGroupPair = 11;  // group-sphere overlap test

// Edge validation: edges of more than kMaxEdgeStates interpolated states are not
// validated (reported with first hit -2); edges are processed longest first by buckets of
// 16 states (bucket 0 the longest).
constexpr int kMaxEdgeStates = 1 << 22;
constexpr int kEdgeBuckets = 64;
__host__ __device__ inline int edge_bucket(int n) {
    const int b = n >> 4;
    return kEdgeBuckets - 1 - (b < kEdgeBuckets - 1 ? b : kEdgeBuckets - 1);
}

constexpr int kMaxGroups = 32;
constexpr float kBroadMargin = 1e-3f;    // metres added to every group bounding radius

struct DevEnv {
    int ns, nb, nc;
    const float4 *words;              // env_words(ns, nb, nc) float4
};

__host__ __device__ inline int env_clusters(int n) { return (n + 31) / 32; }
__host__ __device__ inline int env_cluster_base(int ns, int nb, int nc) { return 2 * ns + (ns + 3) / 4 + 5 * nb + 4 * nc; }
__host__ __device__ inline int env_words(int ns, int nb, int nc) {
    return env_cluster_base(ns, nb, nc) + env_clusters(ns) + env_clusters(nb) + env_clusters(nc);
}

// Shared-memory staging of the robot tables and the environment.
struct SmemTables {
    float *jl, *axn, *axr;
    float4 *sph;
    int *type, *parent, *slink;
    float4 *grp;
    int *glink, *sgrp;
    int4 *lpair;
    int *gso, *gsl;
    float4 *env;                      // staged environment words
};

__host__ __device__ inline size_t align16(size_t x) { return (x + 15) & ~size_t(15); }

__host__ __device__ inline size_t smem_tables_bytes(const DevRobot &R, int nwords) {
    size_t b = 0;
    b += align16(sizeof(float) * 12 * R.L);
    b += align16(sizeof(float) * 4 * R.L) * 2;
    b += align16(sizeof(float4) * R.S);
    b += align16(sizeof(int) * R.L) * 2;
    b += align16(sizeof(int) * R.S);
    b += align16(sizeof(float4) * R.G);
    b += align16(sizeof(int) * R.G);
    b += align16(sizeof(int) * R.S);
    b += align16(sizeof(int4) * R.NPL);
    b += align16(sizeof(int) * (R.G + 1));
    b += align16(sizeof(int) * R.S);
    b += align16(sizeof(float4) * nwords);
    return b;
}

// Per-warp scratch: link poses [L*12], joint-local transforms [L*12], joint state [L], sphere centres [S],
// group bounding spheres in the base frame [G] + their A terms [G], candidate list [32].
__host__ __device__ inline size_t smem_warp_bytes(const DevRobot &R) {
    return align16(sizeof(float) * 12 * R.L) * 2 + align16(sizeof(float) * R.L) +
           align16(sizeof(float4) * R.S) + align16(sizeof(float4) * R.G) + align16(sizeof(float) * R.G) +
           align16(sizeof(int) * kWarp) * 2;
}

struct WarpScratch {
    float *lp;      // link poses
    float *loc;     // joint-local transforms [L*12]
    float *q;       // joint values of the state under test
    float4 *cen;    // sphere centres (x, y, z, r)
    float4 *gb;     // group bounding spheres in the base frame (x, y, z, R)
    float *gA;      // |c|^2 - R^2 of each group sphere
    int *cand;      // candidate obstacle indices of the current chunk
    unsigned *cmask;// their group masks
};

__device__ inline SmemTables carve_tables(unsigned char *base, const DevRobot &R, int nwords) {
    SmemTables t;
    size_t off = 0;
    t.jl = reinterpret_cast<float *>(base + off); off += align16(sizeof(float) * 12 * R.L);
    t.axn = reinterpret_cast<float *>(base + off); off += align16(sizeof(float) * 4 * R.L);
    t.axr = reinterpret_cast<float *>(base + off); off += align16(sizeof(float) * 4 * R.L);
    t.sph = reinterpret_cast<float4 *>(base + off); off += align16(sizeof(float4) * R.S);
    t.type = reinterpret_cast<int *>(base + off); off += align16(sizeof(int) * R.L);
    t.parent = reinterpret_cast<int *>(base + off); off += align16(sizeof(int) * R.L);
    t.slink = reinterpret_cast<int *>(base + off); off += align16(sizeof(int) * R.S);
    t.grp = reinterpret_cast<float4 *>(base + off); off += align16(sizeof(float4) * R.G);
    t.glink = reinterpret_cast<int *>(base + off); off += align16(sizeof(int) * R.G);
    t.sgrp = reinterpret_cast<int *>(base + off); off += align16(sizeof(int) * R.S);
    t.lpair = reinterpret_cast<int4 *>(base + off); off += align16(sizeof(int4) * R.NPL);
    t.gso = reinterpret_cast<int *>(base + off); off += align16(sizeof(int) * (R.G + 1));
    t.gsl = reinterpret_cast<int *>(base + off); off += align16(sizeof(int) * R.S);
    t.env = reinterpret_cast<float4 *>(base + off);
    return t;
}

__device__ inline WarpScratch carve_warp(unsigned char *base, const DevRobot &R, int warp) {
    size_t per = smem_warp_bytes(R);
    unsigned char *p = base + per * warp;
    WarpScratch w;
    size_t off = 0;
    w.lp = reinterpret_cast<float *>(p + off); off += align16(sizeof(float) * 12 * R.L);
    w.loc = reinterpret_cast<float *>(p + off); off += align16(sizeof(float) * 12 * R.L);
    w.q = reinterpret_cast<float *>(p + off); off += align16(sizeof(float) * R.L);
    w.cen = reinterpret_cast<float4 *>(p + off); off += align16(sizeof(float4) * R.S);
    w.gb = reinterpret_cast<float4 *>(p + off); off += align16(sizeof(float4) * R.G);
    w.gA = reinterpret_cast<float *>(p + off); off += align16(sizeof(float) * R.G);
    w.cand = reinterpret_cast<int *>(p + off); off += align16(sizeof(int) * kWarp);
    w.cmask = reinterpret_cast<unsigned *>(p + off);
    return w;
}

__device__ __forceinline__ unsigned smem_u32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

// Polls of a staging wait before it gives up (each poll sleeps ~0.1 us after the first
// few): far beyond the microseconds a copy of at most 227 KB takes.
constexpr int kStageWaitPolls = 1 << 24;

// Stages the robot tables and the environment into shared memory with two bulk
// asynchronous copies (TMA, cp.async.bulk: the robot's staged block and the environment
// words, both 16-byte aligned with sizes that are multiples of 16) completing on one
// mbarrier.  All threads of the block call it; it begins and ends with a block barrier,
// so a block may stage again later (the batched planner does, per problem).  Every
// thread waits on the mbarrier (bounded); if the copies have not completed within the
// limit the robot's fault word is set and false is returned on every thread, and the
// caller must not use the tables.
__device__ inline bool stage_tables(const DevRobot &R, const DevEnv &E, const SmemTables &t, int nwords) {
    __shared__ __align__(8) unsigned long long s_mbar;
    __shared__ int s_fail;
    const unsigned bar = smem_u32(&s_mbar);
    const unsigned bytes_r = R.stage_bytes, bytes_e = 16u * (unsigned)nwords;
    __syncthreads();   // no thread still reads tables this block staged before
    if (threadIdx.x == 0) {
        s_fail = 0;
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        // order earlier generic-proxy accesses of this shared memory before the copies
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes_r + bytes_e)
                     : "memory");
        asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                         smem_u32(t.jl)),
                     "l"(R.stage), "r"(bytes_r), "r"(bar)
                     : "memory");
        if (bytes_e)
            asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                             smem_u32(t.env)),
                         "l"(E.words), "r"(bytes_e), "r"(bar)
                         : "memory");
    }
    __syncthreads();   // the mbarrier is initialised before anyone polls it
    auto poll = [&](int limit) {
        unsigned done = 0;
        for (int it = 0; it < limit; ++it) {
            asm volatile(
                "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n\tselp.u32 %0, 1, 0, p;\n\t}"
                : "=r"(done)
                : "r"(bar)
                : "memory");
            if (done) break;
            if (it > 8) __nanosleep(100);
        }
        return done != 0;
    };
    if (!poll(R.stage_polls)) s_fail = 1;
    __syncthreads();
    const bool ok = s_fail == 0;
    if (!ok) {
        // gave up: the results of this launch are not valid, but the block does not leave
        // while its copies may still write into its shared memory (a second wait, also
        // bounded), and the fault word tells the host
        if (threadIdx.x == 0) {
            poll(kStageWaitPolls);
            if (R.fault) atomicOr(R.fault, 1u);
        }
        __syncthreads();
        return false;
    }
    if (threadIdx.x == 0) asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(bar) : "memory");
    return ok;
}

// ---------------------------------------------------------------------------------
// Forward kinematics (warp-cooperative).  Element e = 4*r + c of a 3x4 product
// C = A * B with B's implicit last row (0 0 0 1), in the reference's multiply4x4
// order (KernelGenerator.h:257-280) with its multiply-adds fused.
// ---------------------------------------------------------------------------------
__device__ __forceinline__ float mul_elem(const float *A, const float *B, int r, int c) {
    float acc = __fmul_rn(A[4 * r + 0], B[0 * 4 + c]);
    acc = __fmaf_rn(A[4 * r + 1], B[1 * 4 + c], acc);
    acc = __fmaf_rn(A[4 * r + 2], B[2 * 4 + c], acc);
    if (c == 3) acc = __fadd_rn(acc, A[4 * r + 3]);
    return acc;
}

// Rodrigues rotation (KernelGenerator.h:305-325), 3x3 block R[3*row + col].
__device__ __forceinline__ void rot33(const float *n4, float s, float c, float *R) {
    const float nx = n4[0], ny = n4[1], nz = n4[2], valid = n4[3];
    const float oc = __fadd_rn(1.f, -c);
    const float iv = __fadd_rn(1.f, -valid);
    R[0] = __fadd_rn(__fmul_rn(__fmaf_rn(__fmul_rn(nx, nx), oc, c), valid), iv);
    R[1] = __fmul_rn(__fmaf_rn(__fmul_rn(nx, ny), oc, -__fmul_rn(nz, s)), valid);
    R[2] = __fmul_rn(__fmaf_rn(__fmul_rn(nx, nz), oc, __fmul_rn(ny, s)), valid);
    R[3] = __fmul_rn(__fmaf_rn(__fmul_rn(ny, nx), oc, __fmul_rn(nz, s)), valid);
    R[4] = __fadd_rn(__fmul_rn(__fmaf_rn(__fmul_rn(ny, ny), oc, c), valid), iv);
    R[5] = __fmul_rn(__fmaf_rn(__fmul_rn(ny, nz), oc, -__fmul_rn(nx, s)), valid);
    R[6] = __fmul_rn(__fmaf_rn(__fmul_rn(nz, nx), oc, -__fmul_rn(ny, s)), valid);
    R[7] = __fmul_rn(__fmaf_rn(__fmul_rn(nz, ny), oc, __fmul_rn(nx, s)), valid);
    R[8] = __fadd_rn(__fmul_rn(__fmaf_rn(__fmul_rn(nz, nz), oc, c), valid), iv);
}

// Joint-local transform of link i (one lane): revolute P * R(axis, q), prismatic
// P * T(axis q), fixed P, in the product order of mul_elem.  Unsupported types get
// the identity and are flagged so that the chain gives them an identity pose.  Computed
// in registers (joint_local_regs) and stored as three float4 rows: the 12-word stride
// between the lanes' transforms then spreads a quarter-warp's stores over all 32 banks
// (scalar stores at that stride hit 8 banks, 4-way conflicts).  `Mout` is 16-byte aligned.
__device__ __forceinline__ void joint_local_regs(const SmemTables &t, int i, float q, float *M);
__device__ __forceinline__ void joint_local(const SmemTables &t, int i, float q, float *Mout) {
    float M[12];
    joint_local_regs(t, i, q, M);
    float4 *o = reinterpret_cast<float4 *>(Mout);
    o[0] = make_float4(M[0], M[1], M[2], M[3]);
    o[1] = make_float4(M[4], M[5], M[6], M[7]);
    o[2] = make_float4(M[8], M[9], M[10], M[11]);
}
__device__ __forceinline__ void joint_local_regs(const SmemTables &t, int i, float q, float *M) {
    const float *P = t.jl + 12 * i;
    const int ty = t.type[i];
    if (ty == 1) {
        float sn, cs, R[9];
        sincosf(q, &sn, &cs);
        rot33(t.axn + 4 * i, sn, cs, R);
#pragma unroll
        for (int r = 0; r < 3; ++r) {
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                float acc = __fmul_rn(P[4 * r], R[c]);
                acc = __fmaf_rn(P[4 * r + 1], R[3 + c], acc);
                M[4 * r + c] = __fmaf_rn(P[4 * r + 2], R[6 + c], acc);
            }
            float acc = __fmul_rn(P[4 * r], 0.f);
            acc = __fmaf_rn(P[4 * r + 1], 0.f, acc);
            acc = __fmaf_rn(P[4 * r + 2], 0.f, acc);
            M[4 * r + 3] = __fadd_rn(acc, P[4 * r + 3]);
        }
    } else if (ty == 2) {
        const float *a = t.axr + 4 * i;
        const float tx = __fmul_rn(a[0], q), ty2 = __fmul_rn(a[1], q), tz = __fmul_rn(a[2], q);
#pragma unroll
        for (int r = 0; r < 3; ++r) {
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                float acc = __fmul_rn(P[4 * r], c == 0 ? 1.f : 0.f);
                acc = __fmaf_rn(P[4 * r + 1], c == 1 ? 1.f : 0.f, acc);
                M[4 * r + c] = __fmaf_rn(P[4 * r + 2], c == 2 ? 1.f : 0.f, acc);
            }
            float acc = __fmul_rn(P[4 * r], tx);
            acc = __fmaf_rn(P[4 * r + 1], ty2, acc);
            acc = __fmaf_rn(P[4 * r + 2], tz, acc);
            M[4 * r + 3] = __fadd_rn(acc, P[4 * r + 3]);
        }
    } else if (ty == 5) {
#pragma unroll
        for (int k = 0; k < 12; ++k) M[k] = P[k];
    } else {
#pragma unroll
        for (int k = 0; k < 12; ++k) M[k] = (k % 5 == 0) ? 1.f : 0.f;
    }
}

// FK of the state in w.q into w.lp.  All lanes of the warp must call it.
// Phase 1: lane i forms the joint-local transform of link i (all links at once).
// Phase 2: lanes 0..11 walk the chain, link_i = link_parent(i) * local_i, one
// element per lane (KernelGenerator.h:369-400; association parent * (pose * motion)).
__device__ inline void warp_fk(const SmemTables &t, int L, const WarpScratch &w, int lane) {
    for (int i = lane; i < L; i += kWarp) joint_local(t, i, w.q[i], w.loc + 12 * i);
    const int r = lane >> 2, c = lane & 3;
    const bool own = lane < 12;
    if (own) w.lp[lane] = (r == c) ? 1.f : 0.f;
    __syncwarp();
    for (int i = 1; i < L; ++i) {
        const int ty = t.type[i];
        if (own) {
            const bool known = ty == 1 || ty == 2 || ty == 5;
            w.lp[12 * i + lane] = known ? mul_elem(w.lp + 12 * t.parent[i], w.loc + 12 * i, r, c)
                                        : ((r == c) ? 1.f : 0.f);
        }
        __syncwarp();
    }
}

// Sphere centre in the base frame (SingleArmStates.cu:340-393).
__device__ __forceinline__ float3 xform_point(const float *T, float x, float y, float z) {
    float3 o;
    o.x = __fadd_rn(__fmaf_rn(T[2], z, __fmaf_rn(T[1], y, __fmul_rn(T[0], x))), T[3]);
    o.y = __fadd_rn(__fmaf_rn(T[6], z, __fmaf_rn(T[5], y, __fmul_rn(T[4], x))), T[7]);
    o.z = __fadd_rn(__fmaf_rn(T[10], z, __fmaf_rn(T[9], y, __fmul_rn(T[8], x))), T[11]);
    return o;
}

__device__ __forceinline__ float3 xform_rows(const float4 r0, const float4 r1, const float4 r2, float x, float y,
                                             float z) {
    float3 o;
    o.x = __fadd_rn(__fmaf_rn(r0.z, z, __fmaf_rn(r0.y, y, __fmul_rn(r0.x, x))), r0.w);
    o.y = __fadd_rn(__fmaf_rn(r1.z, z, __fmaf_rn(r1.y, y, __fmul_rn(r1.x, x))), r1.w);
    o.z = __fadd_rn(__fmaf_rn(r2.z, z, __fmaf_rn(r2.y, y, __fmul_rn(r2.x, x))), r2.w);
    return o;
}

__device__ __forceinline__ float sq3(float dx, float dy, float dz) {
    return __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
}

// ---------------------------------------------------------------------------------
// Collision of one state.  Returns true if it collides.  With COST, costs[0..3] of
// lane 0 receive the warp totals per constraint slot (self, spheres, cuboids,
// cylinders), following the per-pair cost formulas of SelfCollisionConstraint.cu:80-112,
// EnvConstraintSphere.cu:57-96, EnvConstraintCuboid.cu:105-159,
// EnvConstraintCylinder.cu:130-180.
// ---------------------------------------------------------------------------------
template <int SPL, bool COST>
__device__ inline bool warp_collide(const SmemTables &t, const DevRobot &R, const DevEnv &E,
                                    const WarpScratch &w, int lane, float *costs) {
    float cx[SPL], cy[SPL], cz[SPL], cr[SPL];
#pragma unroll
    for (int m = 0; m < SPL; ++m) {
        const int k = lane + kWarp * m;
        if (k < R.S) {
            const float4 s = t.sph[k];
            const float3 p = xform_point(w.lp + 12 * t.slink[k], s.x, s.y, s.z);
            cx[m] = p.x; cy[m] = p.y; cz[m] = p.z; cr[m] = s.w;
            w.cen[k] = make_float4(p.x, p.y, p.z, s.w);
        } else {
            cx[m] = kFar; cy[m] = kFar; cz[m] = kFar; cr[m] = 0.f;
        }
    }
    __syncwarp();

    bool hit = false;
    float c_self = 0.f, c_sph = 0.f, c_box = 0.f, c_cyl = 0.f;
    const float4 *env = t.env;

    // --- environment spheres ---
    if (COST) {
        for (int o = 0; o < E.ns; ++o) {
            const float4 b = env[o];
#pragma unroll
            for (int m = 0; m < SPL; ++m) {
                const float d2 = sq3(cx[m] - b.x, cy[m] - b.y, cz[m] - b.z);
                const float rr = cr[m] + b.w;
                if (d2 < rr * rr) c_sph += fmaxf(0.f, rr - sqrtf(d2));
            }
        }
    } else {
        // Expanded form: d^2 - (rs + ro)^2 = A + B - 2 (c.o + rs ro) with A = |c|^2 - rs^2
        // per robot sphere and B = |o|^2 - ro^2 per obstacle (staged as (2o, 2ro, -B)),
        // so a test is four FMAs and a compare.  Rounding moves the contact surface by
        // ~1e-5 m at workspace scale.
        float A[SPL];
#pragma unroll
        for (int m = 0; m < SPL; ++m) A[m] = __fmaf_rn(cz[m], cz[m], __fmaf_rn(cy[m], cy[m], __fmaf_rn(cx[m], cx[m], -cr[m] * cr[m])));
        const float4 *sx = t.env + E.ns + 5 * E.nb + 4 * E.nc;
        const float *snb = reinterpret_cast<const float *>(sx + E.ns);
        for (int o0 = 0; o0 < E.ns; o0 += 16) {
            const int oe = min(o0 + 16, E.ns);
#pragma unroll 4
            for (int o = o0; o < oe; ++o) {
                const float4 b = sx[o];
                const float nb = snb[o];
#pragma unroll
                for (int m = 0; m < SPL; ++m) {
                    const float v = __fmaf_rn(cx[m], b.x, __fmaf_rn(cy[m], b.y, __fmaf_rn(cz[m], b.z, __fmaf_rn(cr[m], b.w, nb))));
                    hit |= v > A[m];
                }
            }
            if (__any_sync(kFull, hit)) return true;
        }
    }
    env += E.ns;

    // --- cuboids (inverse pose, clamp to [min, max]) ---
    for (int o0 = 0; o0 < E.nb; o0 += 4) {
        const int oe = min(o0 + 4, E.nb);
        for (int o = o0; o < oe; ++o) {
            const float4 r0 = env[5 * o], r1 = env[5 * o + 1], r2 = env[5 * o + 2];
            const float4 mn = env[5 * o + 3], mx = env[5 * o + 4];
#pragma unroll
            for (int m = 0; m < SPL; ++m) {
                const float3 l = xform_rows(r0, r1, r2, cx[m], cy[m], cz[m]);
                const float dx = l.x - fminf(fmaxf(l.x, mn.x), mx.x);
                const float dy = l.y - fminf(fmaxf(l.y, mn.y), mx.y);
                const float dz = l.z - fminf(fmaxf(l.z, mn.z), mx.z);
                const float d2 = sq3(dx, dy, dz);
                const bool h = d2 < cr[m] * cr[m];
                if (COST) { if (h) c_box += cr[m] - sqrtf(d2); }
                hit |= h;
            }
        }
        if (!COST && __any_sync(kFull, hit)) return true;
    }
    env += 5 * E.nb;

    // --- cylinders (finite, local z axis) ---
    for (int o0 = 0; o0 < E.nc; o0 += 4) {
        const int oe = min(o0 + 4, E.nc);
        for (int o = o0; o < oe; ++o) {
            const float4 r0 = env[4 * o], r1 = env[4 * o + 1], r2 = env[4 * o + 2], pr = env[4 * o + 3];
#pragma unroll
            for (int m = 0; m < SPL; ++m) {
                const float3 l = xform_rows(r0, r1, r2, cx[m], cy[m], cz[m]);
                const float dxy = sqrtf(__fmaf_rn(l.y, l.y, __fmul_rn(l.x, l.x)));
                const float dx = dxy - pr.x;
                const float dz = fabsf(l.z) - pr.y;
                const float ox = dx > 0.f ? dx : 0.f, oz = dz > 0.f ? dz : 0.f;
                const float outside = sqrtf(__fmaf_rn(oz, oz, __fmul_rn(ox, ox)));
                const float inside = fminf(fmaxf(dx, dz), 0.f);
                const float pen = cr[m] - (outside + inside);
                if (COST) c_cyl += pen > 0.f ? pen : 0.f;
                hit |= pen > 0.f;
            }
        }
        if (!COST && __any_sync(kFull, hit)) return true;
    }

    // --- self collision pairs ---
    for (int p0 = 0; p0 < R.P; p0 += kWarp * 4) {
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int p = p0 + u * kWarp + lane;
            if (p < R.P) {
                const unsigned ij = __ldg(R.pairs + p);
                const float thr = __ldg(R.thr + p);
                const float4 a = w.cen[ij & 0xffffu], b = w.cen[ij >> 16];
                const float d2 = sq3(a.x - b.x, a.y - b.y, a.z - b.z);
                const bool h = d2 < thr;
                if (COST) { if (h) c_self += sqrtf(thr) - sqrtf(d2); }
                hit |= h;
            }
        }
        if (!COST && __any_sync(kFull, hit)) return true;
    }

    if (COST) {
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            c_self += __shfl_xor_sync(kFull, c_self, off);
            c_sph += __shfl_xor_sync(kFull, c_sph, off);
            c_box += __shfl_xor_sync(kFull, c_box, off);
            c_cyl += __shfl_xor_sync(kFull, c_cyl, off);
        }
        costs[0] = c_self; costs[1] = c_sph; costs[2] = c_box; costs[3] = c_cyl;
    }
    return __any_sync(kFull, hit);
}

// ---------------------------------------------------------------------------------
// Verdict-only collision with a broad phase.  Every sphere-carrying link ("group") has
// a bounding sphere that encloses its collision spheres plus kBroadMargin.  Obstacles
// are taken 32 at a time, one per lane; each lane tests its obstacle against every
// group bounding sphere and keeps a mask of overlapping groups.  Obstacles with a
// non-empty mask are compacted (ballot + popc) into a per-warp candidate list, and
// only the robot spheres of the overlapping groups are tested against them with the
// exact per-sphere formulas.  Self-collision uses the group-pair ranges of the sorted
// pair list the same way.  The broad tests are conservative (a sphere inside its group
// sphere cannot touch an obstacle the group sphere misses, and every distance function
// used is 1-Lipschitz), so the verdict equals that of warp_collide up to floating-point
// rounding at the contact surface.
// ---------------------------------------------------------------------------------
template <int SPL>
__device__ inline bool warp_collide_culled(const SmemTables &t, const DevRobot &R, const DevEnv &E,
                                           const WarpScratch &w, int lane) {
    float cx[SPL], cy[SPL], cz[SPL], cr[SPL], A[SPL];
    unsigned gbit[SPL];
#pragma unroll
    for (int m = 0; m < SPL; ++m) {
        const int k = lane + kWarp * m;
        if (k < R.S) {
            const float4 s = t.sph[k];
            const float3 p = xform_point(w.lp + 12 * t.slink[k], s.x, s.y, s.z);
            cx[m] = p.x; cy[m] = p.y; cz[m] = p.z; cr[m] = s.w;
            gbit[m] = 1u << t.sgrp[k];
            w.cen[k] = make_float4(p.x, p.y, p.z, s.w);
        } else {
            cx[m] = kFar; cy[m] = kFar; cz[m] = kFar; cr[m] = 0.f;
            gbit[m] = 0u;
        }
        A[m] = __fmaf_rn(cz[m], cz[m], __fmaf_rn(cy[m], cy[m], __fmaf_rn(cx[m], cx[m], -cr[m] * cr[m])));
    }
    if (lane < R.G) {
        const float4 g = t.grp[lane];
        const float3 c = xform_point(w.lp + 12 * t.glink[lane], g.x, g.y, g.z);
        w.gb[lane] = make_float4(c.x, c.y, c.z, g.w);
        w.gA[lane] = __fmaf_rn(c.z, c.z, __fmaf_rn(c.y, c.y, __fmaf_rn(c.x, c.x, -g.w * g.w)));
    }
    __syncwarp();
    const unsigned lt = (1u << lane) - 1u;
    bool hit = false;
    const bool count = R.work != nullptr;
    unsigned long long fl = (unsigned long long)R.base_flops;
#define GBMP_CULLED_RETURN(v)                                          \
    do {                                                               \
        if (count && lane == 0) {                                      \
            atomicAdd(R.work, fl);                                     \
            atomicAdd(R.work + 1, 1ull);                               \
        }                                                              \
        return (v);                                                    \
    } while (0)

    // --- environment spheres (expanded form, see warp_collide) ---
    const float4 *sx = t.env + E.ns + 5 * E.nb + 4 * E.nc;
    const float *snb = reinterpret_cast<const float *>(sx + E.ns);
#pragma unroll 1
    for (int o0 = 0; o0 < E.ns; o0 += kWarp) {
        const int o = o0 + lane;
        unsigned mask = 0u;
        if (o < E.ns) {
            const float4 b = sx[o];
            const float nb = snb[o];
#pragma unroll 2
            for (int g = 0; g < R.G; ++g) {
                const float4 gs = w.gb[g];
                const float v = __fmaf_rn(gs.x, b.x, __fmaf_rn(gs.y, b.y, __fmaf_rn(gs.z, b.z, __fmaf_rn(gs.w, b.w, nb))));
                if (v > w.gA[g]) mask |= 1u << g;
            }
        }
        const unsigned bal = __ballot_sync(kFull, mask != 0u);
        if (mask) { const int pos = __popc(bal & lt); w.cand[pos] = o; w.cmask[pos] = mask; }
        __syncwarp();
        const int nc = __popc(bal);
        if (count) fl += (unsigned long long)min(kWarp, E.ns - o0) * R.G * kFlSphereX;
        for (int i = 0; i < nc; ++i) {
            const int oc = w.cand[i];
            const unsigned cm = w.cmask[i];
            const float4 b = sx[oc];
            const float nb = snb[oc];
#pragma unroll
            for (int m = 0; m < SPL; ++m) {
                const float v = __fmaf_rn(cx[m], b.x, __fmaf_rn(cy[m], b.y, __fmaf_rn(cz[m], b.z, __fmaf_rn(cr[m], b.w, nb))));
                hit |= (cm & gbit[m]) && v > A[m];
                if (count) fl += (unsigned long long)__popc(__ballot_sync(kFull, (cm & gbit[m]) != 0u)) * kFlSphereX;
            }
        }
        if (__any_sync(kFull, hit)) GBMP_CULLED_RETURN(true);
    }

    // --- cuboids ---
    const float4 *bx = t.env + E.ns;
#pragma unroll 1
    for (int o0 = 0; o0 < E.nb; o0 += kWarp) {
        const int o = o0 + lane;
        unsigned mask = 0u;
        if (o < E.nb) {
            const float4 r0 = bx[5 * o], r1 = bx[5 * o + 1], r2 = bx[5 * o + 2], mn = bx[5 * o + 3], mx = bx[5 * o + 4];
            for (int g = 0; g < R.G; ++g) {
                const float4 gs = w.gb[g];
                const float3 l = xform_rows(r0, r1, r2, gs.x, gs.y, gs.z);
                const float dx = l.x - fminf(fmaxf(l.x, mn.x), mx.x);
                const float dy = l.y - fminf(fmaxf(l.y, mn.y), mx.y);
                const float dz = l.z - fminf(fmaxf(l.z, mn.z), mx.z);
                if (sq3(dx, dy, dz) < gs.w * gs.w) mask |= 1u << g;
            }
        }
        const unsigned bal = __ballot_sync(kFull, mask != 0u);
        if (mask) { const int pos = __popc(bal & lt); w.cand[pos] = o; w.cmask[pos] = mask; }
        __syncwarp();
        const int nc = __popc(bal);
        if (count) fl += (unsigned long long)min(kWarp, E.nb - o0) * R.G * kFlCuboid;
        for (int i = 0; i < nc; ++i) {
            const int oc = w.cand[i];
            const unsigned cm = w.cmask[i];
            const float4 r0 = bx[5 * oc], r1 = bx[5 * oc + 1], r2 = bx[5 * oc + 2], mn = bx[5 * oc + 3], mx = bx[5 * oc + 4];
#pragma unroll
            for (int m = 0; m < SPL; ++m) {
                if (count) fl += (unsigned long long)__popc(__ballot_sync(kFull, (cm & gbit[m]) != 0u)) * kFlCuboid;
                if (cm & gbit[m]) {
                    const float3 l = xform_rows(r0, r1, r2, cx[m], cy[m], cz[m]);
                    const float dx = l.x - fminf(fmaxf(l.x, mn.x), mx.x);
                    const float dy = l.y - fminf(fmaxf(l.y, mn.y), mx.y);
                    const float dz = l.z - fminf(fmaxf(l.z, mn.z), mx.z);
                    hit |= sq3(dx, dy, dz) < cr[m] * cr[m];
                }
            }
        }
        if (__any_sync(kFull, hit)) GBMP_CULLED_RETURN(true);
    }

    // --- cylinders ---
    const float4 *cyl = t.env + E.ns + 5 * E.nb;
#pragma unroll 1
    for (int o0 = 0; o0 < E.nc; o0 += kWarp) {
        const int o = o0 + lane;
        unsigned mask = 0u;
        if (o < E.nc) {
            const float4 r0 = cyl[4 * o], r1 = cyl[4 * o + 1], r2 = cyl[4 * o + 2], pr = cyl[4 * o + 3];
            for (int g = 0; g < R.G; ++g) {
                const float4 gs = w.gb[g];
                const float3 l = xform_rows(r0, r1, r2, gs.x, gs.y, gs.z);
                const float dx = sqrtf(__fmaf_rn(l.y, l.y, __fmul_rn(l.x, l.x))) - pr.x;
                const float dz = fabsf(l.z) - pr.y;
                const float ox = dx > 0.f ? dx : 0.f, oz = dz > 0.f ? dz : 0.f;
                const float sdf = sqrtf(__fmaf_rn(oz, oz, __fmul_rn(ox, ox))) + fminf(fmaxf(dx, dz), 0.f);
                if (gs.w - sdf > 0.f) mask |= 1u << g;
            }
        }
        const unsigned bal = __ballot_sync(kFull, mask != 0u);
        if (mask) { const int pos = __popc(bal & lt); w.cand[pos] = o; w.cmask[pos] = mask; }
        __syncwarp();
        const int nc = __popc(bal);
        if (count) fl += (unsigned long long)min(kWarp, E.nc - o0) * R.G * kFlCylinder;
        for (int i = 0; i < nc; ++i) {
            const int oc = w.cand[i];
            const unsigned cm = w.cmask[i];
            const float4 r0 = cyl[4 * oc], r1 = cyl[4 * oc + 1], r2 = cyl[4 * oc + 2], pr = cyl[4 * oc + 3];
#pragma unroll
            for (int m = 0; m < SPL; ++m) {
                if (count) fl += (unsigned long long)__popc(__ballot_sync(kFull, (cm & gbit[m]) != 0u)) * kFlCylinder;
                if (cm & gbit[m]) {
                    const float3 l = xform_rows(r0, r1, r2, cx[m], cy[m], cz[m]);
                    const float dx = sqrtf(__fmaf_rn(l.y, l.y, __fmul_rn(l.x, l.x))) - pr.x;
                    const float dz = fabsf(l.z) - pr.y;
                    const float ox = dx > 0.f ? dx : 0.f, oz = dz > 0.f ? dz : 0.f;
                    const float outside = sqrtf(__fmaf_rn(oz, oz, __fmul_rn(ox, ox)));
                    const float inside = fminf(fmaxf(dx, dz), 0.f);
                    hit |= cr[m] - (outside + inside) > 0.f;
                }
            }
        }
        if (__any_sync(kFull, hit)) GBMP_CULLED_RETURN(true);
    }

    // --- self collision: group pairs whose bounding spheres overlap ---
    for (int k0 = 0; k0 < R.NPL; k0 += kWarp) {
        const int k = k0 + lane;
        bool on = false;
        int p0 = 0, p1 = 0;
        if (k < R.NPL) {
            const int4 lp = t.lpair[k];
            const float4 a = w.gb[lp.x], b = w.gb[lp.y];
            const float rr = a.w + b.w;
            on = sq3(a.x - b.x, a.y - b.y, a.z - b.z) < rr * rr;
            p0 = lp.z;
            p1 = lp.w;
        }
        unsigned bal = __ballot_sync(kFull, on);
        if (count) fl += (unsigned long long)min(kWarp, R.NPL - k0) * kFlGroupPair;
        while (bal) {
            const int j = __ffs(bal) - 1;
            bal &= bal - 1u;
            const int q0 = __shfl_sync(kFull, p0, j), q1 = __shfl_sync(kFull, p1, j);
            if (count) fl += (unsigned long long)(q1 - q0) * kFlSelf;
            for (int p = q0 + lane; p < q1; p += kWarp) {
                const unsigned ij = __ldg(R.pairs + p);
                const float thr = __ldg(R.thr + p);
                const float4 a = w.cen[ij & 0xffffu], b = w.cen[ij >> 16];
                hit |= sq3(a.x - b.x, a.y - b.y, a.z - b.z) < thr;
            }
            if (__any_sync(kFull, hit)) GBMP_CULLED_RETURN(true);
        }
    }
    GBMP_CULLED_RETURN(false);
#undef GBMP_CULLED_RETURN
}

// Dispatch on spheres-per-lane.
template <bool COST>
__device__ inline bool warp_collide_dispatch(const SmemTables &t, const DevRobot &R, const DevEnv &E,
                                             const WarpScratch &w, int lane, float *costs) {
    switch (R.spl) {
    case 1: return warp_collide<1, COST>(t, R, E, w, lane, costs);
    case 2: return warp_collide<2, COST>(t, R, E, w, lane, costs);
    case 3: return warp_collide<3, COST>(t, R, E, w, lane, costs);
    case 4: return warp_collide<4, COST>(t, R, E, w, lane, costs);
    case 5: return warp_collide<5, COST>(t, R, E, w, lane, costs);
    case 6: return warp_collide<6, COST>(t, R, E, w, lane, costs);
    case 7: return warp_collide<7, COST>(t, R, E, w, lane, costs);
    default: return warp_collide<8, COST>(t, R, E, w, lane, costs);
    }
}

// Link poses [L*16] (row-major 4x4, last row 0 0 0 1) and sphere centres [S*3] of the
// state whose FK is in w.lp, written to HBM by the warp.
__device__ inline void store_fk(const SmemTables &t, const DevRobot &R, const WarpScratch &w, long long s,
                                float *__restrict__ poses, float *__restrict__ centers, int lane) {
    if (poses) {
        float *P = poses + s * R.L * 16;
        for (int e = lane; e < R.L * 16; e += kWarp) {
            const int li = e >> 4, k = e & 15;
            P[e] = k < 12 ? w.lp[12 * li + k] : (k == 15 ? 1.f : 0.f);
        }
    }
    if (centers) {
        float *C = centers + s * R.S * 3;
        for (int k = lane; k < R.S; k += kWarp) {
            const float4 sp = t.sph[k];
            const float3 p = xform_point(w.lp + 12 * t.slink[k], sp.x, sp.y, sp.z);
            C[3 * k] = p.x; C[3 * k + 1] = p.y; C[3 * k + 2] = p.z;
        }
    }
}

// One state of a collision check, one warp: FK of state s of q, its poses / centres when
// asked for, the collision test, and the outputs (verdict; in cost mode the four
// constraint costs [4][n] and their total).  k_check_states and the batched check run
// this routine, so their outputs are bit-identical.
template <bool COST, int SPL>
__device__ inline void check_state(const SmemTables &t, const DevRobot &R, const DevEnv &E, const WarpScratch &w,
                                   const float *__restrict__ q, long long s, long long n,
                                   unsigned char *__restrict__ verdict, float *__restrict__ costs,
                                   float *__restrict__ total, float *__restrict__ poses, float *__restrict__ centers,
                                   int lane) {
    for (int j = lane; j < R.L; j += kWarp) w.q[j] = q[s * R.L + j];
    __syncwarp();
    warp_fk(t, R.L, w, lane);
    if (poses || centers) store_fk(t, R, w, s, poses, centers, lane);
    float c[4] = {0.f, 0.f, 0.f, 0.f};
    const bool hit = (!COST && R.cull) ? warp_collide_culled<SPL>(t, R, E, w, lane)
                                       : warp_collide<SPL, COST>(t, R, E, w, lane, c);
    if (lane == 0) {
        if (COST) {
            const float tot = ((c[0] + c[1]) + c[2]) + c[3];
            if (costs) { costs[s] = c[0]; costs[n + s] = c[1]; costs[2 * n + s] = c[2]; costs[3 * n + s] = c[3]; }
            if (total) total[s] = tot;
            if (verdict) verdict[s] = tot != 0.f;
        } else if (verdict) {
            verdict[s] = hit;
        }
    }
    __syncwarp();
}

}  // namespace gbmp
