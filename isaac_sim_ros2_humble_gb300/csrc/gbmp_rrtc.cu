// gbmp_rrtc.cu -- parallel RRT-Connect on the device (replaces CPRRTC::RobotSolver::solve,
// cudampl/CPRRTC/src/RobotSolver.cu:348-473 with its kernel :507-799, and the pRRTC
// kernel rrtc<Robot>, pRRTC/src/planning/pRRTC.cu:305-602).
//
// One persistent launch per solve.  Each block is one extension lane of kRrtcWarps
// warps; per iteration a lane
//   1. picks the tree to grow (the smaller tree gets proportionally more lanes,
//      pRRTC.cu:348-371 balance mode 1),
//   2. draws a Philox sample in the joint limits (counter = lane, iteration),
//   3. finds the nearest node of that tree (block-wide argmin over the active joints),
//   4. steers to at most `range` (pRRTC.cu:415-434),
//   5. validates the edge with the checkMotions step rule, one warp per state
//      (FK + self + environment collision, broad phase included),
//   6. appends the node (atomic slot, NaN sentinel until every coordinate is written,
//      pRRTC.cu:447-476 with the sentinel filled correctly),
//   7. tries to connect: finds the nearest node of the other tree and extends towards
//      it in steps of at most `range`, appending every validated step; reaching it
//      solves the problem (RobotSolver.cu:686-794, pRRTC.cu:478-551).
// The first lane to connect records the connection; a trace kernel then walks both
// parent chains into the path buffer (pRRTC.cu:552-581).  Every loop is bounded: the
// lane iteration cap, the node cap and a %globaltimer deadline end the launch with a
// status the host reads.
#include <algorithm>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstring>

#include "gbmp_autotune.h"
#include "gbmp_rrtc.cuh"

namespace gbmp {

// Reset of every problem of a batch: NaN sentinels over the slots the previous solve
// used, roots from the staged start / goal, counters to zero.
__global__ void k_rrtc_batch_reset(BatchProblem *__restrict__ probs, int n, unsigned long long *deadline,
                                   unsigned long long limit_ns) {
    const int p = blockIdx.y;
    if (p == 0 && blockIdx.x == 0 && threadIdx.x == 0) *deadline = global_ns() + limit_ns;
    if (p >= n) return;
    BatchProblem &b = probs[p];
    const int L = b.R.L;
    for (int t = 0; t < 2; ++t) {
        // the words the previous solve of this slot wrote (its stride may differ)
        const long long words = max((long long)b.prev[t], (long long)b.P.stride);
        for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < words;
             i += (long long)gridDim.x * blockDim.x)
            b.P.nodes[t][i] = __int_as_float(0xffffffff);
        // dynamic-domain radii of at least as many nodes back to unset
        if (b.P.radii[t]) {
            const long long nodes = min(words, (long long)b.P.cap);
            for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nodes;
                 i += (long long)gridDim.x * blockDim.x)
                b.P.radii[t][i] = __uint_as_float(kRadiusUnset);
        }
    }
    __syncthreads();
    if (blockIdx.x == 0) {
        for (int j = threadIdx.x; j < L; j += blockDim.x) {
            b.P.nodes[0][j] = b.start[j];
            b.P.nodes[1][j] = b.goal[j];
        }
        if (threadIdx.x == 0) {
            b.P.parent[0][0] = 0;
            b.P.parent[1][0] = 0;
            b.P.size[0] = 1;
            b.P.size[1] = 1;
            for (int k = 0; k < 12; ++k) b.P.state[k] = 0;
        }
    }
}

// Record the node words used, for the next reset.
__global__ void k_rrtc_batch_finish(BatchProblem *__restrict__ probs, int n) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    probs[p].prev[0] = min(probs[p].P.size[0], probs[p].P.cap) * probs[p].P.stride;
    probs[p].prev[1] = min(probs[p].P.size[1], probs[p].P.cap) * probs[p].P.stride;
}

// Goals a single-problem solve stages in its pinned input block; more are copied into the
// goal tree after the reset.
constexpr int kStagedGoals = 64;

// Reset of a single-problem solve, one launch: NaN sentinels over the words the previous
// solve wrote (w[t] words of tree t past its root rows), unset dynamic-domain radii (r[t]),
// the root rows (the start; the staged goals, other goal rows NaN until their copy), the
// roots' parents, the counters and the deadline (the device clock plus the limit, set here
// so that no host round trip reads the clock).  `in` is the mapped pinned input block:
// start [L], then up to kStagedGoals goals [L] each.  The root rows and the words past
// them are written by different loops, so no word has two writers.
__global__ void k_rrtc_init(RrtcDev P, int L, long long w0, long long w1, int r0, int r1,
                            const float *__restrict__ in, int n_goals, unsigned long long limit_ns) {
    const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long nth = (long long)gridDim.x * blockDim.x;
    const float nan = __int_as_float(0xffffffff);
    const long long root0 = P.stride, root1 = (long long)n_goals * P.stride;
    for (long long i = root0 + tid; i < w0; i += nth) P.nodes[0][i] = nan;
    for (long long i = root1 + tid; i < w1; i += nth) P.nodes[1][i] = nan;
    if (P.radii[0])
        for (long long i = tid; i < r0; i += nth) P.radii[0][i] = __uint_as_float(kRadiusUnset);
    if (P.radii[1])
        for (long long i = tid; i < r1; i += nth) P.radii[1][i] = __uint_as_float(kRadiusUnset);
    for (long long i = tid; i < root0; i += nth) P.nodes[0][i] = i < L ? in[i] : nan;
    for (long long i = tid; i < root1; i += nth) {
        const long long g = i / P.stride, j = i - g * P.stride;
        P.nodes[1][i] = (j < L && g < kStagedGoals) ? in[L + g * L + j] : nan;
    }
    for (long long g = tid; g < n_goals; g += nth) P.parent[1][g] = (int)g;
    if (tid == 0) {
        P.parent[0][0] = 0;
        for (int k = 0; k < 64; ++k) P.size[k] = 0;   // sizes, state, deadline, path length
        P.size[0] = 1;
        P.size[1] = n_goals;
        *(unsigned long long *)(P.state + 8) = global_ns() + limit_ns;
    }
}

// Walk both parent chains into the path (start tree root first).  One thread.
__device__ void rrtc_trace_path(const RrtcDev &P, int L) {
    if (P.state[0] != kStSolved) { *P.path_len = 0; return; }
    const int tr = P.state[2];
    const int a = P.state[3], b = P.state[4];
    const int na = tr == 0 ? a : b, nb = tr == 0 ? b : a;   // node in start tree, node in goal tree
    // count
    int len0 = 0, len1 = 0;
    for (int i = na; i >= 0 && len0 <= P.cap; i = (P.parent[0][i] == i ? -1 : P.parent[0][i])) ++len0;
    for (int i = nb; i >= 0 && len1 <= P.cap; i = (P.parent[1][i] == i ? -1 : P.parent[1][i])) ++len1;
    if (len0 + len1 > P.path_cap || len0 > P.cap || len1 > P.cap) { *P.path_len = -(len0 + len1); return; }
    int k = len0 - 1;
    for (int i = na; i >= 0; i = (P.parent[0][i] == i ? -1 : P.parent[0][i]), --k)
        for (int j = 0; j < L; ++j) P.path[k * L + j] = P.nodes[0][(long long)i * P.stride + j];
    k = len0;
    for (int i = nb; i >= 0; i = (P.parent[1][i] == i ? -1 : P.parent[1][i]), ++k)
        for (int j = 0; j < L; ++j) P.path[k * L + j] = P.nodes[1][(long long)i * P.stride + j];
    *P.path_len = len0 + len1;
}

// The trace, then the solve's outcome into the mapped pinned block `out` (state [6], tree
// sizes [2], path length), so that the host reads everything after one synchronisation.
__global__ void k_rrtc_trace(RrtcDev P, int L, int *out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    rrtc_trace_path(P, L);
    for (int k = 0; k < 6; ++k) out[k] = P.state[k];
    out[6] = P.size[0];
    out[7] = P.size[1];
    out[8] = *P.path_len;
}

__global__ void k_rrtc_batch_trace(const BatchProblem *__restrict__ probs, int n, int *__restrict__ summary) {
    const int p = blockIdx.x;
    if (p >= n) return;
    if (threadIdx.x == 0) {
        const RrtcDev &P = probs[p].P;
        rrtc_trace_path(P, probs[p].R.L);   // the single-problem trace (one thread)
        int *o = summary + 8 * p;
        o[0] = P.state[0];
        o[1] = *P.path_len;
        o[2] = min(P.size[0], P.cap);
        o[3] = min(P.size[1], P.cap);
        o[4] = P.state[5];
    }
}

}  // namespace gbmp

using namespace gbmp;

// Edge-check step of a solve: the settings' resolution (or the robot's), or for
// GBMP_STEP_COUNT the step count G in [1, 1e6].  Returns false on invalid settings.
static bool plan_step(const gbmp_rrtc_settings *s, float robot_res, float *res) {
    if (s->step_rule == GBMP_STEP_COUNT) {
        if (!(s->resolution >= 1.f && s->resolution <= 1e6f)) return false;
        *res = floorf(s->resolution);
        return true;
    }
    if (s->step_rule != GBMP_STEP_L2 && s->step_rule != GBMP_STEP_LINF) return false;
    *res = s->resolution > 0.f ? s->resolution : robot_res;
    return *res > 0.f;
}

// Balance strategy of a solve in the device encoding (0 none, 1 size, 2 swap, 3 proportional) and its
// tree ratio; false on an unknown strategy or a non-finite ratio.
static bool plan_balance(const gbmp_rrtc_settings *s, int *balance, float *ratio) {
    switch (s->balance) {
    case GBMP_BALANCE_DEFAULT: *balance = 3; break;
    case GBMP_BALANCE_SIZE: *balance = 1; break;
    case GBMP_BALANCE_SWAP: *balance = 2; break;
    case GBMP_BALANCE_NONE: *balance = 0; break;
    default: return false;
    }
    if (!std::isfinite(s->tree_ratio)) return false;
    *ratio = s->tree_ratio > 0.f ? s->tree_ratio : (*balance == 2 ? 1.0f : 0.5f);
    return true;
}

static bool plan_dd_ok(const gbmp_rrtc_settings *s) {
    return !s->dynamic_domain || (s->dd_alpha >= 0.f && s->dd_alpha < 1.f && s->dd_radius > 0.f &&
                                  s->dd_min_radius > 0.f && std::isfinite(s->dd_radius));
}

struct gbmp_planner_s {
    gbmp_robot robot = nullptr;
    int cap = 0, stride = 0, path_cap = 0;
    void *block = nullptr;
    RrtcDev dev{};
    // tree slots written since the last reset, per tree (all of them after creation or an
    // interrupted solve): only these are re-poisoned before the next solve
    int dirty[2] = {0, 0}, dirty_radii[2] = {0, 0};
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    // the traced path goes straight to pinned host memory (the trace kernel writes it
    // through the mapped pointer), so reading a result takes one synchronisation
    float *h_path = nullptr;
    // mapped pinned block: the outcome the trace kernel writes (16 ints), then the staged
    // start and goals the reset kernel reads
    int *h_io = nullptr, *d_io = nullptr;
};

extern "C" {

gbmp_status gbmp_planner_create(gbmp_robot r, int32_t max_nodes, int32_t path_cap, gbmp_planner *out) {
    GBMP_CHECK_ARG(r && out, "robot/out is NULL");
    *out = nullptr;
    GBMP_CHECK_ARG(max_nodes >= 2 && max_nodes <= (1 << 28), "max_nodes %d outside [2, 2^28]", max_nodes);
    GBMP_CHECK_ARG(path_cap >= 2, "path_cap < 2");
    auto *p = new gbmp_planner_s();
    p->robot = r;
    p->cap = max_nodes;
    p->stride = (r->L + 3) & ~3;
    p->path_cap = path_cap;
    const size_t nodes_b = align16(sizeof(float) * (size_t)max_nodes * p->stride);
    const size_t par_b = align16(sizeof(int) * (size_t)max_nodes);
    const size_t path_b = align16(sizeof(float) * (size_t)path_cap * r->L);
    const size_t rad_b = align16(sizeof(float) * (size_t)max_nodes);   // dynamic-domain radii, per tree
    const size_t bytes = 2 * nodes_b + 2 * par_b + 256 + 2 * rad_b;
    cudaError_t e = cudaMalloc(&p->block, bytes);
    if (e != cudaSuccess) {
        delete p;
        set_error("planner allocation of %zu bytes failed: %s", bytes, cudaGetErrorString(e));
        return e == cudaErrorMemoryAllocation ? GBMP_ERR_OUT_OF_MEMORY : GBMP_ERR_CUDA;
    }
    auto *b = static_cast<unsigned char *>(p->block);
    RrtcDev &D = p->dev;
    D.nodes[0] = (float *)b; D.nodes[1] = (float *)(b + nodes_b);
    D.parent[0] = (int *)(b + 2 * nodes_b); D.parent[1] = (int *)(b + 2 * nodes_b + par_b);
    int *ints = (int *)(b + 2 * nodes_b + 2 * par_b);
    D.size = ints; D.state = ints + 4; D.path_len = ints + 16;
    D.cap = max_nodes; D.stride = p->stride; D.path_cap = path_cap;
    D.radii[0] = (float *)(b + 2 * nodes_b + 2 * par_b + 256);
    D.radii[1] = (float *)(b + 2 * nodes_b + 2 * par_b + 256 + rad_b);
    p->dirty[0] = p->dirty[1] = p->dirty_radii[0] = p->dirty_radii[1] = max_nodes;
    void *mapped = nullptr, *mapped_io = nullptr;
    const size_t io_b = sizeof(int) * 16 + sizeof(float) * (size_t)r->L * (1 + kStagedGoals);
    if (cudaEventCreate(&p->ev0) != cudaSuccess || cudaEventCreate(&p->ev1) != cudaSuccess ||
        cudaHostAlloc((void **)&p->h_path, path_b, cudaHostAllocMapped) != cudaSuccess ||
        cudaHostGetDevicePointer(&mapped, p->h_path, 0) != cudaSuccess ||
        cudaHostAlloc((void **)&p->h_io, io_b, cudaHostAllocMapped) != cudaSuccess ||
        cudaHostGetDevicePointer(&mapped_io, p->h_io, 0) != cudaSuccess) {
        gbmp_planner_destroy(p);
        set_error("planner events or pinned buffers could not be created");
        return GBMP_ERR_CUDA;
    }
    D.path = static_cast<float *>(mapped);
    p->d_io = static_cast<int *>(mapped_io);
    *out = p;
    return GBMP_OK;
}

gbmp_status gbmp_planner_destroy(gbmp_planner p) {
    if (!p) return GBMP_OK;
    if (p->ev0) cudaEventDestroy(p->ev0);
    if (p->ev1) cudaEventDestroy(p->ev1);
    if (p->h_path) cudaFreeHost(p->h_path);
    if (p->h_io) cudaFreeHost(p->h_io);
    if (p->block) cudaFree(p->block);
    delete p;
    return GBMP_OK;
}

gbmp_status gbmp_rrtc_solve(gbmp_planner p, gbmp_env env, const float *h_start, const float *h_goal,
                            const gbmp_rrtc_settings *s, float *h_path, int32_t path_cap, gbmp_rrtc_result *res,
                            void *stream) {
    return gbmp_rrtc_solve_goals(p, env, h_start, h_goal, 1, s, h_path, path_cap, res, stream);
}

gbmp_status gbmp_rrtc_solve_goals(gbmp_planner p, gbmp_env env, const float *h_start, const float *h_goals,
                                  int32_t n_goals, const gbmp_rrtc_settings *s, float *h_path, int32_t path_cap,
                                  gbmp_rrtc_result *res, void *stream) {
    GBMP_CHECK_ARG(p && env && h_start && h_goals && s && res, "NULL argument");
    gbmp_robot r = p->robot;
    const int L = r->L;
    GBMP_CHECK_ARG(n_goals >= 1 && n_goals <= p->cap, "n_goals %d outside [1, %d]", n_goals, p->cap);
    GBMP_CHECK_ARG(s->lanes >= 1 && s->lanes <= (1 << 20), "lanes %d outside [1, 2^20]", s->lanes);
    GBMP_CHECK_ARG(s->range > 0.f && std::isfinite(s->range), "range must be > 0");
    GBMP_CHECK_ARG(s->max_iters >= 1, "max_iters < 1");
    float step_res = 0.f;
    GBMP_CHECK_ARG(plan_step(s, r->resolution, &step_res), "unknown step rule or resolution out of range");
    GBMP_CHECK_ARG(plan_dd_ok(s), "dynamic domain needs 0 <= dd_alpha < 1 and positive radii");
    int balance = 1;
    float tree_ratio = 0.5f;
    GBMP_CHECK_ARG(plan_balance(s, &balance, &tree_ratio), "unknown balance strategy %d or tree ratio", s->balance);
    for (int j = 0; j < L; ++j) GBMP_CHECK_ARG(std::isfinite(h_start[j]), "start not finite");
    for (long long j = 0; j < (long long)n_goals * L; ++j) GBMP_CHECK_ARG(std::isfinite(h_goals[j]), "goal not finite");
    memset(res, 0, sizeof *res);
    cudaStream_t st = (cudaStream_t)stream;
    const RrtcDev &D = p->dev;
    // reset (RobotSolver.cu:361-388 with a float sentinel), one launch: only the slots
    // written since the last reset are re-poisoned (a solve of a 1,000,000-node planner
    // otherwise re-poisons 64 MB of trees); start and goals come from the mapped pinned
    // input block, the goals past kStagedGoals by a copy after the reset
    const long long w0 = (long long)std::max(p->dirty[0], 1) * p->stride;
    const long long w1 = (long long)std::max(p->dirty[1], n_goals) * p->stride;
    const int r0 = s->dynamic_domain ? p->dirty_radii[0] : 0, r1 = s->dynamic_domain ? p->dirty_radii[1] : 0;
    if (s->dynamic_domain) p->dirty_radii[0] = p->dirty_radii[1] = 0;
    float *in = reinterpret_cast<float *>(p->h_io + 16);
    memcpy(in, h_start, sizeof(float) * L);
    memcpy(in + L, h_goals, sizeof(float) * (size_t)std::min(n_goals, kStagedGoals) * L);
    const double lim = s->time_limit_s > 0.0 ? s->time_limit_s : 10.0;
    {
        const long long most = std::max(std::max(w0, w1), (long long)std::max(r0, r1));
        const int blocks = (int)std::max(1LL, std::min<long long>((most + 255) / 256, 8LL * r->num_sms));
        ProfScope ps(GBMP_PROF_OTHER, st);
        k_rrtc_init<<<blocks, 256, 0, st>>>(D, L, w0, w1, r0, r1, reinterpret_cast<const float *>(p->d_io + 16),
                                            n_goals, (unsigned long long)(lim * 1e9));
    }
    GBMP_CUDA(cudaGetLastError());
    if (n_goals > kStagedGoals)
        GBMP_CUDA(cudaMemcpy2DAsync(D.nodes[1] + (size_t)kStagedGoals * p->stride, sizeof(float) * p->stride,
                                    h_goals + (size_t)kStagedGoals * L, sizeof(float) * L, sizeof(float) * L,
                                    n_goals - kStagedGoals, cudaMemcpyHostToDevice, st));
    // until this solve's tree sizes are read back, every slot counts as written
    p->dirty[0] = p->dirty[1] = p->cap;
    if (s->dynamic_domain) p->dirty_radii[0] = p->dirty_radii[1] = p->cap;

    const DevEnv E = env->dev();
    DevRobot DR = r->dev;
    DR.work = nullptr;
    const int nwords = env_words(E.ns, E.nb, E.nc);
    const size_t smem = rrtc_block_smem(DR, nwords, false);
    RrtcParams prm;
    prm.lanes = s->lanes;
    prm.max_iters = s->max_iters;
    prm.rule = s->step_rule;
    prm.range = s->range;
    prm.res = step_res;
    prm.seed = s->seed;
    prm.dd = s->dynamic_domain ? 1 : 0;
    prm.dd_alpha = s->dd_alpha;
    prm.dd_radius = s->dd_radius;
    prm.dd_min = s->dd_min_radius;
    prm.balance = balance;
    prm.tree_ratio = tree_ratio;
    // device deadline: set by the reset kernel
    prm.deadline_ns = 0;
    prm.deadline_ptr = (unsigned long long *)(D.state + 8);
    cudaEvent_t e0 = p->ev0, e1 = p->ev1;
    GBMP_CUDA(cudaEventRecord(e0, st));
    gbmp_status stt = GBMP_OK;
    {
        ProfScope ps(GBMP_PROF_OTHER, st);
        const bool cull = DR.cull != 0;
        const cudaError_t ce = DR.spl <= 4 ? rrtc_launch_lo(DR.spl, cull, s->lanes, smem, st, DR, E, D, prm)
                                           : rrtc_launch_hi(DR.spl, cull, s->lanes, smem, st, DR, E, D, prm);
        if (ce != cudaSuccess) {
            set_error("planning kernel launch (%zu bytes of shared memory): %s", smem, cudaGetErrorString(ce));
            stt = ce == cudaErrorInvalidValue ? GBMP_ERR_CAPACITY : GBMP_ERR_CUDA;
        }
    }
    if (stt) return stt;
    GBMP_CUDA(cudaGetLastError());
    GBMP_CUDA(cudaEventRecord(e1, st));
    {
        ProfScope ps(GBMP_PROF_OTHER, st);
        k_rrtc_trace<<<1, 32, 0, st>>>(D, L, p->d_io);
    }
    GBMP_CUDA(cudaGetLastError());
    GBMP_CUDA(cudaStreamSynchronize(st));
    const volatile int *io = p->h_io;
    int h_state[6], h_size[2];
    for (int k = 0; k < 6; ++k) h_state[k] = io[k];
    h_size[0] = io[6];
    h_size[1] = io[7];
    const int h_len = io[8];
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    p->dirty[0] = std::min(std::max(h_size[0], 1), p->cap);
    p->dirty[1] = std::min(std::max(h_size[1], n_goals), p->cap);
    if (s->dynamic_domain) {
        p->dirty_radii[0] = p->dirty[0];
        p->dirty_radii[1] = p->dirty[1];
    }
    res->status = h_state[0];
    res->solved = h_state[0] == kStSolved;
    res->start_tree_size = std::min(h_size[0], p->cap);
    res->goal_tree_size = std::min(h_size[1], p->cap);
    res->iterations = h_state[5];
    res->kernel_ms = ms;
    res->path_len = 0;
    if (res->solved) {
        if (h_len < 0 || h_len > path_cap || (h_path == nullptr)) {
            res->path_len = h_len < 0 ? -h_len : h_len;
            set_error("path of %d states does not fit the buffer of %d", res->path_len, path_cap);
            return GBMP_ERR_CAPACITY;
        }
        memcpy(h_path, p->h_path, sizeof(float) * (size_t)h_len * L);   // written by the trace, before the sync
        res->path_len = h_len;
        double cost = 0.0;
        for (int k = 1; k < h_len; ++k) {
            double s2 = 0.0;
            for (int j = 0; j < L; ++j)
                if (r->active[j]) {
                    const double d = (double)h_path[k * L + j] - h_path[(k - 1) * L + j];
                    s2 += d * d;
                }
            cost += std::sqrt(s2);
        }
        res->cost = (float)cost;
        return GBMP_OK;
    }
    if (h_state[0] == kStDeadline) {
        set_error("no path within %.3f s", lim);
        return GBMP_ERR_TIMEOUT;
    }
    set_error("no path (status %d: node cap or iteration cap)", h_state[0]);
    return GBMP_ERR_NOT_SOLVED;
}

}  // extern "C"

// ---------------------------------------------------------------------------------
// Batched planning (many heterogeneous problems in one persistent launch).
// ---------------------------------------------------------------------------------
struct gbmp_batch_planner_s {
    int max_problems = 0, cap = 0, max_links = 0, path_cap = 0, stride = 0;
    void *pool = nullptr;                 // per-problem trees, parents, ints, paths
    size_t per_problem = 0;
    BatchProblem *d_table = nullptr;      // device problem table
    BatchProblem *h_table = nullptr;      // pinned host mirror
    float *d_roots = nullptr, *h_roots = nullptr;   // [max_problems * 2 * max_links]
    int *d_summary = nullptr, *h_summary = nullptr; // [max_problems * 8]
    int *h_flags = nullptr, *d_flags = nullptr;     // host-mapped completion words [max_problems]
    // launch in progress (between batch_begin and batch_end)
    int cur_n = 0;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    unsigned long long *d_deadline = nullptr;   // [0] deadline, [1] round-robin counter
    std::vector<int> prev;                // 2 per problem
    // captured graphs by launch shape (a few shapes, least recently used evicted)
    struct Captured {
        long long key[12];
        cudaGraphExec_t exec;
        long long used;
    };
    std::vector<Captured> graphs;
    long long use_clock = 0;
    std::mutex mu;
};

static gbmp_status batch_launch(gbmp_batch_planner b, int n, int lpp, const RrtcParams &prm, int spl, bool cull,
                                size_t smem, double limit_s, cudaStream_t st) {
    GBMP_CUDA(cudaMemcpyAsync(b->d_table, b->h_table, sizeof(BatchProblem) * n, cudaMemcpyHostToDevice, st));
    GBMP_CUDA(cudaMemcpyAsync(b->d_roots, b->h_roots, sizeof(float) * (size_t)n * 2 * b->max_links,
                              cudaMemcpyHostToDevice, st));
    {
        ProfScope ps(GBMP_PROF_OTHER, st);
        k_rrtc_batch_reset<<<dim3(8, n), 256, 0, st>>>(b->d_table, n, b->d_deadline,
                                                      (unsigned long long)(limit_s * 1e9));
    }
    GBMP_CUDA(cudaGetLastError());
    gbmp_status stt = GBMP_OK;
    {
        ProfScope ps(GBMP_PROF_OTHER, st);
        int *rr = (int *)(b->d_deadline + 1);
        const cudaError_t ce = spl <= 4 ? rrtc_batch_launch_lo(spl, cull, n * lpp, smem, st, b->d_table, n, lpp, prm, rr)
                                        : rrtc_batch_launch_hi(spl, cull, n * lpp, smem, st, b->d_table, n, lpp, prm, rr);
        if (ce != cudaSuccess) {
            set_error("planning kernel launch (%zu bytes of shared memory): %s", smem, cudaGetErrorString(ce));
            stt = ce == cudaErrorInvalidValue ? GBMP_ERR_CAPACITY : GBMP_ERR_CUDA;
        }
    }
    if (stt) return stt;
    GBMP_CUDA(cudaGetLastError());
    {
        ProfScope ps(GBMP_PROF_OTHER, st);
        k_rrtc_batch_trace<<<n, 32, 0, st>>>(b->d_table, n, b->d_summary);
    }
    {
        ProfScope ps(GBMP_PROF_OTHER, st);
        k_rrtc_batch_finish<<<(n + 127) / 128, 128, 0, st>>>(b->d_table, n);
    }
    GBMP_CUDA(cudaGetLastError());
    GBMP_CUDA(cudaMemcpyAsync(b->h_summary, b->d_summary, sizeof(int) * 8 * n, cudaMemcpyDeviceToHost, st));
    return GBMP_OK;
}

extern "C" {

gbmp_status gbmp_batch_planner_create(int32_t max_problems, int32_t max_nodes, int32_t max_links, int32_t path_cap,
                                      gbmp_batch_planner *out) {
    GBMP_CHECK_ARG(out, "out is NULL");
    *out = nullptr;
    GBMP_CHECK_ARG(max_problems >= 1 && max_problems <= 65535, "max_problems %d outside [1, 65535]", max_problems);
    GBMP_CHECK_ARG(max_nodes >= 2 && max_nodes <= (1 << 24), "max_nodes %d outside [2, 2^24]", max_nodes);
    GBMP_CHECK_ARG(max_links >= 1 && max_links <= kMaxLinks, "max_links %d outside [1, %d]", max_links, kMaxLinks);
    GBMP_CHECK_ARG(path_cap >= 2, "path_cap < 2");
    auto *b = new gbmp_batch_planner_s();
    b->max_problems = max_problems;
    b->cap = max_nodes;
    b->max_links = max_links;
    b->path_cap = path_cap;
    b->stride = (max_links + 3) & ~3;
    const size_t nodes_b = align16(sizeof(float) * (size_t)max_nodes * b->stride);
    const size_t par_b = align16(sizeof(int) * (size_t)max_nodes);
    const size_t rad_b = align16(sizeof(float) * (size_t)max_nodes);   // dynamic-domain radii, per tree
    b->per_problem = 2 * nodes_b + 2 * par_b + 256 + align16(sizeof(float) * (size_t)path_cap * max_links) + 2 * rad_b;
    cudaError_t e = cudaMalloc(&b->pool, b->per_problem * max_problems);
    if (e == cudaSuccess) e = cudaMalloc(&b->d_table, sizeof(BatchProblem) * max_problems);
    if (e == cudaSuccess) e = cudaMallocHost(&b->h_table, sizeof(BatchProblem) * max_problems);
    if (e == cudaSuccess) e = cudaMalloc(&b->d_roots, sizeof(float) * (size_t)max_problems * 2 * max_links);
    if (e == cudaSuccess) e = cudaMallocHost(&b->h_roots, sizeof(float) * (size_t)max_problems * 2 * max_links);
    if (e == cudaSuccess) e = cudaMalloc(&b->d_summary, sizeof(int) * 8 * max_problems);
    if (e == cudaSuccess) e = cudaMallocHost(&b->h_summary, sizeof(int) * 8 * max_problems);
    if (e == cudaSuccess) e = cudaMalloc(&b->d_deadline, 2 * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaHostAlloc(&b->h_flags, sizeof(int) * max_problems, cudaHostAllocMapped);
    if (e == cudaSuccess) e = cudaHostGetDevicePointer((void **)&b->d_flags, b->h_flags, 0);
    if (e == cudaSuccess) e = cudaEventCreate(&b->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&b->ev1);
    if (e != cudaSuccess) {
        set_error("batch planner allocation failed: %s", cudaGetErrorString(e));
        gbmp_batch_planner_destroy(b);
        return e == cudaErrorMemoryAllocation ? GBMP_ERR_OUT_OF_MEMORY : GBMP_ERR_CUDA;
    }
    // every tree starts fully reset once
    e = cudaMemset(b->pool, 0xff, b->per_problem * max_problems);
    if (e == cudaSuccess)   // every dynamic-domain radius unset (kRadiusUnset = bytes 0x7f)
        e = cudaMemset2D(static_cast<unsigned char *>(b->pool) + b->per_problem - 2 * rad_b, b->per_problem, 0x7f,
                         2 * rad_b, max_problems);
    if (e != cudaSuccess) {
        set_error("batch planner reset failed: %s", cudaGetErrorString(e));
        gbmp_batch_planner_destroy(b);
        return GBMP_ERR_CUDA;
    }
    b->prev.assign(2 * max_problems, 1);
    *out = b;
    return GBMP_OK;
}

gbmp_status gbmp_batch_planner_destroy(gbmp_batch_planner b) {
    if (!b) return GBMP_OK;
    for (auto &g : b->graphs) cudaGraphExecDestroy(g.exec);
    if (b->pool) cudaFree(b->pool);
    if (b->d_table) cudaFree(b->d_table);
    if (b->h_table) cudaFreeHost(b->h_table);
    if (b->d_roots) cudaFree(b->d_roots);
    if (b->h_roots) cudaFreeHost(b->h_roots);
    if (b->d_summary) cudaFree(b->d_summary);
    if (b->h_summary) cudaFreeHost(b->h_summary);
    if (b->d_deadline) cudaFree(b->d_deadline);
    if (b->h_flags) cudaFreeHost(b->h_flags);
    if (b->ev0) cudaEventDestroy(b->ev0);
    if (b->ev1) cudaEventDestroy(b->ev1);
    delete b;
    return GBMP_OK;
}

gbmp_status gbmp_rrtc_solve_batch(gbmp_batch_planner b, int32_t n, const gbmp_rrtc_problem *problems,
                                  const gbmp_rrtc_settings *s, int32_t lanes_per_problem, int32_t use_graph,
                                  gbmp_rrtc_result *results, float *h_paths, void *stream) {
    GBMP_CHECK_ARG(b && problems && s && results, "NULL argument");
    std::lock_guard<std::mutex> lock(b->mu);
    gbmp_status st = gbmp::batch_begin(b, n, problems, s, lanes_per_problem, use_graph, (cudaStream_t)stream);
    if (st) return st;
    return gbmp::batch_end(b, problems, results, h_paths, (cudaStream_t)stream);
}

}  // extern "C"

namespace gbmp {

// Lanes-per-problem candidates of the autotuned batched solve, each timed twice.
static LaneTuner &lane_tuner() {
    static LaneTuner t({4, 8, 16, 32, 64}, 2);
    return t;
}

// Signature of a batched solve's shape: device, problem count, graph use, the multiset of
// per-problem (links, sphere bucket, obstacle bucket), and the settings that change the
// work of a lane.
static gbmp_status batch_shape_key(int n, const gbmp_rrtc_problem *problems, const gbmp_rrtc_settings *s,
                                   int use_graph, uint64_t *key) {
    GBMP_CHECK_ARG(problems && s && n >= 1, "NULL argument or n < 1");
    int dev = 0;
    GBMP_CUDA(cudaGetDevice(&dev));
    ShapeKey k;
    k.add((uint64_t)dev);
    k.add((uint64_t)n);
    k.add((uint64_t)(use_graph != 0));
    std::vector<uint64_t> shapes((size_t)n);
    for (int i = 0; i < n; ++i) {
        GBMP_CHECK_ARG(problems[i].robot && problems[i].env, "problem %d: robot/env is NULL", i);
        const gbmp_env e = problems[i].env;
        shapes[(size_t)i] = ((uint64_t)problems[i].robot->L << 48) | (shape_bucket(problems[i].robot->S) << 24) |
                            shape_bucket((int64_t)e->ns + e->nb + e->nc);
    }
    std::sort(shapes.begin(), shapes.end());
    for (uint64_t v : shapes) k.add(v);
    uint32_t fr = 0, fs = 0;
    memcpy(&fr, &s->range, 4);
    memcpy(&fs, &s->resolution, 4);
    k.add((uint64_t)s->max_iters);
    k.add(((uint64_t)fr << 32) | fs);
    k.add((uint64_t)(uint32_t)s->step_rule);
    k.add((uint64_t)(uint32_t)s->dynamic_domain);
    k.add((uint64_t)(uint32_t)s->balance);
    *key = k.hash;
    return GBMP_OK;
}

}  // namespace gbmp

extern "C" {

gbmp_status gbmp_rrtc_solve_batch_auto(gbmp_batch_planner b, int32_t n, const gbmp_rrtc_problem *problems,
                                       const gbmp_rrtc_settings *s, int32_t use_graph, gbmp_rrtc_result *results,
                                       float *h_paths, int32_t *lanes_used, void *stream) {
    GBMP_CHECK_ARG(b && problems && s && results, "NULL argument");
    GBMP_CHECK_ARG(n >= 1 && n <= b->max_problems, "n %d outside [1, %d]", n, b->max_problems);
    uint64_t key = 0;
    gbmp_status st = gbmp::batch_shape_key(n, problems, s, use_graph, &key);
    if (st) return st;
    const int max_lanes = (int)std::min<long long>(4096, (1LL << 30) / n);
    bool trial = false;
    const int lpp = gbmp::lane_tuner().choose(key, max_lanes, &trial);
    const auto t0 = std::chrono::steady_clock::now();
    st = gbmp_rrtc_solve_batch(b, n, problems, s, lpp, use_graph, results, h_paths, stream);
    const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    if (st == GBMP_OK && trial) gbmp::lane_tuner().report(key, lpp, ms);
    if (lanes_used) *lanes_used = lpp;
    return st;
}

gbmp_status gbmp_batch_autotune_lookup(int32_t n, const gbmp_rrtc_problem *problems, const gbmp_rrtc_settings *s,
                                       int32_t use_graph, int32_t *lanes, double *ms, int32_t capacity,
                                       int32_t *count, int32_t *chosen) {
    GBMP_CHECK_ARG(count && chosen, "NULL argument");
    uint64_t key = 0;
    gbmp_status st = gbmp::batch_shape_key(n, problems, s, use_graph, &key);
    if (st) return st;
    std::vector<int> cand;
    std::vector<double> t;
    int best = -1;
    *count = 0;
    *chosen = -1;
    if (!gbmp::lane_tuner().lookup(key, &cand, &t, &best)) return GBMP_OK;
    *count = (int32_t)cand.size();
    *chosen = best;
    for (int i = 0; i < (int)cand.size() && i < capacity; ++i) {
        if (lanes) lanes[i] = cand[(size_t)i];
        if (ms) ms[i] = t[(size_t)i];
    }
    return GBMP_OK;
}

gbmp_status gbmp_batch_autotune_reset(void) {
    gbmp::lane_tuner().reset();
    return GBMP_OK;
}

}  // extern "C"

namespace gbmp {

gbmp_status batch_begin(gbmp_batch_planner b, int n, const gbmp_rrtc_problem *problems, const gbmp_rrtc_settings *s,
                        int lanes_per_problem, int use_graph, cudaStream_t st) {
    GBMP_CHECK_ARG(n >= 1 && n <= b->max_problems, "n %d outside [1, %d]", n, b->max_problems);
    GBMP_CHECK_ARG(lanes_per_problem >= 1 && lanes_per_problem <= 4096, "lanes_per_problem outside [1, 4096]");
    GBMP_CHECK_ARG((long long)n * lanes_per_problem <= (1LL << 30), "too many blocks");
    GBMP_CHECK_ARG(s->range > 0.f && s->max_iters >= 1, "bad settings");
    GBMP_CHECK_ARG(plan_dd_ok(s), "dynamic domain needs 0 <= dd_alpha < 1 and positive radii");
    int balance = 1;
    float tree_ratio = 0.5f;
    GBMP_CHECK_ARG(plan_balance(s, &balance, &tree_ratio), "unknown balance strategy %d or tree ratio", s->balance);
    float step_res = 0.f;
    GBMP_CHECK_ARG(plan_step(s, problems[0].robot ? problems[0].robot->resolution : 0.f, &step_res),
                   "unknown step rule or resolution out of range");
    int spl = 1;
    bool cull = true;
    size_t smem = 0;
    auto *pool = static_cast<unsigned char *>(b->pool);
    const size_t nodes_b = align16(sizeof(float) * (size_t)b->cap * b->stride);
    const size_t par_b = align16(sizeof(int) * (size_t)b->cap);
    const size_t rad_b = align16(sizeof(float) * (size_t)b->cap);
    for (int i = 0; i < n; ++i) {
        const gbmp_rrtc_problem &pr = problems[i];
        GBMP_CHECK_ARG(pr.robot && pr.env && pr.start && pr.goal, "problem %d has a NULL field", i);
        GBMP_CHECK_ARG(pr.robot->L <= b->max_links, "problem %d: %d links > max_links %d", i, pr.robot->L,
                       b->max_links);
        const DevRobot &R = pr.robot->dev;
        const DevEnv E = pr.env->dev();
        spl = std::max(spl, R.spl);
        cull = cull && R.cull;
        smem = std::max(smem, rrtc_block_smem(R, env_words(E.ns, E.nb, E.nc), true));
        BatchProblem &bp = b->h_table[i];
        bp.R = R;
        bp.R.work = nullptr;
        bp.E = E;
        unsigned char *base = pool + b->per_problem * i;
        bp.P.nodes[0] = (float *)base;
        bp.P.nodes[1] = (float *)(base + nodes_b);
        bp.P.parent[0] = (int *)(base + 2 * nodes_b);
        bp.P.parent[1] = (int *)(base + 2 * nodes_b + par_b);
        int *ints = (int *)(base + 2 * nodes_b + 2 * par_b);
        bp.P.size = ints;
        bp.P.state = ints + 4;
        bp.P.path_len = ints + 16;
        bp.P.path = (float *)(base + 2 * nodes_b + 2 * par_b + 256);
        bp.P.cap = b->cap;
        bp.P.stride = (pr.robot->L + 3) & ~3;   // its own joints, padded to float4 words
        // dynamic-domain radii: the last two regions of the problem's block, reset by every
        // solve (used only when the settings turn the dynamic domain on)
        bp.P.radii[0] = (float *)(base + b->per_problem - 2 * rad_b);
        bp.P.radii[1] = (float *)(base + b->per_problem - rad_b);
        bp.P.path_cap = b->path_cap;
        bp.P.flag = b->d_flags + i;
        bp.seed = pr.seed;
        bp.start = b->d_roots + (size_t)i * 2 * b->max_links;
        bp.goal = bp.start + b->max_links;
        bp.prev[0] = b->prev[2 * i];
        bp.prev[1] = b->prev[2 * i + 1];
        for (int j = 0; j < pr.robot->L; ++j) {
            GBMP_CHECK_ARG(std::isfinite(pr.start[j]) && std::isfinite(pr.goal[j]), "problem %d: start/goal not finite", i);
            b->h_roots[(size_t)i * 2 * b->max_links + j] = pr.start[j];
            b->h_roots[(size_t)i * 2 * b->max_links + b->max_links + j] = pr.goal[j];
        }
        b->h_flags[i] = 0;
    }
    RrtcParams prm;
    prm.lanes = lanes_per_problem;
    prm.max_iters = s->max_iters;
    prm.rule = s->step_rule;
    prm.range = s->range;
    prm.res = step_res;
    prm.seed = 0;
    prm.deadline_ns = 0;
    prm.deadline_ptr = b->d_deadline;
    prm.dd = s->dynamic_domain ? 1 : 0;
    prm.dd_alpha = s->dd_alpha;
    prm.dd_radius = s->dd_radius;
    prm.dd_min = s->dd_min_radius;
    prm.balance = balance;
    prm.tree_ratio = tree_ratio;
    const double lim = s->time_limit_s > 0.0 ? s->time_limit_s : 10.0;
    b->cur_n = n;
    GBMP_CUDA(cudaEventRecord(b->ev0, st));
    if (use_graph) {
        float dd_f[3] = {prm.dd_alpha, prm.dd_radius, prm.dd_min};
        unsigned dd_bits[3];
        memcpy(dd_bits, dd_f, sizeof dd_bits);
        unsigned tr_bits = 0;
        memcpy(&tr_bits, &prm.tree_ratio, sizeof tr_bits);
        const long long key[12] = {n, lanes_per_problem, (long long)smem, spl, cull, s->max_iters,
                                   (long long)(lim * 1e6), (long long)(prm.range * 1e6) ^ ((long long)(prm.res * 1e9) << 20),
                                   prm.dd ? (long long)dd_bits[0] | ((long long)dd_bits[1] << 32) : -1,
                                   prm.dd ? (long long)dd_bits[2] : -1, prm.balance, (long long)tr_bits};
        cudaGraphExec_t exec = nullptr;
        for (auto &g : b->graphs)
            if (memcmp(key, g.key, sizeof key) == 0) { exec = g.exec; g.used = ++b->use_clock; }
        if (!exec) {
            if (b->graphs.size() >= 8) {
                auto lru = std::min_element(b->graphs.begin(), b->graphs.end(),
                                            [](const gbmp_batch_planner_s::Captured &x,
                                               const gbmp_batch_planner_s::Captured &y) { return x.used < y.used; });
                cudaGraphExecDestroy(lru->exec);
                b->graphs.erase(lru);
            }
            cudaStream_t cap_st;
            GBMP_CUDA(cudaStreamCreateWithFlags(&cap_st, cudaStreamNonBlocking));
            GBMP_CUDA(cudaStreamBeginCapture(cap_st, cudaStreamCaptureModeThreadLocal));
            gbmp_status bs = batch_launch(b, n, lanes_per_problem, prm, spl, cull, smem, lim, cap_st);
            cudaGraph_t g = nullptr;
            cudaError_t ce = cudaStreamEndCapture(cap_st, &g);
            cudaStreamDestroy(cap_st);
            if (bs) { if (g) cudaGraphDestroy(g); return bs; }
            if (ce != cudaSuccess) { set_error("graph capture failed: %s", cudaGetErrorString(ce)); return GBMP_ERR_CUDA; }
            ce = cudaGraphInstantiate(&exec, g, 0);
            cudaGraphDestroy(g);
            if (ce != cudaSuccess) { set_error("graph instantiate failed: %s", cudaGetErrorString(ce)); return GBMP_ERR_CUDA; }
            gbmp_batch_planner_s::Captured c;
            memcpy(c.key, key, sizeof key);
            c.exec = exec;
            c.used = ++b->use_clock;
            b->graphs.push_back(c);
        }
        count_launch(4);
        GBMP_CUDA(cudaGraphLaunch(exec, st));
    } else {
        gbmp_status bs = batch_launch(b, n, lanes_per_problem, prm, spl, cull, smem, lim, st);
        if (bs) return bs;
    }
    GBMP_CUDA(cudaEventRecord(b->ev1, st));
    return GBMP_OK;
}

int batch_flag(gbmp_batch_planner b, int i) { return *(volatile int *)(b->h_flags + i); }

gbmp_status batch_copy_path(gbmp_batch_planner b, int i, int L, int len, float *h_path, cudaStream_t st) {
    const float *src = b->h_table[i].P.path;
    GBMP_CUDA(cudaMemcpyAsync(h_path, src, sizeof(float) * (size_t)len * L, cudaMemcpyDeviceToHost, st));
    GBMP_CUDA(cudaStreamSynchronize(st));
    return GBMP_OK;
}

gbmp_status batch_end(gbmp_batch_planner b, const gbmp_rrtc_problem *problems, gbmp_rrtc_result *results,
                      float *h_paths, cudaStream_t st) {
    const int n = b->cur_n;
    GBMP_CUDA(cudaStreamSynchronize(st));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, b->ev0, b->ev1);
    int max_len = 0;
    for (int i = 0; i < n; ++i) {
        const int *o = b->h_summary + 8 * i;
        gbmp_rrtc_result &r = results[i];
        memset(&r, 0, sizeof r);
        r.status = o[0];
        r.solved = o[0] == kStSolved && o[1] > 0;
        r.path_len = o[1] > 0 ? o[1] : 0;
        r.start_tree_size = o[2];
        r.goal_tree_size = o[3];
        r.iterations = o[4];
        r.kernel_ms = ms;
        b->prev[2 * i] = std::max(o[2], 1) * b->h_table[i].P.stride;
        b->prev[2 * i + 1] = std::max(o[3], 1) * b->h_table[i].P.stride;
        max_len = std::max(max_len, r.path_len);
    }
    if (h_paths && max_len > 0) {
        // one pitched copy: rows of max_len * max_links floats from every problem's path buffer
        const size_t pitch_src = b->per_problem;
        const size_t row = sizeof(float) * (size_t)max_len * b->max_links;
        const size_t pitch_dst = sizeof(float) * (size_t)b->path_cap * b->max_links;
        if (row <= pitch_dst) {
            GBMP_CUDA(cudaMemcpy2DAsync(h_paths, pitch_dst, b->h_table[0].P.path, pitch_src, row, n,
                                        cudaMemcpyDeviceToHost, st));
            GBMP_CUDA(cudaStreamSynchronize(st));
        }
        for (int i = 0; i < n; ++i) {
            gbmp_rrtc_result &r = results[i];
            if (!r.solved) continue;
            const int L = problems[i].robot->L;
            const float *pth = h_paths + (size_t)i * b->path_cap * b->max_links;
            double cost = 0.0;
            for (int k = 1; k < r.path_len; ++k) {
                double s2 = 0.0;
                for (int j = 0; j < L; ++j)
                    if (problems[i].robot->active[j]) {
                        const double d = (double)pth[k * L + j] - pth[(k - 1) * L + j];
                        s2 += d * d;
                    }
                cost += std::sqrt(s2);
            }
            r.cost = (float)cost;
        }
    }
    return GBMP_OK;
}

std::mutex &batch_mutex(gbmp_batch_planner b) { return b->mu; }

}  // namespace gbmp

