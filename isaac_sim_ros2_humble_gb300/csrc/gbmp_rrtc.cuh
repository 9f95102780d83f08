// gbmp_rrtc.cuh -- types and kernel declarations of the parallel RRT-Connect planner
// (gbmp_rrtc.cu).  The planning kernels are defined in gbmp_rrtc_device.cuh and
// instantiated, one spheres-per-lane range each, in the gbmp_rrtc_k*.cu / gbmp_rrtc_b*.cu
// translation units so that they compile in parallel.
#pragma once

#include "gbmp_chunk_device.cuh"
#include "gbmp_internal.h"

namespace gbmp {

constexpr int kRrtcWarps = 4;
constexpr int kRrtcThreads = kRrtcWarps * kWarp;
// States per chunk of the planner's edge checks: an extension of at most `range` has a
// dozen states or so, split over the lane's four warps, so chunks stay small (and so
// does the per-warp chunk scratch in shared memory).
constexpr int kRrtcChunk = 4;

// Shared memory of a planning block: staged tables, four warp scratches, the lane's
// joint vectors and flags, and, when the edge checks run by chunks (batched planning,
// robots of at most 32 sphere groups), four chunk scratches.
__host__ __device__ inline size_t rrtc_misc_bytes() { return align16(6 * kMaxLinks * 4 + 256); }
__host__ __device__ inline size_t rrtc_block_smem(const DevRobot &R, int nwords, bool chunks) {
    return smem_tables_bytes(R, nwords) + smem_warp_bytes(R) * kRrtcWarps + rrtc_misc_bytes() +
           (chunks && R.cull ? smem_chunk_bytes(R, kRrtcChunk) * kRrtcWarps : 0);
}

enum : int { kStRunning = 0, kStSolved = 1, kStNodeCap = 2, kStIterCap = 3, kStDeadline = 4 };

struct RrtcDev {
    float *nodes[2];          // [cap * stride], NaN until written
    float *radii[2];          // [cap] dynamic-domain radii (kRadiusUnset until a failure), or null
    int *parent[2];           // [cap]
    int *size;                // [2] allocated slots per tree
    int *state;               // [0] status, [1] winning lane, [2] tree of the new node,
                              // [3] node in that tree, [4] node in the other tree, [5] max iteration
    float *path;              // [path_cap * L]
    int *path_len;            // [1], -1 if the path buffer was too small
    int cap, stride, path_cap;
    volatile int *flag;       // host-mapped completion word (batched solves) or null:
                              // path length + 1 when solved, -status when ended without a path
};

struct RrtcParams {
    int lanes, max_iters, rule;
    float range, res;
    unsigned long long seed;
    unsigned long long deadline_ns;   // absolute %globaltimer value, or
    const unsigned long long *deadline_ptr;   // read from device memory when non-null
    int dd = 0;                       // dynamic domain on (needs RrtcDev::radii)
    float dd_alpha = 0.f, dd_radius = 0.f, dd_min = 0.f;
    int balance = 3;                  // 0 none, 1 pRRTC size, 2 pRRTC swap, 3 proportional
    float tree_ratio = 0.5f;
};

// Lane hash in [0, 1) (Fibonacci hashing of the lane index): the share of lanes below h
// stands for pRRTC's block index over the block count, whatever the lane count and
// however batched lanes are numbered.
__host__ __device__ inline float lane_hash(int lane) {
    return (float)(((unsigned)lane * 2654435769u) >> 8) * (1.0f / 16777216.0f);
}

// Tree a lane grows (pRRTC.cu:348-371).  n0, n1: tree sizes; cur: the lane's tree in its
// previous iteration, -1 at its first (half the lanes per tree, pRRTC's iteration 1).
// Strategy 3 (the default) splits the lanes in proportion to the other tree's share at
// every size; strategy 1 (pRRTC's) does so while the trees differ by less than 1.5 x
// lanes nodes, else grows tree 0 while its share is below tree_ratio; strategy 2 swaps a
// lane's tree while the size difference relative to it is below tree_ratio.  (Under
// strategy 1 every lane grows the smaller tree once they differ: a tree trapped in a
// pocket of free space then takes all lanes, the other tree stops growing, and an
// unsolvable problem runs to its iteration cap or deadline instead of its node cap.)
__host__ __device__ inline int balance_tree(int balance, float tree_ratio, int lanes, int n0, int n1, float h,
                                            int cur) {
    if (cur < 0 || balance == 0) return h < 0.5f ? 0 : 1;
    if (balance == 3) return h < 1.f - (float)n0 / (float)(n0 + n1 > 1 ? n0 + n1 : 1) ? 0 : 1;
    if (balance == 2) {
        const int nt = cur == 0 ? n0 : n1, no = cur == 0 ? n1 : n0;
        const float ratio = (float)abs(nt - no) / (float)(nt > 1 ? nt : 1);
        return ratio < tree_ratio ? 1 - cur : cur;
    }
    const float ratio = (float)n0 / (float)(n0 + n1 > 1 ? n0 + n1 : 1);
    if ((float)abs(n0 - n1) < 1.5f * (float)lanes) return h < 1.f - ratio ? 0 : 1;
    return ratio < tree_ratio ? 0 : 1;
}

// Dynamic-domain radius of a node that has not failed yet (the bytes 0x7f of a memset;
// 3.4e38, so it never rejects a sample).
constexpr unsigned kRadiusUnset = 0x7f7f7f7fu;

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// A problem of a batched launch: its robot, scene, trees and Philox key.
struct BatchProblem {
    DevRobot R;
    DevEnv E;
    RrtcDev P;
    unsigned long long seed;
    const float *start, *goal;      // device copies of the roots
    int prev[2];                    // node words the previous solve wrote (to reset)
};

// Launchers of the planning kernels, defined by the instantiation units: *_lo for 1 to 4
// spheres per lane, *_hi for 5 to 8.  Each sets the kernel's dynamic shared-memory limit
// to `smem` and launches `grid` blocks of kRrtcThreads on `st`; the CUDA error of either
// step is returned.
cudaError_t rrtc_launch_lo(int spl, bool cull, int grid, size_t smem, cudaStream_t st, const DevRobot &R,
                           const DevEnv &E, const RrtcDev &P, const RrtcParams &prm);
cudaError_t rrtc_launch_hi(int spl, bool cull, int grid, size_t smem, cudaStream_t st, const DevRobot &R,
                           const DevEnv &E, const RrtcDev &P, const RrtcParams &prm);
cudaError_t rrtc_batch_launch_lo(int spl, bool cull, int grid, size_t smem, cudaStream_t st,
                                 const BatchProblem *probs, int n, int lanes_per_problem, const RrtcParams &prm,
                                 int *rr);
cudaError_t rrtc_batch_launch_hi(int spl, bool cull, int grid, size_t smem, cudaStream_t st,
                                 const BatchProblem *probs, int n, int lanes_per_problem, const RrtcParams &prm,
                                 int *rr);

}  // namespace gbmp
