// gbmp_rrtc_device.cuh -- device code of the parallel RRT-Connect planner: the
// extension lane shared by the single-problem and batched planning kernels, and those
// kernels.  Included only by the instantiation units gbmp_rrtc_k*.cu / gbmp_rrtc_b*.cu.
#pragma once

#include <climits>

#include "gbmp_philox.h"
#include "gbmp_rrtc.cuh"

namespace gbmp {

// Bounded compare-and-swap update of a node's radius: after a failed extension (set to
// dd_radius if unset, else shrink towards dd_min) or a successful one (grow if set).  A
// radius is a sampling heuristic, so an update that loses 64 races in a row is dropped.
__device__ inline void dd_update(float *radius, bool failed, const RrtcParams &prm) {
    unsigned *p = reinterpret_cast<unsigned *>(radius);
    for (int tries = 0; tries < 64; ++tries) {
        const unsigned old = *(volatile unsigned *)p;
        float nw;
        if (old == kRadiusUnset) {
            if (!failed) return;
            nw = prm.dd_radius;
        } else {
            const float r = __uint_as_float(old);
            nw = failed ? fmaxf(__fmul_rn(r, __fadd_rn(1.f, -prm.dd_alpha)), prm.dd_min)
                        : __fmul_rn(r, __fadd_rn(1.f, prm.dd_alpha));
        }
        if (atomicCAS(p, old, __float_as_uint(nw)) == old) return;
    }
}

// Squared active-joint distance of one node (NW float4 words) from the query held in
// registers, accumulated joint by joint in index order; inactive joints add exactly 0.
// `written` clears if any coordinate still holds the NaN sentinel.  The words are read
// through L1 (the blocks on one SM scan the same trees): a node is written once, from
// the sentinel to its final value, so a line cached before the write can only show the
// sentinel, and the node is skipped as not yet written, as it is when the scan simply
// runs before the write (measured: shelf p50 0.82 against 0.86 ms, uneven batch 553-564
// against 574-579 ms).
template <int NW>
__device__ __forceinline__ float node_dist(const float4 *__restrict__ y, const float (&qr)[4 * NW], unsigned am, int L,
                                           bool &written) {
    float4 v4[NW];
#pragma unroll
    for (int k = 0; k < NW; ++k) v4[k] = __ldca(y + k);
    float s = 0.f;
#pragma unroll
    for (int k = 0; k < NW; ++k) {
        const float v[4] = {v4[k].x, v4[k].y, v4[k].z, v4[k].w};
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            const int j = 4 * k + c;
            if (j < L) {
                written &= v[c] == v[c];
                const float d = ((am >> j) & 1u) ? __fadd_rn(qr[j], -v[c]) : 0.f;
                s = __fmaf_rn(d, d, s);
            }
        }
    }
    return s;
}

// Per-thread part of the nearest-node scan for trees of at most 4 * NW joints: nodes as
// float4 words, two nodes per step (the second clamped to the last node, so both loads
// are always issued).
template <int NW>
__device__ __forceinline__ void scan_nearest(const float *__restrict__ nodes, int size, int stride, int L,
                                             const unsigned char *act, const float *q, float &best, int &bi) {
    float qr[4 * NW];
    unsigned am = 0u;
#pragma unroll
    for (int j = 0; j < 4 * NW; ++j) {
        qr[j] = j < L ? q[j] : 0.f;
        if (j < L && act[j]) am |= 1u << j;
    }
    const int bd = blockDim.x;
    for (int i = threadIdx.x; i < size; i += 2 * bd) {
        const int i2 = i + bd;
        bool w1 = true, w2 = i2 < size;
        const float s1 = node_dist<NW>(reinterpret_cast<const float4 *>(nodes + (long long)i * stride), qr, am, L, w1);
        const float s2 =
            node_dist<NW>(reinterpret_cast<const float4 *>(nodes + (long long)min(i2, size - 1) * stride), qr, am, L, w2);
        if (w1 && (s1 < best || (s1 == best && i < bi))) { best = s1; bi = i; }
        if (w2 && (s2 < best || (s2 == best && i2 < bi))) { best = s2; bi = i2; }
    }
}

// Block-wide argmin of the squared active-joint distance from q to the written nodes
// of one tree (ties to the lower index).  Returns the node index (or -1) to every
// thread.  Trees of up to 16 joints (stride a multiple of 4, 16-byte aligned) are read
// as float4 words with the query in registers; longer chains coordinate by coordinate.
__device__ inline int block_nearest(const float *__restrict__ nodes, int size, int stride, int L,
                             const unsigned char *act, const float *q, float *s_d, int *s_i) {
    float best = __int_as_float(0x7f800000);
    int bi = INT_MAX;
    const bool vec = (stride & 3) == 0 && (reinterpret_cast<unsigned long long>(nodes) & 15ull) == 0 && L <= 16;
    if (vec && L <= 4) {
        scan_nearest<1>(nodes, size, stride, L, act, q, best, bi);
    } else if (vec && L <= 8) {
        scan_nearest<2>(nodes, size, stride, L, act, q, best, bi);
    } else if (vec && L <= 12) {
        scan_nearest<3>(nodes, size, stride, L, act, q, best, bi);
    } else if (vec) {
        scan_nearest<4>(nodes, size, stride, L, act, q, best, bi);
    } else {
        for (int i = threadIdx.x; i < size; i += blockDim.x) {
            const float *y = nodes + (long long)i * stride;
            float s = 0.f;
            bool written = true;
            for (int j = 0; j < L; ++j) {
                const float v = __ldcg(y + j);
                written &= v == v;
                if (act[j]) {
                    const float d = __fadd_rn(q[j], -v);
                    s = __fmaf_rn(d, d, s);
                }
            }
            if (written && (s < best || (s == best && i < bi))) { best = s; bi = i; }
        }
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        const float ob = __shfl_xor_sync(kFull, best, off);
        const int oi = __shfl_xor_sync(kFull, bi, off);
        if (ob < best || (ob == best && oi < bi)) { best = ob; bi = oi; }
    }
    const int warp = threadIdx.x / kWarp, lane = threadIdx.x & 31;
    if (lane == 0) { s_d[warp] = best; s_i[warp] = bi; }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < kRrtcWarps; ++w)
            if (s_d[w] < s_d[0] || (s_d[w] == s_d[0] && s_i[w] < s_i[0])) { s_d[0] = s_d[w]; s_i[0] = s_i[w]; }
    }
    __syncthreads();
    const int r = s_i[0];
    __syncthreads();
    return r == INT_MAX ? -1 : r;
}

// Validate the edge a -> b (full joint vectors in shared memory) with the step rule of
// checkMotions: n = floor(metric / res) + 1 states, dir = (b - a) / n, state k = a +
// dir * k, the last state is b (for GBMP_STEP_COUNT, pRRTC's granularity G = res:
// n = G + 1 and dir = (b - a) / G, so the states are at k / G).  The states are checked in
// the direction the edge takes in a returned path, so that a path check (which walks the
// path from the start root to the goal root) meets exactly the states checked here: the
// interpolated states of a -> b and b -> a differ, and a thin contact can lie between the
// states of one direction and on a state of the other.  old_first: a is the node already
// in the tree (start tree edges), state 0 (= a) is skipped unless n == 1; otherwise
// (goal tree edges, the new node first) b is the node already in the tree and the last
// state (= b) is skipped, and with n == 1 the one state checked is a.  CHUNK (batched
// planning, robots of at most 32 sphere groups): the states are split into chunks of
// consecutive states, one chunk per warp at a time, each with one broad phase for its
// states (warp_edge_chunk, whose narrow tests are the per-state ones): measured 487
// against 531 ms on the uneven batch, whose time is the trees of the problems without a
// path growing to their node cap.  Otherwise one warp per state, which keeps the
// single-problem kernel at 5 blocks per SM (its p50 time to solution is 4 % longer with
// chunks).  Returns true if every state is collision-free.
template <int SPL, bool CULL, bool CHUNK>
__device__ bool block_edge_free(const SmemTables &t, const DevRobot &R, const DevEnv &E, const WarpScratch &w,
                                const WarpScratch &wc, const ChunkScratch &cs, const float *a, const float *b,
                                float res, int rule, bool old_first, int *s_flag, float *s_dir, int *s_n) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x / kWarp;
    if (threadIdx.x == 0) {
        float d2 = 0.f, dinf = 0.f;
        for (int j = 0; j < R.L; ++j) {
            const float d = __fadd_rn(a[j], -b[j]);
            d2 = __fmaf_rn(d, d, d2);
            dinf = fmaxf(dinf, fabsf(d));
        }
        if (rule == GBMP_STEP_COUNT) {
            *s_n = (int)res + 1;   // res in [1, 1e6] (checked by the host): G equal steps
        } else {
            const float metric = rule == GBMP_STEP_LINF ? dinf : __fsqrt_rn(d2);
            const float ratio = __fdiv_rn(metric, res);
            *s_n = ratio < 1e6f ? (int)ratio + 1 : 1000001;
        }
        *s_flag = 0;
    }
    __syncthreads();
    const int n = *s_n;
    // checkMotions divides the edge by n (its last state replaced by b); the count rule
    // by n - 1 = G, so that state k lies at k / G of the edge
    const float parts = rule == GBMP_STEP_COUNT ? (float)(n - 1) : (float)n;
    for (int j = threadIdx.x; j < R.L; j += blockDim.x) s_dir[j] = __fdiv_rn(__fadd_rn(b[j], -a[j]), parts);
    __syncthreads();
    const int first = old_first ? (n == 1 ? 0 : 1) : 0;
    const int last = old_first ? n : (n == 1 ? 1 : n - 1);   // exclusive
    if (CULL && CHUNK) {
        // chunks of `per` states; warp v takes chunk v of every round of four.  The chunk
        // routine replaces state n - 1 by b; the new-node-first single state is a, so it
        // runs as state 0 of two
        const int nstates = (!old_first && n == 1) ? 2 : n;
        const int per = min(kRrtcChunk, (last - first + kRrtcWarps - 1) / kRrtcWarps);
        for (int c0 = first; c0 < last; c0 += per * kRrtcWarps) {
            const int s0 = c0 + warp * per, s1 = min(s0 + per, last);
            int h = -1;
            if (s0 < s1)
                h = warp_edge_chunk<SPL, kRrtcChunk, false>(t, R, E, wc, cs, lane, a, b, s_dir, s0, s1, nstates);
            if (h >= 0 && lane == 0) *s_flag = 1;
            __syncthreads();
            const bool any = *s_flag != 0;
            __syncthreads();
            if (any) return false;
        }
        return true;
    }
    for (int k0 = first; k0 < last; k0 += kRrtcWarps) {
        const int k = k0 + warp;
        bool hit = false;
        if (k < last) {
            for (int j = lane; j < R.L; j += kWarp)
                w.q[j] = (old_first && k == n - 1) ? b[j] : __fmaf_rn(s_dir[j], (float)k, a[j]);
            __syncwarp();
            warp_fk(t, R.L, w, lane);
            hit = CULL ? warp_collide_culled<SPL>(t, R, E, w, lane)
                       : warp_collide<SPL, false>(t, R, E, w, lane, nullptr);
        }
        if (hit && lane == 0) *s_flag = 1;
        __syncthreads();
        const bool any = *s_flag != 0;
        __syncthreads();
        if (any) return false;
    }
    return true;
}

// Append q to tree `tr` with parent `par`; returns the slot or -1 when the tree is full.
__device__ inline int block_append(const RrtcDev &P, int tr, const float *q, int par, int L, int *s_idx) {
    if (threadIdx.x == 0) {
        const int idx = atomicAdd(P.size + tr, 1);
        *s_idx = idx < P.cap ? idx : -1;
        if (idx >= P.cap) atomicCAS(P.state, kStRunning, kStNodeCap);
    }
    __syncthreads();
    const int idx = *s_idx;
    if (idx >= 0) {
        for (int j = threadIdx.x; j < L; j += blockDim.x) __stcg(P.nodes[tr] + (long long)idx * P.stride + j, q[j]);
        if (threadIdx.x == 0) P.parent[tr][idx] = par;
        __threadfence();
    }
    __syncthreads();
    return idx;
}

// Walk both parent chains into the path (start tree root first); one thread.  Returns
// the number of states, or minus the required size when the buffer is too small.
__device__ inline int trace_path(const RrtcDev &P, int L) {
    const int tr = P.state[2];
    const int a = P.state[3], b = P.state[4];
    const int na = tr == 0 ? a : b, nb = tr == 0 ? b : a;
    int len0 = 0, len1 = 0;
    for (int i = na; i >= 0 && len0 <= P.cap; i = (P.parent[0][i] == i ? -1 : P.parent[0][i])) ++len0;
    for (int i = nb; i >= 0 && len1 <= P.cap; i = (P.parent[1][i] == i ? -1 : P.parent[1][i])) ++len1;
    if (len0 + len1 > P.path_cap || len0 > P.cap || len1 > P.cap) return -(len0 + len1);
    int k = len0 - 1;
    for (int i = na; i >= 0; i = (P.parent[0][i] == i ? -1 : P.parent[0][i]), --k)
        for (int j = 0; j < L; ++j) P.path[k * L + j] = __ldcg(P.nodes[0] + (long long)i * P.stride + j);
    k = len0;
    for (int i = nb; i >= 0; i = (P.parent[1][i] == i ? -1 : P.parent[1][i]), ++k)
        for (int j = 0; j < L; ++j) P.path[k * L + j] = __ldcg(P.nodes[1] + (long long)i * P.stride + j);
    return len0 + len1;
}

// Publish the end of a problem to the host-mapped completion word once (state[10]
// elects the writer).
__device__ inline void publish_end(const RrtcDev &P, int value) {
    if (!P.flag) return;
    if (atomicCAS(P.state + 10, 0, 1) == 0) {
        __threadfence_system();
        *P.flag = value;
        __threadfence_system();
    }
}

// One extension lane of one problem (the body of both the single-problem and the
// batched planning kernels).  All threads of the block call it.
template <int SPL, bool CULL, bool CHUNK>
__device__ void rrtc_lane(const DevRobot &R, const DevEnv &E, const RrtcDev &P, const RrtcParams &prm,
                          const int lane_id) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int nwords = env_words(E.ns, E.nb, E.nc);
    SmemTables t = carve_tables(smem, R, nwords);
    if (!stage_tables(R, E, t, nwords)) return;
    unsigned char *p = smem + smem_tables_bytes(R, nwords);
    WarpScratch w = carve_warp(p, R, threadIdx.x / kWarp);
    p += smem_warp_bytes(R) * kRrtcWarps;
    float *q_s = reinterpret_cast<float *>(p);          // sample / steered node
    float *q_a = q_s + kMaxLinks;                        // nearest node / current node
    float *q_b = q_a + kMaxLinks;                        // connect target
    float *q_c = q_b + kMaxLinks;                        // next connect step
    float *s_dir = q_c + kMaxLinks;
    float *s_d = s_dir + kMaxLinks;                      // [kRrtcWarps]
    int *s_i = reinterpret_cast<int *>(s_d + kRrtcWarps);
    int *s_misc = s_i + kRrtcWarps;                      // [8]
    unsigned char *act = reinterpret_cast<unsigned char *>(s_misc + 8);
    ChunkScratch cs{};
    WarpScratch wc{};
    if (CULL && CHUNK) carve_chunk(p + rrtc_misc_bytes(), R, kRrtcChunk, threadIdx.x / kWarp, cs, wc);
    for (int j = threadIdx.x; j < R.L; j += blockDim.x) act[j] = R.active[j];
    __syncthreads();

    const int L = R.L;
    int cur_tree = -1;   // thread 0: the tree of this lane's previous iteration
    for (int it = 0;; ++it) {
        if (threadIdx.x == 0) {
            int st = *(volatile int *)P.state;
            if (st == kStRunning && it >= prm.max_iters) st = kStIterCap;
            if (st == kStRunning && global_ns() > (prm.deadline_ptr ? *prm.deadline_ptr : prm.deadline_ns)) {
                atomicCAS(P.state, kStRunning, kStDeadline);
                st = kStDeadline;
            }
            s_misc[0] = st;
            // tree choice by pRRTC's balance rule from the current tree sizes
            const int n0 = *(volatile int *)(P.size), n1 = *(volatile int *)(P.size + 1);
            cur_tree = balance_tree(prm.balance, prm.tree_ratio, prm.lanes, n0, n1, lane_hash(lane_id), cur_tree);
            s_misc[1] = cur_tree;
            s_misc[2] = min(n0, P.cap);
            s_misc[3] = min(n1, P.cap);
        }
        __syncthreads();
        if (s_misc[0] != kStRunning) {
            if (threadIdx.x == 0 && s_misc[0] == kStIterCap) atomicCAS(P.state, kStRunning, kStIterCap);
            break;
        }
        if (threadIdx.x == 0) atomicMax(P.state + 5, it + 1);
        const int tr = s_misc[1], ot = 1 - tr;
        const int size_t_ = tr == 0 ? s_misc[2] : s_misc[3];
        const int size_o = tr == 0 ? s_misc[3] : s_misc[2];
        // 2. sample
        for (int j = threadIdx.x; j < L; j += blockDim.x) {
            if (act[j]) {
                const float u = philox_uniform(prm.seed, ((unsigned long long)lane_id << 32) | (unsigned)it, (unsigned)j);
                q_s[j] = __fmaf_rn(u, __fadd_rn(R.upper[j], -R.lower[j]), R.lower[j]);
            } else {
                q_s[j] = R.defv[j];
            }
        }
        __syncthreads();
        // 3. nearest node in the tree being grown
        const int nn = block_nearest(P.nodes[tr], size_t_, P.stride, L, act, q_s, s_d, s_i);
        if (nn < 0) continue;
        for (int j = threadIdx.x; j < L; j += blockDim.x) q_a[j] = __ldcg(P.nodes[tr] + (long long)nn * P.stride + j);
        __syncthreads();
        // 4. steer to at most `range` (active joints)
        if (threadIdx.x == 0) {
            float s = 0.f;
            for (int j = 0; j < L; ++j)
                if (act[j]) { const float d = __fadd_rn(q_s[j], -q_a[j]); s = __fmaf_rn(d, d, s); }
            const float d = __fsqrt_rn(s);
            s_d[0] = d > prm.range ? __fdiv_rn(prm.range, d) : 1.f;
            // dynamic domain: a sample beyond the nearest node's radius is skipped
            s_i[1] = (prm.dd && __uint_as_float(*(volatile unsigned *)(P.radii[tr] + nn)) < d) ? 1 : 0;
        }
        __syncthreads();
        const float scale = s_d[0];
        const bool outside = s_i[1] != 0;
        __syncthreads();
        if (outside) continue;
        for (int j = threadIdx.x; j < L; j += blockDim.x)
            if (act[j] && scale < 1.f) q_s[j] = __fmaf_rn(scale, __fadd_rn(q_s[j], -q_a[j]), q_a[j]);
        __syncthreads();
        // 5. validate nn -> new, in path order (start tree: nn first; goal tree: new first)
        if (!block_edge_free<SPL, CULL, CHUNK>(t, R, E, w, wc, cs, tr == 0 ? q_a : q_s, tr == 0 ? q_s : q_a, prm.res, prm.rule,
                                        tr == 0, s_misc + 4, s_dir, s_misc + 5)) {
            if (prm.dd && threadIdx.x == 0) dd_update(P.radii[tr] + nn, true, prm);
            continue;
        }
        // 6. append
        int cur = block_append(P, tr, q_s, nn, L, s_misc + 6);
        if (cur < 0) break;
        if (prm.dd && threadIdx.x == 0) dd_update(P.radii[tr] + nn, false, prm);
        // 7. connect towards the nearest node of the other tree
        const int tgt = block_nearest(P.nodes[ot], size_o, P.stride, L, act, q_s, s_d, s_i);
        if (tgt < 0) continue;
        for (int j = threadIdx.x; j < L; j += blockDim.x) {
            q_b[j] = __ldcg(P.nodes[ot] + (long long)tgt * P.stride + j);
            q_a[j] = q_s[j];
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            float s = 0.f;
            for (int j = 0; j < L; ++j)
                if (act[j]) { const float d = __fadd_rn(q_b[j], -q_a[j]); s = __fmaf_rn(d, d, s); }
            const float d = __fsqrt_rn(s);
            const float ne = ceilf(__fdiv_rn(d, prm.range));
            s_misc[7] = ne < 1e6f ? max(1, (int)ne) : 1000000;
        }
        __syncthreads();
        const int n_ext = s_misc[7];
        __syncthreads();
        bool connected = true;
        for (int e = 1; e <= n_ext; ++e) {
            if (threadIdx.x == 0) s_misc[4] = *(volatile int *)P.state;
            __syncthreads();
            const bool stop = s_misc[4] != kStRunning;
            __syncthreads();
            if (stop) { connected = false; break; }
            for (int j = threadIdx.x; j < L; j += blockDim.x)
                q_c[j] = (e == n_ext) ? q_b[j]
                                      : __fmaf_rn(__fdiv_rn(__fadd_rn(q_b[j], -q_s[j]), (float)n_ext), (float)e, q_s[j]);
            __syncthreads();
            // in path order: the last step joins the goal tree's node to the start tree's
            // (start tree first), every other step runs away from its tree's root
            if (!block_edge_free<SPL, CULL, CHUNK>(t, R, E, w, wc, cs, tr == 0 ? q_a : q_c, tr == 0 ? q_c : q_a, prm.res, prm.rule,
                                            tr == 0, s_misc + 4, s_dir, s_misc + 5)) {
                connected = false;
                break;
            }
            if (e < n_ext) {
                cur = block_append(P, tr, q_c, cur, L, s_misc + 6);
                if (cur < 0) { connected = false; break; }
                for (int j = threadIdx.x; j < L; j += blockDim.x) q_a[j] = q_c[j];
                __syncthreads();
            }
        }
        if (connected && threadIdx.x == 0) {
            if (atomicCAS(P.state, kStRunning, kStSolved) == kStRunning) {
                P.state[1] = lane_id;
                P.state[2] = tr;
                P.state[3] = cur;
                P.state[4] = tgt;
                __threadfence();
                if (P.flag) {
                    // the winner traces at once so the host can take this result while the
                    // launch continues for other problems
                    const int len = trace_path(P, L);
                    *P.path_len = len;
                    publish_end(P, len > 0 ? len + 1 : -5);
                }
            }
        }
        __syncthreads();
    }
}

template <int SPL, bool CULL>
__global__ void __launch_bounds__(kRrtcThreads, 5) k_rrtc(DevRobot R, DevEnv E, RrtcDev P, RrtcParams prm) {
    rrtc_lane<SPL, CULL, false>(R, E, P, prm, blockIdx.x);
}

// Batched planning: block b serves problem b % n as lane b / n, so every problem gets
// lanes from the first wave of resident blocks.  The problem's descriptors are copied
// into shared memory once.  Bounded to 128 registers (four blocks per SM): the chunked
// edge checks otherwise take the kernel to 168.
template <int SPL, bool CULL>
__global__ void __launch_bounds__(kRrtcThreads, 4) k_rrtc_batch(const BatchProblem *__restrict__ probs, int n,
                                                            int lanes_per_problem, RrtcParams prm, int *rr) {
    __shared__ DevRobot sR;
    __shared__ DevEnv sE;
    __shared__ RrtcDev sP;
    __shared__ unsigned long long sSeed;
    __shared__ int sLane, sNext;
    int p = blockIdx.x % n;
    // A block stays with a problem until it ends (solved, capped or deadline), then
    // migrates to a problem that is still running, so the lanes of easy problems end up
    // helping the hard ones.  Each stay ends a problem, so there are at most n hops.
    for (int hop = 0; hop <= n; ++hop) {
        if (threadIdx.x == 0) {
            sR = probs[p].R;
            sE = probs[p].E;
            sP = probs[p].P;
            sSeed = probs[p].seed;
            sLane = atomicAdd(probs[p].P.state + 6, 1);
            atomicAdd(probs[p].P.state + 7, 1);
        }
        __syncthreads();
        RrtcParams q = prm;
        q.lanes = lanes_per_problem;
        q.seed = sSeed;
        rrtc_lane<SPL, CULL, CULL>(sR, sE, sP, q, sLane);
        __syncthreads();
        if (threadIdx.x == 0) {
            // the last lane to leave an ended, unsolved problem publishes its end
            __threadfence();
            if (atomicSub(sP.state + 7, 1) == 1) {
                const int stt = *(volatile int *)sP.state;
                if (stt != kStRunning && stt != kStSolved) publish_end(sP, -stt);
            }
        }
        if (threadIdx.x == 0) {
            int next = -1;
            const int start = (int)((unsigned)atomicAdd(rr, 1) % (unsigned)n);
            for (int k = 0; k < n; ++k) {
                const int c = (start + k) % n;
                if (*(volatile int *)probs[c].P.state == kStRunning) { next = c; break; }
            }
            sNext = next;
        }
        __syncthreads();
        if (sNext < 0) break;
        p = sNext;
        __syncthreads();
    }
}


// Launcher of the single-problem kernel for spheres-per-lane counts A..A+3 (see
// gbmp_rrtc.cuh).
template <int SPL>
inline cudaError_t rrtc_launch_one(bool cull, int grid, size_t smem, cudaStream_t st, const DevRobot &R,
                                   const DevEnv &E, const RrtcDev &P, const RrtcParams &prm) {
    auto kern = cull ? k_rrtc<SPL, true> : k_rrtc<SPL, false>;
    cudaError_t ce = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (ce != cudaSuccess) return ce;
    kern<<<grid, kRrtcThreads, smem, st>>>(R, E, P, prm);
    return cudaGetLastError();
}

template <int SPL>
inline cudaError_t rrtc_batch_launch_one(bool cull, int grid, size_t smem, cudaStream_t st, const BatchProblem *probs,
                                         int n, int lpp, const RrtcParams &prm, int *rr) {
    auto kern = cull ? k_rrtc_batch<SPL, true> : k_rrtc_batch<SPL, false>;
    cudaError_t ce = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (ce != cudaSuccess) return ce;
    kern<<<grid, kRrtcThreads, smem, st>>>(probs, n, lpp, prm, rr);
    return cudaGetLastError();
}

#define GBMP_RRTC_DEFINE_LAUNCHER(NAME, A)                                                                    \
    cudaError_t NAME(int spl, bool cull, int grid, size_t smem, cudaStream_t st, const DevRobot &R,           \
                     const DevEnv &E, const RrtcDev &P, const RrtcParams &prm) {                              \
        switch (spl) {                                                                                        \
        case A: return rrtc_launch_one<A>(cull, grid, smem, st, R, E, P, prm);                                \
        case A + 1: return rrtc_launch_one<A + 1>(cull, grid, smem, st, R, E, P, prm);                        \
        case A + 2: return rrtc_launch_one<A + 2>(cull, grid, smem, st, R, E, P, prm);                        \
        default: return rrtc_launch_one<A + 3>(cull, grid, smem, st, R, E, P, prm);                           \
        }                                                                                                     \
    }

#define GBMP_RRTC_DEFINE_BATCH_LAUNCHER(NAME, A)                                                              \
    cudaError_t NAME(int spl, bool cull, int grid, size_t smem, cudaStream_t st, const BatchProblem *probs,   \
                     int n, int lpp, const RrtcParams &prm, int *rr) {                                        \
        switch (spl) {                                                                                        \
        case A: return rrtc_batch_launch_one<A>(cull, grid, smem, st, probs, n, lpp, prm, rr);                \
        case A + 1: return rrtc_batch_launch_one<A + 1>(cull, grid, smem, st, probs, n, lpp, prm, rr);        \
        case A + 2: return rrtc_batch_launch_one<A + 2>(cull, grid, smem, st, probs, n, lpp, prm, rr);        \
        default: return rrtc_batch_launch_one<A + 3>(cull, grid, smem, st, probs, n, lpp, prm, rr);           \
        }                                                                                                     \
    }

}  // namespace gbmp
