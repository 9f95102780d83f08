// gbmp_order.h -- the orders in which edge validation visits an edge's interpolated
// states.  Plain integer code, compiled for the device by the edge kernels and for the
// host by tests/cpp/order_check.cpp.
//
// With the first hit asked for, states go in order, so the hit found is the lowest
// colliding index.  With only the verdict asked for (what the reference's checkMotions
// returns), an edge is infeasible as soon as any of its states collides, so the states are
// visited coarse to fine: the first ones (a colliding start), the last (a colliding goal),
// then the ones between in 16 interleaved passes taken in bit-reversed order of their
// offsets (0, 8, 4, 12, 2, ...), so that a colliding stretch of the edge is met after a
// fraction of the states before it.  Either way every state is visited exactly once, so a
// free edge has every state checked.
#pragma once

#if defined(__CUDACC__)
#define GBMP_ORDER_FN __host__ __device__ __forceinline__
#else
#define GBMP_ORDER_FN inline
#endif

namespace gbmp {

constexpr int kFirstChunk = 4;   // states of an edge's first chunk
constexpr int kOrderPasses = 16;  // interleaved passes of the coarse-to-fine orders

struct StateRange {
    int x, y;   // states [x, y)
};

// p in [0, 16) with its four bits reversed: the offset of pass p.
GBMP_ORDER_FN int order_pass_offset(int p) {
#if defined(__CUDA_ARCH__)
    return (int)(__brev((unsigned)p) >> 28);
#else
    return ((p & 1) << 3) | ((p & 2) << 1) | ((p & 4) >> 1) | ((p & 8) >> 3);
#endif
}

// Chunks of an edge of n states, K states a chunk after a first chunk of kFirstChunk.
GBMP_ORDER_FN int edge_chunk_count(int n, int K, bool any) {
    if (n <= kFirstChunk) return 1;
    if (!any) return 1 + (n - kFirstChunk + K - 1) / K;
    const int ts = n - K > kFirstChunk ? n - K : kFirstChunk;   // the last chunk is [ts, n)
    return 2 + (ts - kFirstChunk + K - 1) / K;
}

// States of chunk idx (0 <= idx < edge_chunk_count).  In state order: [0, 4), then K at a
// time.  Coarse to fine (`any`): [0, 4), the last K states, then the K-state chunks
// between them, chunk j = [4 + jK, min(ts, 4 + (j + 1)K)), in the 16 passes (pass p holds
// the chunks o, o + 16, o + 32, ... with o = order_pass_offset(p)).
GBMP_ORDER_FN StateRange edge_chunk_range(int idx, int n, int K, bool any) {
    if (idx == 0) return StateRange{0, n < kFirstChunk ? n : kFirstChunk};
    if (!any) {
        const int a = kFirstChunk + (idx - 1) * K;
        return StateRange{a, a + K < n ? a + K : n};
    }
    const int ts = n - K > kFirstChunk ? n - K : kFirstChunk;
    if (idx == 1) return StateRange{ts, n};
    const int nm = (ts - kFirstChunk + K - 1) / K;
    int r = idx - 2, o = 0;
    if (r >= nm) return StateRange{0, 0};   // idx past the last chunk
    for (int p = 0;; ++p) {   // r < nm, so the pass is found within 16 steps
        o = order_pass_offset(p);
        const int sz = (nm - o + kOrderPasses - 1) / kOrderPasses;   // nm - o + 15 >= 0
        if (r < sz) break;
        r -= sz;
    }
    const int a = kFirstChunk + (o + r * kOrderPasses) * K;
    return StateRange{a, a + K < ts ? a + K : ts};
}

// State checked at step c (0 <= c < n) of an edge of n states, state by state, coarse to
// fine: the first state, the last, then the states between in the 16 passes.
GBMP_ORDER_FN int verdict_order_state(int c, int n) {
    if (c == 0 || n <= 2) return c;
    if (c == 1) return n - 1;
    const int m = n - 2;   // states 1 .. n-2
    int r = c - 2;
    if (r >= m) return 0;   // c past the last state
    for (int p = 0;; ++p) {   // r < m, so the pass is found within 16 steps
        const int o = order_pass_offset(p);
        const int sz = (m - o + kOrderPasses - 1) / kOrderPasses;   // m - o + 15 >= 0
        if (r < sz) return 1 + o + r * kOrderPasses;
        r -= sz;
    }
}

}  // namespace gbmp
