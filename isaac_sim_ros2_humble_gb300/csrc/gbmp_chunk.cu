// gbmp_chunk.cu -- the edge-validation kernel (one warp per edge, the edge's states in
// chunks of consecutive states; the chunk routines are in gbmp_chunk_device.cuh), its
// launch set-up, and FK alone by chunks of consecutive states (gbmp_fk).
#include "gbmp_chunk_device.cuh"
#include "gbmp_order.h"

namespace gbmp {

// Warps per block of the chunk kernel.  Two blocks of 8 warps per SM at 128 registers
// per thread: measured faster than 2 x 10 warps at 96 registers or 3 x 8 warps at 80,
// where the chunk routine spills.
constexpr int kChunkWarps = 8;

// Edge validation by chunks: a warp takes the next edge of `order` (a shared counter; the
// edges come longest first, so the last edges taken are the shortest and the warps end
// together), walks its states in chunks of consecutive states and stops at the first chunk
// that holds a colliding state.  One warp per edge, so no state past that hit is placed in
// a later chunk.  Writes the edge's outputs (ok, first hit; -2 for an edge too long to
// validate).
//
// The chunk orders are gbmp_order.h's: state order when the first hit is asked for,
// coarse to fine when only the verdict is.  On the 65,536 edges of the 8-DOF benchmark
// (uniform endpoints, 82 % colliding) the coarse-to-fine order checks 4.94 M states
// against 8.89 M, 4.19 M of them on the free edges; 8 passes give 4.97 M (5.01 M in plain
// order), 4 passes 5.06 M, a full bit-reversed order of the chunks 4.96 M.

template <int SPL, int K, bool CNT>
__global__ void __launch_bounds__(kChunkWarps *kWarp, 2)
    k_edge_chunk(DevRobot R, DevEnv E, const float *__restrict__ from, const float *__restrict__ to,
                 const int *__restrict__ nsteps, const float *__restrict__ dir, const int *__restrict__ order,
                 long long n_edges, int *__restrict__ next, unsigned char *__restrict__ ok_out,
                 int *__restrict__ first_hit_out) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int nwords = env_words(E.ns, E.nb, E.nc);
    SmemTables t = carve_tables(smem, R, nwords);
    if (!stage_tables(R, E, t, nwords)) return;
    const int warp = threadIdx.x / kWarp;
    WarpScratch w;
    ChunkScratch cs;
    carve_chunk(smem + smem_tables_bytes(R, nwords), R, K, warp, cs, w);
    const int lane = threadIdx.x & 31;
    const bool any = first_hit_out == nullptr;
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
            const int nch = edge_chunk_count(n, K, any);
            for (int c = 0; c < nch; ++c) {
                const StateRange r = edge_chunk_range(c, n, K, any);
                const int h = warp_edge_chunk<SPL, K, CNT>(t, R, E, w, cs, lane, from + off, to + off, dir + off, r.x,
                                                           r.y, n);
                __syncwarp();
                if (h >= 0) { hit = h; break; }
            }
        }
        if (lane == 0) {
            if (ok_out) ok_out[e] = hit == -1;
            if (first_hit_out) first_hit_out[e] = hit;
        }
        __syncwarp();
    }
}

#define GBMP_CHUNK_SWITCH(spl, K, ...)                                                       \
    do {                                                                                     \
        if ((K) == 10) {                                                                     \
            constexpr int KK = 10;                                                            \
            switch (spl) {                                                                   \
            case 1: { constexpr int SPL = 1; __VA_ARGS__; } break;                           \
            case 2: { constexpr int SPL = 2; __VA_ARGS__; } break;                           \
            case 3: { constexpr int SPL = 3; __VA_ARGS__; } break;                           \
            case 4: { constexpr int SPL = 4; __VA_ARGS__; } break;                           \
            case 5: { constexpr int SPL = 5; __VA_ARGS__; } break;                           \
            case 6: { constexpr int SPL = 6; __VA_ARGS__; } break;                           \
            case 7: { constexpr int SPL = 7; __VA_ARGS__; } break;                           \
            default: { constexpr int SPL = 8; __VA_ARGS__; } break;                          \
            }                                                                                \
        } else {                                                                             \
            constexpr int KK = 4;                                                            \
            switch (spl) {                                                                   \
            case 1: { constexpr int SPL = 1; __VA_ARGS__; } break;                           \
            case 2: { constexpr int SPL = 2; __VA_ARGS__; } break;                           \
            case 3: { constexpr int SPL = 3; __VA_ARGS__; } break;                           \
            case 4: { constexpr int SPL = 4; __VA_ARGS__; } break;                           \
            case 5: { constexpr int SPL = 5; __VA_ARGS__; } break;                           \
            case 6: { constexpr int SPL = 6; __VA_ARGS__; } break;                           \
            case 7: { constexpr int SPL = 7; __VA_ARGS__; } break;                           \
            default: { constexpr int SPL = 8; __VA_ARGS__; } break;                          \
            }                                                                                \
        }                                                                                    \
    } while (0)

// States per chunk: 10 (three pose-row lanes per state fill 30 of 32 lanes in the chunk
// FK; measured 8.22 ms against 8.43 for 8 on the 65,536-edge benchmark call), 4 for
// robots of more than 16 links, whose pose block per state is larger.
int edge_chunk_states(const DevRobot &R, int form) {
    if (!R.cull || form == 1) return 0;
    if (form == 4 || form == 10) return form;
    return R.L <= 16 ? 10 : 4;
}

gbmp_status edge_chunk_prepare(const DevRobot &R, const DevEnv &E, int num_sms, int K, size_t *smem, int *grid) {
    *smem = smem_tables_bytes(R, env_words(E.ns, E.nb, E.nc)) + smem_chunk_bytes(R, K) * kChunkWarps;
    gbmp_status st = GBMP_OK;
    GBMP_CHUNK_SWITCH(R.spl, K, {
        const void *fn = R.work ? (const void *)k_edge_chunk<SPL, KK, true> : (const void *)k_edge_chunk<SPL, KK, false>;
        st = ensure_smem_optin(fn);
        if (st) return st;
        int per_sm = 0;
        GBMP_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kChunkWarps * kWarp, *smem));
        if (per_sm < 1) {
            set_error("chunked edge kernel does not fit on an SM (%zu bytes of shared memory)", *smem);
            st = GBMP_ERR_CAPACITY;
        }
        *grid = per_sm * num_sms;
    });
    return st;
}

gbmp_status edge_chunk_launch(const DevRobot &R, const DevEnv &E, int K, int grid, size_t smem, cudaStream_t s,
                              const float *from, const float *to, const int *nsteps, const float *dir,
                              const int *order, long long n_edges, int *next, unsigned char *ok, int *first_hit) {
    // the grid is the resident blocks, at most one warp per edge
    const long long need = (n_edges + kChunkWarps - 1) / kChunkWarps;
    if (need < grid) grid = (int)need;
    GBMP_CHUNK_SWITCH(R.spl, K, {
        if (R.work)
            k_edge_chunk<SPL, KK, true><<<grid, kChunkWarps * kWarp, smem, s>>>(R, E, from, to, nsteps, dir, order,
                                                                                n_edges, next, ok, first_hit);
        else
            k_edge_chunk<SPL, KK, false><<<grid, kChunkWarps * kWarp, smem, s>>>(R, E, from, to, nsteps, dir, order,
                                                                                 n_edges, next, ok, first_hit);
    });
    GBMP_CUDA(cudaGetLastError());
    return GBMP_OK;
}

// ---------------------------------------------------------------------------------
// FK alone (gbmp_fk): chunks of kFkChunk consecutive states per warp, the chunk FK above,
// then the chunk's link poses and sphere centres written out.  The poses of consecutive
// states are consecutive in memory, so a chunk's poses are one block that the warp writes
// as 16-byte words, 512 contiguous bytes per store (float4 rows from shared memory, the
// constant last row 0 0 0 1 built in registers); the sphere centres of the chunk are
// likewise one block, written lane by lane in order.
// ---------------------------------------------------------------------------------
constexpr int kFkChunk = 10;

__host__ __device__ inline size_t smem_fk_chunk_warp(const DevRobot &R) {
    return 2 * align16(sizeof(float) * 12 * R.L * kFkChunk);
}

__global__ void __launch_bounds__(kChunkWarps *kWarp)
    k_fk_chunk(DevRobot R, const float *__restrict__ q, long long n, float *__restrict__ poses,
               float *__restrict__ centers, int vec) {
    extern __shared__ __align__(16) unsigned char smem[];
    const DevEnv E{0, 0, 0, nullptr};
    SmemTables t = carve_tables(smem, R, 0);
    if (!stage_tables(R, E, t, 0)) return;
    const int warp = threadIdx.x / kWarp, lane = threadIdx.x & 31;
    unsigned char *wbase = smem + smem_tables_bytes(R, 0) + smem_fk_chunk_warp(R) * warp;
    float *lpK = reinterpret_cast<float *>(wbase);
    float *locK = reinterpret_cast<float *>(wbase + align16(sizeof(float) * 12 * R.L * kFkChunk));
    const int L = R.L, S = R.S;
    const long long nchunks = (n + kFkChunk - 1) / kFkChunk;
    const long long nw = (long long)gridDim.x * kChunkWarps;
    for (long long c = blockIdx.x * (long long)kChunkWarps + warp; c < nchunks; c += nw) {
        const long long s0 = c * kFkChunk;
        const int ks = (int)min((long long)kFkChunk, n - s0);
        const float *qc = q + s0 * L;
        warp_fk_chunk_q<kFkChunk>(t, L, ks, [&](int k, int i) { return qc[k * L + i]; }, locK, lpK, lane);
        if (poses) {
            if (vec) {
                float4 *P4 = reinterpret_cast<float4 *>(poses + s0 * L * 16);
                const float4 *rows = reinterpret_cast<const float4 *>(lpK);
                for (int f = lane; f < ks * L * 4; f += kWarp) {
                    const int r = f & 3, kl = f >> 2;   // kl = k * L + link
                    P4[f] = r < 3 ? rows[3 * kl + r] : make_float4(0.f, 0.f, 0.f, 1.f);
                }
            } else {
                float *P = poses + s0 * L * 16;
                for (int e = lane; e < ks * L * 16; e += kWarp) {
                    const int kl = e >> 4, k = e & 15;
                    P[e] = k < 12 ? lpK[12 * kl + k] : (k == 15 ? 1.f : 0.f);
                }
            }
        }
        if (centers) {
            float *Cc = centers + s0 * S * 3;
            for (int p = lane; p < ks * S; p += kWarp) {
                const int k = p / S, j = p - k * S;
                const float4 sp = t.sph[j];
                const float3 c3 = xform_point_a16(lpK + 12 * (k * L + t.slink[j]), sp.x, sp.y, sp.z);
                Cc[3 * p] = c3.x;
                Cc[3 * p + 1] = c3.y;
                Cc[3 * p + 2] = c3.z;
            }
        }
        __syncwarp();
    }
}

gbmp_status fk_chunk_launch(const DevRobot &R, int num_sms, const float *q, long long n, float *poses,
                            float *centers, cudaStream_t s) {
    const size_t smem = smem_tables_bytes(R, 0) + smem_fk_chunk_warp(R) * kChunkWarps;
    gbmp_status st = ensure_smem_optin((const void *)k_fk_chunk);
    if (st) return st;
    int per_sm = 0;
    GBMP_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_fk_chunk, kChunkWarps * kWarp, smem));
    if (per_sm < 1) {
        set_error("FK kernel does not fit on an SM (%zu bytes of shared memory)", smem);
        return GBMP_ERR_CAPACITY;
    }
    long long grid = (long long)per_sm * num_sms;
    const long long need = ((n + kFkChunk - 1) / kFkChunk + kChunkWarps - 1) / kChunkWarps;
    if (need < grid) grid = need;
    const int vec = (reinterpret_cast<uintptr_t>(poses) & 15u) == 0;
    k_fk_chunk<<<(int)grid, kChunkWarps * kWarp, smem, s>>>(R, q, n, poses, centers, vec);
    GBMP_CUDA(cudaGetLastError());
    return GBMP_OK;
}

}  // namespace gbmp
