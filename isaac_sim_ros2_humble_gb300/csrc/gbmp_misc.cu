// gbmp_misc.cu -- state-manager kernels of libgbmp: nearest neighbour, steer and
// counter-based sampling, with their C-ABI entry points.
#include <climits>

#include "gbmp_internal.h"
#include "gbmp_philox.h"

namespace gbmp {

// Nearest candidate per query over the active joints; one warp per query.  The
// squared distance is accumulated in joint order with fused multiply-adds
// (SingleArmStates.cu:1285-1300); the argmin key is (distance, candidate position).
__global__ void __launch_bounds__(256)
    k_nearest(const float *__restrict__ tree, const int *__restrict__ cand, long long ncand,
              const float *__restrict__ queries, long long Q, int L, const unsigned char *__restrict__ active,
              int *__restrict__ out) {
    __shared__ float qs[8][kMaxLinks];
    __shared__ unsigned char act[kMaxLinks];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int j = threadIdx.x; j < L; j += blockDim.x) act[j] = active[j];
    __syncthreads();
    const long long nw = (long long)gridDim.x * (blockDim.x >> 5);
    for (long long q = blockIdx.x * (long long)(blockDim.x >> 5) + warp; q < Q; q += nw) {
        for (int j = lane; j < L; j += 32) qs[warp][j] = queries[q * L + j];
        __syncwarp();
        float best = __int_as_float(0x7f800000);
        long long bpos = LLONG_MAX;
        for (long long c = lane; c < ncand; c += 32) {
            const long long idx = cand ? cand[c] : c;
            const float *y = tree + idx * L;
            float s = 0.f;
            for (int j = 0; j < L; ++j)
                if (act[j]) {
                    const float d = __fadd_rn(qs[warp][j], -y[j]);
                    s = __fmaf_rn(d, d, s);
                }
            if (s < best) { best = s; bpos = c; }
        }
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            const float ob = __shfl_xor_sync(kFull, best, off);
            const long long op = __shfl_xor_sync(kFull, bpos, off);
            if (ob < best || (ob == best && op < bpos)) { best = ob; bpos = op; }
        }
        if (lane == 0) out[q] = bpos == LLONG_MAX ? -1 : (int)(cand ? cand[bpos] : bpos);
        __syncwarp();
    }
}

// Steer: limit the L2 step from the source state to max_distance (SingleArmStates.cu:1501-1521).
__global__ void k_steer(const float *__restrict__ from, const int *__restrict__ idx, float *__restrict__ to,
                        long long n, int L, float max_d) {
    const long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (k >= n) return;
    const float *f = from + (idx ? (long long)idx[k] : k) * L;
    float *t = to + k * L;
    float s = 0.f;
    for (int j = 0; j < L; ++j) {
        const float d = __fadd_rn(f[j], -t[j]);
        s = __fmaf_rn(d, d, s);
    }
    const float d = __fsqrt_rn(s);
    if (d > max_d) {
        const float sc = __fdiv_rn(max_d, d);
        for (int j = 0; j < L; ++j) t[j] = __fmaf_rn(sc, __fadd_rn(t[j], -f[j]), f[j]);
    }
}

// Gather rows of L floats by index, one thread per output element (coalesced stores).
__global__ void k_gather_states(const float *__restrict__ src, long long M, const int *__restrict__ idx, long long n,
                                int L, float *__restrict__ dst, int *__restrict__ bad) {
    const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (e >= n * L) return;
    const long long k = e / L;
    const int j = (int)(e - k * L);
    const int i = idx[k];
    if (i >= 0 && i < M) {
        dst[e] = src[(long long)i * L + j];
    } else {
        dst[e] = __int_as_float(0x7fffffff);
        if (bad && j == 0) *bad = 1;
    }
}

// Uniform sample in [lower, upper) per active joint, default value otherwise.
__global__ void k_sample(DevRobot R, unsigned long long seed, unsigned long long offset, long long n,
                         float *__restrict__ q) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n * R.L) return;
    const long long k = i / R.L;
    const int j = (int)(i % R.L);
    if (!R.active[j]) {
        q[i] = R.defv[j];
        return;
    }
    const float u = philox_uniform(seed, offset + (unsigned long long)k, (unsigned)j);
    const float lo = R.lower[j], hi = R.upper[j];
    q[i] = __fmaf_rn(u, __fadd_rn(hi, -lo), lo);
}

}  // namespace gbmp

using namespace gbmp;

extern "C" {

gbmp_status gbmp_nearest(gbmp_robot r, const float *d_tree, int64_t M, const int32_t *d_cand, int64_t n_cand,
                         const float *d_queries, int64_t Q, int32_t *d_out, void *stream) {
    GBMP_CHECK_ARG(r, "robot is NULL");
    GBMP_CHECK_ARG(M >= 0 && Q >= 0 && n_cand >= 0, "negative size");
    if (Q == 0) return GBMP_OK;
    GBMP_CHECK_ARG(d_queries && d_out, "queries/out is NULL");
    // SingleArmStates.cu:1359-1370: the manager and every candidate group must be non-empty.
    GBMP_CHECK_ARG(M > 0, "manager is empty");
    const long long nc = d_cand ? n_cand : M;
    GBMP_CHECK_ARG(nc > 0, "candidate group is empty");
    GBMP_CHECK_ARG(d_tree, "tree is NULL");
    const long long blocks = std::min<long long>((Q + 7) / 8, 64LL * r->num_sms);
    ProfScope ps(GBMP_PROF_OTHER, (cudaStream_t)stream);
    k_nearest<<<(unsigned)blocks, 256, 0, (cudaStream_t)stream>>>(d_tree, d_cand, nc, d_queries, Q, r->L,
                                                                  r->dev.active, d_out);
    GBMP_CUDA(cudaGetLastError());
    return GBMP_OK;
}

gbmp_status gbmp_steer(gbmp_robot r, const float *d_from, const int32_t *d_idx, float *d_to, int64_t n,
                       float max_distance, void *stream) {
    GBMP_CHECK_ARG(r, "robot is NULL");
    GBMP_CHECK_ARG(n >= 0, "n < 0");
    if (n == 0) return GBMP_OK;
    GBMP_CHECK_ARG(d_from && d_to, "from/to is NULL");
    const unsigned blocks = (unsigned)((n + 255) / 256);
    ProfScope ps(GBMP_PROF_OTHER, (cudaStream_t)stream);
    k_steer<<<blocks, 256, 0, (cudaStream_t)stream>>>(d_from, d_idx, d_to, n, r->L, max_distance);
    GBMP_CUDA(cudaGetLastError());
    return GBMP_OK;
}

gbmp_status gbmp_gather_states(int32_t L, const float *d_src, int64_t M, const int32_t *d_idx, int64_t n,
                               float *d_dst, int32_t *d_bad, void *stream) {
    GBMP_CHECK_ARG(L >= 1, "L < 1");
    GBMP_CHECK_ARG(M >= 0 && n >= 0, "negative count");
    GBMP_CHECK_ARG(n <= (1LL << 40) / L, "n too large");
    if (n == 0) return GBMP_OK;
    GBMP_CHECK_ARG(d_idx && d_dst, "idx/dst is NULL");
    GBMP_CHECK_ARG(d_src || M == 0, "src is NULL");
    const long long total = n * (long long)L;
    const unsigned long long blocks = (unsigned long long)((total + 255) / 256);
    GBMP_CHECK_ARG(blocks <= 0x7fffffffull, "n too large");
    ProfScope ps(GBMP_PROF_OTHER, (cudaStream_t)stream);
    k_gather_states<<<(unsigned)blocks, 256, 0, (cudaStream_t)stream>>>(d_src, M, d_idx, n, L, d_dst, d_bad);
    GBMP_CUDA(cudaGetLastError());
    return GBMP_OK;
}

gbmp_status gbmp_sample(gbmp_robot r, uint64_t seed, uint64_t offset, int64_t n, float *d_q, void *stream) {
    GBMP_CHECK_ARG(r, "robot is NULL");
    GBMP_CHECK_ARG(n >= 0, "n < 0");
    if (n == 0) return GBMP_OK;
    GBMP_CHECK_ARG(d_q, "q is NULL");
    const long long total = n * r->L;
    const unsigned blocks = (unsigned)((total + 255) / 256);
    ProfScope ps(GBMP_PROF_OTHER, (cudaStream_t)stream);
    k_sample<<<blocks, 256, 0, (cudaStream_t)stream>>>(r->dev, seed, offset, n, d_q);
    GBMP_CUDA(cudaGetLastError());
    return GBMP_OK;
}

}  // extern "C"
