// gbmp_project.cu -- projection of joint states onto a task-space region and the joint
// limits, replacing SingleArmSpace::projectStates (SingleArmSpace.cu:1631-1662) with
// TaskSpaceConstraint::computeGradientAndError / computeCost
// (TaskSpaceConstraint.cu:66-139, :167-396) and BoundaryConstraint
// (BoundaryConstraint.cu:36-155).
//
// One warp per state, all iterations in one launch (the reference launches FK, one
// gradient kernel per constraint, a gradient sum and an update kernel per iteration,
// each followed by a device synchronisation, and allocates the Jacobian buffers on
// every call).  Per iteration: the warp's FK (warp_fk), lane 0 the task frame and its
// dead-banded error, lane j the Jacobian column of joint j, lanes 0..35 the 6x6 normal
// matrix J_a J_a^T + 1e-4 I over the active joints, lane 0 its Gauss-Jordan inverse,
// lane j the step of joint j (pseudo-inverse row times error, plus the joint-limit
// pull), applied with step 1.  Arithmetic is written with explicit rounding in the
// reference's operation order.
#include "gbmp_internal.h"

namespace gbmp {
namespace {

struct ProjParams {
    int task_link, use_boundary, iterations;
    float offset[16], reference[6], tolerance[6];
};

// Per-warp scratch after the WarpScratch block: Jacobian [L*6], augmented matrix
// [6*12], frame values v[6], error[6], invertible flag.
__host__ __device__ inline size_t proj_warp_bytes(const DevRobot &R) {
    return align16(sizeof(float) * 6 * R.L) + align16(sizeof(float) * 72) + align16(sizeof(float) * 16);
}

__device__ __forceinline__ float dot3(float a0, float a1, float a2, float b0, float b1, float b2) {
    return __fadd_rn(__fadd_rn(__fmul_rn(a0, b0), __fmul_rn(a1, b1)), __fmul_rn(a2, b2));
}

// Rows 0..2 of (link pose, implicit last row 0 0 0 1) x offset (TaskSpaceConstraint.cu:47-63),
// then x, y, z, roll, pitch, yaw of the result.
__device__ void task_frame(const float *T, const float *off, float *v) {
    float P[12];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c)
            P[4 * r + c] = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(T[4 * r], off[c]), __fmul_rn(T[4 * r + 1], off[4 + c])),
                                               __fmul_rn(T[4 * r + 2], off[8 + c])),
                                     __fmul_rn(T[4 * r + 3], off[12 + c]));
    v[0] = P[3]; v[1] = P[7]; v[2] = P[11];
    v[4] = asinf(-P[8]);
    v[3] = atan2f(P[9], P[10]);
    v[5] = atan2f(P[4], P[0]);
}

__device__ __forceinline__ float dead(float diff, float tol) {
    return copysignf(fmaxf(__fadd_rn(fabsf(diff), -tol), 0.0f), diff);
}

__global__ void __launch_bounds__(kWarpsPerBlock *kWarp)
    k_project(DevRobot R, ProjParams p, float *__restrict__ qall, long long n, float *__restrict__ task_cost,
              float *__restrict__ bound_cost) {
    extern __shared__ __align__(16) unsigned char smem[];
    DevEnv E0{0, 0, 0, nullptr};
    SmemTables t = carve_tables(smem, R, 0);
    stage_tables(R, E0, t, 0);
    const int warp = threadIdx.x / kWarp, lane = threadIdx.x & 31;
    unsigned char *wbase = smem + smem_tables_bytes(R, 0);
    WarpScratch w = carve_warp(wbase, R, warp);
    unsigned char *xb = wbase + smem_warp_bytes(R) * kWarpsPerBlock + proj_warp_bytes(R) * warp;
    float *J = reinterpret_cast<float *>(xb);
    float *aug = reinterpret_cast<float *>(xb + align16(sizeof(float) * 6 * R.L));
    float *misc = aug + 72;   // v[0..5], err[6..11], invertible [12]
    __syncthreads();
    const int L = R.L;
    const long long nw = (long long)gridDim.x * kWarpsPerBlock;
    for (long long s = blockIdx.x * (long long)kWarpsPerBlock + warp; s < n; s += nw) {
        float *qs = qall + s * L;
        for (int j = lane; j < L; j += kWarp) w.q[j] = qs[j];
        __syncwarp();
        for (int it = 0; it < p.iterations; ++it) {
            warp_fk(t, L, w, lane);
            float gt[2] = {0.f, 0.f};   // task step of joints lane and lane + 32
            if (p.task_link >= 0) {
                if (lane == 0) {
                    float v[6];
                    task_frame(w.lp + 12 * p.task_link, p.offset, v);
                    for (int k = 0; k < 6; ++k) misc[k] = v[k];
                    misc[6] = dead(__fadd_rn(p.reference[3], -v[3]), p.tolerance[3]);
                    misc[7] = dead(__fadd_rn(p.reference[4], -v[4]), p.tolerance[4]);
                    misc[8] = dead(__fadd_rn(p.reference[5], -v[5]), p.tolerance[5]);
                    misc[9] = dead(__fadd_rn(p.reference[0], -v[0]), p.tolerance[0]);
                    misc[10] = dead(__fadd_rn(p.reference[1], -v[1]), p.tolerance[1]);
                    misc[11] = dead(__fadd_rn(p.reference[2], -v[2]), p.tolerance[2]);
                }
                __syncwarp();
                for (int j = lane; j < L; j += kWarp) {   // Jacobian column j
                    float *c = J + 6 * j;
                    float c0 = 0.f, c1 = 0.f, c2 = 0.f, c3 = 0.f, c4 = 0.f, c5 = 0.f;
                    if (j <= p.task_link) {
                        const float *T = w.lp + 12 * j;
                        const float *a = t.axr + 4 * j;
                        const float w0 = dot3(T[0], T[1], T[2], a[0], a[1], a[2]);
                        const float w1 = dot3(T[4], T[5], T[6], a[0], a[1], a[2]);
                        const float w2 = dot3(T[8], T[9], T[10], a[0], a[1], a[2]);
                        if (t.type[j] == 1) {
                            const float d0 = __fadd_rn(misc[0], -T[3]), d1 = __fadd_rn(misc[1], -T[7]),
                                        d2 = __fadd_rn(misc[2], -T[11]);
                            c0 = w0; c1 = w1; c2 = w2;
                            c3 = __fadd_rn(__fmul_rn(w1, d2), -__fmul_rn(w2, d1));
                            c4 = __fadd_rn(__fmul_rn(w2, d0), -__fmul_rn(w0, d2));
                            c5 = __fadd_rn(__fmul_rn(w0, d1), -__fmul_rn(w1, d0));
                        } else if (t.type[j] == 2) {
                            c3 = w0; c4 = w1; c5 = w2;
                        }
                    }
                    c[0] = c0; c[1] = c1; c[2] = c2; c[3] = c3; c[4] = c4; c[5] = c5;
                }
                __syncwarp();
                for (int e = lane; e < 72; e += kWarp) {   // [J_a J_a^T + 1e-4 I | I]
                    const int i = e / 12, jj = e - 12 * i;
                    float val;
                    if (jj < 6) {
                        float sum = 0.0f;
                        for (int k = 0; k < L; ++k)
                            if (R.active[k]) sum = __fadd_rn(sum, __fmul_rn(J[6 * k + i], J[6 * k + jj]));
                        val = (i == jj) ? __fadd_rn(sum, 1e-4f) : sum;
                    } else {
                        val = (jj - 6 == i) ? 1.0f : 0.0f;
                    }
                    aug[e] = val;
                }
                __syncwarp();
                if (lane == 0) {   // Gauss-Jordan without pivoting (TaskSpaceConstraint.cu:305-350)
                    float ok = 1.f;
                    for (int i = 0; i < 6; ++i) {
                        const float pivot = aug[12 * i + i];
                        if (fabsf(pivot) < 1e-8f) { ok = 0.f; break; }
                        for (int j = 0; j < 12; ++j) aug[12 * i + j] = __fdiv_rn(aug[12 * i + j], pivot);
                        for (int k = 0; k < 6; ++k)
                            if (k != i) {
                                const float f = aug[12 * k + i];
                                for (int j = 0; j < 12; ++j)
                                    aug[12 * k + j] = __fadd_rn(aug[12 * k + j], -__fmul_rn(f, aug[12 * i + j]));
                            }
                    }
                    misc[12] = ok;
                }
                __syncwarp();
                const bool invertible = misc[12] != 0.f;
#pragma unroll
                for (int u = 0; u < 2; ++u) {
                    const int j = lane + kWarp * u;
                    if (j < L && R.active[j] && invertible) {
                        float g = 0.0f;
                        for (int i = 0; i < 6; ++i) {
                            float sum = 0.0f;
                            for (int m = 0; m < 6; ++m) sum = __fadd_rn(sum, __fmul_rn(J[6 * j + m], aug[12 * m + 6 + i]));
                            g = __fadd_rn(g, __fmul_rn(sum, misc[6 + i]));
                        }
                        gt[u] = g;
                    }
                }
            }
#pragma unroll
            for (int u = 0; u < 2; ++u) {
                const int j = lane + kWarp * u;
                if (j < L && R.active[j]) {
                    const float qv = w.q[j];
                    float gb = 0.f;
                    if (p.use_boundary) {
                        const float lo = R.lower[j], hi = R.upper[j];
                        if (qv < lo) gb = __fadd_rn(lo, -qv);
                        else if (qv > hi) gb = __fadd_rn(hi, -qv);
                    }
                    w.q[j] = __fadd_rn(qv, __fadd_rn(gt[u], gb));
                }
            }
            __syncwarp();
        }
        warp_fk(t, L, w, lane);
        if (lane == 0) {
            float tc = 0.f, bc = 0.f;
            if (p.task_link >= 0) {
                float v[6];
                task_frame(w.lp + 12 * p.task_link, p.offset, v);
                for (int k = 0; k < 6; ++k) {
                    const float d = __fadd_rn(v[k], -p.reference[k]), tl = p.tolerance[k];
                    tc = __fadd_rn(tc, fmaxf(__fadd_rn(__fmul_rn(d, d), -__fmul_rn(tl, tl)), 0.f));
                }
                tc = __fsqrt_rn(tc);
                if (tc < 1e-4f) tc = 0.f;
            }
            if (p.use_boundary) {
                for (int j = 0; j < L; ++j) {
                    if (!R.active[j]) continue;
                    const float qv = w.q[j], lo = R.lower[j], hi = R.upper[j];
                    if (qv < lo) bc = __fadd_rn(bc, __fmul_rn(__fadd_rn(lo, -qv), __fadd_rn(lo, -qv)));
                    else if (qv > hi) bc = __fadd_rn(bc, __fmul_rn(__fadd_rn(qv, -hi), __fadd_rn(qv, -hi)));
                }
                bc = bc < 1e-4f ? 0.f : __fsqrt_rn(bc);
            }
            if (task_cost) task_cost[s] = tc;
            if (bound_cost) bound_cost[s] = bc;
        }
        for (int j = lane; j < L; j += kWarp) qs[j] = w.q[j];
        __syncwarp();
    }
}

}  // namespace
}  // namespace gbmp

using namespace gbmp;

extern "C" gbmp_status gbmp_project_states(gbmp_robot r, const gbmp_projection *proj, float *d_q, int64_t n,
                                           float *d_task_cost, float *d_bound_cost, void *stream) {
    GBMP_CHECK_ARG(r && proj, "robot/projection is NULL");
    GBMP_CHECK_ARG(n >= 0, "n < 0");
    GBMP_CHECK_ARG(proj->task_link >= -1 && proj->task_link < r->L, "task_link %d outside [-1, %d)", proj->task_link,
                   r->L);
    GBMP_CHECK_ARG(proj->iterations >= 0 && proj->iterations <= 1000, "iterations %d outside [0, 1000]",
                   proj->iterations);
    GBMP_CHECK_ARG(r->L <= 2 * kWarp, "projection supports at most %d links", 2 * kWarp);
    if (n == 0) return GBMP_OK;
    GBMP_CHECK_ARG(d_q, "q is NULL");
    ProjParams p;
    p.task_link = proj->task_link;
    p.use_boundary = proj->use_boundary != 0;
    p.iterations = proj->iterations;
    for (int k = 0; k < 16; ++k) p.offset[k] = proj->offset[k];
    for (int k = 0; k < 6; ++k) {
        p.reference[k] = proj->reference[k];
        p.tolerance[k] = proj->tolerance[k];
    }
    const size_t smem = smem_tables_bytes(r->dev, 0) + (smem_warp_bytes(r->dev) + proj_warp_bytes(r->dev)) * kWarpsPerBlock;
    GBMP_CUDA(cudaFuncSetAttribute(k_project, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024));
    int per_sm = 0;
    GBMP_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_project, kWarpsPerBlock * kWarp, smem));
    if (per_sm < 1) {
        set_error("projection kernel does not fit on an SM (%zu bytes of shared memory)", smem);
        return GBMP_ERR_CAPACITY;
    }
    long long grid = (long long)per_sm * r->num_sms;
    const long long need = (n + kWarpsPerBlock - 1) / kWarpsPerBlock;
    if (need < grid) grid = need;
    ProfScope ps(GBMP_PROF_OTHER, (cudaStream_t)stream);
    k_project<<<(unsigned)grid, kWarpsPerBlock * kWarp, smem, (cudaStream_t)stream>>>(r->dev, p, d_q, n, d_task_cost,
                                                                                   d_bound_cost);
    GBMP_CUDA(cudaGetLastError());
    return GBMP_OK;
}
