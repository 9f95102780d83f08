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
#include <cmath>

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
    return align16(sizeof(float) * 6 * R.L) + align16(sizeof(float) * 72) + align16(sizeof(float) * 24);
}

// Per-warp scratch of the constrained-motion kernel: the projection scratch, then the
// goal, the previous and the last recorded state (kMaxLinks floats each).
__host__ __device__ inline size_t cm_warp_bytes(const DevRobot &R) {
    return proj_warp_bytes(R) + 3 * sizeof(float) * kMaxLinks;
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

// One projection pass on the state in w.q (TaskSpaceConstraint::computeGradientAndError,
// TaskSpaceConstraint.cu:167-396; BoundaryConstraint.cu:36-155; update_with_grad, step 1):
// FK, the dead-banded task error and its damped pseudo-inverse step, the joint-limit
// pull, both added to the active joints.  Returns, on every lane, the total error the
// gradient kernels record for the state before the update: the norm of the dead-banded
// task error plus the norm of the limit violations (SingleArmStates.cu:847-871).
__device__ float proj_pass(const SmemTables &t, const DevRobot &R, const ProjParams &p, const WarpScratch &w,
                           float *J, float *aug, float *misc, int lane) {
    const int L = R.L;
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
            float e2 = 0.f;
            for (int k = 6; k < 12; ++k) e2 = __fadd_rn(e2, __fmul_rn(misc[k], misc[k]));
            misc[13] = __fsqrt_rn(e2);
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
    } else if (lane == 0) {
        misc[13] = 0.f;
    }
    __syncwarp();
    float err = misc[13];
    if (p.use_boundary && lane == 0) {   // norm of the limit violations, joint order
        float v2 = 0.f;
        for (int j = 0; j < L; ++j) {
            if (!R.active[j]) continue;
            const float qv = w.q[j], lo = R.lower[j], hi = R.upper[j];
            float g = 0.f;
            if (qv < lo) g = __fadd_rn(lo, -qv);
            else if (qv > hi) g = __fadd_rn(hi, -qv);
            v2 = __fadd_rn(v2, __fmul_rn(g, g));
        }
        misc[14] = __fsqrt_rn(v2);
    }
    __syncwarp();
    if (p.use_boundary) err = __fadd_rn(err, misc[14]);
    __syncwarp();
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
    return err;
}

// computeCost of the task-space constraint (TaskSpaceConstraint.cu:140-176, zero below
// 1e-4) and of the joint limits (BoundaryConstraint.cu:36-95, zero below 1e-4 before the
// square root) for the state in w.q whose FK is in w.lp.  Lane 0.
__device__ void proj_costs(const DevRobot &R, const ProjParams &p, const WarpScratch &w, float *tc_out,
                           float *bc_out) {
    const int L = R.L;
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
    *tc_out = tc;
    *bc_out = bc;
}

__global__ void __launch_bounds__(kWarpsPerBlock *kWarp)
    k_project(DevRobot R, ProjParams p, float *__restrict__ qall, long long n, float *__restrict__ task_cost,
              float *__restrict__ bound_cost) {
    extern __shared__ __align__(16) unsigned char smem[];
    DevEnv E0{0, 0, 0, nullptr};
    SmemTables t = carve_tables(smem, R, 0);
    if (!stage_tables(R, E0, t, 0)) return;
    const int warp = threadIdx.x / kWarp, lane = threadIdx.x & 31;
    unsigned char *wbase = smem + smem_tables_bytes(R, 0);
    WarpScratch w = carve_warp(wbase, R, warp);
    unsigned char *xb = wbase + smem_warp_bytes(R) * kWarpsPerBlock + proj_warp_bytes(R) * warp;
    float *J = reinterpret_cast<float *>(xb);
    float *aug = reinterpret_cast<float *>(xb + align16(sizeof(float) * 6 * R.L));
    float *misc = aug + 72;   // v[0..5], err[6..11], invertible [12], error norms [13], [14]
    __syncthreads();
    const int L = R.L;
    const long long nw = (long long)gridDim.x * kWarpsPerBlock;
    for (long long s = blockIdx.x * (long long)kWarpsPerBlock + warp; s < n; s += nw) {
        float *qs = qall + s * L;
        for (int j = lane; j < L; j += kWarp) w.q[j] = qs[j];
        __syncwarp();
        for (int it = 0; it < p.iterations; ++it) proj_pass(t, R, p, w, J, aug, misc, lane);
        warp_fk(t, L, w, lane);
        if (lane == 0) {
            float tc = 0.f, bc = 0.f;
            proj_costs(R, p, w, &tc, &bc);
            if (task_cost) task_cost[s] = tc;
            if (bound_cost) bound_cost[s] = bc;
        }
        for (int j = lane; j < L; j += kWarp) qs[j] = w.q[j];
        __syncwarp();
    }
}

// Constrained motions (SingleArmSpace::computeConstrainedMotions, SingleArmSpace.cu:1049-1366),
// one warp per motion and every iteration in one launch (the reference runs a host loop of
// up to 10,000 iterations, each with an approach kernel, two projection passes of several
// kernels, three check kernels, device synchronisations and a copy of every state to the
// host, and then collision-checks the recorded states).  Per iteration: every joint moves
// `res` along the unit direction to the goal (approachKernel, :855-886); two projection
// passes (proj_pass); the motion stops approaching when the second pass's error exceeds
// 1e-3 (checkIfCostIsZero), when the state is farther from the goal than before or moved
// more than 5 res (checkValidOfApproaching); otherwise the state is recorded and checked
// as checkStates checks it (collision, task-space cost and limit cost all zero; checks
// end at the first failure), and reaching the goal within `res` ends the motion as
// achieved (checkAchieveGoal).  ok = achieved and every recorded state passed; cost = L2
// length over all joints of the recorded states; count = recorded states (the first
// `cap` are written to `states` when it is not null).
template <int SPL, bool CULL>
__global__ void __launch_bounds__(kWarpsPerBlock *kWarp)
    k_constrained_motion(DevRobot R, DevEnv E, ProjParams p, const float *__restrict__ from,
                         const float *__restrict__ to, long long n, float res, int max_iters,
                         unsigned char *__restrict__ ok_out, float *__restrict__ cost_out,
                         int *__restrict__ count_out, float *__restrict__ states, int cap) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int nwords = env_words(E.ns, E.nb, E.nc);
    SmemTables t = carve_tables(smem, R, nwords);
    if (!stage_tables(R, E, t, nwords)) return;
    const int warp = threadIdx.x / kWarp, lane = threadIdx.x & 31;
    unsigned char *wbase = smem + smem_tables_bytes(R, nwords);
    WarpScratch w = carve_warp(wbase, R, warp);
    unsigned char *xb = wbase + smem_warp_bytes(R) * kWarpsPerBlock + cm_warp_bytes(R) * warp;
    float *J = reinterpret_cast<float *>(xb);
    float *aug = reinterpret_cast<float *>(xb + align16(sizeof(float) * 6 * R.L));
    float *misc = aug + 72;
    float *goal = reinterpret_cast<float *>(xb + proj_warp_bytes(R));
    float *prev = goal + kMaxLinks;
    float *last = prev + kMaxLinks;
    __syncthreads();
    const int L = R.L;
    const long long nw = (long long)gridDim.x * kWarpsPerBlock;
    for (long long s = blockIdx.x * (long long)kWarpsPerBlock + warp; s < n; s += nw) {
        for (int j = lane; j < L; j += kWarp) {
            w.q[j] = from[s * L + j];
            goal[j] = to[s * L + j];
        }
        __syncwarp();
        bool achieved = false, feasible = true;
        int steps = 0;
        double len = 0.0;
        for (int it = 0; it < max_iters; ++it) {
            for (int j = lane; j < L; j += kWarp) prev[j] = w.q[j];
            if (lane == 0) {
                float nrm = 0.f;
                for (int j = 0; j < L; ++j) {
                    const float d = __fadd_rn(goal[j], -w.q[j]);
                    nrm = __fadd_rn(nrm, __fmul_rn(d, d));
                }
                misc[15] = __fsqrt_rn(nrm);
            }
            __syncwarp();
            const float nrm = misc[15];
            if (nrm > 1e-6f)
                for (int j = lane; j < L; j += kWarp)
                    w.q[j] = __fadd_rn(w.q[j], __fmul_rn(__fdiv_rn(__fadd_rn(goal[j], -w.q[j]), nrm), res));
            __syncwarp();
            proj_pass(t, R, p, w, J, aug, misc, lane);
            const float err = proj_pass(t, R, p, w, J, aug, misc, lane);
            if (err > 1e-3f) break;
            if (lane == 0) {
                float dpg = 0.f, dcg = 0.f, dpc = 0.f;
                for (int j = 0; j < L; ++j) {
                    const float a = __fadd_rn(prev[j], -goal[j]), b = __fadd_rn(w.q[j], -goal[j]),
                                c = __fadd_rn(prev[j], -w.q[j]);
                    dpg = __fadd_rn(dpg, __fmul_rn(a, a));
                    dcg = __fadd_rn(dcg, __fmul_rn(b, b));
                    dpc = __fadd_rn(dpc, __fmul_rn(c, c));
                }
                const float cg = __fsqrt_rn(dcg);
                misc[15] = (cg > __fsqrt_rn(dpg) || __fsqrt_rn(dpc) > __fmul_rn(res, 5.0f)) ? 0.f : 1.f;
                misc[16] = cg;
                if (misc[15] != 0.f && steps > 0) {
                    double s2 = 0.0;
                    for (int j = 0; j < L; ++j) {
                        const double d = (double)__fadd_rn(w.q[j], -last[j]);
                        s2 += d * d;
                    }
                    len += sqrt(s2);
                }
            }
            __syncwarp();
            if (misc[15] == 0.f) break;   // stopped approaching: this state is not recorded
            const float to_goal = misc[16];
            if (states && steps < cap)
                for (int j = lane; j < L; j += kWarp) states[(s * cap + steps) * L + j] = w.q[j];
            for (int j = lane; j < L; j += kWarp) last[j] = w.q[j];
            ++steps;
            if (feasible) {   // checkStates on the recorded state
                warp_fk(t, L, w, lane);
                const bool hit = CULL ? warp_collide_culled<SPL>(t, R, E, w, lane)
                                      : warp_collide<SPL, false>(t, R, E, w, lane, nullptr);
                if (lane == 0) {
                    float tc = 0.f, bc = 0.f;
                    proj_costs(R, p, w, &tc, &bc);
                    misc[15] = (hit || tc != 0.f || bc != 0.f) ? 0.f : 1.f;
                }
                __syncwarp();
                feasible = misc[15] != 0.f;
                __syncwarp();
            }
            if (to_goal < res) {
                achieved = true;
                break;
            }
        }
        if (lane == 0) {
            const bool ok = achieved && feasible;
            if (ok_out) ok_out[s] = ok;
            if (cost_out) cost_out[s] = ok ? (float)len : 0.f;
            if (count_out) count_out[s] = steps;
        }
        __syncwarp();
    }
}

}  // namespace
}  // namespace gbmp

using namespace gbmp;

// Space Jacobian of every link (SingleArmStates::calculateSpaceJacobian with
// kin_space_jacobian_per_link_kernel, SingleArmStates.cu:223-338, :793-817): for link i
// and joint j, w = R_j a_j (a_j the joint's axis as given, R_j the rotation of link j's
// pose) and p the pose positions; column j is (w, w x (p_i - p_j)) for a revolute
// joint, (0, w) for a prismatic one, and zero for link 0, joint 0, j > i and other joint
// types (joint order, not ancestry, as the reference has it).  Output [n][L][L][6]
// (state, link, joint, column).  One warp per state: FK, then the lanes over (i, j).
__global__ void __launch_bounds__(kWarpsPerBlock *kWarp)
    k_space_jacobian(DevRobot R, const float *__restrict__ q, long long n, float *__restrict__ jac) {
    extern __shared__ __align__(16) unsigned char smem[];
    DevEnv E0{0, 0, 0, nullptr};
    SmemTables t = carve_tables(smem, R, 0);
    if (!stage_tables(R, E0, t, 0)) return;
    const int warp = threadIdx.x / kWarp, lane = threadIdx.x & 31;
    WarpScratch w = carve_warp(smem + smem_tables_bytes(R, 0), R, warp);
    __syncthreads();
    const int L = R.L;
    const long long nw = (long long)gridDim.x * kWarpsPerBlock;
    for (long long s = blockIdx.x * (long long)kWarpsPerBlock + warp; s < n; s += nw) {
        for (int j = lane; j < L; j += kWarp) w.q[j] = q[s * L + j];
        __syncwarp();
        warp_fk(t, L, w, lane);
        float *out = jac + s * L * L * 6;
        for (int e = lane; e < L * L; e += kWarp) {
            const int i = e / L, j = e - i * L;
            float c[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
            const int ty = t.type[j];
            if (i > 0 && j > 0 && j <= i && (ty == 1 || ty == 2)) {
                const float *Tj = w.lp + 12 * j, *Ti = w.lp + 12 * i;
                const float *a = t.axr + 4 * j;
                const float w0 = dot3(Tj[0], Tj[1], Tj[2], a[0], a[1], a[2]);
                const float w1 = dot3(Tj[4], Tj[5], Tj[6], a[0], a[1], a[2]);
                const float w2 = dot3(Tj[8], Tj[9], Tj[10], a[0], a[1], a[2]);
                if (ty == 1) {
                    const float d0 = __fadd_rn(Ti[3], -Tj[3]), d1 = __fadd_rn(Ti[7], -Tj[7]),
                                d2 = __fadd_rn(Ti[11], -Tj[11]);
                    c[0] = w0; c[1] = w1; c[2] = w2;
                    c[3] = __fadd_rn(__fmul_rn(w1, d2), -__fmul_rn(w2, d1));
                    c[4] = __fadd_rn(__fmul_rn(w2, d0), -__fmul_rn(w0, d2));
                    c[5] = __fadd_rn(__fmul_rn(w0, d1), -__fmul_rn(w1, d0));
                } else {
                    c[3] = w0; c[4] = w1; c[5] = w2;
                }
            }
#pragma unroll
            for (int k = 0; k < 6; ++k) out[6 * e + k] = c[k];
        }
        __syncwarp();
    }
}

extern "C" gbmp_status gbmp_space_jacobian(gbmp_robot r, const float *d_q, int64_t n, float *d_jac, void *stream) {
    GBMP_CHECK_ARG(r, "robot is NULL");
    GBMP_CHECK_ARG(n >= 0, "n < 0");
    if (n == 0) return GBMP_OK;
    GBMP_CHECK_ARG(d_q && d_jac, "q/jacobian is NULL");
    const size_t smem = smem_tables_bytes(r->dev, 0) + smem_warp_bytes(r->dev) * kWarpsPerBlock;
    gbmp_status so = ensure_smem_optin((const void *)k_space_jacobian);
    if (so) return so;
    int per_sm = 0;
    GBMP_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_space_jacobian, kWarpsPerBlock * kWarp, smem));
    if (per_sm < 1) {
        set_error("Jacobian kernel does not fit on an SM (%zu bytes of shared memory)", smem);
        return GBMP_ERR_CAPACITY;
    }
    long long grid = (long long)per_sm * r->num_sms;
    const long long need = (n + kWarpsPerBlock - 1) / kWarpsPerBlock;
    if (need < grid) grid = need;
    ProfScope ps(GBMP_PROF_OTHER, (cudaStream_t)stream);
    k_space_jacobian<<<(unsigned)grid, kWarpsPerBlock * kWarp, smem, (cudaStream_t)stream>>>(r->dev, d_q, n, d_jac);
    GBMP_CUDA(cudaGetLastError());
    return GBMP_OK;
}

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
    gbmp_status so = ensure_smem_optin((const void *)k_project);
    if (so) return so;
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

extern "C" gbmp_status gbmp_constrained_motions(gbmp_robot r, gbmp_env env, const gbmp_projection *proj,
                                                const float *d_from, const float *d_to, int64_t n, float resolution,
                                                int32_t max_iterations, uint8_t *d_ok, float *d_cost,
                                                int32_t *d_num_states, float *d_states, int32_t states_cap,
                                                void *stream) {
    GBMP_CHECK_ARG(r && env && proj, "robot/env/projection is NULL");
    GBMP_CHECK_ARG(n >= 0, "n < 0");
    GBMP_CHECK_ARG(proj->task_link >= -1 && proj->task_link < r->L, "task_link %d outside [-1, %d)", proj->task_link,
                   r->L);
    GBMP_CHECK_ARG(max_iterations >= 1 && max_iterations <= 1000000, "max_iterations %d outside [1, 1e6]",
                   max_iterations);
    GBMP_CHECK_ARG(!d_states || states_cap >= 1, "states_cap < 1 with a states buffer");
    GBMP_CHECK_ARG(r->L <= 2 * kWarp, "constrained motions support at most %d links", 2 * kWarp);
    if (n == 0) return GBMP_OK;
    GBMP_CHECK_ARG(d_from && d_to, "from/to is NULL");
    const float res = resolution > 0.f ? resolution : r->resolution;
    GBMP_CHECK_ARG(std::isfinite(res), "resolution is not finite");
    ProjParams p;
    p.task_link = proj->task_link;
    p.use_boundary = proj->use_boundary != 0;
    p.iterations = 2;
    for (int k = 0; k < 16; ++k) p.offset[k] = proj->offset[k];
    for (int k = 0; k < 6; ++k) {
        p.reference[k] = proj->reference[k];
        p.tolerance[k] = proj->tolerance[k];
    }
    const DevEnv E = env->dev();
    DevRobot D = r->dev;
    D.work = nullptr;
    const int nwords = env_words(E.ns, E.nb, E.nc);
    const size_t smem = smem_tables_bytes(D, nwords) + (smem_warp_bytes(D) + cm_warp_bytes(D)) * kWarpsPerBlock;
    const void *fn = D.cull ? (const void *)k_constrained_motion<8, true> : (const void *)k_constrained_motion<8, false>;
    gbmp_status st = ensure_smem_optin(fn);
    if (st) return st;
    int per_sm = 0;
    GBMP_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kWarpsPerBlock * kWarp, smem));
    if (per_sm < 1) {
        set_error("constrained-motion kernel does not fit on an SM (%zu bytes of shared memory)", smem);
        return GBMP_ERR_CAPACITY;
    }
    long long grid = (long long)per_sm * r->num_sms;
    const long long need = (n + kWarpsPerBlock - 1) / kWarpsPerBlock;
    if (need < grid) grid = need;
    cudaStream_t s = (cudaStream_t)stream;
    ProfScope ps(GBMP_PROF_OTHER, s);
    if (D.cull)
        k_constrained_motion<8, true><<<(unsigned)grid, kWarpsPerBlock * kWarp, smem, s>>>(
            D, E, p, d_from, d_to, n, res, max_iterations, d_ok, d_cost, d_num_states, d_states, states_cap);
    else
        k_constrained_motion<8, false><<<(unsigned)grid, kWarpsPerBlock * kWarp, smem, s>>>(
            D, E, p, d_from, d_to, n, res, max_iterations, d_ok, d_cost, d_num_states, d_states, states_cap);
    GBMP_CUDA(cudaGetLastError());
    return GBMP_OK;
}
