/*
 * gbmp_oracle.h -- CPU restatement of the reference motion-planning hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This code is the checker for the CUDA product
 * path and the timed CPU baseline; the product never links or calls it.
 *
 * Every function restates one piece of CUDAMPLib / CPRRTC arithmetic and cites
 * the reference file:line it follows (paths relative to the reference tree).
 * The FP32 functions keep the reference's operation order; the FP64 functions
 * are the high-precision truth used for tolerance checks.
 *
 * Pinning: the FK, edge-step and interpolation restatements are checked in
 * tests against the reference's own generated kernels, compiled for the CPU from
 * cudampl/CUDAMPLib/include/spaces/KernelGenerator.h by oracle/ref_build.py.  The
 * collision-cost restatements cannot be pinned the same way (the constraint kernels
 * live in .cu files that need Eigen, thrust and CUDA launches); they are checked
 * against hand-computed cases and FP64 signed clearances.
 */
#ifndef GBMP_ORACLE_H
#define GBMP_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Joint type codes, cudampl/CUDAMPLib/include/states/SingleArmStates.h:190-195. */
#define OR_REVOLUTE 1
#define OR_PRISMATIC 2
#define OR_FIXED 5

typedef struct or_robot {
    int32_t L;                 /* links == joints (joint i drives link i)        */
    const int32_t *type;       /* [L]                                            */
    const float *pose;         /* [L*16] row-major joint origin in parent frame  */
    const float *axis;         /* [L*3]                                          */
    const int32_t *parent;     /* [L]  parent[i] < i, parent[0] < 0              */
    int32_t S;                 /* collision spheres                              */
    const int32_t *sph_link;   /* [S]                                            */
    const float *sph_pos;      /* [S*3] centre in link frame                     */
    const float *sph_r;        /* [S]                                            */
} or_robot;

typedef struct or_env {
    int32_t ns;                /* obstacle spheres                               */
    const float *sph;          /* [ns*4] x y z r                                 */
    int32_t nb;                /* cuboids                                        */
    const float *box_inv;      /* [nb*12] inverse pose 3x4 row-major             */
    const float *box_min;      /* [nb*3]                                         */
    const float *box_max;      /* [nb*3]                                         */
    int32_t nc;                /* cylinders (local z axis)                       */
    const float *cyl_inv;      /* [nc*12]                                        */
    const float *cyl_r;        /* [nc]                                           */
    const float *cyl_h;        /* [nc] full height                               */
} or_env;

/* ---- kinematics ---- */
void or_fk_f32(const or_robot *r, const float *q, int64_t n, float *poses);
void or_fk_f64(const or_robot *r, const double *q, int64_t n, double *poses);
void or_sphere_centers_f32(const or_robot *r, const float *poses, int64_t n, float *centers);
void or_sphere_centers_f64(const or_robot *r, const double *poses, int64_t n, double *centers);

/* ---- collision model ---- */
int32_t or_self_pairs(const or_robot *r, const uint8_t *enables, int32_t *pairs, float *thr_sq, int32_t cap);
void or_inverse_pose(const float *pos, const float *rot, float *inv);

/* costs: SoA out[4*n]: slot 0 self, 1 env spheres, 2 cuboids, 3 cylinders */
void or_check_states(const or_robot *r, const or_env *e, int32_t npairs, const int32_t *pairs,
                     const float *thr_sq, const float *q, int64_t n, float *costs, float *total,
                     int32_t nthreads);
void or_clearance_f64(const or_robot *r, const or_env *e, int32_t npairs, const int32_t *pairs,
                      const double *q, int64_t n, double *clearance, int32_t nthreads);

/* ---- edges ---- */
#define OR_STEP_L2 0
#define OR_STEP_LINF 1
#define OR_STEP_COUNT 2   /* `res` equal steps (pRRTC granularity): n = res + 1, dir = (to - from) / res */
int32_t or_edge_steps(const float *from, const float *to, int32_t J, float res, int32_t rule,
                      float *dir, float *length);
void or_edge_state(const float *from, const float *to, const float *dir, int32_t J, int32_t n,
                   int32_t k, float *out);
void or_check_motions(const or_robot *r, const or_env *e, int32_t npairs, const int32_t *pairs,
                      const float *thr_sq, const float *from, const float *to, int64_t E,
                      float res, int32_t rule, int32_t early_exit, uint8_t *ok, int32_t *first_hit,
                      int32_t *num_steps, float *length, int32_t nthreads);

/* ---- state-manager kernels ---- */
void or_nearest(const float *tree, int64_t M, int32_t J, const uint8_t *active,
                const int32_t *cand, int64_t ncand, const float *queries, int64_t Q,
                int32_t *out, int32_t nthreads);
void or_steer(const float *from, float *to, int64_t n, int32_t J, float max_distance);
void or_sample(const float *lower, const float *upper, const uint8_t *active, const float *defv,
               int32_t J, uint64_t seed, uint64_t offset, int64_t n, float *q);

int32_t or_rrtc(const or_robot *r, const or_env *e, int32_t np, const int32_t *pairs, const float *thr,
                const float *start, const float *goal, const uint8_t *active, const float *lower,
                const float *upper, const float *defv, float range, float res, int32_t rule, uint64_t seed,
                int32_t max_nodes, int32_t max_iters, float *path, int32_t path_cap, int32_t *path_len,
                float *cost, int32_t *iters, int32_t *tree_sizes);
/* Tree a lane grows, pRRTC.cu:348-371 (balance 0 none, 1 proportional / smaller tree,
 * 2 VAMP swap); h the lane's hash in [0, 1); cur its previous tree or -1. */
int32_t or_balance_tree(int32_t balance, float tree_ratio, int32_t lanes, int32_t n0, int32_t n1, float h,
                        int32_t cur);
/* Lane-parallel RRT-Connect in synchronous rounds (the device planner's per-lane rule:
 * RobotSolver.cu:562-796, pRRTC.cu:340-601).  Returns 1 when solved. */
int32_t or_rrtc_lanes(const or_robot *r, const or_env *e, int32_t np, const int32_t *pairs, const float *thr,
                      const float *start, const float *goal, const uint8_t *active, const float *lower,
                      const float *upper, const float *defv, float range, float res, int32_t rule, uint64_t seed,
                      int32_t lanes, int32_t balance, float tree_ratio, int32_t max_nodes, int32_t max_iters,
                      float *path, int32_t path_cap, int32_t *path_len, float *cost, int32_t *iters,
                      int32_t *tree_sizes, int32_t nthreads);

int32_t or_num_threads(void);

/* ---- constraint projection ----
 * SingleArmSpace::projectStates (SingleArmSpace.cu:1631-1662): `iterations` rounds of
 * FK, the task-space gradient (TaskSpaceConstraint.cu:167-396: damped pseudo-inverse of
 * the task link's geometric Jacobian times the dead-banded pose error) plus the
 * joint-limit gradient (BoundaryConstraint.cu:104-155), added to the active joints with
 * step 1 (update_with_grad).  task_link < 0 disables the task-space constraint.
 * After the rounds, the final costs (TaskSpaceConstraint.cu:66-139,
 * BoundaryConstraint.cu:36-88) go to task_cost[n] / bound_cost[n] (either may be NULL). */
typedef struct or_projection {
    int32_t task_link;
    float offset[16];          /* pose of the constrained frame in the task link       */
    float reference[6];        /* x, y, z, roll, pitch, yaw                           */
    float tolerance[6];
    int32_t use_boundary;
    int32_t iterations;
} or_projection;
void or_project(const or_robot *r, const uint8_t *active, const float *lower, const float *upper,
                const or_projection *p, float *q, int64_t n, float *task_cost, float *bound_cost,
                int32_t nthreads);

/* Constrained motions (SingleArmSpace.cu:1049-1366): ok[n], cost[n], count[n] recorded
 * states, states [n * cap * L] or NULL. */
void or_constrained_motions(const or_robot *r, const or_env *e, int32_t np, const int32_t *pairs,
                            const float *thr, const uint8_t *active, const float *lower, const float *upper,
                            const or_projection *p, const float *from, const float *to, int64_t n, float res,
                            int32_t max_iters, uint8_t *ok, float *cost, int32_t *count, float *states, int32_t cap,
                            int32_t nthreads);

#ifdef __cplusplus
}
#endif
#endif
