/*
 * gbmp.h -- C-ABI of the GB300 motion-planning hot path (libgbmp.so).
 *
 * Plain C types only: opaque handles, pointers and sizes.  Every function
 * returns a gbmp_status; nothing throws across the boundary and nothing calls
 * exit().  gbmp_last_error() returns a message for the calling thread's last
 * failure.
 *
 * Memory: every array argument named d_* is DEVICE memory (cudaMalloc'd, or a
 * torch CUDA tensor's data pointer); every h_* argument is HOST memory.  Arrays
 * of joint values are row-major [n x L] "full" vectors with one entry per link
 * (fixed joints included), the layout of the reference's SingleArmStates
 * (cudampl/CUDAMPLib/src/states/SingleArmStates.cu:435).
 *
 * Streams: `stream` is a cudaStream_t passed as void* (NULL = legacy default
 * stream).  Calls are stream-ordered and asynchronous unless documented
 * otherwise.  Handles may be used from several threads if each thread uses its
 * own stream; a handle must outlive the work queued with it.
 */
#ifndef GBMP_H
#define GBMP_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(_WIN32)
#define GBMP_API __declspec(dllexport)
#else
#define GBMP_API __attribute__((visibility("default")))
#endif

#define GBMP_VERSION_MAJOR 0
#define GBMP_VERSION_MINOR 1

typedef int32_t gbmp_status;
enum {
    GBMP_OK = 0,
    GBMP_ERR_INVALID_ARGUMENT = 1, /* reference: std::runtime_error (SingleArmSpace.cu:65-77, :657-664) */
    GBMP_ERR_OUT_OF_MEMORY = 2,    /* reference: isValid()=false / nullptr (base/States.h:39-52)        */
    GBMP_ERR_CUDA = 3,
    GBMP_ERR_CODEGEN = 4,          /* runtime FK code generation / NVRTC failure                         */
    GBMP_ERR_CAPACITY = 5,         /* a table does not fit the kernel limits (see gbmp_limits)           */
    GBMP_ERR_TIMEOUT = 6,          /* a device-side wait or iteration cap gave up                        */
    GBMP_ERR_NOT_SOLVED = 7,       /* planner finished without a path                                    */
    GBMP_ERR_UNSUPPORTED = 8
};

/* Joint types, cudampl/CUDAMPLib/include/states/SingleArmStates.h:190-195. */
#define GBMP_JOINT_REVOLUTE 1
#define GBMP_JOINT_PRISMATIC 2
#define GBMP_JOINT_FIXED 5

typedef struct gbmp_robot_s *gbmp_robot;
typedef struct gbmp_env_s *gbmp_env;

/* Kinematic tree and collision-sphere model.  Same tables as the constructor of
 * CUDAMPLib::SingleArmSpace (cudampl/CUDAMPLib/include/spaces/SingleArmSpace.h:24-40)
 * and CPRRTC::RobotSolver (cudampl/CPRRTC/include/RobotSolver.h:84-101), filled by
 * RobotInfo (src/foliation_planner/include/foliation_planner/robot_info.hpp:13-220). */
typedef struct gbmp_robot_desc {
    int32_t num_links;              /* L: links == joints; joint i drives link i          */
    const int32_t *joint_types;     /* [L]                                                 */
    const float *joint_poses;       /* [L*16] row-major 4x4 joint origin in parent frame  */
    const float *joint_axes;        /* [L*3]                                              */
    const int32_t *parent;          /* [L] parent[i] < i; parent[0] < 0                   */
    int32_t num_spheres;            /* S                                                   */
    const int32_t *sphere_link;     /* [S]                                                 */
    const float *sphere_pos;        /* [S*3] centre in the link frame                      */
    const float *sphere_radius;     /* [S]                                                 */
    const uint8_t *active_joints;   /* [L] 1 = planning joint                              */
    const float *lower;             /* [L]                                                 */
    const float *upper;             /* [L]                                                 */
    const float *default_values;    /* [L] value of inactive joints                        */
    const uint8_t *self_enables;    /* [L*L] link-pair self-collision mask, NULL = all     */
    float resolution;               /* edge interpolation step (SingleArmSpace.h:39)       */
} gbmp_robot_desc;

/* Robot flags. */
#define GBMP_ROBOT_GENERIC 0x0      /* table-driven kernels compiled ahead of time         */
#define GBMP_ROBOT_CODEGEN 0x1      /* also generate + NVRTC-compile robot-specific kernels */

typedef struct gbmp_limits {
    int32_t max_links;
    int32_t max_spheres;
    int32_t max_self_pairs;
    int32_t max_env_words;          /* float4 words of an environment kept in shared memory */
} gbmp_limits;

GBMP_API const char *gbmp_last_error(void);
GBMP_API const char *gbmp_status_string(gbmp_status s);
GBMP_API gbmp_status gbmp_get_limits(gbmp_limits *out);
GBMP_API gbmp_status gbmp_device_count(int32_t *count);

/* Replaces SingleArmSpace::SingleArmSpace (SingleArmSpace.cu:10-161): validates the
 * tree (parent[i] < i, :63-69), uploads the tables, builds the self-collision pair
 * list (SelfCollisionConstraint.cu:28-38) and, with GBMP_ROBOT_CODEGEN, generates
 * and compiles the robot-specific kernels (replacing KernelGenerator.h:222-406 +
 * NvrtcUtil.h:58-148).  Synchronous. */
GBMP_API gbmp_status gbmp_robot_create(const gbmp_robot_desc *desc, int32_t flags, gbmp_robot *out);
GBMP_API gbmp_status gbmp_robot_destroy(gbmp_robot robot);
GBMP_API gbmp_status gbmp_robot_info(gbmp_robot robot, int32_t *num_links, int32_t *num_spheres,
                            int32_t *num_self_pairs, int32_t *dim, int32_t *codegen_active);
/* Host copy of the self-collision pair list: h_pairs [2*P] (i, j), h_thr_sq [P]. */
GBMP_API gbmp_status gbmp_robot_self_pairs(gbmp_robot robot, int32_t *h_pairs, float *h_thr_sq, int32_t cap);
/* Host copies of the joint tables given at creation, each [L] and each optional: the
 * active map (1 = planning joint), the value inactive joints take, and the limits.
 * Callers that hold active-joint vectors (the reference's Configuration / vector<float>
 * of `dim` values) build full vectors from these. */
GBMP_API gbmp_status gbmp_robot_joints(gbmp_robot robot, uint8_t *h_active, float *h_default, float *h_lower,
                              float *h_upper);
/* Device-side health of a robot handle: *status = GBMP_ERR_TIMEOUT when a kernel working
 * for it gave up a bounded device-side wait (its results are then not valid; the kernels
 * stage tables into shared memory with asynchronous bulk copies and wait for them with a
 * limit), GBMP_OK otherwise.  Synchronous (reads one word).  No reference counterpart
 * (the reference exits the process on a CUDA error, util.h:12-19). */
GBMP_API gbmp_status gbmp_robot_device_status(gbmp_robot robot, int32_t *status);
/* Test control of the bounded staging wait of one robot handle's kernels: `polls` polls
 * before a block gives up (0: at once, so the give-up path runs and reports through
 * gbmp_robot_device_status; -1: the default, far beyond any copy).  A block that gives up
 * still waits, again bounded, for its copies in flight before it leaves.  The fault word
 * stays set for the handle's life.  No reference counterpart. */
GBMP_API gbmp_status gbmp_robot_set_stage_wait(gbmp_robot robot, int32_t polls);
/* Select the kernel family used by later calls: 0 table-driven, 1 generated. */
GBMP_API gbmp_status gbmp_robot_use_codegen(gbmp_robot robot, int32_t enable);
/* The generated kernels of a robot created with GBMP_ROBOT_CODEGEN (the reference writes
 * its generated source to a file, SingleArmSpace.cu:98-123): the CUDA C++ source
 * (copied when `source` is non-NULL and `capacity` suffices; *source_len = bytes incl.
 * the terminating 0), the cache key *hash, *cache = 0 compiled by this call, 1 found in
 * the in-process cache, 2 read from the GBMP_CODEGEN_CACHE directory, and the NVRTC time
 * *compile_ms (0 when cached).  Any output may be NULL. */
GBMP_API gbmp_status gbmp_robot_codegen_info(gbmp_robot robot, char *source, int64_t capacity, int64_t *source_len,
                                    uint64_t *hash, int32_t *cache, double *compile_ms);

/* Replaces the constructors of EnvConstraintSphere (EnvConstraintSphere.h:21-25),
 * EnvConstraintCuboid (EnvConstraintCuboid.h:23-29; pos[3], row-major rotation[9],
 * min[3], max[3] in the box frame) and EnvConstraintCylinder (EnvConstraintCylinder.h:23-29;
 * pos, rotation, radius, full height along local z).  Any count may be 0.  Synchronous. */
GBMP_API gbmp_status gbmp_env_create(int32_t n_spheres, const float *h_sphere_pos, const float *h_sphere_radius,
                            int32_t n_cuboids, const float *h_cuboid_pos, const float *h_cuboid_rot,
                            const float *h_cuboid_min, const float *h_cuboid_max,
                            int32_t n_cylinders, const float *h_cyl_pos, const float *h_cyl_rot,
                            const float *h_cyl_radius, const float *h_cyl_height, gbmp_env *out);
GBMP_API gbmp_status gbmp_env_destroy(gbmp_env env);
GBMP_API gbmp_status gbmp_env_counts(gbmp_env env, int32_t *n_spheres, int32_t *n_cuboids, int32_t *n_cylinders);

/* Forward kinematics, replacing SingleArmStates::update (SingleArmStates.cu:696-723:
 * generated FK kernel KernelGenerator.h:353-403 + sphere transform :340-393).
 * d_q [n*L]; d_poses [n*L*16] row-major 4x4 or NULL; d_centers [n*S*3] or NULL. */
GBMP_API gbmp_status gbmp_fk(gbmp_robot robot, const float *d_q, int64_t n, float *d_poses,
                    float *d_centers, void *stream);

/* Space Jacobian of every link, replacing SingleArmStates::calculateSpaceJacobian
 * (SingleArmStates.cu:223-338, :793-817): d_jac [n*L*L*6], state s, link i, joint j at
 * ((s * L + i) * L + j) * 6: for a revolute joint j <= i (j > 0, i > 0) the column
 * (w, w x (p_i - p_j)) with w the joint's axis in the base frame and p the link
 * positions, for a prismatic one (0, w), otherwise zero (joint order decides, as in the
 * reference). */
GBMP_API gbmp_status gbmp_space_jacobian(gbmp_robot robot, const float *d_q, int64_t n, float *d_jac,
                                         void *stream);

/* Collision check of n states, replacing SingleArmSpace::checkStates
 * (SingleArmSpace.cu:1572-1602) with the four collision constraints
 * (SelfCollisionConstraint.cu:60-133, EnvConstraintSphere.cu:35-117,
 * EnvConstraintCuboid.cu:84-171, EnvConstraintCylinder.cu:107-196) and
 * calculateTotalCosts (base/States.cu:5-21).
 * mode GBMP_CHECK_VERDICT: d_verdict[n] = 1 if the state collides (any-hit, early exit).
 * mode GBMP_CHECK_COST: also d_costs[4*n] (SoA slots: 0 self, 1 spheres, 2 cuboids,
 * 3 cylinders; NULL allowed) and d_total[n] (NULL allowed); verdict = total != 0. */
#define GBMP_CHECK_VERDICT 0
#define GBMP_CHECK_COST 1
GBMP_API gbmp_status gbmp_check_states(gbmp_robot robot, gbmp_env env, const float *d_q, int64_t n,
                              int32_t mode, uint8_t *d_verdict, float *d_costs, float *d_total,
                              void *stream);
/* gbmp_check_states that also writes the FK it computed, replacing the pair
 * SingleArmStates::update (SingleArmStates.cu:696-723) + SingleArmSpace::checkStates
 * (SingleArmSpace.cu:1572-1602) with one FK per state: d_poses [n*L*16] row-major 4x4
 * link poses and d_centers [n*S*3] sphere centres, each NULL allowed, exactly as gbmp_fk
 * writes them.  Verdicts and costs are those of gbmp_check_states. */
GBMP_API gbmp_status gbmp_check_states_fk(gbmp_robot robot, gbmp_env env, const float *d_q, int64_t n,
                                          int32_t mode, uint8_t *d_verdict, float *d_costs, float *d_total,
                                          float *d_poses, float *d_centers, void *stream);

/* State checks of many (robot, scene) requests in one launch (no reference counterpart:
 * the reference checks one space's states per checkStates call, SingleArmSpace.cu:
 * 1572-1602).  Each request names its robot, scene, states and outputs (the arguments of
 * gbmp_check_states_fk); its outputs are bit-identical to that call's.  The handle owns a
 * pinned and a device descriptor table of max_requests entries, so a run allocates
 * nothing; a run waits (on the host) until the previous run's descriptors have been
 * uploaded, so one handle serves one stream at a time (use one handle per stream).  All
 * robots must live on the device the handle was created on.  Requests with n = 0 are
 * skipped. */
typedef struct gbmp_check_batch_s *gbmp_check_batch;
typedef struct gbmp_check_request {
    gbmp_robot robot;
    gbmp_env env;
    const float *d_q;         /* [n x L] */
    int64_t n;
    uint8_t *d_verdict;       /* [n] or NULL */
    float *d_costs;           /* [4 x n] (GBMP_CHECK_COST) or NULL */
    float *d_total;           /* [n] (GBMP_CHECK_COST) or NULL */
    float *d_poses;           /* [n x L x 16] or NULL */
    float *d_centers;         /* [n x S x 3] or NULL */
} gbmp_check_request;
GBMP_API gbmp_status gbmp_check_batch_create(int32_t max_requests, gbmp_check_batch *out);
GBMP_API gbmp_status gbmp_check_batch_run(gbmp_check_batch batch, const gbmp_check_request *requests,
                                          int32_t n_requests, int32_t mode, void *stream);
GBMP_API gbmp_status gbmp_check_batch_destroy(gbmp_check_batch batch);

/* Edge validation, replacing SingleArmSpace::checkMotions / checkUnconstrainedMotions
 * (SingleArmSpace.cu:628-848; step rule KernelGenerator.h:408-465, interpolation
 * :467-522, feasibility SingleArmSpace.cu:603-626).  Edge k runs from d_from[k] to
 * d_to[k] ([E*L] each).  States are generated on the fly, never materialised.
 * Outputs (device, any may be NULL): d_ok[E] 1 = collision-free; d_first_hit[E] lowest
 * colliding state index, -1 for a free edge, -2 for an edge of more than 4,194,304
 * interpolated states, which is not validated (d_ok 0); d_length[E] L2 length (the
 * reference's motion cost); d_num_steps[E] interpolated state count (4,194,305 for an edge
 * that is too long).  step_rule GBMP_STEP_L2 is the reference rule; GBMP_STEP_LINF
 * bounds the per-joint step by `resolution` instead.  resolution <= 0 uses the robot's
 * resolution.  Asynchronous: three launches on `stream`, no host synchronisation (the
 * reference reads step counts back to the host, SingleArmSpace.cu:728-739).  The working
 * memory belongs to the robot handle: calls with one robot on different streams must be
 * ordered by the caller.  Each edge is validated by one warp, stopping at a colliding
 * state; the edges are taken longest first.  Robots of up to 32 sphere-carrying links are
 * validated by chunks of consecutive states (10 states; 4 for robots of more than 16
 * links), others state by state; gbmp_robot_set_edge_form overrides the form for one
 * robot handle.  With d_first_hit the chunks go in state order (the first 4 states, then
 * the chunks in turn) and the edge stops at its lowest colliding state.  Without it (the
 * reference's outputs: verdict and cost) the chunks go coarse to fine -- the first 4
 * states, the last chunk, then the chunks between in 8 interleaved passes -- and the
 * edge stops at the first colliding state met: the same verdicts, fewer states checked
 * on colliding edges. */
#define GBMP_STEP_L2 0
#define GBMP_STEP_LINF 1
/* pRRTC's `granularity` (pRRTC/src/planning/pRRTC.cu:430-440): every edge is checked at
 * a fixed count of equal steps, `resolution` rounded down to an integer G in [1, 1e6]:
 * the states at k / G of the edge (k = 0..G in gbmp_check_edges, k = 1..G in the
 * planners, whose edge start is already a tree node). */
#define GBMP_STEP_COUNT 2
GBMP_API gbmp_status gbmp_check_edges(gbmp_robot robot, gbmp_env env, const float *d_from, const float *d_to,
                             int64_t n_edges, float resolution, int32_t step_rule, uint8_t *d_ok,
                             int32_t *d_first_hit, float *d_length, int32_t *d_num_steps, void *stream);

/* Tuning and test control of the edge-validation form of one robot handle: 0 automatic
 * (the default), 1 state by state, 4 or 10 consecutive states per chunk (chunks need a
 * robot of at most 32 sphere-carrying links; others stay state by state).  Results do
 * not depend on the form.  No counterpart in the reference. */
GBMP_API gbmp_status gbmp_robot_set_edge_form(gbmp_robot robot, int32_t form);

/* gbmp_check_edges without any allocation: same arguments, kernels and results (both
 * entry points run one implementation), but its working memory is a fixed 4.5 MiB device
 * array inside the library (one per device) instead of a buffer grown with cudaMalloc.
 * No counterpart in the reference, whose checkMotions allocates and frees its state
 * buffers on every call.
 * For callers that must not allocate device memory: a control loop with a latency bound
 * (cudaMalloc / cudaFree can block and cudaFree synchronises the device), a process whose
 * device memory is fully reserved up front, or code that runs while memory is exhausted.
 * Limits: n_edges <= 65536 and n_edges * num_links <= 1,048,576; larger calls return
 * GBMP_ERR_CAPACITY with a message and do nothing (use gbmp_check_edges or split them).
 * The scratch's counters must start at zero: every call zeroes them on `stream` before
 * its first kernel; all other scratch is written before it is read.
 * Calls on one device share the scratch: calls whose work overlaps on the device (other
 * streams, other host threads) race and give wrong results; order them on one stream or
 * synchronise between them.  Different devices do not share it.
 * The first call on each device (n_edges = 0 is enough) looks up the scratch's device
 * address with that device current; a caller that captures streams makes that first
 * call before it begins a capture.  The address belongs to the device's context and is
 * kept for the life of the process: do not call this entry point on a device after
 * cudaDeviceReset of that device.  Asynchronous like gbmp_check_edges. */
GBMP_API gbmp_status gbmp_check_edges_noalloc(gbmp_robot robot, gbmp_env env, const float *d_from,
                                     const float *d_to, int64_t n_edges, float resolution,
                                     int32_t step_rule, uint8_t *d_ok, int32_t *d_first_hit,
                                     float *d_length, int32_t *d_num_steps, void *stream);

/* Nearest neighbour, replacing SingleArmStateManager::find_the_nearest_neighbors
 * (SingleArmStates.cu:1265-1431).  d_tree [M*L]; candidate indices d_cand [n_cand]
 * (NULL = all M nodes); d_queries [Q*L]; d_out [Q] index of the nearest candidate by
 * L2 distance over the robot's active joints; exact ties go to the lowest candidate
 * position. */
GBMP_API gbmp_status gbmp_nearest(gbmp_robot robot, const float *d_tree, int64_t M, const int32_t *d_cand,
                         int64_t n_cand, const float *d_queries, int64_t Q, int32_t *d_out, void *stream);

/* Steer, replacing SingleArmStateManager::interpolateToStates (SingleArmStates.cu:1488-1557)
 * and SingleArmSpace::interpolate (SingleArmSpace.cu:219-249, :1368-1409): d_to[k] is moved
 * onto the segment from d_tree[d_idx[k]] (or d_from[k] when d_idx is NULL) so that its L2
 * distance is at most max_distance.  In place on d_to [n*L]. */
GBMP_API gbmp_status gbmp_steer(gbmp_robot robot, const float *d_from, const int32_t *d_idx, float *d_to,
                       int64_t n, float max_distance, void *stream);

/* Gather of stored states by index, replacing SingleArmStateManager::get_states
 * (SingleArmStates.cu:1433-1453, one cudaMemcpy per index there): d_dst[k] = d_src[d_idx[k]]
 * for k < n, rows of L floats, one launch.  An index outside [0, M) gives a row of NaN
 * and sets *d_bad to 1 when d_bad is not NULL (d_bad is only ever set, never cleared). */
GBMP_API gbmp_status gbmp_gather_states(int32_t L, const float *d_src, int64_t M, const int32_t *d_idx, int64_t n,
                               float *d_dst, int32_t *d_bad, void *stream);

/* Uniform samples within the joint limits, inactive joints at their defaults, replacing
 * SingleArmSpace::sample / sampleConfigurations (SingleArmSpace.cu:184-217, :251-403).
 * Counter-based Philox4x32-10: sample k, joint j uses counter (offset + k, j) and key seed,
 * so the stream is reproducible independent of the launch shape.  d_q [n*L]. */
GBMP_API gbmp_status gbmp_sample(gbmp_robot robot, uint64_t seed, uint64_t offset, int64_t n, float *d_q,
                        void *stream);

/* Projection onto a task-space region and the joint limits, replacing
 * SingleArmSpace::projectStates (SingleArmSpace.cu:1631-1662) with the projectable
 * TaskSpaceConstraint (TaskSpaceConstraint.cu:66-396) and BoundaryConstraint
 * (BoundaryConstraint.cu:36-155).  `iterations` rounds (the reference uses 10) of: FK;
 * the pose (x, y, z, roll, pitch, yaw) of `offset` in link `task_link`; the error
 * reference - pose with each component shrunk by its tolerance; the step
 * J_a^T (J_a J_a^T + 1e-4 I)^-1 error over the active joints (J: geometric Jacobian,
 * angular rows first); plus, with use_boundary, the pull back inside the limits; added to
 * the active joints.  The Euler-angle error is used as an angular error, as in the
 * reference, so orientation targets converge only near zero roll / pitch / yaw of the
 * constrained frame (choose `offset` accordingly, or loosen the orientation tolerances).
 * In place on d_q [n*L]; d_task_cost / d_bound_cost [n] (NULL allowed) get the final
 * costs of computeCost (0 below 1e-4).  task_link = -1 disables the task-space part. */
typedef struct gbmp_projection {
    int32_t task_link;
    float offset[16];      /* row-major 4x4 pose of the constrained frame in the task link */
    float reference[6];    /* x, y, z, roll, pitch, yaw in the base frame */
    float tolerance[6];
    int32_t use_boundary;
    int32_t iterations;
} gbmp_projection;
GBMP_API gbmp_status gbmp_project_states(gbmp_robot robot, const gbmp_projection *proj, float *d_q, int64_t n,
                                float *d_task_cost, float *d_bound_cost, void *stream);

/* Constrained motions, replacing SingleArmSpace::computeConstrainedMotions
 * (SingleArmSpace.cu:1049-1366), which checkMotions (:636-639, :1466-1477) and
 * getPathFromWaypoints (:1416-1419, :1479-1564) use when the space holds projectable
 * constraints.  Motion k walks from d_from[k] towards d_to[k] ([n*L] each): every
 * iteration moves all joints by `resolution` (<= 0: the robot's) along the unit direction
 * to the goal, then runs two projection passes of `proj` (its `iterations` is ignored);
 * the motion stops when the second pass's total error (task error norm + limit violation
 * norm) exceeds 1e-3, when the state is farther from the goal than the previous one or
 * moved more than 5 x resolution, or after max_iterations (the reference uses 10000);
 * each state reached while still approaching is recorded, and coming within
 * `resolution` of the goal achieves the motion.  d_ok[k] = 1 when the motion was
 * achieved and every recorded state is collision-free with zero task-space and
 * joint-limit cost (checkStates); d_cost[k] its length (L2 over all joints of the
 * recorded states, 0 when not ok); d_num_states[k] the number of recorded states; with
 * d_states [n * states_cap * L] non-NULL the first states_cap recorded states of each
 * motion.  Outputs may be NULL.  One launch, asynchronous on `stream`. */
GBMP_API gbmp_status gbmp_constrained_motions(gbmp_robot robot, gbmp_env env, const gbmp_projection *proj,
                                              const float *d_from, const float *d_to, int64_t n, float resolution,
                                              int32_t max_iterations, uint8_t *d_ok, float *d_cost,
                                              int32_t *d_num_states, float *d_states, int32_t states_cap,
                                              void *stream);

/* ---- parallel RRT-Connect ----
 * Replaces CPRRTC::RobotSolver (cudampl/CPRRTC/include/RobotSolver.h:84-101,
 * cudampl/CPRRTC/src/RobotSolver.cu:348-473) and pRRTC::solve (pRRTC/src/planning/
 * pRRTC.cu:607-766, settings pRRTC_settings.hh:3-16).  A planner owns two device-resident
 * trees of max_nodes nodes each and a path buffer; it can be reused for many solves with
 * the same robot (one solve at a time per planner). */
typedef struct gbmp_planner_s *gbmp_planner;

typedef struct gbmp_rrtc_settings {
    int32_t lanes;          /* parallel extension lanes (one 4-warp block each)          */
    int32_t max_iters;      /* iteration cap per lane                                    */
    float range;            /* maximum extension length, L2 over active joints            */
    float resolution;       /* edge collision-check step (<= 0: the robot's resolution)   */
    int32_t step_rule;      /* GBMP_STEP_L2, GBMP_STEP_LINF or GBMP_STEP_COUNT             */
    uint64_t seed;          /* Philox key; sample (lane, iteration, joint)                */
    double time_limit_s;    /* device-side deadline (<= 0: 10 s)                          */
    /* pRRTC's dynamic domain (pRRTC/src/planning/pRRTC.cu:418-424, :456-467, :584-596),
     * in single-problem and batched solves: a sample farther from its nearest node than that node's
     * radius is skipped; a failed extension sets the node's radius to dd_radius, or
     * shrinks it by (1 - dd_alpha) down to dd_min_radius; a successful one grows it by
     * (1 + dd_alpha).  0 = off (the other three are then ignored). */
    int32_t dynamic_domain;
    float dd_alpha;
    float dd_radius;
    float dd_min_radius;
    /* Tree balancing, the tree each lane grows per iteration (pRRTC/src/planning/
     * pRRTC.cu:348-371, pRRTC_settings.hh:10-11).  GBMP_BALANCE_DEFAULT (0): lanes split in
     * proportion to the other tree's share of the nodes, at every size.  GBMP_BALANCE_SIZE:
     * pRRTC strategy 1, the same while the trees differ by less than 1.5 x lanes nodes,
     * else every lane grows tree 0 when its share is below tree_ratio and tree 1 otherwise
     * (so a tree trapped in a pocket of free space takes every lane and an unsolvable
     * problem runs to its iteration cap or deadline rather than its node cap).
     * GBMP_BALANCE_SWAP: pRRTC strategy 2, a lane keeps its tree and swaps while the size
     * difference relative to its tree is below tree_ratio.  GBMP_BALANCE_NONE (pRRTC's
     * 0): half the lanes per tree.  tree_ratio <= 0 takes pRRTC's default for the
     * strategy (0.5, or 1.0 for strategy 2). */
    int32_t balance;
    float tree_ratio;
} gbmp_rrtc_settings;
#define GBMP_BALANCE_DEFAULT 0
#define GBMP_BALANCE_SIZE 1
#define GBMP_BALANCE_SWAP 2
#define GBMP_BALANCE_NONE 3

typedef struct gbmp_rrtc_result {
    int32_t solved;
    int32_t status;         /* 1 solved, 2 node cap, 3 iteration cap, 4 deadline            */
    int32_t path_len;       /* states in h_path (start first, goal last)                    */
    float cost;             /* path length, L2 over active joints                           */
    int32_t start_tree_size, goal_tree_size;
    int32_t iterations;     /* largest lane iteration reached                               */
    double kernel_ms;       /* device time of the planning launch                           */
} gbmp_rrtc_result;

/* A planner owns its trees (two of max_nodes nodes), a pinned path buffer of path_cap
 * states and a pinned input / outcome block; a solve resets only the tree slots the
 * previous solve wrote, in one launch, and reads its outcome after one synchronisation.
 * Solves on one planner must not overlap (one at a time, from any thread). */
GBMP_API gbmp_status gbmp_planner_create(gbmp_robot robot, int32_t max_nodes, int32_t path_cap,
                                         gbmp_planner *out);
GBMP_API gbmp_status gbmp_planner_destroy(gbmp_planner planner);
/* Several goals, replacing pRRTC::solve's goal list (pRRTC/src/planning/Planners.hh:75-78,
 * pRRTC.cu:640-700): every goal is a root of the goal tree, and the path ends at the
 * goal its chain reaches.  h_goals: [n_goals * L] full joint vectors, n_goals >= 1 and at
 * most the planner's max_nodes.  Otherwise as gbmp_rrtc_solve. */
GBMP_API gbmp_status gbmp_rrtc_solve_goals(gbmp_planner planner, gbmp_env env, const float *h_start,
                                           const float *h_goals, int32_t n_goals,
                                           const gbmp_rrtc_settings *settings, float *h_path, int32_t path_cap,
                                           gbmp_rrtc_result *result, void *stream);
/* h_start / h_goal: full joint vectors [L].  h_path: [path_cap * L] host buffer.
 * Returns GBMP_OK when solved, GBMP_ERR_NOT_SOLVED / GBMP_ERR_TIMEOUT otherwise (the
 * result struct is filled in every case).  Synchronous on `stream`. */
GBMP_API gbmp_status gbmp_rrtc_solve(gbmp_planner planner, gbmp_env env, const float *h_start,
                                     const float *h_goal, const gbmp_rrtc_settings *settings, float *h_path,
                                     int32_t path_cap, gbmp_rrtc_result *result, void *stream);

/* ---- batched planning ----
 * Many heterogeneous problems (different robots, scenes, start/goal) in one persistent
 * launch: block b serves problem b % n as lane b / n.  The reference has no batched
 * form; each result equals what the same problem gives on its own up to the lane
 * interleaving (the first connection found wins).  With use_graph the whole solve
 * (table upload, reset, planning, trace, result copy) is a captured CUDA graph that is
 * replayed while the shape (n, lanes, settings, launch footprint) stays the same.
 * h_paths: [n * path_cap * max_links] floats; problem i's path starts at
 * i * path_cap * max_links with its robot's L floats per state. */
typedef struct gbmp_batch_planner_s *gbmp_batch_planner;

typedef struct gbmp_rrtc_problem {
    gbmp_robot robot;
    gbmp_env env;
    const float *start;     /* host [L] */
    const float *goal;      /* host [L] */
    uint64_t seed;
} gbmp_rrtc_problem;

GBMP_API gbmp_status gbmp_batch_planner_create(int32_t max_problems, int32_t max_nodes, int32_t max_links,
                                               int32_t path_cap, gbmp_batch_planner *out);
GBMP_API gbmp_status gbmp_batch_planner_destroy(gbmp_batch_planner planner);
GBMP_API gbmp_status gbmp_rrtc_solve_batch(gbmp_batch_planner planner, int32_t n, const gbmp_rrtc_problem *problems,
                                           const gbmp_rrtc_settings *settings, int32_t lanes_per_problem,
                                           int32_t use_graph, gbmp_rrtc_result *results, float *h_paths,
                                           void *stream);
/* gbmp_rrtc_solve_batch with the lanes per problem chosen by the library's launch-shape
 * autotuner (no reference counterpart).  Decisions are keyed by the batch's shape: device,
 * problem count, use_graph, the multiset of per-problem (links, sphere count bucket,
 * obstacle count bucket) and the settings that change a lane's work (max_iters, range,
 * resolution, step rule, dynamic domain, balance).  Each new key tries the candidates 4,
 * 8, 16, 32 and 64 lanes per problem (those within the block limit) twice each on the
 * caller's own solves, timed on the host around the synchronous solve, then keeps the
 * candidate with the least time for every later solve of the key.  Results are those of
 * gbmp_rrtc_solve_batch with that lane count; *lanes_used (NULL allowed) returns it.
 * The decisions are kept in the process (all planners share them). */
GBMP_API gbmp_status gbmp_rrtc_solve_batch_auto(gbmp_batch_planner planner, int32_t n,
                                                const gbmp_rrtc_problem *problems,
                                                const gbmp_rrtc_settings *settings, int32_t use_graph,
                                                gbmp_rrtc_result *results, float *h_paths, int32_t *lanes_used,
                                                void *stream);
/* The autotuner's record for the shape of (problems, settings, use_graph): *count
 * candidates (0: shape not seen), their lanes and least times in ms (-1: not tried yet;
 * first `capacity` entries written, NULL allowed) and *chosen, the decided lanes per
 * problem or -1 while still exploring. */
GBMP_API gbmp_status gbmp_batch_autotune_lookup(int32_t n, const gbmp_rrtc_problem *problems,
                                                const gbmp_rrtc_settings *settings, int32_t use_graph,
                                                int32_t *lanes, double *ms, int32_t capacity, int32_t *count,
                                                int32_t *chosen);
/* Forgets every autotuner decision of the process. */
GBMP_API gbmp_status gbmp_batch_autotune_reset(void);

/* ---- continuous-batching request server ----
 * No counterpart in the reference (its callers run one request at a time).  Robots and
 * environments are registered once and stay resident; FK+collision requests are
 * batched as they arrive (grouped by robot and environment, all groups of a batch in one
 * gbmp_check_batch_run launch, batches overlapping on `num_streams` streams) and admitted while the in-flight
 * device bytes stay within hbm_budget_bytes; plan requests are solved in batched,
 * graph-captured launches by `plan_workers` threads with device-resident trees.
 * Host buffers passed to submit must stay valid until gbmp_server_wait returns. */
typedef struct gbmp_server_s *gbmp_server;

typedef struct gbmp_server_config {
    int32_t num_streams;          /* concurrent check batches                       */
    int64_t hbm_budget_bytes;     /* device bytes of in-flight check batches        */
    int64_t max_batch_states;     /* states per check batch                         */
    int32_t plan_workers;         /* threads solving plan batches (0: no planning)  */
    int32_t plan_batch;           /* problems per plan batch                        */
    int32_t plan_lanes;           /* lanes per problem                              */
    int32_t planner_max_nodes;    /* nodes per tree per problem                     */
    int32_t plan_path_cap;        /* path buffer per problem (states)               */
    int32_t plan_max_iters;
    float plan_range;
    float plan_resolution;
    int32_t step_rule;
    double plan_time_limit_s;
    /* Blocks of one plan launch.  Plan launches are persistent: their blocks hold their
     * SMs until the problems end, and check launches (on higher-priority streams) cannot
     * preempt them, so a plan launch that fills every SM delays every check behind it.
     * Capping the plan blocks leaves room on each SM for check blocks, at the price of plan
     * throughput: on one GB300 at 2000 req/s of the 70 % check / 30 % plan stream, a cap of
     * 3 blocks per SM over two plan workers (228 blocks each) cut the median latency from
     * 392 to 164 ms and the check p99 from 1.30 to 0.75 s, but served 1198 instead of 1498
     * req/s.  0: no cap (the planning kernel fits 5 blocks per SM). */
    int32_t plan_max_blocks;
} gbmp_server_config;

typedef struct gbmp_request_info {
    gbmp_status status;
    int32_t solved;
    int32_t path_len;
    float cost;
    double latency_ms;            /* submit to completion                            */
    double queue_ms;              /* submit to dispatch                              */
} gbmp_request_info;

typedef struct gbmp_server_metrics {
    int64_t completed, batches, plan_batches, states_checked, budget_in_use;
    double check_p50_ms, check_p95_ms, check_p99_ms;
    double plan_p50_ms, plan_p95_ms, plan_p99_ms;
    double elapsed_s;
} gbmp_server_metrics;

GBMP_API gbmp_status gbmp_server_create(const gbmp_server_config *config, gbmp_server *out);
GBMP_API gbmp_status gbmp_server_add_robot(gbmp_server server, gbmp_robot robot, int32_t *robot_id);
GBMP_API gbmp_status gbmp_server_add_env(gbmp_server server, gbmp_env env, int32_t *env_id);
GBMP_API gbmp_status gbmp_server_start(gbmp_server server);
/* h_q [n * L] (L of the robot); h_verdict [n] receives 1 for colliding states. */
GBMP_API gbmp_status gbmp_server_submit_check(gbmp_server server, int32_t robot_id, int32_t env_id, const float *h_q,
                                              int64_t n, uint8_t *h_verdict, int64_t *ticket);
/* h_path [path_cap * L] receives the path (start first) when solved. */
GBMP_API gbmp_status gbmp_server_submit_plan(gbmp_server server, int32_t robot_id, int32_t env_id,
                                             const float *h_start, const float *h_goal, uint64_t seed, float *h_path,
                                             int32_t path_cap, int64_t *ticket);
/* Blocks until the request finishes (or timeout_s passes: GBMP_ERR_TIMEOUT, the ticket
 * stays valid); info->status is the request's own status. */
GBMP_API gbmp_status gbmp_server_wait(gbmp_server server, int64_t ticket, double timeout_s, gbmp_request_info *info);
GBMP_API gbmp_status gbmp_server_stats(gbmp_server server, gbmp_server_metrics *out);
/* Stops the worker threads after the batches in flight finish. */
GBMP_API gbmp_status gbmp_server_destroy(gbmp_server server);

/* ---- instrumentation ----
 * With profiling enabled, CUDA events are recorded on the launching stream around
 * every launch of the named kernel families; gbmp_profile_read() waits for them and
 * returns the accumulated device time and launch count.  gbmp_launch_count() counts
 * every kernel launch made by the library since load. */
#define GBMP_PROF_EDGE_WAVE 0
#define GBMP_PROF_CHECK_STATES 1
#define GBMP_PROF_FK 2
#define GBMP_PROF_OTHER 3
GBMP_API gbmp_status gbmp_profile_enable(int32_t enable);
GBMP_API gbmp_status gbmp_profile_reset(void);
GBMP_API gbmp_status gbmp_profile_read(int32_t family, double *ms, int64_t *launches);
GBMP_API gbmp_status gbmp_launch_count(int64_t *count);
/* Executed-work accounting of the broad-phase collision kernels: while enabled, every
 * checked state adds the floating-point operations its tests executed (same weights as
 * the roofline model) and 1 to the state count.  Enabling resets the counters.  The
 * counting adds work, so time a batch with it off. */
GBMP_API gbmp_status gbmp_work_counting(int32_t enable);
GBMP_API gbmp_status gbmp_work_read(uint64_t *flops, uint64_t *states);

/* FP32 fused-multiply-add throughput of the current device, measured with a
 * register-resident FMA loop over `seconds` of wall time (the CUDA-core roofline
 * denominator for the FK + collision kernels).  Synchronous. */
GBMP_API gbmp_status gbmp_measure_fp32_peak(double seconds, double *tflops);

#ifdef __cplusplus
}
#endif
#endif /* GBMP_H */
