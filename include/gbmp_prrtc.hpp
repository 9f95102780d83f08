/*
 * gbmp_prrtc.hpp -- pRRTC's planning interface over libgbmp (header-only C++17).
 *
 * Mirrors pRRTC/src/planning/Planners.hh:12-23 (PlannerResult) and :75-78
 * (pRRTC::solve), pRRTC_settings.hh:3-16, and the shape and environment types of
 * pRRTC/src/collision/shapes.hh and environment.hh:11-45 (same names and fields), so a
 * caller written against pRRTC compiles against this header.  The planning itself is
 * gbmp_rrtc_solve_goals: every goal a root of the goal tree (pRRTC.cu:686-693), each
 * edge checked at `granularity` equal steps (GBMP_STEP_COUNT), `num_new_configs`
 * extension lanes, `range` steering, `max_samples` nodes per tree, `max_iters` lane
 * iterations, Philox samples with key 1 (pRRTC seeds its generators with 1), the
 * dynamic domain with its dd_* settings, and tree balancing by `balance` (0 none, 1
 * size, 2 swap) with `tree_ratio` (pRRTC.cu:348-371).
 *
 * The reference's Robot types carry generated FK and collision code.  Here a Robot type
 * names the libgbmp robot model to plan for and the configuration layout:
 *
 *     struct MyArm {
 *         static constexpr std::size_t dimension = 7;          // active joints
 *         using Configuration = std::array<float, dimension>;  // active-joint values
 *         static gbmp_robot handle();                          // from gbmp_robot_create
 *     };
 *
 * Scene conversion (exact: the same set of colliding sphere positions):
 *   - spheres stay spheres;
 *   - a capsule (segment x1 + t v, t in [0, 1], radius r) is the union of a cylinder
 *     around the segment and two spheres at its ends; a z-aligned capsule uses only zv,
 *     as the reference's sphere_z_aligned_capsule does (pRRTC/src/planning/utils.cuh);
 *   - a cuboid (centre, three unit axes, half extents) is an oriented box whose
 *     rotation has the axes as columns; a z-aligned cuboid uses the x-y parts of its
 *     first two axes and the z axis, as sphere_z_aligned_cuboid does;
 *   - `cylinders` are not tested by the reference's sphere_environment_in_collision and
 *     are not converted either.
 * Errors other than "no path" are thrown as std::runtime_error with gbmp_last_error().
 */
#pragma once

#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "gbmp.h"

struct pRRTC_settings {
    int max_samples = 1000000;
    int max_iters = 1000000;
    int num_new_configs = 600;
    int granularity = 64;
    float range = 0.5;

    int balance = 1;
    float tree_ratio = 0.5;

    bool dynamic_domain = true;
    float dd_alpha = 0.0001;
    float dd_radius = 4.0;
    float dd_min_radius = 1.0;
};

template <typename Robot>
struct PlannerResult {
    bool solved = false;
    std::vector<typename Robot::Configuration> path;
    int start_tree_size = 0;
    int goal_tree_size = 0;
    int path_length = 0;
    int iters = 0;
    float cost = 0.0;
    std::size_t wall_ns = 0;     // wall time of solve
    std::size_t kernel_ns = 0;   // the planning launch
    std::size_t copy_ns = 0;     // the rest of the library call: uploads, resets, path download
};

namespace ppln::collision {

template <typename DataT>
struct Shape {
    std::string name;
    DataT min_distance = 0;   // distance from the origin to the shape's surface
};

template <typename DataT>
struct Sphere : public Shape<DataT> {
    DataT x{}, y{}, z{}, r{};
    Sphere() = default;
    explicit Sphere(DataT x_, DataT y_, DataT z_, DataT r_) : x(x_), y(y_), z(z_), r(r_) {
        this->min_distance = std::sqrt(x * x + y * y + z * z) - r;
    }
};

template <typename DataT>
struct Cuboid : public Shape<DataT> {
    DataT x{}, y{}, z{};
    DataT axis_1_x{}, axis_1_y{}, axis_1_z{};
    DataT axis_2_x{}, axis_2_y{}, axis_2_z{};
    DataT axis_3_x{}, axis_3_y{}, axis_3_z{};
    DataT axis_1_r{}, axis_2_r{}, axis_3_r{};
    Cuboid() = default;
    explicit Cuboid(DataT x_, DataT y_, DataT z_, DataT a1x, DataT a1y, DataT a1z, DataT a2x, DataT a2y, DataT a2z,
                    DataT a3x, DataT a3y, DataT a3z, DataT r1, DataT r2, DataT r3)
        : x(x_), y(y_), z(z_), axis_1_x(a1x), axis_1_y(a1y), axis_1_z(a1z), axis_2_x(a2x), axis_2_y(a2y),
          axis_2_z(a2z), axis_3_x(a3x), axis_3_y(a3y), axis_3_z(a3z), axis_1_r(r1), axis_2_r(r2), axis_3_r(r3) {
        // the origin's excess over each half extent along each axis
        const DataT e1 = std::max(DataT(0), std::abs(a1x * x + a1y * y + a1z * z) - r1);
        const DataT e2 = std::max(DataT(0), std::abs(a2x * x + a2y * y + a2z * z) - r2);
        const DataT e3 = std::max(DataT(0), std::abs(a3x * x + a3y * y + a3z * z) - r3);
        this->min_distance = std::sqrt(e1 * e1 + e2 * e2 + e3 * e3);
    }
};

template <typename DataT>
struct Cylinder : public Shape<DataT> {
    DataT x1{}, y1{}, z1{};   // first end
    DataT xv{}, yv{}, zv{};   // to the second end
    DataT r{};
    DataT rdv{};              // 1 / |v|^2
    Cylinder() = default;
    explicit Cylinder(DataT x1_, DataT y1_, DataT z1_, DataT xv_, DataT yv_, DataT zv_, DataT r_, DataT rdv_)
        : x1(x1_), y1(y1_), z1(z1_), xv(xv_), yv(yv_), zv(zv_), r(r_), rdv(rdv_) {
        // closest point of the segment to the origin
        const DataT t = std::clamp(-(x1 * xv + y1 * yv + z1 * zv) * rdv, DataT(0), DataT(1));
        const DataT px = x1 + t * xv, py = y1 + t * yv, pz = z1 + t * zv;
        this->min_distance = std::sqrt(px * px + py * py + pz * pz) - r;
    }
};

template <typename DataT>
using Capsule = Cylinder<DataT>;

template <typename DataT>
struct Environment {
    Sphere<DataT> *spheres = nullptr;
    unsigned int num_spheres = 0;

    Capsule<DataT> *capsules = nullptr;
    unsigned int num_capsules = 0;

    Capsule<DataT> *z_aligned_capsules = nullptr;
    unsigned int num_z_aligned_capsules = 0;

    Cylinder<DataT> *cylinders = nullptr;
    unsigned int num_cylinders = 0;

    Cuboid<DataT> *cuboids = nullptr;
    unsigned int num_cuboids = 0;

    Cuboid<DataT> *z_aligned_cuboids = nullptr;
    unsigned int num_z_aligned_cuboids = 0;

    Environment() = default;
    Environment(const Environment &) = delete;
    Environment &operator=(const Environment &) = delete;
    // owns its arrays, allocated with new[] (environment.hh:37-44)
    ~Environment() {
        delete[] spheres;
        delete[] capsules;
        delete[] cuboids;
        delete[] z_aligned_capsules;
        delete[] cylinders;
        delete[] z_aligned_cuboids;
    }
};

}  // namespace ppln::collision

namespace gbmp_prrtc_detail {

inline void check(gbmp_status s) {
    if (s != GBMP_OK) throw std::runtime_error(gbmp_last_error());
}

// Spheres, oriented boxes and cylinders of libgbmp for a pRRTC environment.
struct SceneArrays {
    std::vector<float> sph_pos, sph_r;
    std::vector<float> box_pos, box_rot, box_min, box_max;
    std::vector<float> cyl_pos, cyl_rot, cyl_r, cyl_h;

    void sphere(float x, float y, float z, float r) {
        sph_pos.insert(sph_pos.end(), {x, y, z});
        sph_r.push_back(r);
    }
    // the segment a -> a + v with radius r: a cylinder about it (local z along v) and
    // a sphere at each end
    void capsule(float ax, float ay, float az, float vx, float vy, float vz, float r) {
        sphere(ax, ay, az, r);
        sphere(ax + vx, ay + vy, az + vz, r);
        const float len = std::sqrt(vx * vx + vy * vy + vz * vz);
        if (!(len > 0.f)) return;
        const float zx = vx / len, zy = vy / len, zz = vz / len;
        // a unit vector off the axis, then the right-handed completion
        float ux = 1.f, uy = 0.f, uz = 0.f;
        if (std::abs(zx) > 0.9f) { ux = 0.f; uy = 1.f; }
        float xx = uy * zz - uz * zy, xy = uz * zx - ux * zz, xz = ux * zy - uy * zx;
        const float xn = std::sqrt(xx * xx + xy * xy + xz * xz);
        xx /= xn; xy /= xn; xz /= xn;
        const float yx = zy * xz - zz * xy, yy = zz * xx - zx * xz, yz = zx * xy - zy * xx;
        cyl_pos.insert(cyl_pos.end(), {ax + 0.5f * vx, ay + 0.5f * vy, az + 0.5f * vz});
        cyl_rot.insert(cyl_rot.end(), {xx, yx, zx, xy, yy, zy, xz, yz, zz});   // columns x, y, z
        cyl_r.push_back(r);
        cyl_h.push_back(len);
    }
    void cuboid(float x, float y, float z, const float a1[3], const float a2[3], const float a3[3], float r1,
                float r2, float r3) {
        box_pos.insert(box_pos.end(), {x, y, z});
        box_rot.insert(box_rot.end(), {a1[0], a2[0], a3[0], a1[1], a2[1], a3[1], a1[2], a2[2], a3[2]});
        box_min.insert(box_min.end(), {-r1, -r2, -r3});
        box_max.insert(box_max.end(), {r1, r2, r3});
    }
};

// The libgbmp form of a pRRTC environment (pure conversion, no device work).
inline SceneArrays scene_arrays(const ppln::collision::Environment<float> &e) {
    SceneArrays a;
    for (unsigned i = 0; i < e.num_spheres; ++i) a.sphere(e.spheres[i].x, e.spheres[i].y, e.spheres[i].z, e.spheres[i].r);
    for (unsigned i = 0; i < e.num_capsules; ++i) {
        const auto &c = e.capsules[i];
        a.capsule(c.x1, c.y1, c.z1, c.xv, c.yv, c.zv, c.r);
    }
    for (unsigned i = 0; i < e.num_z_aligned_capsules; ++i) {
        const auto &c = e.z_aligned_capsules[i];
        a.capsule(c.x1, c.y1, c.z1, 0.f, 0.f, c.zv, c.r);
    }
    for (unsigned i = 0; i < e.num_cuboids; ++i) {
        const auto &c = e.cuboids[i];
        const float a1[3] = {c.axis_1_x, c.axis_1_y, c.axis_1_z}, a2[3] = {c.axis_2_x, c.axis_2_y, c.axis_2_z},
                    a3[3] = {c.axis_3_x, c.axis_3_y, c.axis_3_z};
        a.cuboid(c.x, c.y, c.z, a1, a2, a3, c.axis_1_r, c.axis_2_r, c.axis_3_r);
    }
    for (unsigned i = 0; i < e.num_z_aligned_cuboids; ++i) {
        const auto &c = e.z_aligned_cuboids[i];
        const float a1[3] = {c.axis_1_x, c.axis_1_y, 0.f}, a2[3] = {c.axis_2_x, c.axis_2_y, 0.f},
                    a3[3] = {0.f, 0.f, 1.f};
        a.cuboid(c.x, c.y, c.z, a1, a2, a3, c.axis_1_r, c.axis_2_r, c.axis_3_r);
    }
    return a;
}

inline gbmp_env make_env(const ppln::collision::Environment<float> &e) {
    SceneArrays a = scene_arrays(e);
    gbmp_env env = nullptr;
    check(gbmp_env_create((int32_t)a.sph_r.size(), a.sph_pos.data(), a.sph_r.data(), (int32_t)a.box_min.size() / 3,
                          a.box_pos.data(), a.box_rot.data(), a.box_min.data(), a.box_max.data(),
                          (int32_t)a.cyl_r.size(), a.cyl_pos.data(), a.cyl_rot.data(), a.cyl_r.data(), a.cyl_h.data(),
                          &env));
    return env;
}

}  // namespace gbmp_prrtc_detail

namespace pRRTC {

template <typename Robot>
PlannerResult<Robot> solve(typename Robot::Configuration &start, std::vector<typename Robot::Configuration> &goals,
                           ppln::collision::Environment<float> &environment, pRRTC_settings &settings) {
    using Clock = std::chrono::steady_clock;
    using gbmp_prrtc_detail::check;
    const auto t0 = Clock::now();
    PlannerResult<Robot> out;
    if (goals.empty()) throw std::invalid_argument("pRRTC::solve: no goals");
    if (settings.balance != 0 && settings.balance != 1 && settings.balance != 2)
        throw std::invalid_argument("pRRTC::solve: balance must be 0, 1 or 2");
    gbmp_robot robot = Robot::handle();
    int32_t L = 0, S = 0, P = 0, dim = 0, cg = 0;
    check(gbmp_robot_info(robot, &L, &S, &P, &dim, &cg));
    if ((std::size_t)dim != Robot::dimension)
        throw std::invalid_argument("pRRTC::solve: Robot::dimension differs from the robot's active joints");
    std::vector<uint8_t> act(L);
    std::vector<float> defv(L);
    check(gbmp_robot_joints(robot, act.data(), defv.data(), nullptr, nullptr));
    auto full = [&](const typename Robot::Configuration &c, float *dst) {
        std::size_t k = 0;
        for (int j = 0; j < L; ++j) dst[j] = act[j] ? c[k++] : defv[j];
    };
    std::vector<float> h_start(L), h_goals((std::size_t)L * goals.size());
    full(start, h_start.data());
    for (std::size_t g = 0; g < goals.size(); ++g) full(goals[g], h_goals.data() + g * L);

    gbmp_env env = gbmp_prrtc_detail::make_env(environment);
    gbmp_planner planner = nullptr;
    const int32_t path_cap = (int32_t)std::min<long long>(2LL * settings.max_samples + 2, 1 << 20);
    gbmp_status st = gbmp_planner_create(robot, settings.max_samples, path_cap, &planner);
    if (st != GBMP_OK) {
        gbmp_env_destroy(env);
        check(st);
    }
    gbmp_rrtc_settings s{};
    s.lanes = settings.num_new_configs;
    s.max_iters = settings.max_iters;
    s.range = settings.range;
    s.resolution = (float)settings.granularity;
    s.step_rule = GBMP_STEP_COUNT;
    s.seed = 1;
    s.time_limit_s = 3600.0;
    s.dynamic_domain = settings.dynamic_domain ? 1 : 0;
    s.dd_alpha = settings.dd_alpha;
    s.dd_radius = settings.dd_radius;
    s.dd_min_radius = settings.dd_min_radius;
    s.balance = settings.balance == 0 ? GBMP_BALANCE_NONE : (settings.balance == 2 ? GBMP_BALANCE_SWAP : GBMP_BALANCE_SIZE);
    s.tree_ratio = settings.tree_ratio;
    // uninitialised: only the rows of the returned path are ever written or read
    std::unique_ptr<float[]> path(new float[(std::size_t)path_cap * L]);
    gbmp_rrtc_result r{};
    const auto t1 = Clock::now();
    st = gbmp_rrtc_solve_goals(planner, env, h_start.data(), h_goals.data(), (int32_t)goals.size(), &s, path.get(),
                               path_cap, &r, nullptr);
    const auto t2 = Clock::now();
    gbmp_planner_destroy(planner);
    gbmp_env_destroy(env);
    if (st != GBMP_OK && st != GBMP_ERR_NOT_SOLVED && st != GBMP_ERR_TIMEOUT) check(st);

    out.solved = r.solved != 0;
    out.start_tree_size = r.start_tree_size;
    out.goal_tree_size = r.goal_tree_size;
    out.iters = r.iterations;
    if (out.solved) {
        out.path_length = r.path_len;
        out.cost = r.cost;
        out.path.resize(r.path_len);
        for (int i = 0; i < r.path_len; ++i) {
            std::size_t k = 0;
            for (int j = 0; j < L; ++j)
                if (act[j]) out.path[i][k++] = path[(std::size_t)i * L + j];
        }
    }
    const auto ns = [](Clock::duration d) {
        return (std::size_t)std::chrono::duration_cast<std::chrono::nanoseconds>(d).count();
    };
    out.kernel_ns = (std::size_t)(r.kernel_ms * 1e6);
    const std::size_t call_ns = ns(t2 - t1);
    out.copy_ns = call_ns > out.kernel_ns ? call_ns - out.kernel_ns : 0;
    out.wall_ns = ns(Clock::now() - t0);
    return out;
}

}  // namespace pRRTC
