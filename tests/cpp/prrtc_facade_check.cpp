// prrtc_facade_check.cpp -- drives include/gbmp_prrtc.hpp the way pRRTC's callers do
// (pRRTC/scripts/*.cpp: fill a ppln::collision::Environment, call pRRTC::solve<Robot>
// with a start, a list of goals and pRRTC_settings) for a 7-DOF arm built from tables.
// Usage: prrtc_facade_check <problem.txt> <results.txt>.  Problem file, one item per
// line: "L dim S", joint types, poses [L*16], axes [L*3], parents, sphere links, sphere
// positions [S*3], radii, active map, lower, upper, defaults, link-pair mask [L*L];
// then "ns" and ns lines "x y z r"; "nc" and nc lines "x1 y1 z1 xv yv zv r" (capsules);
// "nzc" and z-aligned capsules likewise; "nb" and nb lines "x y z a1(3) a2(3) a3(3) r1 r2
// r3" (cuboids); "nzb" and z-aligned cuboids likewise; the start [dim]; "ng" and ng goals
// [dim]; "max_samples max_iters num_new_configs granularity range".
// Results: lines "name count" then the values.
#include <array>
#include <cstdio>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include "gbmp_prrtc.hpp"

static gbmp_robot g_robot = nullptr;

struct TestArm {
    static constexpr std::size_t dimension = 7;
    using Configuration = std::array<float, dimension>;
    static gbmp_robot handle() { return g_robot; }
};

template <class T>
static std::vector<T> read_n(std::istream &in, std::size_t n) {
    std::vector<T> v(n);
    for (auto &x : v) in >> x;
    return v;
}

int main(int argc, char **argv) {
    if (argc != 3) return 2;
    std::ifstream in(argv[1]);
    int L = 0, dim = 0, S = 0;
    in >> L >> dim >> S;
    if (!in || dim != (int)TestArm::dimension) return 3;
    auto types = read_n<int>(in, L);
    auto poses = read_n<float>(in, 16 * L);
    auto axes = read_n<float>(in, 3 * L);
    auto parent = read_n<int>(in, L);
    auto slink = read_n<int>(in, S);
    auto spos = read_n<float>(in, 3 * S);
    auto srad = read_n<float>(in, S);
    auto active_i = read_n<int>(in, L);
    auto lower = read_n<float>(in, L);
    auto upper = read_n<float>(in, L);
    auto defv = read_n<float>(in, L);
    auto enables_i = read_n<int>(in, L * L);
    std::vector<uint8_t> active(active_i.begin(), active_i.end()), enables(enables_i.begin(), enables_i.end());
    gbmp_robot_desc desc{};
    desc.num_links = L;
    desc.joint_types = types.data();
    desc.joint_poses = poses.data();
    desc.joint_axes = axes.data();
    desc.parent = parent.data();
    desc.num_spheres = S;
    desc.sphere_link = slink.data();
    desc.sphere_pos = spos.data();
    desc.sphere_radius = srad.data();
    desc.active_joints = active.data();
    desc.lower = lower.data();
    desc.upper = upper.data();
    desc.default_values = defv.data();
    desc.self_enables = enables.data();
    desc.resolution = 0.01f;
    if (gbmp_robot_create(&desc, GBMP_ROBOT_GENERIC, &g_robot) != GBMP_OK) {
        std::cerr << gbmp_last_error() << "\n";
        return 4;
    }

    ppln::collision::Environment<float> env;
    unsigned n = 0;
    in >> n;
    env.num_spheres = n;
    env.spheres = new ppln::collision::Sphere<float>[n];
    for (unsigned i = 0; i < n; ++i) {
        float x, y, z, r;
        in >> x >> y >> z >> r;
        env.spheres[i] = ppln::collision::Sphere<float>(x, y, z, r);
    }
    auto read_capsules = [&](ppln::collision::Capsule<float> *&arr, unsigned &cnt) {
        in >> cnt;
        arr = new ppln::collision::Capsule<float>[cnt];
        for (unsigned i = 0; i < cnt; ++i) {
            float x1, y1, z1, xv, yv, zv, r;
            in >> x1 >> y1 >> z1 >> xv >> yv >> zv >> r;
            arr[i] = ppln::collision::Capsule<float>(x1, y1, z1, xv, yv, zv, r, 1.f / (xv * xv + yv * yv + zv * zv));
        }
    };
    read_capsules(env.capsules, env.num_capsules);
    read_capsules(env.z_aligned_capsules, env.num_z_aligned_capsules);
    auto read_cuboids = [&](ppln::collision::Cuboid<float> *&arr, unsigned &cnt) {
        in >> cnt;
        arr = new ppln::collision::Cuboid<float>[cnt];
        for (unsigned i = 0; i < cnt; ++i) {
            float v[15];
            for (float &x : v) in >> x;
            arr[i] = ppln::collision::Cuboid<float>(v[0], v[1], v[2], v[3], v[4], v[5], v[6], v[7], v[8], v[9], v[10],
                                                    v[11], v[12], v[13], v[14]);
        }
    };
    read_cuboids(env.cuboids, env.num_cuboids);
    read_cuboids(env.z_aligned_cuboids, env.num_z_aligned_cuboids);

    TestArm::Configuration start{};
    for (auto &x : start) in >> x;
    int ng = 0;
    in >> ng;
    std::vector<TestArm::Configuration> goals(ng);
    for (auto &g : goals)
        for (auto &x : g) in >> x;
    pRRTC_settings settings;
    in >> settings.max_samples >> settings.max_iters >> settings.num_new_configs >> settings.granularity >>
        settings.range;
    if (!in) return 5;

    PlannerResult<TestArm> res;
    try {
        res = pRRTC::solve<TestArm>(start, goals, env, settings);
    } catch (const std::exception &e) {
        std::cerr << "solve: " << e.what() << "\n";
        return 6;
    }
    std::ofstream out(argv[2]);
    out << "solved 1\n" << (res.solved ? 1 : 0) << "\n";
    out << "sizes 4\n"
        << res.start_tree_size << " " << res.goal_tree_size << " " << res.path_length << " " << res.iters << "\n";
    out << "cost 1\n" << res.cost << "\n";
    out << "times 3\n" << res.wall_ns << " " << res.kernel_ns << " " << res.copy_ns << "\n";
    out << "path " << res.path.size() * TestArm::dimension << "\n";
    for (auto &c : res.path)
        for (float x : c) {
            char b[32];
            std::snprintf(b, sizeof b, "%.9g ", x);
            out << b;
        }
    out << "\n";
    gbmp_robot_destroy(g_robot);
    return 0;
}
