// prrtc_scene_dump.cpp -- prints the libgbmp scene that include/gbmp_prrtc.hpp makes
// of a pRRTC environment (gbmp_prrtc_detail::scene_arrays; no device work, no library).
// Usage: prrtc_scene_dump <shapes.txt> <out.txt>.  Input: "ns" and ns lines "x y z r";
// "nc" and capsules "x1 y1 z1 xv yv zv r"; "nzc" and z-aligned capsules; "nb" and
// cuboids "x y z a1(3) a2(3) a3(3) r1 r2 r3"; "nzb" and z-aligned cuboids.  Output:
// lines "name count" then the values, for the sphere, box and cylinder arrays.
#include <cstdio>
#include <fstream>
#include <string>
#include <vector>

#include "gbmp_prrtc.hpp"

int main(int argc, char **argv) {
    if (argc != 3) return 2;
    std::ifstream in(argv[1]);
    ppln::collision::Environment<float> env;
    in >> env.num_spheres;
    env.spheres = new ppln::collision::Sphere<float>[env.num_spheres];
    for (unsigned i = 0; i < env.num_spheres; ++i) {
        float v[4];
        for (float &x : v) in >> x;
        env.spheres[i] = ppln::collision::Sphere<float>(v[0], v[1], v[2], v[3]);
    }
    auto caps = [&](ppln::collision::Capsule<float> *&arr, unsigned &cnt) {
        in >> cnt;
        arr = new ppln::collision::Capsule<float>[cnt];
        for (unsigned i = 0; i < cnt; ++i) {
            float v[7];
            for (float &x : v) in >> x;
            arr[i] = ppln::collision::Capsule<float>(v[0], v[1], v[2], v[3], v[4], v[5], v[6],
                                                     1.f / (v[3] * v[3] + v[4] * v[4] + v[5] * v[5]));
        }
    };
    auto cubs = [&](ppln::collision::Cuboid<float> *&arr, unsigned &cnt) {
        in >> cnt;
        arr = new ppln::collision::Cuboid<float>[cnt];
        for (unsigned i = 0; i < cnt; ++i) {
            float v[15];
            for (float &x : v) in >> x;
            arr[i] = ppln::collision::Cuboid<float>(v[0], v[1], v[2], v[3], v[4], v[5], v[6], v[7], v[8], v[9], v[10],
                                                    v[11], v[12], v[13], v[14]);
        }
    };
    caps(env.capsules, env.num_capsules);
    caps(env.z_aligned_capsules, env.num_z_aligned_capsules);
    cubs(env.cuboids, env.num_cuboids);
    cubs(env.z_aligned_cuboids, env.num_z_aligned_cuboids);
    if (!in) return 3;
    const gbmp_prrtc_detail::SceneArrays a = gbmp_prrtc_detail::scene_arrays(env);
    std::ofstream out(argv[2]);
    auto put = [&](const char *name, const std::vector<float> &v) {
        out << name << " " << v.size() << "\n";
        for (float x : v) {
            char b[32];
            std::snprintf(b, sizeof b, "%.9g ", x);
            out << b;
        }
        out << "\n";
    };
    put("sph_pos", a.sph_pos);
    put("sph_r", a.sph_r);
    put("box_pos", a.box_pos);
    put("box_rot", a.box_rot);
    put("box_min", a.box_min);
    put("box_max", a.box_max);
    put("cyl_pos", a.cyl_pos);
    put("cyl_rot", a.cyl_rot);
    put("cyl_r", a.cyl_r);
    put("cyl_h", a.cyl_h);
    return 0;
}
