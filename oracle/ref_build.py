"""Recipe that builds the reference-pinning tools under oracle/_ref/ (test infrastructure).

The reference's FK, edge-step and interpolation kernels are CUDA source generated at
run time by cudampl/CUDAMPLib/include/spaces/KernelGenerator.h (header-only, standard
C++).  This recipe
  1. compiles oracle/ref_gen.cpp against that header, included unmodified from the
     reference tree, into oracle/_ref/ref_gen;
  2. for a given robot, runs ref_gen to obtain the reference's generated kernels and
     compiles them as host C++ (oracle/ref_shim.h maps the CUDA qualifiers; every
     kernel is one thread per configuration without shared memory) into a small
     shared library with launch loops.
Outputs go to oracle/_ref/ only.  Without the reference tree nothing is built and
callers get None.
"""
from __future__ import annotations

import ctypes as C
import hashlib
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
# The reference tree (read-only); GBMP_REFERENCE_ROOT points elsewhere when it lies elsewhere.
REF_ROOT = os.environ.get("GBMP_REFERENCE_ROOT", "/root/reference")
REF_INCLUDE = os.path.join(REF_ROOT, "cudampl/CUDAMPLib/include")
GEN = os.path.join(OUT, "ref_gen")

_HARNESS = r'''
#include "ref_shim.h"
%(fk)s
%(step)s
%(interp)s
extern "C" void ref_fk(const float *q, int n, float *poses) {
    blockDim.x = 1;
    for (int i = 0; i < n; ++i) { blockIdx.x = i; threadIdx.x = 0; kin_forward_nvrtc_kernel(q, n, poses); }
}
extern "C" void ref_step(float *from, float *to, int n, float res, int *ns, float *dir, float *dist) {
    blockDim.x = 1;
    for (int i = 0; i < n; ++i) { blockIdx.x = i; threadIdx.x = 0; get_step_nvrtc_kernel(from, to, n, res, ns, dir, dist); }
}
extern "C" void ref_interp(const float *from, const float *to, int n, const int *start, int *ns,
                           const float *dir, float *out) {
    blockDim.x = 1;
    for (int i = 0; i < n; ++i) { blockIdx.x = i; threadIdx.x = 0;
        calculate_interpolated_state_nvrtc_kernel(from, to, n, start, ns, dir, out); }
}
'''


def available() -> bool:
    return os.path.exists(os.path.join(REF_INCLUDE, "spaces", "KernelGenerator.h"))


# The reference's kernels are compiled by NVRTC / nvcc with multiply-add contraction on
# (their default).  GCC forms fused multiply-adds from -O2 on under -ffp-contract=fast,
# with FMA instructions enabled (-mfma where the target needs the flag, as x86-64 does;
# aarch64 has them in the base ISA).
_HOST_FLAGS = ["-O2", "-ffp-contract=fast", "-shared", "-fPIC", "-pthread"]


def _host_library(tag: str, src: str, std: str) -> str:
    """Compile `src` (host C++ around reference code) into oracle/_ref/, cached by a hash
    of the source, the shims and the flags; returns the library path."""
    shims = "".join(open(os.path.join(HERE, f)).read() for f in ("ref_shim.h", "ref_block_shim.h"))
    key = hashlib.sha1((src + shims + " ".join(_HOST_FLAGS) + std).encode()).hexdigest()[:16]
    so = os.path.join(OUT, f"{tag}_{key}.so")
    if not os.path.exists(so):
        os.makedirs(OUT, exist_ok=True)
        cpp = os.path.join(OUT, f"{tag}_{key}.cpp")
        with open(cpp, "w") as fh:
            fh.write(src)
        cmd = ["g++", std] + _HOST_FLAGS + ["-I" + HERE, cpp, "-o", so]
        try:
            subprocess.run(cmd[:2] + ["-mfma"] + cmd[2:], check=True, capture_output=True)
        except subprocess.CalledProcessError:
            subprocess.run(cmd, check=True)
    return so


def build(force: bool = False):
    """Build oracle/_ref/ref_gen when the reference tree is present; returns its path or None."""
    if not available():
        return None
    os.makedirs(OUT, exist_ok=True)
    src = os.path.join(HERE, "ref_gen.cpp")
    if force or not os.path.exists(GEN) or os.path.getmtime(GEN) < os.path.getmtime(src):
        subprocess.run(["g++", "-O1", "-std=c++17", "-I" + REF_INCLUDE, "-include", "vector", src, "-o", GEN],
                       check=True)
    return GEN


def _robot_text(robot) -> str:
    L = robot.num_links
    f = lambda a: " ".join(repr(float(x)) for x in np.asarray(a, np.float64).reshape(-1))
    return "\n".join([str(L), " ".join(str(int(t)) for t in robot.joint_types), f(robot.joint_poses.reshape(-1)),
                      f(robot.joint_axes.reshape(-1)), " ".join(str(int(p)) for p in robot.parent)]) + "\n"


def robot_kernels(robot):
    """ctypes library with ref_fk / ref_step / ref_interp for `robot`, or None."""
    gen = build()
    if gen is None:
        return None
    text = _robot_text(robot)
    out = subprocess.run([gen], input=text, capture_output=True, text=True, check=True).stdout
    parts = {}
    cur = None
    for line in out.splitlines(keepends=True):
        if line.startswith("//@@ "):
            cur = line.split()[1]
            parts[cur] = ""
        elif cur:
            parts[cur] += line
    lib = C.CDLL(_host_library("ref_kernels", _HARNESS % parts, "-std=c++17"))
    f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
    i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
    lib.ref_fk.argtypes = [f32p, C.c_int, f32p]
    lib.ref_step.argtypes = [f32p, f32p, C.c_int, C.c_float, i32p, f32p, f32p]
    lib.ref_interp.argtypes = [f32p, f32p, C.c_int, i32p, i32p, f32p, f32p]
    return lib


# ---------------------------------------------------------------------------------
# Collision-cost kernels (cudampl/CUDAMPLib/src/constraints/*.cu).  Those files also
# hold the constraint classes, which need the reference's headers (Eigen, CUDA
# runtime); the recipe takes from them, unmodified, only the four cost kernels, the two
# inverse-pose helpers and the body of the self-collision constructor (the pair list),
# and compiles those for the host with oracle/ref_block_shim.h.
# ---------------------------------------------------------------------------------
REF_SRC = os.path.join(REF_ROOT, "cudampl/CUDAMPLib/src/constraints")

_COST_HARNESS = r'''
#include "ref_block_shim.h"
#include <algorithm>

namespace CUDAMPLib {
float sdata[1024];   // the kernels' extern __shared__ array (256 floats a block)

// util.h's flattening of the link-pair mask (only fills the unused device copy here)
inline std::vector<int> boolMatrixFlatten(const std::vector<std::vector<bool>> &m) {
    std::vector<int> out;
    for (const auto &row : m)
        for (bool b : row) out.push_back(b ? 1 : 0);
    return out;
}

%(cuboid_inv)s

%(k_sphere)s

%(k_cuboid)s

%(k_cylinder)s

%(k_self)s

struct RefSelfPairs {
    int *d_self_collision_enables_map = nullptr;
    int num_of_self_collision_check_ = 0;
    int *d_collision_sphere_indices_1 = nullptr;
    int *d_collision_sphere_indices_2 = nullptr;
    float *d_collision_distance_threshold = nullptr;
    std::vector<int> collision_sphere_indices_1;
    std::vector<int> collision_sphere_indices_2;
    std::vector<float> collision_distance_threshold;
    void build(const std::string &constraint_name, const std::vector<int> &self_collision_spheres_map,
               const std::vector<float> &self_collision_spheres_radius,
               const std::vector<std::vector<bool>> &self_collision_enables_map)
%(self_ctor)s
    ~RefSelfPairs() {
        cudaFree(d_self_collision_enables_map);
        cudaFree(d_collision_sphere_indices_1);
        cudaFree(d_collision_sphere_indices_2);
        cudaFree(d_collision_distance_threshold);
    }
};
}  // namespace CUDAMPLib

%(cylinder_inv)s

static std::vector<float> ref_inverse_poses(bool cylinder, const float *pos, const float *rot, int O) {
    std::vector<float> inv(12 * (size_t)O);
    for (int o = 0; o < O; ++o) {
        std::vector<float> p(pos + 3 * o, pos + 3 * o + 3), r(rot + 9 * o, rot + 9 * o + 9);
        std::vector<float> m = cylinder ? ::computeInversePoseMatrix(p, r) : CUDAMPLib::computeInversePoseMatrix(p, r);
        std::copy(m.begin(), m.begin() + 12, inv.begin() + 12 * (size_t)o);
    }
    return inv;
}

extern "C" {
// centres [n*S*3], radius [S]; one block of 256 threads per configuration, as computeCost
void ref_cost_sphere(const float *c, const float *r, int S, int n, const float *op, const float *orad, int O,
                     float *out) {
    ref_block_launch(n, 256, [&] { CUDAMPLib::computeAndSumCollisionCostKernel(c, r, S, n, op, orad, O, out); });
}
void ref_cost_cuboid(const float *c, const float *r, int S, int n, const float *pos, const float *rot,
                     const float *mn, const float *mx, int O, float *out) {
    std::vector<float> inv = ref_inverse_poses(false, pos, rot, O);
    ref_block_launch(n, 256, [&] {
        CUDAMPLib::computeAndSumCuboidCollisionCostKernel(c, r, S, n, inv.data(), mn, mx, O, out);
    });
}
void ref_cost_cylinder(const float *c, const float *r, int S, int n, const float *pos, const float *rot,
                       const float *crad, const float *chei, int O, float *out) {
    std::vector<float> inv = ref_inverse_poses(true, pos, rot, O);
    ref_block_launch(n, 256, [&] {
        CUDAMPLib::computeAndSumCylinderCollisionCostKernel(c, r, S, n, inv.data(), crad, chei, O, out);
    });
}
// sphere_link [S], enables [L*L] (row-major 0/1); returns the pair count
int ref_cost_self(const float *c, const int *sphere_link, const float *r, const unsigned char *enables, int S, int L,
                  int n, float *out) {
    std::vector<int> map(sphere_link, sphere_link + S);
    std::vector<float> rad(r, r + S);
    std::vector<std::vector<bool>> en(L, std::vector<bool>(L));
    for (int i = 0; i < L; ++i)
        for (int j = 0; j < L; ++j) en[i][j] = enables[i * L + j] != 0;
    CUDAMPLib::RefSelfPairs sp;
    sp.build("self_collision_constraint", map, rad, en);
    const int P = sp.num_of_self_collision_check_;
    ref_block_launch(n, 256, [&] {
        CUDAMPLib::computeAndSumSelfCollisionCostKernel(c, n, S, P, sp.d_collision_sphere_indices_1,
                                                        sp.d_collision_sphere_indices_2,
                                                        sp.d_collision_distance_threshold, out);
    });
    return P;
}
}
'''


def _extract(text: str, start: str, body_only: bool = False) -> str:
    """The definition beginning at `start` (through its matching closing brace), or only
    its braced body; comments and literals are skipped while matching."""
    i = text.index(start)
    j = text.index("{", i)
    depth, k, n = 0, j, len(text)
    while k < n:
        if text.startswith("//", k):
            k = text.index("\n", k)
            continue
        if text.startswith("/*", k):
            k = text.index("*/", k) + 2
            continue
        c = text[k]
        if c in "\"'":
            k += 1
            while text[k] != c:
                k += 2 if text[k] == "\\" else 1
        elif c == "{":
            depth += 1
        elif c == "}":
            depth -= 1
            if depth == 0:
                break
        k += 1
    return text[j:k + 1] if body_only else text[i:k + 1]


def cost_available() -> bool:
    return all(os.path.exists(os.path.join(REF_SRC, f)) for f in
               ("EnvConstraintSphere.cu", "EnvConstraintCuboid.cu", "EnvConstraintCylinder.cu",
                "SelfCollisionConstraint.cu"))


def cost_kernels():
    """ctypes library with ref_cost_{self,sphere,cuboid,cylinder} built from the
    reference's own cost kernels, or None without the reference tree."""
    if not cost_available():
        return None
    os.makedirs(OUT, exist_ok=True)
    rd = lambda f: open(os.path.join(REF_SRC, f)).read()
    sph, cub, cyl, slf = (rd("EnvConstraintSphere.cu"), rd("EnvConstraintCuboid.cu"), rd("EnvConstraintCylinder.cu"),
                          rd("SelfCollisionConstraint.cu"))
    parts = dict(
        cuboid_inv=_extract(cub, "std::vector<float> computeInversePoseMatrix("),
        cylinder_inv=_extract(cyl, "std::vector<float> computeInversePoseMatrix("),
        k_sphere=_extract(sph, "__global__ void computeAndSumCollisionCostKernel("),
        k_cuboid=_extract(cub, "__global__ void computeAndSumCuboidCollisionCostKernel("),
        k_cylinder=_extract(cyl, "__global__ void computeAndSumCylinderCollisionCostKernel("),
        k_self=_extract(slf, "__global__ void computeAndSumSelfCollisionCostKernel("),
        self_ctor=_extract(slf, "SelfCollisionConstraint::SelfCollisionConstraint(", body_only=True),
    )
    lib = C.CDLL(_host_library("ref_costs", _COST_HARNESS % parts, "-std=c++20"))
    f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
    i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
    u8p = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")
    lib.ref_cost_sphere.argtypes = [f32p, f32p, C.c_int, C.c_int, f32p, f32p, C.c_int, f32p]
    lib.ref_cost_cuboid.argtypes = [f32p, f32p, C.c_int, C.c_int, f32p, f32p, f32p, f32p, C.c_int, f32p]
    lib.ref_cost_cylinder.argtypes = [f32p, f32p, C.c_int, C.c_int, f32p, f32p, f32p, f32p, C.c_int, f32p]
    lib.ref_cost_self.argtypes = [f32p, i32p, f32p, u8p, C.c_int, C.c_int, C.c_int, f32p]
    lib.ref_cost_self.restype = C.c_int
    return lib


# The state manager's nearest-neighbour and steer kernels and the sphere transform of
# SingleArmStates::update (cudampl/CUDAMPLib/src/states/SingleArmStates.cu), taken the
# same way.
REF_STATES = os.path.join(REF_ROOT, "cudampl/CUDAMPLib/src/states/SingleArmStates.cu")

_MANAGER_HARNESS = r'''
#include "ref_block_shim.h"

namespace CUDAMPLib {
alignas(16) char shared_mem[256 * 8];   // the NN kernel's extern __shared__ array

%(k_nn)s

%(k_steer)s

%(k_spheres)s
}  // namespace CUDAMPLib

extern "C" {
// one block of 256 threads per query, one group holding candidate indices cand[G]
void ref_nearest(float *query, int Q, float *tree, int *cand, int G, int L, int *active, int *out) {
    ref_block_launch(Q, 256, [&] {
        CUDAMPLib::find_the_nearest_neighbors_kernel(query, Q, tree, cand, G, L, active, 1, 0, out);
    });
}
// sphere centres [n*S*3] from link poses [n*L*16]; 256 threads a block, as update()
void ref_sphere_centers(int n, int L, int S, int *map, float *pos, float *poses, float *out) {
    ref_block_launch((n * S + 255) / 256, 256, [&] {
        CUDAMPLib::update_self_collision_spheres_kernel(n, L, S, map, pos, poses, out);
    });
}
// in place on to[n*L]; 256 threads a block, as interpolateToStates
void ref_steer(float *to, int n, float *tree, int L, int *nn, float max_distance) {
    ref_block_launch((n + 255) / 256, 256, [&] {
        CUDAMPLib::interpolate_to_states(to, n, tree, L, nn, max_distance);
    });
}
}
'''


def manager_available() -> bool:
    return os.path.exists(REF_STATES)


def manager_kernels():
    """ctypes library with ref_nearest / ref_steer / ref_sphere_centers built from the
    reference's own state kernels, or None without the reference tree."""
    if not manager_available():
        return None
    os.makedirs(OUT, exist_ok=True)
    text = open(REF_STATES).read()
    src = _MANAGER_HARNESS % dict(k_nn=_extract(text, "__global__ void find_the_nearest_neighbors_kernel("),
                                  k_steer=_extract(text, "__global__ void interpolate_to_states("),
                                  k_spheres=_extract(text, "__global__ void update_self_collision_spheres_kernel("))
    lib = C.CDLL(_host_library("ref_manager", src, "-std=c++20"))
    f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
    i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
    lib.ref_nearest.argtypes = [f32p, C.c_int, f32p, i32p, C.c_int, C.c_int, i32p, i32p]
    lib.ref_steer.argtypes = [f32p, C.c_int, f32p, C.c_int, i32p, C.c_float]
    lib.ref_sphere_centers.argtypes = [C.c_int, C.c_int, C.c_int, i32p, f32p, f32p, f32p]
    return lib


# SingleArmSpace::projectStates (SingleArmSpace.cu:1631-1712): the table FK kernel and its
# helpers (SingleArmStates.cu:11-221), the task-space and boundary gradient and cost
# kernels (TaskSpaceConstraint.cu, BoundaryConstraint.cu), the gradient sum
# (SingleArmStates.cu:819-845) and update_with_grad (SingleArmSpace.cu:1604-1626), taken
# the same way.  Each source's kernels sit in a namespace of their own (the two
# constraint files both name their kernel computeGradientErrorKernel and both define
# multiply4x4).
REF_SPACE = os.path.join(REF_ROOT, "cudampl/CUDAMPLib/src/spaces/SingleArmSpace.cu")
REF_TASK = os.path.join(REF_SRC, "TaskSpaceConstraint.cu")
REF_BOUND = os.path.join(REF_SRC, "BoundaryConstraint.cu")

_PROJECT_HARNESS = r'''
#include "ref_block_shim.h"
#include <vector>

#define CUDAMPLib_UNKNOWN 0
#define CUDAMPLib_REVOLUTE 1
#define CUDAMPLib_PRISMATIC 2
#define CUDAMPLib_FIXED 5

namespace CUDAMPLib {
namespace fk {
%(fk)s
}
namespace ts {
%(ts)s
}
namespace bd {
%(bd)s
}
namespace sp {
%(sp)s
}
}  // namespace CUDAMPLib

// The table-driven FK kernel alone (SingleArmStates::calculateForwardKinematics):
// link poses [n*L*16] of q [n*L].
extern "C" void ref_table_fk(int n, int L, int *types, float *poses, float *axes, int *parent, float *q,
                             float *out) {
    ref_serial_launch((n + 255) / 256, 256, [&] {
        CUDAMPLib::fk::kin_forward_kernel(q, L, n, types, poses, L, axes, parent, out);
    });
}

// `iterations` rounds of projectStates on q [n*L] (in place), then the final costs of
// both constraints (each output optional; a disabled constraint's cost is 0).
extern "C" void ref_project(int n, int L, int *types, float *poses, float *axes, int *parent, int *active,
                            float *lower, float *upper, int task_link, float *offset, float *reference,
                            float *tolerance, int use_boundary, int iterations, float *q, float *task_cost,
                            float *bound_cost) {
    using namespace CUDAMPLib;
    int A = 0;
    for (int j = 0; j < L; ++j) A += active[j] != 0;
    std::vector<float> lp((size_t)n * L * 16), jac((size_t)n * L * 6), jinv((size_t)n * A * 6 + 1);
    std::vector<float> grad(2 * (size_t)n * L, 0.f), cost(2 * (size_t)n, 0.f), tgrad((size_t)n * L, 0.f);
    std::vector<int> idx;
    if (task_link >= 0) idx.push_back(0);
    if (use_boundary) idx.push_back(1);
    const int nb = (n + 255) / 256, nbj = (n * L + 255) / 256;
    auto fk_all = [&] {
        ref_serial_launch(nb, 256, [&] { fk::kin_forward_kernel(q, L, n, types, poses, L, axes, parent, lp.data()); });
    };
    for (int it = 0; it < iterations; ++it) {
        fk_all();
        if (task_link >= 0)
            ref_serial_launch(nb, 256, [&] {
                ts::computeGradientErrorKernel(n, lp.data(), L, L, types, axes, task_link, offset, reference, tolerance,
                                               active, A, jac.data(), jinv.data(), grad.data(), cost.data());
            });
        if (use_boundary)
            ref_serial_launch(nb, 256, [&] {
                bd::computeGradientErrorKernel(q, active, lower, upper, n, L, cost.data() + n,
                                               grad.data() + (size_t)n * L);
            });
        if (idx.empty()) continue;
        ref_serial_launch(nbj, 256, [&] {
            fk::sum_gradients_kernel(n, L, 2, idx.data(), (int)idx.size(), grad.data(), tgrad.data());
        });
        ref_serial_launch(nbj, 256, [&] { sp::update_with_grad(q, tgrad.data(), 1.0f, n, L, active); });
    }
    fk_all();
    if (task_cost) {
        if (task_link >= 0)
            ref_serial_launch(nb, 256, [&] {
                ts::computeTaskSpaceCostKernel(n, lp.data(), L, task_link, offset, reference, tolerance, 0.0001f,
                                               task_cost);
            });
        else
            for (int i = 0; i < n; ++i) task_cost[i] = 0.f;
    }
    if (bound_cost) {
        if (use_boundary)
            ref_serial_launch(nb, 256, [&] {
                bd::computeBoundaryCostKernel(q, active, lower, upper, n, L, 0.0001f, bound_cost);
            });
        else
            for (int i = 0; i < n; ++i) bound_cost[i] = 0.f;
    }
}
'''


def project_available() -> bool:
    return all(os.path.exists(f) for f in (REF_STATES, REF_SPACE, REF_TASK, REF_BOUND))


def project_kernels():
    """ctypes library with ref_project (the reference's projection kernels) and
    ref_table_fk (its table-driven FK kernel), or None without the reference tree."""
    if not project_available():
        return None
    st, sp_, ts_, bd_ = (open(f).read() for f in (REF_STATES, REF_SPACE, REF_TASK, REF_BOUND))
    fk_names = ["__device__ __forceinline__ void multiply4x4(", "__device__ __forceinline__ void set_identity(",
                "__device__ __forceinline__ void fixed_joint_fn_cuda(",
                "__device__ __forceinline__ void make_rotation_axis_angle(",
                "__device__ __forceinline__ void revolute_joint_fn_cuda(",
                "__device__ __forceinline__ void prism_joint_fn_cuda(", "__global__ void kin_forward_kernel(",
                "__global__ void sum_gradients_kernel("]
    parts = dict(
        fk="\n\n".join(_extract(st, n) for n in fk_names),
        ts="\n\n".join(_extract(ts_, n) for n in ("__device__ __forceinline__ void multiply4x4(",
                                                   "__global__ void computeTaskSpaceCostKernel(",
                                                   "__global__ void computeGradientErrorKernel(")),
        bd="\n\n".join(_extract(bd_, n) for n in ("__global__ void computeBoundaryCostKernel(",
                                                   "__global__ void computeGradientErrorKernel(")),
        sp=_extract(sp_, "__global__ void update_with_grad("),
    )
    lib = C.CDLL(_host_library("ref_project", _PROJECT_HARNESS % parts, "-std=c++20"))
    f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
    i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
    lib.ref_table_fk.argtypes = [C.c_int, C.c_int, i32p, f32p, f32p, i32p, f32p, f32p]
    lib.ref_project.argtypes = [C.c_int, C.c_int, i32p, f32p, f32p, i32p, i32p, f32p, f32p, C.c_int, f32p, f32p,
                                f32p, C.c_int, C.c_int, f32p, f32p, f32p]
    return lib


# pRRTC's sphere-versus-environment test (pRRTC/src/planning/utils.cuh:15-242: the shape
# distance functions and sphere_environment_in_collision), over the reference's own
# shape and environment types (pRRTC/src/collision/shapes.hh, environment.hh, math.hh,
# included where they lie).
REF_PRRTC = os.path.join(REF_ROOT, "pRRTC/src")

_PRRTC_HARNESS = r'''
#include <array>
#include "ref_block_shim.h"
#include "shapes.hh"
#include "environment.hh"

namespace ppln::device_utils {
// the device overload of abs for floats
constexpr float abs(float x) { return x < 0.f ? -x : x; }
}

%(utils)s
}  // namespace ppln::device_utils

// Per configuration, 1 if any of its S spheres (centres cen [n*S*3], radii rad [S])
// collides with the environment: spheres [ns*4] (x y z r), capsules and z-aligned
// capsules [*7] (x1 y1 z1 xv yv zv r), cuboids and z-aligned cuboids [*15] (x y z,
// three axes, three half extents).
extern "C" void ref_prrtc_collide(int n, int S, float *cen, float *rad, int ns, float *sph, int nc, float *cap,
                                  int nzc, float *zcap, int nb, float *cub, int nzb, float *zcub,
                                  unsigned char *out) {
    using namespace ppln::collision;
    Environment<float> env;
    env.spheres = new Sphere<float>[ns];
    env.num_spheres = ns;
    for (int i = 0; i < ns; ++i) env.spheres[i] = Sphere<float>(sph[4 * i], sph[4 * i + 1], sph[4 * i + 2], sph[4 * i + 3]);
    auto caps = [](float *c, int k) {
        Capsule<float> *a = new Capsule<float>[k];
        for (int i = 0; i < k; ++i) {
            float *v = c + 7 * i;
            a[i] = Capsule<float>(v[0], v[1], v[2], v[3], v[4], v[5], v[6], 1.f / (v[3] * v[3] + v[4] * v[4] + v[5] * v[5]));
        }
        return a;
    };
    auto cubs = [](float *c, int k) {
        Cuboid<float> *a = new Cuboid<float>[k];
        for (int i = 0; i < k; ++i) {
            float *v = c + 15 * i;
            a[i] = Cuboid<float>(v[0], v[1], v[2], v[3], v[4], v[5], v[6], v[7], v[8], v[9], v[10], v[11], v[12],
                                 v[13], v[14]);
        }
        return a;
    };
    env.capsules = caps(cap, nc);
    env.num_capsules = nc;
    env.z_aligned_capsules = caps(zcap, nzc);
    env.num_z_aligned_capsules = nzc;
    env.cylinders = nullptr;
    env.num_cylinders = 0;
    env.cuboids = cubs(cub, nb);
    env.num_cuboids = nb;
    env.z_aligned_cuboids = cubs(zcub, nzb);
    env.num_z_aligned_cuboids = nzb;
    for (int s = 0; s < n; ++s) {
        bool hit = false;
        for (int k = 0; k < S && !hit; ++k) {
            const float *c = cen + 3 * ((size_t)s * S + k);
            hit = ppln::device_utils::sphere_environment_in_collision(&env, c[0], c[1], c[2], rad[k]);
        }
        out[s] = hit ? 1 : 0;
    }
}
'''


def prrtc_available() -> bool:
    return os.path.exists(os.path.join(REF_PRRTC, "planning", "utils.cuh")) and \
        os.path.exists(os.path.join(REF_PRRTC, "collision", "shapes.hh"))


def prrtc_collision():
    """ctypes library with ref_prrtc_collide (pRRTC's own sphere / capsule / cuboid
    tests), or None without the reference tree."""
    if not prrtc_available():
        return None
    text = open(os.path.join(REF_PRRTC, "planning", "utils.cuh")).read()
    sig = "__device__ __forceinline__ bool sphere_environment_in_collision("
    i = text.index("namespace ppln::device_utils {")
    end = text.index(sig) + len(_extract(text, sig))
    src = _PRRTC_HARNESS % dict(utils=text[i:end])
    so_path = _host_library("ref_prrtc", src.replace('#include "shapes.hh"', '#include "%s"' % os.path.join(
        REF_PRRTC, "collision", "shapes.hh")).replace('#include "environment.hh"', '#include "%s"' % os.path.join(
            REF_PRRTC, "collision", "environment.hh")), "-std=c++20")
    lib = C.CDLL(so_path)
    f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
    u8p = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")
    lib.ref_prrtc_collide.argtypes = [C.c_int, C.c_int, f32p, f32p, C.c_int, f32p, C.c_int, f32p, C.c_int, f32p,
                                      C.c_int, f32p, C.c_int, f32p, u8p]
    return lib


def build_all():
    """Every reference-pinning tool that the reference tree allows (none without it):
    the kernel generator, the collision-cost, state, projection and pRRTC collision
    libraries.  Returns the names built."""
    built = []
    if build() is not None:
        built.append("ref_gen")
    for name, fn in (("costs", cost_kernels), ("manager", manager_kernels), ("project", project_kernels),
                     ("prrtc", prrtc_collision)):
        if fn() is not None:
            built.append(name)
    return built


if __name__ == "__main__":
    print(build(force=True), build_all())
