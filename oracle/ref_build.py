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
REF_INCLUDE = "/root/reference/cudampl/CUDAMPLib/include"
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
    key = hashlib.sha1(text.encode()).hexdigest()[:16]
    so = os.path.join(OUT, f"ref_kernels_{key}.so")
    if not os.path.exists(so):
        out = subprocess.run([gen], input=text, capture_output=True, text=True, check=True).stdout
        parts = {}
        cur = None
        for line in out.splitlines(keepends=True):
            if line.startswith("//@@ "):
                cur = line.split()[1]
                parts[cur] = ""
            elif cur:
                parts[cur] += line
        cpp = os.path.join(OUT, f"ref_kernels_{key}.cpp")
        with open(cpp, "w") as fh:
            fh.write(_HARNESS % parts)
        # NVRTC contracts multiply-adds by default (fmad=true); -ffp-contract=fast with FMA
        # instructions mirrors that on the host.
        cmd = ["g++", "-O1", "-std=c++17", "-shared", "-fPIC", "-ffp-contract=fast", "-I" + HERE, cpp, "-o", so]
        try:
            subprocess.run(cmd[:5] + ["-mfma"] + cmd[5:], check=True, capture_output=True)
        except subprocess.CalledProcessError:
            subprocess.run(cmd, check=True)
    lib = C.CDLL(so)
    f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
    i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
    lib.ref_fk.argtypes = [f32p, C.c_int, f32p]
    lib.ref_step.argtypes = [f32p, f32p, C.c_int, C.c_float, i32p, f32p, f32p]
    lib.ref_interp.argtypes = [f32p, f32p, C.c_int, i32p, i32p, f32p, f32p]
    return lib


if __name__ == "__main__":
    print(build(force=True))
