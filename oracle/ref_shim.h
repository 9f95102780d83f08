// ref_shim.h -- lets the reference's generated CUDA kernels compile as host C++.
//
// TEST INFRASTRUCTURE ONLY.  The reference emits its FK / step / interpolation
// kernels as CUDA source strings (cudampl/CUDAMPLib/include/spaces/KernelGenerator.h)
// and compiles them with NVRTC.  Those kernels use one thread per configuration and
// no shared memory or barriers, so each "thread" can run as a plain function call
// with threadIdx / blockIdx / blockDim set by the caller (see ref_launch below).
#pragma once
#include <cmath>

struct RefDim3 {
    unsigned x, y, z;
};
static RefDim3 threadIdx = {0, 0, 0}, blockIdx = {0, 0, 0}, blockDim = {1, 1, 1};

#define __global__
#define __device__
#define __forceinline__ inline
#define __constant__ static
