// ref_block_shim.h -- lets the reference's collision-cost kernels run as host C++.
//
// TEST INFRASTRUCTURE ONLY.  The cost kernels of cudampl/CUDAMPLib/src/constraints/
// (EnvConstraintSphere.cu, EnvConstraintCuboid.cu, EnvConstraintCylinder.cu,
// SelfCollisionConstraint.cu) take one block per configuration, stride their threads
// over the pairs and reduce the per-thread sums in shared memory between
// __syncthreads() barriers.  Here every CUDA thread of a block is a host thread:
// threadIdx / blockIdx are thread-local, __syncthreads() is a std::barrier over the
// block's threads, and the blocks of a launch run one after another (each thread walks
// the blocks in order, with a barrier between blocks), so the one shared array can
// serve every block.  The reduction tree, the per-thread strides and therefore the
// summation order are the reference's own.
#pragma once
#include <barrier>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

struct RefDim3 {
    unsigned x, y, z;
};
inline thread_local RefDim3 threadIdx = {0, 0, 0};
inline thread_local RefDim3 blockIdx = {0, 0, 0};
inline RefDim3 blockDim = {1, 1, 1};
inline std::barrier<> *ref_block_barrier = nullptr;

#define __global__
#define __device__
#define __host__
#define __forceinline__ inline
#define __shared__
#define __restrict__ __restrict

inline void __syncthreads() { ref_block_barrier->arrive_and_wait(); }

// CUDA's device overloads of min / max for floats (fminf / fmaxf semantics).
inline float max(float a, float b) { return fmaxf(a, b); }
inline float min(float a, float b) { return fminf(a, b); }

// Host stand-ins for the allocation calls of the constructors (host memory).
enum RefMemcpyKind { cudaMemcpyHostToDevice = 1, cudaMemcpyDeviceToHost = 2, cudaMemcpyDeviceToDevice = 3 };
template <class T>
inline int cudaMalloc(T **p, size_t bytes) {
    *p = static_cast<T *>(std::malloc(bytes ? bytes : 1));
    return 0;
}
inline int cudaMemcpy(void *dst, const void *src, size_t bytes, int) {
    if (bytes) std::memcpy(dst, src, bytes);
    return 0;
}
inline int cudaFree(void *p) {
    std::free(p);
    return 0;
}

// Runs `kernel()` for every (block, thread) of a launch on the calling thread, in order;
// for kernels without barriers or shared memory.
template <class F>
inline void ref_serial_launch(int grid, int block, F kernel) {
    blockDim = {(unsigned)block, 1, 1};
    for (int b = 0; b < grid; ++b) {
        blockIdx = {(unsigned)b, 0, 0};
        for (int t = 0; t < block; ++t) {
            threadIdx = {(unsigned)t, 0, 0};
            kernel();
        }
    }
}

// Runs `kernel()` as a launch of `grid` blocks of `block` threads.
template <class F>
inline void ref_block_launch(int grid, int block, F kernel) {
    std::barrier<> bar(block);
    ref_block_barrier = &bar;
    blockDim = {(unsigned)block, 1, 1};
    std::vector<std::thread> th;
    th.reserve(block);
    for (int t = 0; t < block; ++t)
        th.emplace_back([&, t] {
            threadIdx = {(unsigned)t, 0, 0};
            for (int b = 0; b < grid; ++b) {
                blockIdx = {(unsigned)b, 0, 0};
                kernel();
                bar.arrive_and_wait();   // the next block reuses the shared array
            }
        });
    for (auto &x : th) x.join();
    ref_block_barrier = nullptr;
}
