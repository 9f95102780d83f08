// ref_gen.cpp -- emits the reference's own generated CUDA kernels for a robot.
//
// TEST INFRASTRUCTURE ONLY.  Built by oracle/ref_build.py against the reference tree
// (cudampl/CUDAMPLib/include/spaces/KernelGenerator.h, included unmodified from where
// it lies).  Reads a robot description from stdin:
//   L
//   joint_types[L]
//   joint_poses[L*16]   (row-major)
//   joint_axes[L*3]
//   parent[L]
// and writes, separated by lines "//@@ <name>", the reference's FK kernel
// (genForwardKinematicsKernelCode), step kernel (genGetStepKernelCode) and
// interpolation kernel (genCalculateInterpolatedStateKernelCode).
#include <iostream>
#include <string>
#include <vector>

#include "spaces/KernelGenerator.h"

int main() {
    int L = 0;
    if (!(std::cin >> L) || L <= 0) return 2;
    std::vector<int> types(L), parent(L);
    std::vector<float> poses(16 * L), axes(3 * L);
    for (auto &t : types) std::cin >> t;
    for (auto &p : poses) std::cin >> p;
    for (auto &a : axes) std::cin >> a;
    for (auto &p : parent) std::cin >> p;
    if (!std::cin) return 3;
    std::cout << "//@@ fk\n"
              << CUDAMPLib::genForwardKinematicsKernelCode(types, L, L, poses, axes, parent) << "\n";
    std::cout << "//@@ step\n" << CUDAMPLib::genGetStepKernelCode(L) << "\n";
    std::cout << "//@@ interp\n" << CUDAMPLib::genCalculateInterpolatedStateKernelCode(L) << "\n";
    return 0;
}
