/*
 * Compiles libMobility's own NBody CUDA kernels (solvers/NBody/extra/NbodyRPY.cu,
 * "fast" schedule, GPU Gems 3 tiling, :26-97) for sm_103a into a cubin, straight
 * from the reference checkout.  TEST INFRASTRUCTURE ONLY: the GPU parity tests
 * load the cubin through oracle/ref_gpu_launcher.cpp to check libmobility_gb300
 * against the reference's own kernel on the same GB300, and to time it.
 *
 * Only explicit instantiations live here; the kernel code is the reference's.
 */
#include "solvers/NBody/extra/NbodyRPY.cu"

namespace nbody_rpy {
template __global__ void computeRPYBatchedFastGPU<OpenBoundary, real3>(
    const real3 *, const real3 *, const real3 *, real3 *, real3 *, Constants,
    blocksToCompute, int, int);
template __global__ void computeRPYBatchedFastGPU<BottomWall, real3>(
    const real3 *, const real3 *, const real3 *, real3 *, real3 *, Constants,
    blocksToCompute, int, int);
} // namespace nbody_rpy
