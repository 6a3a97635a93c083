/*
 * Host shim for the reference's CUDA kernels -- TEST INFRASTRUCTURE.
 *
 * Force-included in front of Ax_cone_gpu.cu lines 1-297 and 339-776 (the
 * device functions and kernels; the two cudaMalloc-based launchers are left
 * out) so that the reference's own kernel code compiles with g++.  Kernels
 * become plain functions; blockIdx/threadIdx become thread-local variables
 * set by the launch emulation in ref_shim_tail.inc, which must be compiled in
 * the same translation unit.
 */
#ifndef ASDPOCS_REF_SHIM_HEAD_H
#define ASDPOCS_REF_SHIM_HEAD_H
#define __global__
#define __device__
struct ref_dim3 {
  unsigned x, y, z;
};
static thread_local ref_dim3 blockIdx;
static thread_local ref_dim3 threadIdx;
#endif
