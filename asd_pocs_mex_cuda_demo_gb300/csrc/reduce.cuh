// Deterministic grid reductions in FP64 (internal).
//
// Each block reduces its values in a fixed tree order and stores the block
// partial; the last block to finish (atomic ticket) sums the partials in
// block order.  The result is bit-identical from run to run and independent
// of block scheduling, so a reconstruction gives the same scalars alone and
// inside a batch.  The ticket is reset by the last block, which makes the
// kernels replayable inside a CUDA graph.
#pragma once
#include "common.cuh"

namespace asd {

template <int NT, int K>
__device__ __forceinline__ void block_sum(double (&v)[K], double *sh) {
  // sh: K * (NT/32) doubles of shared memory
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < K; k++) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
  }
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k < K; k++) sh[k * (NT / 32) + warp] = v[k];
  }
  __syncthreads();
  if (warp == 0) {
#pragma unroll
    for (int k = 0; k < K; k++) {
      double t = lane < NT / 32 ? sh[k * (NT / 32) + lane] : 0.0;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
      v[k] = t;
    }
  }
  __syncthreads();
}

// Grid-wide deterministic sum of K values per thread over the blocks
// blockIdx.x = 0..nblocks-1 (blockIdx.y selects an independent reduction
// through `partials`/`counter`).  `partials` holds nblocks*K doubles.  Returns true in every thread of the last
// block, where `tot` then holds the totals; other blocks return false.
template <int NT, int K>
__device__ __forceinline__ bool grid_sum(double (&v)[K], double *partials,
                                         unsigned *counter, int nblocks,
                                         double (&tot)[K]) {
  __shared__ double sh[K * (NT / 32)];
  __shared__ bool last;
  block_sum<NT, K>(v, sh);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < K; k++) partials[(long long)blockIdx.x * K + k] = v[k];
    __threadfence();
    const unsigned t = atomicAdd(counter, 1u);
    last = (t == (unsigned)nblocks - 1);
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
  double acc[K];
#pragma unroll
  for (int k = 0; k < K; k++) {
    acc[k] = 0.0;
    for (int b = threadIdx.x; b < nblocks; b += NT)
      acc[k] += ((volatile double *)partials)[(long long)b * K + k];
  }
  block_sum<NT, K>(acc, sh);  // totals land in warp 0
  __shared__ double bc[K];
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < K; k++) bc[k] = acc[k];
    *counter = 0u;
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < K; k++) tot[k] = bc[k];
  return true;
}

}  // namespace asd
