// Deterministic grid reductions (internal).
//
// GB300 executes FP64 at a small fraction of its FP32 rate, so everything
// inside a block stays in FP32: each warp sums its 32 values with an FP32
// xor butterfly and warp 0 sums the per-warp totals (a 256-value pairwise
// tree: relative error <= 8 roundings, ~5e-7).  Only the block partials are
// accumulated in FP64, by the last block to finish (atomic ticket), in block
// order -- so the result is bit-identical from run to run and independent of
// scheduling; a reconstruction gives the same scalars alone and inside a
// batch.  The ticket is reset by the last block, which keeps the kernels
// replayable inside a CUDA graph.
#pragma once
#include "common.cuh"

namespace asd {

// Block totals (valid in warp 0 after the call), FP32 tree; sh holds
// K * (NT/32) floats.  Every thread of the block must call it.
template <int NT, int K>
__device__ __forceinline__ void block_sum_f(const float (&v)[K], float (&out)[K],
                                            float *sh) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < K; k++) {
    float s = v[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) sh[k * (NT / 32) + warp] = s;
  }
  __syncthreads();
  if (warp == 0) {
#pragma unroll
    for (int k = 0; k < K; k++) {
      float t = lane < NT / 32 ? sh[k * (NT / 32) + lane] : 0.f;
#pragma unroll
      for (int o = NT / 64; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
      out[k] = t;
    }
  }
  __syncthreads();
}

// The last block's part of grid_sum: the FP64 totals of `nblocks` block
// partials (K values each) in a fixed order -- each of the first NT threads
// a strided subset, a warp butterfly, then the warps in order -- and the
// ticket reset.  Every thread of the block must call it (a block may have
// more than NT threads; the others only wait); all get the totals.
template <int NT, int K>
__device__ __forceinline__ void grid_sum_final(const double *partials,
                                               unsigned *counter, int nblocks,
                                               double (&tot)[K]) {
  __shared__ double sh[K * (NT / 32)];
  __shared__ double bc[K];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const bool in = threadIdx.x < NT;  // warp-uniform (NT is a multiple of 32)
#pragma unroll
  for (int k = 0; k < K; k++) {
    double a = 0.0;
    if (in)
      for (int b = threadIdx.x; b < nblocks; b += NT)
        a += ((volatile const double *)partials)[(long long)b * K + k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
    if (lane == 0 && in) sh[k * (NT / 32) + warp] = a;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < K; k++) {
      double a = 0.0;
      for (int w = 0; w < NT / 32; w++) a += sh[k * (NT / 32) + w];
      bc[k] = a;
    }
    *counter = 0u;
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < K; k++) tot[k] = bc[k];
  __syncthreads();  // sh / bc may be reused by the next call
}

// Grid-wide deterministic sum of K values per thread over the blocks
// bid = 0..nblocks-1 of one reduction (other grid dimensions select
// independent reductions through `partials`/`counter`).  `partials` holds
// nblocks*K doubles.  Returns true in every thread of the last block, where
// `tot` then holds the totals; other blocks return false.
template <int NT, int K>
__device__ __forceinline__ bool grid_sum(const float (&v)[K], double *partials,
                                         unsigned *counter, int bid,
                                         int nblocks, double (&tot)[K]) {
  static_assert(K <= kMaxReduceK, "partials are sized for kMaxReduceK values");
  __shared__ float shf[K * (NT / 32)];
  __shared__ bool last;
  float bs[K];
  block_sum_f<NT, K>(v, bs, shf);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < K; k++) partials[(long long)bid * K + k] = (double)bs[k];
    __threadfence();
    const unsigned t = atomicAdd(counter, 1u);
    last = (t == (unsigned)nblocks - 1);
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
  grid_sum_final<NT, K>(partials, counter, nblocks, tot);
  return true;
}

}  // namespace asd

namespace asd {

// FP64 variant for the FP64 entry points (the mex-level TV): every level of
// the reduction in FP64, same deterministic last-block scheme.
template <int NT>
__device__ __forceinline__ bool grid_sum_d(double v, double *partials,
                                           unsigned *counter, int nblocks,
                                           double &tot) {
  __shared__ double sh[NT / 32];
  __shared__ bool last;
  __shared__ double bc;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if (lane == 0) sh[warp] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < NT / 32; w++) s += sh[w];
    partials[inst_block()] = s;
    __threadfence();
    last = atomicAdd(counter, 1u) == (unsigned)nblocks - 1;
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
  double a = 0.0;
  for (int b = threadIdx.x; b < nblocks; b += NT) a += ((volatile double *)partials)[b];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
  __syncthreads();
  if (lane == 0) sh[warp] = a;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < NT / 32; w++) s += sh[w];
    bc = s;
    *counter = 0u;
  }
  __syncthreads();
  tot = bc;
  return true;
}

}  // namespace asd
