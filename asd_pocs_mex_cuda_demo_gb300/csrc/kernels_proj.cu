// Projector kernels for sm_103a: Ax (ray-driven, one warp per ray) and Atx
// (voxel-driven, one thread per voxel), standalone and fused with the SART
// per-view update.  Compiled with -fmad=false (see projector.cuh).
#include "kernels.h"
#include "projector.cuh"
#include "reduce.cuh"

namespace asd {

namespace {

constexpr int kAxWarps = 4;            // rays per Ax block
constexpr int kAxThreads = kAxWarps * 32;
constexpr int kTileX = 32, kTileY = 8; // Atx voxel tile (x fastest)
constexpr int kAtxThreads = kTileX * kTileY;

__device__ __forceinline__ void tile_voxel(const Dims &D, int &ix, int &iy,
                                           int &iz) {
  const int tx = (D.nx + kTileX - 1) / kTileX;
  const int ty = (D.ny + kTileY - 1) / kTileY;
  int b = blockIdx.x;
  const int bx = b % tx;
  b /= tx;
  const int by = b % ty;
  iz = b / ty;
  ix = bx * kTileX + (threadIdx.x % kTileX);
  iy = by * kTileY + (threadIdx.x / kTileX);
}

int atx_blocks(const Dims &d) {
  return ((d.nx + kTileX - 1) / kTileX) * ((d.ny + kTileY - 1) / kTileY) * d.nz;
}

// ------------------------------------------------------------- standalone
__global__ void __launch_bounds__(kAxThreads)
    k_ax(const float *__restrict__ x, float *__restrict__ y,
         float *__restrict__ sr, ViewGeo G, Dims D) {
  const int lane = threadIdx.x & 31;
  const long long r = (long long)blockIdx.x * kAxWarps + (threadIdx.x >> 5);
  if (r >= (long long)D.na * D.nb) return;  // whole warp exits together
  const int ia = (int)(r % D.na), ib = (int)(r / D.na);
  const RayMarch R = ray_setup(G, D, G.y_det[ia], G.z_det[ib]);
  float ys = 0.f, ss = 0.f;
  ray_columns(R, lane, 32, [&](long long i) { return __ldg(x + i); }, ys, ss);
  ys = warp_sum(ys);
  ss = warp_sum(ss);
  if (lane == 0) {
    y[r] = ys * G.scale;
    sr[r] = ss * G.scale;
  }
}

__global__ void __launch_bounds__(kAtxThreads)
    k_atx(float *__restrict__ x, const float *__restrict__ yv,
          float *__restrict__ sc, ViewGeo G, Dims D) {
  int ix, iy, iz;
  tile_voxel(D, ix, iy, iz);
  if (ix >= D.nx || iy >= D.ny) return;
  const VoxelWin w = voxel_window(G, D, ix, iy, iz);
  float acc = 0.f, accl = 0.f;
  voxel_backproject(G, D, w, [&](long long i) { return __ldg(yv + i); }, acc,
                    accl);
  const long long idx = ((long long)iz * D.ny + iy) * D.nx + ix;
  x[idx] = acc * G.scale;
  sc[idx] = accl * G.scale;
}

// ------------------------------------------------------------- fused SART
__device__ __forceinline__ ViewGeo view_of(const Inst &I, int view) {
  ViewGeo g = I.g;
  const float2 t = I.trig[view];
  g.cos_phi = t.x;
  g.sin_phi = t.y;
  return g;
}

// ASD_POCS_cuda.m:117-123: [proj,sumR]=Ax(m); sumR(sumR==0)=1;
// cor0=P(:,ii)-proj; dd2+=||cor0||^2; cor=cor0./sumR.
__global__ void __launch_bounds__(kAxThreads)
    k_sart_ax(const Inst *__restrict__ insts, Dims D, int view) {
  const Inst &I = insts[blockIdx.y];
  if (((volatile int *)&I.s->done)[0]) return;
  const ViewGeo G = view_of(I, view);
  const int lane = threadIdx.x & 31;
  const long long nr = (long long)D.na * D.nb;
  const long long r = (long long)blockIdx.x * kAxWarps + (threadIdx.x >> 5);
  double part[1] = {0.0};
  if (r < nr) {
    const int ia = (int)(r % D.na), ib = (int)(r / D.na);
    const RayMarch R = ray_setup(G, D, G.y_det[ia], G.z_det[ib]);
    float ys = 0.f, ss = 0.f;
    const float *m = I.m;
    ray_columns(R, lane, 32, [&](long long i) { return m[i]; }, ys, ss);
    ys = warp_sum(ys);
    ss = warp_sum(ss);
    if (lane == 0) {
      const float yv = ys * G.scale, srv = ss * G.scale;
      const float c0 = I.P[(long long)view * nr + r] - yv;
      I.cor[r] = c0 / (srv == 0.f ? 1.f : srv);
      part[0] = (double)c0 * (double)c0;
    }
  }
  double tot[1];
  if (grid_sum<kAxThreads, 1>(part, I.partials, I.counter, gridDim.x, tot)) {
    if (threadIdx.x == 0) I.s->dd2_acc += tot[0];
  }
}

// ASD_POCS_cuda.m:125-131: [bProj,sumC]=Atx(cor); sumC(sumC==0)=1;
// m = m + beta*(bProj./sumC); m(m<0)=0.
__global__ void __launch_bounds__(kAtxThreads)
    k_sart_atx(const Inst *__restrict__ insts, Dims D, int view) {
  const Inst &I = insts[blockIdx.y];
  if (((volatile int *)&I.s->done)[0]) return;
  const ViewGeo G = view_of(I, view);
  int ix, iy, iz;
  tile_voxel(D, ix, iy, iz);
  if (ix >= D.nx || iy >= D.ny) return;
  const VoxelWin w = voxel_window(G, D, ix, iy, iz);
  float acc = 0.f, accl = 0.f;
  const float *cor = I.cor;
  voxel_backproject(G, D, w, [&](long long i) { return cor[i]; }, acc, accl);
  const float bp = acc * G.scale, scv = accl * G.scale;
  const float beta = (float)I.s->beta;
  const long long idx = ((long long)iz * D.ny + iy) * D.nx + ix;
  const float mn = I.m[idx] + beta * (bp / (scv == 0.f ? 1.f : scv));
  I.m[idx] = mn < 0.f ? 0.f : mn;
}

}  // namespace

cudaError_t launch_ax(const float *x, float *y, float *sr, const ViewGeo &g,
                      const Dims &d, cudaStream_t st) {
  const long long nr = (long long)d.na * d.nb;
  if (nr == 0) return cudaSuccess;
  const unsigned blocks = (unsigned)((nr + kAxWarps - 1) / kAxWarps);
  k_ax<<<blocks, kAxThreads, 0, st>>>(x, y, sr, g, d);
  return cudaGetLastError();
}

cudaError_t launch_atx(float *x, const float *y, float *sc, const ViewGeo &g,
                       const Dims &d, cudaStream_t st) {
  const int blocks = atx_blocks(d);
  if (blocks == 0) return cudaSuccess;
  k_atx<<<blocks, kAtxThreads, 0, st>>>(x, y, sc, g, d);
  return cudaGetLastError();
}

cudaError_t launch_sart_ax(const Inst *insts, int batch, const Dims &d,
                           int view, cudaStream_t st) {
  const long long nr = (long long)d.na * d.nb;
  const unsigned blocks = (unsigned)((nr + kAxWarps - 1) / kAxWarps);
  k_sart_ax<<<dim3(blocks, batch), kAxThreads, 0, st>>>(insts, d, view);
  return cudaGetLastError();
}

cudaError_t launch_sart_atx(const Inst *insts, int batch, const Dims &d,
                            int view, cudaStream_t st) {
  k_sart_atx<<<dim3(atx_blocks(d), batch), kAtxThreads, 0, st>>>(insts, d,
                                                                 view);
  return cudaGetLastError();
}

int reduce_blocks_for(const Dims &d) {
  const long long nr = (long long)d.na * d.nb;
  const long long ax = (nr + kAxWarps - 1) / kAxWarps;
  const long long at = atx_blocks(d);
  return (int)(ax > at ? ax : at);
}

}  // namespace asd
