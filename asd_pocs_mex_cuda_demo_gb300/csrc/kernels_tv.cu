// TV steepest-descent kernels (imgTVGradMin.cpp / imgTVGradMin3D.cpp) and
// the per-iteration ASD-POCS scalar steps (ASD_POCS_cuda.m:137-170), sm_103a.
//
// The TV global norm forces a grid-wide dependency in every step, so a step
// is two passes over the image: the first recomputes the stencil only for
// ||v||^2 (deterministic grid sum), the second recomputes it and writes
// m - (alpha*d/||v||)*v into the other buffer of a ping-pong pair.  Nothing
// but the image is stored: 12 bytes per voxel per step in FP32.
#include "kernels.h"
#include "reduce.cuh"

namespace asd {

namespace {

constexpr int kTileX = 32, kTileY = 8;
constexpr int kThreads = kTileX * kTileY;

__host__ __device__ inline int tiles(int nx, int ny, int nz) {
  return ((nx + kTileX - 1) / kTileX) * ((ny + kTileY - 1) / kTileY) * nz;
}

__device__ __forceinline__ bool tile_voxel(int nx, int ny, int &ix, int &iy,
                                           int &iz) {
  const int tx = (nx + kTileX - 1) / kTileX;
  const int ty = (ny + kTileY - 1) / kTileY;
  int b = blockIdx.x;
  const int bx = b % tx;
  b /= tx;
  const int by = b % ty;
  iz = b / ty;
  ix = bx * kTileX + (threadIdx.x % kTileX);
  iy = by * kTileY + (threadIdx.x / kTileX);
  return ix < nx && iy < ny;
}

// num / sqrt(den): exact operations in FP64 (the mex-level entry points);
// the hardware reciprocal square root in FP32 (the device-resident path,
// within a few ulp of the FP64 stencil's value).
__device__ __forceinline__ double tv_q(double num, double den) {
  return num / sqrt(den);
}
__device__ __forceinline__ float tv_q(float num, float den) {
  return num * rsqrtf(den);
}

template <class T>
__device__ __forceinline__ T tv_eps();
template <>
__device__ __forceinline__ double tv_eps<double>() {
  return 1e-8;
}
template <>
__device__ __forceinline__ float tv_eps<float>() {
  return 1e-8f;
}

// Zero-padded read of the image (the reference's (n+2)-wide bordered copy).
template <class T>
struct Img {
  const T *p;
  int nx, ny, nz;
  __device__ __forceinline__ T operator()(int x, int y, int z) const {
    if (x < 0 || y < 0 || z < 0 || x >= nx || y >= ny || z >= nz) return T(0);
    return p[((long long)z * ny + y) * nx + x];
  }
};

template <class T>
__device__ __forceinline__ T sqr(T v) {
  return v * v;
}

// imgTVGradMin.cpp:84-97 (x = row index r, fastest; y = column index c).
template <class T>
__device__ __forceinline__ T tv_grad2(const Img<T> &u, int x, int y) {
  const T eps = tv_eps<T>();
  const T c0 = u(x, y, 0);
  const T xm = u(x - 1, y, 0), ym = u(x, y - 1, 0);
  const T xp = u(x + 1, y, 0), yp = u(x, y + 1, 0);
  const T xpym = u(x + 1, y - 1, 0), xmyp = u(x - 1, y + 1, 0);
  const T g1 = tv_q((c0 - xm) + (c0 - ym), eps + sqr(c0 - xm) + sqr(c0 - ym));
  const T g2 = tv_q(-(xp - c0), eps + sqr(xp - c0) + sqr(xp - xpym));
  const T g3 = tv_q(-(yp - c0), eps + sqr(yp - c0) + sqr(yp - xmyp));
  return g1 + g2 + g3;
}

// imgTVGradMin3D.cpp:114-140 (image index x + y*Nx + z*Nx*Ny).
template <class T>
__device__ __forceinline__ T tv_grad3(const Img<T> &u, int x, int y, int z) {
  const T eps = tv_eps<T>();
  const T c0 = u(x, y, z);
  const T xm = u(x - 1, y, z), ym = u(x, y - 1, z), zm = u(x, y, z - 1);
  const T xp = u(x + 1, y, z), yp = u(x, y + 1, z), zp = u(x, y, z + 1);
  const T xm_zp = u(x - 1, y, z + 1), ym_zp = u(x, y - 1, z + 1);
  const T xm_yp = u(x - 1, y + 1, z), yp_zm = u(x, y + 1, z - 1);
  const T xp_ym = u(x + 1, y - 1, z), xp_zm = u(x + 1, y, z - 1);
  const T g1 = tv_q(T(6) * c0 - T(2) * (xm + ym + zm),
                    eps + sqr(c0 - xm) + sqr(c0 - ym) + sqr(c0 - zm));
  const T g2 = tv_q(T(2) * c0 - T(2) * zp,
                    eps + sqr(zp - xm_zp) + sqr(zp - ym_zp) + sqr(zp - c0));
  const T g3 = tv_q(T(2) * c0 - T(2) * yp,
                    eps + sqr(yp - xm_yp) + sqr(yp - c0) + sqr(yp - yp_zm));
  const T g4 = tv_q(T(2) * c0 - T(2) * xp,
                    eps + sqr(xp - c0) + sqr(xp - xp_ym) + sqr(xp - xp_zm));
  return g1 + g2 + g3 + g4;
}

template <class T>
__device__ __forceinline__ T tv_grad(const Img<T> &u, int x, int y, int z) {
  return u.nz >= 2 ? tv_grad3(u, x, y, z) : tv_grad2(u, x, y);
}

// --------------------------------------------------- standalone TV kernels
// scal[0] = d, scal[1] = ||v||^2 of the current step.
// Grid sum of one value per thread: FP32 within warps for the FP32 path,
// FP64 throughout for the FP64 entry points.
__device__ __forceinline__ bool sum_all(float v, double *partials,
                                        unsigned *counter, double &tot) {
  const float vv[1] = {v};
  double t[1];
  const bool last = grid_sum<kThreads, 1>(vv, partials, counter, gridDim.x, t);
  tot = t[0];
  return last;
}
__device__ __forceinline__ bool sum_all(double v, double *partials,
                                        unsigned *counter, double &tot) {
  return grid_sum_d<kThreads>(v, partials, counter, gridDim.x, tot);
}

template <class T>
__global__ void __launch_bounds__(kThreads)
    k_tv_dist(const T *__restrict__ img, const T *__restrict__ old, int nx,
              int ny, int nz, double *scal, double *partials,
              unsigned *counter) {
  int ix, iy, iz;
  T v = T(0);
  if (tile_voxel(nx, ny, ix, iy, iz)) {
    const long long i = ((long long)iz * ny + iy) * nx + ix;
    const T d = img[i] - (old ? old[i] : T(0));
    v = d * d;
  }
  double tot;
  if (sum_all(v, partials, counter, tot))
    if (threadIdx.x == 0) scal[0] = sqrt(tot);
}

template <class T>
__global__ void __launch_bounds__(kThreads)
    k_tv_norm(const T *__restrict__ src, int nx, int ny, int nz, double alpha,
              double *scal, double *partials, unsigned *counter) {
  int ix, iy, iz;
  T v = T(0);
  const Img<T> u{src, nx, ny, nz};
  if (tile_voxel(nx, ny, ix, iy, iz)) {
    const T g = tv_grad(u, ix, iy, iz);
    v = g * g;
  }
  double tot;
  if (sum_all(v, partials, counter, tot))
    if (threadIdx.x == 0) {
      scal[1] = sqrt(tot);
      scal[2] = alpha * scal[0] / scal[1];
      *(float *)(scal + 3) = (float)scal[2];  // for the FP32 update pass
    }
}

// img -= alpha*d*v/norm   (imgTVGradMin.cpp:104-107)
template <class T>
__global__ void __launch_bounds__(kThreads)
    k_tv_update(const T *__restrict__ src, T *__restrict__ dst, int nx, int ny,
                int nz, double alpha, const double *scal, int clamp) {
  int ix, iy, iz;
  if (!tile_voxel(nx, ny, ix, iy, iz)) return;
  const Img<T> u{src, nx, ny, nz};
  const T g = tv_grad(u, ix, iy, iz);
  const long long i = ((long long)iz * ny + iy) * nx + ix;
  T r;
  if (sizeof(T) == 8) {
    r = (T)((double)src[i] - alpha * scal[0] * (double)g / scal[1]);
  } else {
    const float coef = *(const float *)(scal + 3);
    r = src[i] - coef * g;
  }
  if (clamp && r < T(0)) r = T(0);
  dst[i] = r;
}

template <class T>
__global__ void k_copy_clamp(const T *__restrict__ src, T *__restrict__ dst,
                             long long n, int clamp) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    T v = src[i];
    if (clamp && v < T(0)) v = T(0);
    dst[i] = v;
  }
}

template <class T>
cudaError_t tv_minimize(T *img, const T *old, T *wa, T *wb, double *scal,
                        double *partials, unsigned *counter, int nx, int ny,
                        int nz, double alpha, int n_iter, int pos,
                        cudaStream_t st) {
  const int blocks = tiles(nx, ny, nz);
  if (blocks == 0) return cudaSuccess;
  if (blocks > kMaxPartials) return cudaErrorInvalidValue;
  k_tv_dist<T><<<blocks, kThreads, 0, st>>>(img, old, nx, ny, nz, scal,
                                            partials, counter);
  const T *src = img;
  T *bufs[2] = {wa, wb};
  for (int it = 0; it < n_iter; it++) {
    T *dst = (it == n_iter - 1) ? img : bufs[it & 1];
    if (dst == src) dst = bufs[(it + 1) & 1];
    k_tv_norm<T><<<blocks, kThreads, 0, st>>>(src, nx, ny, nz, alpha, scal,
                                              partials, counter);
    const int clamp_now = (it == n_iter - 1) && pos == 1;
    k_tv_update<T><<<blocks, kThreads, 0, st>>>(src, dst, nx, ny, nz, alpha,
                                                scal, clamp_now);
    src = dst;
  }
  if (n_iter > 0 && src != img) {
    const long long n = (long long)nx * ny * nz;
    k_copy_clamp<T><<<(unsigned)((n + 255) / 256), 256, 0, st>>>(src, img, n, 0);
  }
  return cudaGetLastError();
}

// ------------------------------------------- batched ASD-POCS scalar steps
__device__ __forceinline__ bool inst_done(const Inst &I) {
  return ((volatile int *)&I.s->done)[0] != 0;
}

// After the SART sweep (ASD_POCS_cuda.m:137-149): dd, m_res, RMSE, dp and the
// stop test; also d = ||m - m_k1|| for the TV step (imgTVGradMin.cpp:57-60).
__global__ void __launch_bounds__(kThreads)
    k_after_sweep(const Inst *__restrict__ insts, Dims D) {
  const Inst &I = insts[blockIdx.y];
  if (inst_done(I)) return;
  int ix, iy, iz;
  float v[3] = {0.f, 0.f, 0.f};
  if (tile_voxel(D.nx, D.ny, ix, iy, iz)) {
    const long long i = ((long long)iz * D.ny + iy) * D.nx + ix;
    const float m = I.m[i];
    I.m_res[i] = m;
    const float a = m - I.m_pre[i];
    const float b = m - I.m_k1[i];
    v[0] = a * a;
    v[1] = b * b;
    if (I.I0) {
      const float c = m - I.I0[i];
      v[2] = c * c;
    }
  }
  double tot[3];
  if (grid_sum<kThreads, 3>(v, I.partials, I.counter, gridDim.x, tot)) {
    if (threadIdx.x == 0) {
      Scalars *s = I.s;
      const double N = (double)D.nx * D.ny * D.nz;
      s->dd2 = s->dd2_acc;
      s->dd2_acc = 0.0;
      s->dp = sqrt(tot[0]);
      if (s->has_ref) I.rmse[s->k - 1] = sqrt(tot[2] / N);
      s->iterations = s->k;
      if (s->dp / N <= s->stopRelChg) {
        s->done = 1;
      } else {
        s->d_tv = sqrt(tot[1]);
      }
    }
  }
}

__device__ __forceinline__ const float *tv_src(const Inst &I, int step) {
  return step == 0 ? I.m : ((step & 1) ? I.tv_b : I.tv_c);
}
__device__ __forceinline__ float *tv_dst(const Inst &I, int step) {
  return (step & 1) ? I.tv_c : I.tv_b;
}

// ||v||^2 of TV step `step`; last block sets tv_coef = alpha*d/||v||.
__global__ void __launch_bounds__(kThreads)
    k_tv_norm_batch(const Inst *__restrict__ insts, Dims D, int step) {
  const Inst &I = insts[blockIdx.y];
  if (inst_done(I) || step >= I.s->ng) return;
  int ix, iy, iz;
  float v[1] = {0.f};
  const Img<float> u{tv_src(I, step), D.nx, D.ny, D.nz};
  if (tile_voxel(D.nx, D.ny, ix, iy, iz)) {
    const float g = tv_grad(u, ix, iy, iz);
    v[0] = g * g;
  }
  double tot[1];
  if (grid_sum<kThreads, 1>(v, I.partials, I.counter, gridDim.x, tot))
    if (threadIdx.x == 0) {
      I.s->tv_coef = I.s->alpha * I.s->d_tv / sqrt(tot[0]);
      I.s->tv_coef_f = (float)I.s->tv_coef;
    }
}

__global__ void __launch_bounds__(kThreads)
    k_tv_update_batch(const Inst *__restrict__ insts, Dims D, int step) {
  const Inst &I = insts[blockIdx.y];
  if (inst_done(I) || step >= I.s->ng) return;
  int ix, iy, iz;
  if (!tile_voxel(D.nx, D.ny, ix, iy, iz)) return;
  const float *src = tv_src(I, step);
  const Img<float> u{src, D.nx, D.ny, D.nz};
  const float g = tv_grad(u, ix, iy, iz);
  const long long i = ((long long)iz * D.ny + iy) * D.nx + ix;
  const float coef = I.s->tv_coef_f;
  tv_dst(I, step)[i] = src[i] - coef * g;
}

// End of an iteration (ASD_POCS_cuda.m:155-170 after TV): positivity
// (imgTVGradMin.cpp:110-116), dg, alpha/beta updates, next k.
__global__ void __launch_bounds__(kThreads)
    k_finish_iter(const Inst *__restrict__ insts, Dims D) {
  const Inst &I = insts[blockIdx.y];
  if (inst_done(I)) return;
  const int ng = I.s->ng;
  int ix, iy, iz;
  float v[1] = {0.f};
  if (tile_voxel(D.nx, D.ny, ix, iy, iz)) {
    const long long i = ((long long)iz * D.ny + iy) * D.nx + ix;
    const float f0 = I.m[i];
    float mn = f0;
    if (ng > 0) {
      mn = tv_dst(I, ng - 1)[i];
      if (mn < 0.f) mn = 0.f;
    }
    const float dlt = mn - f0;
    v[0] = dlt * dlt;
    I.m[i] = mn;
    I.m_pre[i] = mn;
  }
  double tot[1];
  if (grid_sum<kThreads, 1>(v, I.partials, I.counter, gridDim.x, tot)) {
    if (threadIdx.x == 0) {
      Scalars *s = I.s;
      s->dg = sqrt(tot[0]);
      if (s->dg > s->r_max * s->dp && sqrt(s->dd2) > s->epsilon)
        s->alpha = s->alpha * s->alpha_red;
      s->beta = s->beta * s->beta_red;
      s->beta_f = (float)s->beta;
      if (s->k >= s->maxIter) {
        s->done = 1;
      } else {
        s->k = s->k + 1;
      }
    }
  }
}

}  // namespace

cudaError_t tv_minimize_f64(double *img, const double *img_old, double *wa,
                            double *wb, double *scal, double *partials,
                            unsigned *counter, int nx, int ny, int nz,
                            double alpha, int n_iter, int pos,
                            cudaStream_t st) {
  return tv_minimize<double>(img, img_old, wa, wb, scal, partials, counter, nx,
                             ny, nz, alpha, n_iter, pos, st);
}
cudaError_t tv_minimize_f32(float *img, const float *img_old, float *wa,
                            float *wb, double *scal, double *partials,
                            unsigned *counter, int nx, int ny, int nz,
                            double alpha, int n_iter, int pos,
                            cudaStream_t st) {
  return tv_minimize<float>(img, img_old, wa, wb, scal, partials, counter, nx,
                            ny, nz, alpha, n_iter, pos, st);
}

cudaError_t launch_iter_begin(const Inst *, int, cudaStream_t) {
  return cudaSuccess;
}

cudaError_t launch_after_sweep(const Inst *insts, int batch, const Dims &d,
                               cudaStream_t st) {
  k_after_sweep<<<dim3(tiles(d.nx, d.ny, d.nz), batch), kThreads, 0, st>>>(
      insts, d);
  return cudaGetLastError();
}

cudaError_t launch_tv_step(const Inst *insts, int batch, const Dims &d,
                           int step, int ng, cudaStream_t st) {
  (void)ng;
  const dim3 grid(tiles(d.nx, d.ny, d.nz), batch);
  k_tv_norm_batch<<<grid, kThreads, 0, st>>>(insts, d, step);
  k_tv_update_batch<<<grid, kThreads, 0, st>>>(insts, d, step);
  return cudaGetLastError();
}

cudaError_t launch_finish_iter(const Inst *insts, int batch, const Dims &d,
                               int ng, cudaStream_t st) {
  (void)ng;
  k_finish_iter<<<dim3(tiles(d.nx, d.ny, d.nz), batch), kThreads, 0, st>>>(
      insts, d);
  return cudaGetLastError();
}

}  // namespace asd
