// TV steepest-descent kernels (imgTVGradMin.cpp / imgTVGradMin3D.cpp) and
// the per-iteration ASD-POCS scalar steps (ASD_POCS_cuda.m:137-170), sm_103a.
//
// Device-resident path (FP32 image, FP64 scalars): one kernel per TV step.
// A step computes the updated image m' = m - (alpha*d/||v||) v(m) (zero
// outside the image, as the reference's padded copy), writes it, and
// evaluates the stencil of m' for the next step's ||v'||^2 (deterministic
// grid sum) -- so it reads the image once and writes it once (8 bytes per
// voxel), and the ||v|| that every step needs before it can update comes out
// of the previous kernel.  2-D: warps walk down strips of columns with the
// stencils in registers (k_tv_walk2d).  Cone beam: blocks walk down z over
// (x, y) tiles, a thread holding the stencils of eight rows of a column in
// registers and the slices staged in shared memory (k_tv_walk3d).  The
// end-of-sweep kernel provides ||v|| of the first step; the last step also
// applies the positivity constraint and the alpha/beta step control.
#include <type_traits>
#include "kernels.h"
#include "reduce.cuh"

namespace asd {

namespace {

constexpr int kThreads = kTileThreads;

// num / sqrt(den): exact operations in FP64 (the mex-level entry points);
// the hardware reciprocal square root in FP32 (the device-resident path,
// within a few ulp of the FP64 stencil's value).
__device__ __forceinline__ double tv_q(double num, double den) {
  return num / sqrt(den);
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

template <class T>
__device__ __forceinline__ T sqr(T v) {
  return v * v;
}

// imgTVGradMin.cpp:84-97; u(dx, dy, dz) reads the image at an offset from
// the voxel (zero outside the image).  x = row index r (fastest).
template <class T, class U>
__device__ __forceinline__ T tv_grad2(const U &u) {
  const T eps = tv_eps<T>();
  const T c0 = u(0, 0, 0);
  const T xm = u(-1, 0, 0), ym = u(0, -1, 0);
  const T xp = u(1, 0, 0), yp = u(0, 1, 0);
  const T xpym = u(1, -1, 0), xmyp = u(-1, 1, 0);
  const T g1 = tv_q((c0 - xm) + (c0 - ym), eps + sqr(c0 - xm) + sqr(c0 - ym));
  const T g2 = tv_q(-(xp - c0), eps + sqr(xp - c0) + sqr(xp - xpym));
  const T g3 = tv_q(-(yp - c0), eps + sqr(yp - c0) + sqr(yp - xmyp));
  return g1 + g2 + g3;
}

// FP32 form of the 2-D stencil with every rounding explicit, so that a
// kernel holding its terms in registers reproduces it bit for bit.  With
// dx = f(x,y) - f(x-1,y), dy = f(x,y) - f(x,y-1) at a voxel, its terms are
//   r = 1/sqrt(eps + dx^2 + dy^2),  g1 = (dx + dy) * r,  q = dx * r,
//   t = dy * r
// and v(x,y) = (g1(x,y) - q(x+1,y)) - t(x,y+1): the reference's second and
// third terms (FP64 there) are the right neighbour's q and the lower
// neighbour's t -- the same differences under the same square root, whose
// two squares the reference sums in the other order for the third.  1/sqrt
// is the approximate reciprocal square root; den >= eps is never
// subnormal, so flushing subnormals changes nothing.
__device__ __forceinline__ float tv_rsqrt(float x) {
  float r;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}
struct Tv2Terms {
  float g1, q, t;
};
__device__ __forceinline__ Tv2Terms tv2_terms(float dx, float dy) {
  const float eps = tv_eps<float>();
  const float r = tv_rsqrt(__fmaf_rn(dy, dy, __fmaf_rn(dx, dx, eps)));
  return Tv2Terms{__fmul_rn(__fadd_rn(dx, dy), r), __fmul_rn(dx, r), __fmul_rn(dy, r)};
}
__device__ __forceinline__ float tv2_combine(float g1, float q_right, float t_below) {
  return __fsub_rn(__fsub_rn(g1, q_right), t_below);
}
template <class U>
__device__ __forceinline__ float tv_grad2f(const U &u) {
  const float c0 = u(0, 0, 0);
  const float xm = u(-1, 0, 0), ym = u(0, -1, 0);
  const float xp = u(1, 0, 0), yp = u(0, 1, 0);
  const float xpym = u(1, -1, 0), xmyp = u(-1, 1, 0);
  const Tv2Terms here = tv2_terms(__fsub_rn(c0, xm), __fsub_rn(c0, ym));
  const Tv2Terms right = tv2_terms(__fsub_rn(xp, c0), __fsub_rn(xp, xpym));
  const Tv2Terms below = tv2_terms(__fsub_rn(yp, xmyp), __fsub_rn(yp, c0));
  return tv2_combine(here.g1, right.q, below.t);
}

// imgTVGradMin3D.cpp:114-140 (image index x + y*Nx + z*Nx*Ny).
template <class T, class U>
__device__ __forceinline__ T tv_grad3(const U &u) {
  const T eps = tv_eps<T>();
  const T c0 = u(0, 0, 0);
  const T xm = u(-1, 0, 0), ym = u(0, -1, 0), zm = u(0, 0, -1);
  const T xp = u(1, 0, 0), yp = u(0, 1, 0), zp = u(0, 0, 1);
  const T xm_zp = u(-1, 0, 1), ym_zp = u(0, -1, 1);
  const T xm_yp = u(-1, 1, 0), yp_zm = u(0, 1, -1);
  const T xp_ym = u(1, -1, 0), xp_zm = u(1, 0, -1);
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

// FP32 form of the 3-D stencil with every rounding explicit.  At a voxel
// with differences dx, dy, dz to its -x, -y, -z neighbours,
//   r = 1/sqrt(eps + dx^2 + dy^2 + dz^2),
// and the denominators of the reference's second to fourth terms are those
// of the +z, +y and +x neighbours' first terms (r+z, r+y, r+x).  All four
// terms carry a factor 2, so v = 2 u with
//   u = (3c - ((xm + ym) + zm)) r + (c - yp) r+y + (c - xp) r+x + (c - zp) r+z
// evaluated left to right, each later term by one fused multiply-add
// (tv3_u).  Scaling by 2 is exact, so the TV step's m - coef v is
// m - (2 coef) u and ||v||^2 = 4 sum u^2; the z walk (k_tv_walk3d), the end
// of the sweep and the FP32 device entry point all use this one form.
__device__ __forceinline__ float tv3_r(float dx, float dy, float dz) {
  return tv_rsqrt(__fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmaf_rn(dx, dx, tv_eps<float>()))));
}
// u's in-slice terms: (3c - ((xm + ym) + zm)) r + (c - yp) r+y + (c - xp) r+x
__device__ __forceinline__ float tv3_inslice(float c, float xm, float ym, float zm, float xp,
                                             float yp, float r, float rx, float ry) {
  const float sum = __fadd_rn(__fadd_rn(xm, ym), zm);
  float t = __fmul_rn(__fmaf_rn(3.f, c, -sum), r);
  t = __fmaf_rn(__fsub_rn(c, yp), ry, t);
  return __fmaf_rn(__fsub_rn(c, xp), rx, t);
}
// u from the in-slice terms s and the +z neighbour
__device__ __forceinline__ float tv3_u(float s, float c, float zp, float rz) {
  return __fmaf_rn(__fsub_rn(c, zp), rz, s);
}
template <class U>
__device__ __forceinline__ float tv_grad3f(const U &u) {
  const float c = u(0, 0, 0);
  const float xm = u(-1, 0, 0), ym = u(0, -1, 0), zm = u(0, 0, -1);
  const float xp = u(1, 0, 0), yp = u(0, 1, 0), zp = u(0, 0, 1);
  const float r = tv3_r(__fsub_rn(c, xm), __fsub_rn(c, ym), __fsub_rn(c, zm));
  const float rx = tv3_r(__fsub_rn(xp, c), __fsub_rn(xp, u(1, -1, 0)), __fsub_rn(xp, u(1, 0, -1)));
  const float ry = tv3_r(__fsub_rn(yp, u(-1, 1, 0)), __fsub_rn(yp, c), __fsub_rn(yp, u(0, 1, -1)));
  const float rz = tv3_r(__fsub_rn(zp, u(-1, 0, 1)), __fsub_rn(zp, u(0, -1, 1)), __fsub_rn(zp, c));
  return __fmul_rn(2.f, tv3_u(tv3_inslice(c, xm, ym, zm, xp, yp, r, rx, ry), c, zp, rz));
}

template <class T, class U>
__device__ __forceinline__ T tv_grad(const U &u, bool is3d) {
  if (is3d) {
    if constexpr (std::is_same<T, float>::value)
      return tv_grad3f(u);
    else
      return tv_grad3<T>(u);
  }
  if constexpr (std::is_same<T, float>::value)
    return tv_grad2f(u);
  else
    return tv_grad2<T>(u);
}

// Global-memory accessor with zero padding (standalone entry points).
template <class T>
struct GlobalAt {
  const T *p;
  int nx, ny, nz, x, y, z;
  __device__ __forceinline__ T operator()(int dx, int dy, int dz) const {
    const int xx = x + dx, yy = y + dy, zz = z + dz;
    if (xx < 0 || yy < 0 || zz < 0 || xx >= nx || yy >= ny || zz >= nz) return T(0);
    return p[((long long)zz * ny + yy) * nx + xx];
  }
};

// --------------------------------------------------- standalone TV kernels
// scal[0] = d, scal[1] = ||v||, scal[2] = alpha*d/||v|| (+ FP32 copy at 3).
__device__ __forceinline__ bool sum_all(float v, double *partials,
                                        unsigned *counter, double &tot) {
  const float vv[1] = {v};
  double t[1];
  const bool last = grid_sum<kThreads, 1>(vv, partials, counter, inst_block(),
                                          inst_blocks(), t);
  tot = t[0];
  return last;
}
__device__ __forceinline__ bool sum_all(double v, double *partials,
                                        unsigned *counter, double &tot) {
  return grid_sum_d<kThreads>(v, partials, counter, inst_blocks(), tot);
}

template <class T>
__global__ void __launch_bounds__(kThreads)
    k_tv_dist(const T *__restrict__ img, const T *__restrict__ old, int nx,
              int ny, int nz, double *scal, double *partials,
              unsigned *counter) {
  int ix, iy, iz;
  T v = T(0);
  if (tile_voxel(nx, ny, nz, ix, iy, iz)) {
    const long long i = ((long long)iz * ny + iy) * nx + ix;
    const T d = ASD_IN(i, (long long)nx * ny * nz) ? img[i] - (old ? old[i] : T(0)) : T(0);
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
  if (tile_voxel(nx, ny, nz, ix, iy, iz)) {
    const T g = tv_grad<T>(GlobalAt<T>{src, nx, ny, nz, ix, iy, iz}, nz >= 2);
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
  if (!tile_voxel(nx, ny, nz, ix, iy, iz)) return;
  const T g = tv_grad<T>(GlobalAt<T>{src, nx, ny, nz, ix, iy, iz}, nz >= 2);
  const long long i = ((long long)iz * ny + iy) * nx + ix;
  if (!ASD_IN(i, (long long)nx * ny * nz)) return;
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
  const dim3 grid = tile_grid(nx, ny, nz, 1);
  if ((long long)grid.x * grid.y > kMaxPartials || tile_rows(ny, nz) > kMaxGridRows)
    return cudaErrorInvalidValue;
  k_tv_dist<T><<<grid, kThreads, 0, st>>>(img, old, nx, ny, nz, scal, partials,
                                          counter);
  const T *src = img;
  T *bufs[2] = {wa, wb};
  for (int it = 0; it < n_iter; it++) {
    T *dst = (it == n_iter - 1) ? img : bufs[it & 1];
    if (dst == src) dst = bufs[(it + 1) & 1];
    k_tv_norm<T><<<grid, kThreads, 0, st>>>(src, nx, ny, nz, alpha, scal,
                                            partials, counter);
    const int clamp_now = (it == n_iter - 1) && pos == 1;
    k_tv_update<T><<<grid, kThreads, 0, st>>>(src, dst, nx, ny, nz, alpha,
                                              scal, clamp_now);
    src = dst;
  }
  if (n_iter > 0 && src != img) {
    const long long n = (long long)nx * ny * nz;
    k_copy_clamp<T><<<(unsigned)((n + 255) / 256), 256, 0, st>>>(src, img, n, 0);
  }
  return cudaGetLastError();
}

// ------------------------------------------- batched ASD-POCS: tiled steps
// Shared tile of an image with a halo of H voxels (zero outside the image).
template <int H, bool k3D>
struct Tile {
  static constexpr int W = kTileX + 2 * H, Hh = kTileY + 2 * H;
  static constexpr int D = k3D ? 1 + 2 * H : 1;
  float v[D][Hh][W];
};

template <int H, bool k3D>
struct TileAt {  // accessor centred on tile position (tx, ty, tz)
  const Tile<H, k3D> &t;
  int tx, ty, tz;
  __device__ __forceinline__ float operator()(int dx, int dy, int dz) const {
    return t.v[tz + dz][ty + dy][tx + dx];
  }
};

// Loads the tile (origin x0, y0 of the block, slice z) with its halo.
template <int H, bool k3D>
__device__ __forceinline__ void load_tile(Tile<H, k3D> &t, const float *src,
                                          const Dims &D, int x0, int y0,
                                          int z) {
  constexpr int W = Tile<H, k3D>::W, Hh = Tile<H, k3D>::Hh, Dd = Tile<H, k3D>::D;
  for (int k = threadIdx.x; k < W * Hh * Dd; k += kThreads) {
    const int tx = k % W, ty = (k / W) % Hh, tz = k / (W * Hh);
    const int x = x0 - H + tx, y = y0 - H + ty, zz = k3D ? z - H + tz : z;
    float v = 0.f;
    const long long si = ((long long)zz * D.ny + y) * D.nx + x;
    if (x >= 0 && y >= 0 && zz >= 0 && x < D.nx && y < D.ny && zz < D.nz &&
        ASD_IN(si, (long long)D.nx * D.ny * D.nz))
      v = src[si];
    t.v[tz][ty][tx] = v;
  }
}

__device__ __forceinline__ bool inst_done(const Inst &I) {
  return ((volatile int *)&I.s->done)[0] != 0;
}

__device__ __forceinline__ const float *tv_src(const Inst &I, int step) {
  return step == 0 ? I.m : ((step & 1) ? I.tv_b : I.tv_c);
}
__device__ __forceinline__ float *tv_dst(const Inst &I, int step) {
  return (step & 1) ? I.tv_c : I.tv_b;
}

// End-of-iteration scalars (ASD_POCS_cuda.m:166-170) by the last block.
__device__ __forceinline__ void finish_scalars(Scalars *s, double dg2) {
  s->dg = sqrt(dg2);
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

// The sweep's scalars from the totals of (m - m_pre)^2, (m - m_k1)^2,
// (m - I0)^2 and v(m)^2 (ASD_POCS_cuda.m:137-149, imgTVGradMin.cpp:57-60).
__device__ __forceinline__ void sweep_scalars(const Inst &I, const double (&tot)[4]) {
  Scalars *s = I.s;
  const double N = (double)I.d.nx * I.d.ny * I.d.nz;
  s->dd2 = s->dd2_acc;
  s->dd2_acc = 0.0;
  s->dp = sqrt(tot[0]);
  if (s->has_ref) I.rmse[s->k - 1] = sqrt(tot[2] / N);
  s->iterations = s->k;
  if (s->dp / N <= s->stopRelChg) {
    s->done = 1;
  } else {
    s->d_tv = sqrt(tot[1]);
    s->tv_coef = s->alpha * s->d_tv / sqrt(tot[3]);
    s->tv_coef_f = (float)s->tv_coef;
  }
}

// After the SART sweep (ASD_POCS_cuda.m:137-149): dd, m_res, RMSE, dp and the
// stop test; d = ||m - m_k1|| (imgTVGradMin.cpp:57-60) and ||v|| of the first
// TV step, giving its step size alpha*d/||v||.
template <bool k3D>
__global__ void __launch_bounds__(kThreads)
    k_after_sweep(const Inst *__restrict__ insts, const int *__restrict__ zmap) {
  __shared__ Tile<1, k3D> t;
  pdl_enter();
  const Inst &I = insts[zmap ? zmap[blockIdx.z] : blockIdx.z];
  if (inst_done(I)) return;
  const Dims D = I.d;
  const OwnBlock ob = own_block(group_grid(D.nx, D.ny, D.nz, 1));
  if (ob.bid < 0) return;
  const bool tv = I.s->ng > 0;
  const int tx = threadIdx.x % kTileX, ty = threadIdx.x / kTileX;
  float v[4] = {0.f, 0.f, 0.f, 0.f};
  for (int g = 0; g < kTilesPerBlock; g++) {
    int x0, y0, z;
    if (!group_tile(D.ny, D.nz, g, x0, y0, z)) break;
    if (tv) {
      load_tile(t, I.m, D, x0, y0, z);
      __syncthreads();
    }
    const int ix = x0 + tx, iy = y0 + ty;
    const unsigned i = ((unsigned)z * D.ny + iy) * D.nx + ix;
    if (ix < D.nx && iy < D.ny && ASD_IN(i, (long long)D.nx * D.ny * D.nz)) {
      const float m = I.m[i];
      I.m_res[i] = m;
      const float a = m - I.m_pre[i];
      const float b = m - I.m_k1[i];
      v[0] += a * a;
      v[1] += b * b;
      if (I.I0) {
        const float c = m - I.I0[i];
        v[2] += c * c;
      }
      if (tv) {
        const float gr =
            tv_grad<float>(TileAt<1, k3D>{t, tx + 1, ty + 1, k3D ? 1 : 0}, k3D);
        v[3] += gr * gr;
      }
    }
    __syncthreads();  // the tile is reused by the next group member
  }
  double tot[4];
  if (grid_sum<kThreads, 4>(v, I.partials, I.counter, ob.bid, ob.nblocks, tot)) {
    if (threadIdx.x == 0) sweep_scalars(I, tot);
  }
}

// 2-D TV step (imgTVGradMin.cpp:62-116: m' = m - alpha*d*v(m)/||v(m)||,
// positivity after the last step) as column walks.  A warp owns a strip of
// 64 image columns (lane l: columns xs - 2 + 2l and the next) and walks
// down it a row at a time, holding everything in registers: each new row
// of m gives, with one shuffle from each neighbour lane, the stencil terms
// of that row
// (tv2_terms), which complete v(m) one row up; m' = m - coef * v(m) follows
// (zero outside the image), and the same walk over the rows of m' completes
// v(m') two rows up.  The lanes at the strip's edges only feed their
// neighbours, so a strip writes its 60 middle columns (strips overlap by
// four columns) and a walk over output rows [y0, y1) reads rows
// y0 - 2 .. y1 + 1.  A step reads m once and writes m' once (8 bytes per
// voxel) and evaluates two stencils per voxel, both in registers.
//
// ||v(m')||^2 (or, in the last step, the positivity-change norm) is summed
// per band of 16 output rows of a strip -- lanes in row order, then an xor
// butterfly -- and the walk that finishes last sums the band partials of
// the instance in order; walks of `bands` consecutive bands (chosen by the
// host from the batch size) therefore give the same bits for every choice.
constexpr int kWalkWarps = 4;
constexpr int kWalkOut = 60;   // output columns of a strip
constexpr int kBandRows = 16;  // output rows of a partial
constexpr int kWalkChunk = 4;  // rows per chunk (a band ends at a chunk's end)
constexpr int kWalkRing = 8;  // rows of m in flight per warp (shared-memory ring)
static_assert(4 % kWalkChunk == 0 && kBandRows % 4 == 0, "bands and the steady chunks line up");
static_assert(kWalkRing % kWalkChunk == 0 && (kWalkRing & (kWalkRing - 1)) == 0,
              "a chunk's rows sit in consecutive ring slots");

__host__ __device__ __forceinline__ int walk_strips(int nx) {
  return (nx + kWalkOut - 1) / kWalkOut;
}
__host__ __device__ __forceinline__ int walk_bands(int ny) {
  return (ny + kBandRows - 1) / kBandRows;
}

// The running stencil of one field along a walk: the previous row's values
// and its partly combined v, (g1 - q_right), waiting for the row below.
struct WalkField {
  float pa, pb;  // previous row, columns a and b
  float ca, cb;  // g1 - q_right of the previous row
  // Takes row j (fa, fb); returns v of row j - 1 in va, vb.
  __device__ __forceinline__ void push(float fa, float fb, float &va, float &vb) {
    const float fl = __shfl_up_sync(0xffffffffu, fb, 1);  // column a - 1
    const Tv2Terms ta = tv2_terms(__fsub_rn(fa, fl), __fsub_rn(fa, pa));
    const Tv2Terms tb = tv2_terms(__fsub_rn(fb, fa), __fsub_rn(fb, pb));
    const float qr = __shfl_down_sync(0xffffffffu, ta.q, 1);  // q of column b + 1
    va = __fsub_rn(ca, ta.t);
    vb = __fsub_rn(cb, tb.t);
    ca = __fsub_rn(ta.g1, tb.q);
    cb = __fsub_rn(tb.g1, qr);
    pa = fa;
    pb = fb;
  }
};

// kMode 0: m' and ||v(m')||^2; 1: m' only (the single, last step);
// 2: the last of several steps -- positivity, the change norm, and m' into
// the image and m_pre.  kPair: nx is even, so a lane's two columns are both
// inside or both outside the image and 8-byte aligned (one access each).
// 4- and 8-byte asynchronous copies into shared memory, zero-filled when
// `valid` is false (nothing is read then; `gmem` must still be mapped)
__device__ __forceinline__ void cp_async_4(float *smem, const float *gmem, bool valid) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(
                   (unsigned)__cvta_generic_to_shared(smem)),
               "l"(gmem), "r"(valid ? 4 : 0)
               : "memory");
}
__device__ __forceinline__ void cp_async_8(float *smem, const float *gmem, bool valid) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(
                   (unsigned)__cvta_generic_to_shared(smem)),
               "l"(gmem), "r"(valid ? 8 : 0)
               : "memory");
}

template <int kMode, bool kPair>
__device__ __forceinline__ void tv_walk(const Inst &I, int step, int y0, int y1, int xa,
                                        int strip, int S, float coef, float2 *ring,
                                        float2 *ring0) {
  const Dims D = I.d;
  const int lane = threadIdx.x & 31;
  const float *src = tv_src(I, step);
  float *dst = tv_dst(I, step);
  float *const im = I.m, *const impre = I.m_pre;
  const bool ina = xa >= 0 && xa < D.nx, inb = xa + 1 >= 0 && xa + 1 < D.nx;
  const bool outl = lane >= 1 && lane <= 30;
  const bool outa = outl && ina, outb = outl && inb;
  const int jl0 = y0 - 2, jl1 = min(D.ny, y1 + 2);  // rows of m read
  const int j1 = y1 + 2;                            // rows walked: jl0 .. j1 - 1
  const float coef_a = ina ? coef : 0.f, coef_b = inb ? coef : 0.f;
  const long long N2 = (long long)D.nx * D.ny;  // bounds-checked builds
  // Rows of m stream through a ring of kWalkRing rows per warp (each lane
  // its two columns), copied asynchronously kWalkRing - 1 rows ahead of the
  // one in use and zero-filled outside the image and the walk; one copy
  // group per row, so "row j has landed" is a fixed wait depth.
  // The finishing step (kMode 2) also streams the rows of the pre-TV image
  // (the positivity-change norm's reference) through a second ring.
  float2 *const my = ring + lane;  // slot s of this lane: my[32 * s]
  float2 *const my0 = ring0 + lane;
  const float *la = src + (ina ? xa : 0), *lb = src + (inb ? xa + 1 : 0);
  const float *l0a = im + (ina ? xa : 0), *l0b = im + (inb ? xa + 1 : 0);
  auto fetch = [&](int j, int slot) {
    const bool r = (unsigned)j < (unsigned)jl1;  // 0 <= j < jl1
    const int off = r ? j * D.nx : 0;
    float *d = (float *)(my + 32 * slot);
    float *d0 = (float *)(my0 + 32 * slot);
    const bool va = r && ina && ASD_IN((long long)off + xa, N2) &&
                    (!kPair || ASD_IN((long long)off + xa + 1, N2));
    const bool vb = r && inb && ASD_IN((long long)off + xa + 1, N2);
    if (kPair) {
      cp_async_8(d, la + off, va);
      if (kMode == 2) cp_async_8(d0, l0a + off, va);
    } else {
      cp_async_4(d, la + off, va);
      cp_async_4(d + 1, lb + off, vb);
      if (kMode == 2) {
        cp_async_4(d0, l0a + off, va);
        cp_async_4(d0 + 1, l0b + off, vb);
      }
    }
    asm volatile("cp.async.commit_group;\n" ::: "memory");
  };
  for (int k = 0; k < kWalkRing - 1; k++) fetch(jl0 + k, k);
  WalkField f1{0.f, 0.f, 0.f, 0.f}, f2{0.f, 0.f, 0.f, 0.f};
  float acc = 0.f;
  // one partial from the band whose last output row is o
  auto flush = [&](int o) {
#pragma unroll
    for (int w = 16; w > 0; w >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, w);
    if (lane == 0) I.partials[(o / kBandRows) * S + strip] = (double)acc;
    acc = 0.f;
  };
  // row j of m in: v(m) and m' of row j - 1, v(m') of row j - 2
  // rslot: ring slot of row j; its predecessor's slot receives row
  // j + kWalkRing - 1
  auto walk_row = [&](auto checked, int j, int rslot) {
    constexpr bool kC = decltype(checked)::value;
    // the pre-TV image at output row j - 1 (landed a row ago), read before
    // its slot receives row j + kWalkRing - 1
    const float2 f0 = kMode == 2 ? my0[32 * ((rslot + kWalkRing - 1) & (kWalkRing - 1))]
                                 : make_float2(0.f, 0.f);
    fetch(j + kWalkRing - 1, (rslot + kWalkRing - 1) & (kWalkRing - 1));
    asm volatile("cp.async.wait_group %0;\n" ::"n"(kWalkRing - 1) : "memory");
    const float2 mab = my[32 * rslot];
    const float m1a = f1.pa, m1b = f1.pb;
    float va, vb;
    f1.push(mab.x, mab.y, va, vb);
    const int o1 = j - 1;
    float pa, pb;
    if (kC) {
      const bool row1 = o1 >= 0 && o1 < D.ny;
      pa = (row1 && ina) ? __fmaf_rn(-coef, va, m1a) : 0.f;
      pb = (row1 && inb) ? __fmaf_rn(-coef, vb, m1b) : 0.f;
    } else {
      pa = __fmaf_rn(-coef_a, va, m1a);
      pb = __fmaf_rn(-coef_b, vb, m1b);
    }
    const bool out1 = !kC || (o1 >= y0 && o1 < y1);  // warp-uniform
    if (kMode == 2) {
      if (out1) {
        const int i = o1 * D.nx + xa;
        const float mca = pa < 0.f ? 0.f : pa;  // imgTVGradMin.cpp:110-116
        const float mcb = pb < 0.f ? 0.f : pb;
        if (kPair) {
          if (outa && ASD_IN(i + 1, N2) && ASD_IN(i, N2)) {
            const float da = mca - f0.x, db = mcb - f0.y;
            acc += da * da;
            acc += db * db;
            *(float2 *)(im + i) = make_float2(mca, mcb);
            *(float2 *)(impre + i) = make_float2(mca, mcb);
          }
        } else {
          if (outa && ASD_IN(i, N2)) {
            const float d = mca - f0.x;
            acc += d * d;
            im[i] = mca;
            impre[i] = mca;
          }
          if (outb && ASD_IN(i + 1, N2)) {
            const float d = mcb - f0.y;
            acc += d * d;
            im[i + 1] = mcb;
            impre[i + 1] = mcb;
          }
        }
      }
    } else {
      if (out1) {
        const int i = o1 * D.nx + xa;
        if (kPair) {
          if (outa && ASD_IN(i, N2) && ASD_IN(i + 1, N2)) *(float2 *)(dst + i) = make_float2(pa, pb);
        } else {
          if (outa && ASD_IN(i, N2)) dst[i] = pa;
          if (outb && ASD_IN(i + 1, N2)) dst[i + 1] = pb;
        }
      }
      if (kMode == 0) {
        float wa, wb;
        f2.push(pa, pb, wa, wb);
        const int o2 = j - 2;
        if (!kC || (o2 >= y0 && o2 < y1)) {
          if (outa) acc += wa * wa;
          if (outb) acc += wb * wb;
        }
      }
    }
    if (kC && kMode != 1) {
      const int o = kMode == 2 ? o1 : j - 2;
      if (o >= y0 && o < y1 && ((o + 1) % kBandRows == 0 || o + 1 == y1)) flush(o);
    }
  };
  // steady chunks: outputs of rows j0 - 2 .. j0 + 1 all inside [y0, y1 - 1)
  for (int j0 = jl0; j0 < j1; j0 += kWalkChunk) {
    const int s0 = (j0 - jl0) & (kWalkRing - 1);  // chunks never wrap the ring
    if (kMode == 0 && j0 >= y0 + 2 && j0 <= y1 - 3) {
#pragma unroll
      for (int k = 0; k < kWalkChunk; k++) walk_row(std::false_type(), j0 + k, s0 + k);
      // bands start at multiples of 32 (so does y0) and steady chunks at
      // y0 - 2 plus a multiple of 4: a band can only end at a chunk's end
      if ((j0 + 2) % kBandRows == 0) flush(j0 + 1);
    } else {
#pragma unroll
      for (int k = 0; k < kWalkChunk; k++) walk_row(std::true_type(), j0 + k, s0 + k);
    }
  }
  asm volatile("cp.async.wait_group 0;\n" ::: "memory");  // the ring's last copies
}

__global__ void __launch_bounds__(kWalkWarps * 32, 8)
    k_tv_walk2d(const Inst *__restrict__ insts, int step, int bands,
                const int *__restrict__ zmap) {
  __shared__ float2 ring[kWalkWarps][kWalkRing * 32], ring0[kWalkWarps][kWalkRing * 32];
  pdl_enter();
  const Inst &I = insts[zmap ? zmap[blockIdx.z] : blockIdx.z];
  if (inst_done(I)) return;
  const int ng = I.s->ng;
  if (step >= ng) return;
  const Dims D = I.d;
  const int S = walk_strips(D.nx), NB = walk_bands(D.ny);
  const int per_strip = (NB + bands - 1) / bands;
  const int walks = S * per_strip;
  const int w = blockIdx.x * kWalkWarps + (threadIdx.x >> 5);
  if (w >= walks) return;  // warp-uniform
  const int lane = threadIdx.x & 31;
  const int strip = w % S, b0 = (w / S) * bands;
  const int y0 = b0 * kBandRows, y1 = min(D.ny, (b0 + bands) * kBandRows);
  const int xa = strip * kWalkOut - 2 + 2 * lane;
  const bool last = step == ng - 1;
  const float coef = I.s->tv_coef_f;
  const bool pair = (D.nx & 1) == 0;
  float2 *const rg = ring[threadIdx.x >> 5], *const rg0 = ring0[threadIdx.x >> 5];
  if (!last)
    pair ? tv_walk<0, true>(I, step, y0, y1, xa, strip, S, coef, rg, rg0)
         : tv_walk<0, false>(I, step, y0, y1, xa, strip, S, coef, rg, rg0);
  else if (ng == 1)
    pair ? tv_walk<1, true>(I, step, y0, y1, xa, strip, S, coef, rg, rg0)
         : tv_walk<1, false>(I, step, y0, y1, xa, strip, S, coef, rg, rg0);
  else
    pair ? tv_walk<2, true>(I, step, y0, y1, xa, strip, S, coef, rg, rg0)
         : tv_walk<2, false>(I, step, y0, y1, xa, strip, S, coef, rg, rg0);
  if (last && ng == 1) return;  // nothing to sum: k_finish_iter ends the iteration
  // the walk that finishes last sums the instance's band partials
  unsigned ticket = 0;
  if (lane == 0) {
    __threadfence();
    ticket = atomicAdd(I.counter, 1u);
  }
  ticket = __shfl_sync(0xffffffffu, ticket, 0);
  if (ticket != (unsigned)walks - 1) return;
  __threadfence();
  const int P = S * NB;
  double a = 0.0;
  for (int p = lane; p < P; p += 32) a += ((volatile const double *)I.partials)[p];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
  if (lane == 0) {
    *I.counter = 0u;
    Scalars *s = I.s;
    if (last) {
      finish_scalars(s, a);
    } else {
      s->tv_coef = s->alpha * s->d_tv / sqrt(a);
      s->tv_coef_f = (float)s->tv_coef;
    }
  }
}

// End of the SART sweep for 2-D instances as column walks (the work of
// k_after_sweep<false>): the same strips, bands and ring as k_tv_walk2d,
// streaming m, m_pre, m_k1 and the reference image I0 through four rings.
// Each output voxel copies m to m_res and adds (m - m_pre)^2, (m - m_k1)^2,
// (m - I0)^2 and v(m)^2 (tv2_terms, the TV step's own stencil) to its
// band's four partials; the walk that finishes last sums them in order and
// sets the iteration's scalars (ASD_POCS_cuda.m:137-149).
template <bool kPair>
__device__ __forceinline__ void sweep_walk(const Inst &I, int y0, int y1, int xa, int strip,
                                           int S, bool tv, float2 (*ring)[kWalkRing * 32]) {
  const Dims D = I.d;
  const int lane = threadIdx.x & 31;
  const bool ina = xa >= 0 && xa < D.nx, inb = xa + 1 >= 0 && xa + 1 < D.nx;
  const bool outl = lane >= 1 && lane <= 30;
  const bool outa = outl && ina, outb = outl && inb;
  const bool ref = I.I0 != nullptr;
  float *const mres = I.m_res;
  const float *srcs[4] = {I.m, I.m_pre, I.m_k1, ref ? I.I0 : I.m};
  const int jl0 = y0 - 1, jl1 = min(D.ny, y1 + 1);  // rows read
  const long long N2 = (long long)D.nx * D.ny;       // bounds-checked builds
  auto fetch = [&](int j, int slot) {
    const bool r = (unsigned)j < (unsigned)jl1;
    const int off = r ? j * D.nx : 0;
    const bool va = r && ina && ASD_IN((long long)off + xa, N2) &&
                    (!kPair || ASD_IN((long long)off + xa + 1, N2));
    const bool vb = r && inb && ASD_IN((long long)off + xa + 1, N2);
#pragma unroll
    for (int a = 0; a < 4; a++) {
      float *d = (float *)&ring[a][32 * slot + lane];
      const float *g = srcs[a] + off;
      if (kPair) {
        cp_async_8(d, g + (ina ? xa : 0), va);
      } else {
        cp_async_4(d, g + (ina ? xa : 0), va);
        cp_async_4(d + 1, g + (inb ? xa + 1 : 0), vb);
      }
    }
    asm volatile("cp.async.commit_group;\n" ::: "memory");
  };
  for (int k = 0; k < kWalkRing - 1; k++) fetch(jl0 + k, k);
  WalkField f1{0.f, 0.f, 0.f, 0.f};
  float acc[4] = {0.f, 0.f, 0.f, 0.f};
  const int ntot = y1 + 1 - jl0;  // rows jl0 .. y1
  for (int n = 0; n < ntot; n++) {
    const int j = jl0 + n, slot = n & (kWalkRing - 1);
    const int oslot = (slot + kWalkRing - 1) & (kWalkRing - 1);  // row j - 1
    // row j - 1's other arrays, read before that slot receives row
    // j + kWalkRing - 1
    const float2 mo = ring[0][32 * oslot + lane];
    const float2 pre = ring[1][32 * oslot + lane];
    const float2 k1 = ring[2][32 * oslot + lane];
    const float2 i0 = ring[3][32 * oslot + lane];
    fetch(j + kWalkRing - 1, oslot);
    asm volatile("cp.async.wait_group %0;\n" ::"n"(kWalkRing - 1) : "memory");
    const float2 m = ring[0][32 * slot + lane];
    float va = 0.f, vb = 0.f;
    if (tv) f1.push(m.x, m.y, va, vb);  // warp-uniform
    const int o = j - 1;
    if (o < y0 || o >= y1) continue;  // warp-uniform
    const int i = o * D.nx + xa;
    auto add = [&](float mv, float pv, float kv, float iv, float v) {
      const float a = mv - pv, b = mv - kv;
      acc[0] += a * a;
      acc[1] += b * b;
      if (ref) {
        const float c = mv - iv;
        acc[2] += c * c;
      }
      acc[3] += v * v;
    };
    if (outa) {
      add(mo.x, pre.x, k1.x, i0.x, va);
      if (!kPair && ASD_IN(i, N2)) mres[i] = mo.x;
    }
    if (outb) {
      add(mo.y, pre.y, k1.y, i0.y, vb);
      if (!kPair && ASD_IN(i + 1, N2)) mres[i + 1] = mo.y;
    }
    if (kPair && outa && ASD_IN(i, N2) && ASD_IN(i + 1, N2)) *(float2 *)(mres + i) = mo;
    if ((o + 1) % kBandRows == 0 || o + 1 == y1) {
#pragma unroll
      for (int k = 0; k < 4; k++) {
#pragma unroll
        for (int w = 16; w > 0; w >>= 1) acc[k] += __shfl_xor_sync(0xffffffffu, acc[k], w);
        if (lane == 0) I.partials[((long long)(o / kBandRows) * S + strip) * 4 + k] = (double)acc[k];
        acc[k] = 0.f;
      }
    }
  }
  asm volatile("cp.async.wait_group 0;\n" ::: "memory");
}

__global__ void __launch_bounds__(kWalkWarps * 32)
    k_after_sweep_walk2d(const Inst *__restrict__ insts, int bands,
                         const int *__restrict__ zmap) {
  __shared__ float2 ring[kWalkWarps][4][kWalkRing * 32];
  pdl_enter();
  const Inst &I = insts[zmap ? zmap[blockIdx.z] : blockIdx.z];
  if (inst_done(I)) return;
  const Dims D = I.d;
  const int S = walk_strips(D.nx), NB = walk_bands(D.ny);
  const int per_strip = (NB + bands - 1) / bands;
  const int walks = S * per_strip;
  const int w = blockIdx.x * kWalkWarps + (threadIdx.x >> 5);
  if (w >= walks) return;  // warp-uniform
  const int lane = threadIdx.x & 31;
  const int strip = w % S, b0 = (w / S) * bands;
  const int y0 = b0 * kBandRows, y1 = min(D.ny, (b0 + bands) * kBandRows);
  const int xa = strip * kWalkOut - 2 + 2 * lane;
  const bool tv = I.s->ng > 0;
  if ((D.nx & 1) == 0)
    sweep_walk<true>(I, y0, y1, xa, strip, S, tv, ring[threadIdx.x >> 5]);
  else
    sweep_walk<false>(I, y0, y1, xa, strip, S, tv, ring[threadIdx.x >> 5]);
  unsigned ticket = 0;
  if (lane == 0) {
    __threadfence();
    ticket = atomicAdd(I.counter, 1u);
  }
  ticket = __shfl_sync(0xffffffffu, ticket, 0);
  if (ticket != (unsigned)walks - 1) return;
  __threadfence();
  const int P = S * NB;
  double tot[4];
#pragma unroll
  for (int k = 0; k < 4; k++) {
    double a = 0.0;
    for (int p = lane; p < P; p += 32) a += ((volatile const double *)I.partials)[p * 4 + k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
    tot[k] = a;
  }
  if (lane == 0) {
    *I.counter = 0u;
    sweep_scalars(I, tot);
  }
}

// Cone-beam TV step (imgTVGradMin3D.cpp:83-170) as z walks with the
// stencils in registers.  A block of kZWarps warps owns an (x, y) tile of
// 28 x kZTY output voxels and walks down z through a range of slices: lane
// l holds image column x0 - 4 + l (outputs x0 - 2 .. x0 + 25, x0 a multiple
// of 28, so that the staged columns start on a 16-byte boundary), warp w
// the kZR rows y0 - 1 + kZR w .. (the tile and one row either side).  Each
// slice of m is staged by cp.async (16-byte copies when rows are 16-byte
// aligned), two slices ahead, into a ring of four slices of kZRows x 32
// voxels (zeros outside the image), from which a thread reads its rows and
// the row on either side.
//
// The stencil is the FP32 form above (tv3_r, tv3_inslice, tv3_u: v = 2 u,
// m' = m - (2 coef) u, ||v||^2 = 4 sum u^2).  Each voxel's stencil is a
// state of two registers carried down z (ZWalkField): its value at the last
// slice in and u's in-slice terms there; the next slice gives r+z and
// completes u.  x neighbours come by shuffles, y
// neighbours from the thread's other rows, and r of the row below a thread's
// last row is evaluated again by the thread itself, so the staged slice is
// the only exchange between warps for m.  Per slice k:
//   m(k) in: r(k); u(m) of slice k - 1 and m' = m - 2 coef u (zero outside
//            the image); the in-slice terms of slice k;
//   m'(k - 1): the same walk one slice behind on m' (the rows above and
//            below each warp's rows through shared memory), giving u(m') of
//            slice k - 2 on the tile: ||v(m')||^2.
// A step reads each voxel once and writes it once.  ||v(m')||^2 (or the
// last step's positivity-change norm) is summed per tile and slab of 16
// slices, and the block that finishes last sums the slab partials in order;
// walks of `slabs` consecutive slabs (host-chosen) give the same bits for
// every choice.
constexpr int kZTX = 28;                   // output columns of a tile
constexpr int kZR = 8;                     // rows of a thread
constexpr int kZWarps = 4;
constexpr int kZThreads = kZWarps * 32;
constexpr int kZTY = kZWarps * kZR - 2;    // output rows of a tile
constexpr int kZRows = kZWarps * kZR + 2;  // staged rows
constexpr int kZSlab = 16;                 // slices of a partial
constexpr int kZMinBlocks = 3;             // resident blocks per SM
constexpr int kZCopies = (kZRows * 8 + kZThreads - 1) / kZThreads;  // 16-byte copies of a thread
static_assert(kZTX + 4 == 32 && kZThreads % 8 == 0, "lane = staged column");

struct ZShared {
  float m[4][kZRows][32];  // ring of staged slices of m
  float p[2][kZRows][32];  // m' of two slices: the first and last row of each warp
  float red[kZThreads / 32];
};

// tiles: output columns [28 t - 2, 28 t + 26), rows [kZTY t, kZTY (t + 1))
__host__ __device__ __forceinline__ int zwalk_tiles_x(int nx) { return (nx + 2 + kZTX - 1) / kZTX; }
__host__ __device__ __forceinline__ int zwalk_tiles_y(int ny) { return (ny + kZTY - 1) / kZTY; }
__host__ __device__ __forceinline__ int zwalk_slabs(int nz) { return (nz + kZSlab - 1) / kZSlab; }

// The stencil state of one field at a thread's rows: c the value at the last
// slice in, s the in-slice part of u there; cb the value of the row below
// the thread's last row.
struct ZWalkField {
  float c[kZR], s[kZR];
  float cb;
};
// Slice k of a field comes in (n: the thread's rows; na, nb: the rows above
// and below): u of slice k - 1 into u[] (when kU), and the state moves to
// slice k.
template <bool kU>
__device__ __forceinline__ void zfield_push(ZWalkField &f, const float (&n)[kZR], float na,
                                            float nb, float (&u)[kZR]) {
  float r[kZR + 1], xm[kZR];
#pragma unroll
  for (int i = 0; i <= kZR; i++) {
    const float v = i < kZR ? n[i] : nb;
    const float up = i == 0 ? na : n[i - 1];
    const float prev = i < kZR ? f.c[i] : f.cb;
    const float l = __shfl_up_sync(0xffffffffu, v, 1);
    r[i] = tv3_r(__fsub_rn(v, l), __fsub_rn(v, up), __fsub_rn(v, prev));
    if (i < kZR) xm[i] = l;
  }
#pragma unroll
  for (int i = 0; i < kZR; i++) {
    if (kU) u[i] = tv3_u(f.s[i], f.c[i], n[i], r[i]);
    const float up = i == 0 ? na : n[i - 1];
    const float below = i + 1 < kZR ? n[i + 1] : nb;
    const float xp = __shfl_down_sync(0xffffffffu, n[i], 1);
    const float rx = __shfl_down_sync(0xffffffffu, r[i], 1);
    f.s[i] = tv3_inslice(n[i], xm[i], up, f.c[i], xp, below, r[i], rx, r[i + 1]);
    f.c[i] = n[i];
  }
  f.cb = nb;
}

// kMode as in tv_walk: 0 m' and ||v(m')||^2; 1 m' only; 2 the finishing step.
// kVec: rows of the image start on 16-byte boundaries (16-byte staging).
template <int kMode, bool kVec>
__device__ __forceinline__ void tv_zwalk(const Inst &I, int step, int x0, int y0, int z0,
                                         int z1, float coef, float &acc, int tile, int ntiles,
                                         ZShared &sh) {
  const Dims D = I.d;
  const float *src = tv_src(I, step);
  float *dst = tv_dst(I, step);
  float *const im = I.m, *const impre = I.m_pre;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const long long plane = (long long)D.nx * D.ny, nvox = plane * D.nz;
  const int gx = x0 - 4 + lane;
  const bool colin = gx >= 0 && gx < D.nx;
  const int sy = kZR * warp + 1;  // staged row of the thread's first row
  const float coef2 = 2.f * coef;
  // bit i: the thread's row i lies in the image (x, y) / is an output voxel
  unsigned rin = 0u, rout = 0u;
#pragma unroll
  for (int i = 0; i < kZR; i++) {
    const int gy = y0 - 2 + sy + i;
    if (colin && gy >= 0 && gy < D.ny) {
      rin |= 1u << i;
      if (lane >= 2 && lane < 30 && sy + i >= 2 && sy + i < kZRows - 2) rout |= 1u << i;
    }
  }
  const long long row0 = (long long)(y0 - 2 + sy) * D.nx + gx;  // (x, y) of the first row
  // staging.  kVec: thread t copies 4 columns (group t & 7) of rows
  // t / 8 + j T / 8; otherwise warp w copies rows w + j kZWarps, a column per
  // lane.  Bit j of smask: that copy lies in the image (x, y).
  constexpr int kSR = kVec ? kZCopies : (kZRows + kZWarps - 1) / kZWarps;
  constexpr int kRowStep = kVec ? kZThreads / 8 : kZWarps;
  const int srow0 = kVec ? (int)threadIdx.x / 8 : warp;
  const int scol = kVec ? x0 - 4 + 4 * (threadIdx.x & 7) : gx;
  unsigned smask = 0u;
#pragma unroll
  for (int j = 0; j < kSR; j++) {
    const int srow = srow0 + j * kRowStep, gy = y0 - 2 + srow;
    if (srow < kZRows && scol >= 0 && scol < D.nx && gy >= 0 && gy < D.ny) smask |= 1u << j;
  }
  const long long soff = (long long)(y0 - 2 + srow0) * D.nx + scol;
  const int sstep = kRowStep * D.nx;
  const unsigned sbase = (unsigned)__cvta_generic_to_shared(
      kVec ? &sh.m[0][srow0][4 * (threadIdx.x & 7)] : &sh.m[0][srow0][lane]);
  auto zin = [&](int z) { return z >= 0 && z < D.nz; };
  auto stage = [&](int z) {  // slice z into ring slot z & 3
    const unsigned m = zin(z) ? smask : 0u;
    const long long zo = z * plane + soff;
    const unsigned sa = sbase + (unsigned)(z & 3) * (unsigned)sizeof(sh.m[0]);
#pragma unroll
    for (int j = 0; j < kSR; j++) {
      if (srow0 + j * kRowStep >= kZRows) break;
      const long long gi = zo + (long long)j * sstep;
      const bool in = ((m >> j) & 1u) && ASD_IN(gi, nvox) && (!kVec || ASD_IN(gi + 3, nvox));
      const float *g = in ? src + gi : src;
      const unsigned d = sa + (unsigned)(j * kRowStep * 32 * 4);
      if (kVec)
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(d), "l"(g),
                     "r"(in ? 16 : 0)
                     : "memory");
      else
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(d), "l"(g),
                     "r"(in ? 4 : 0)
                     : "memory");
    }
    asm volatile("cp.async.commit_group;\n" ::: "memory");
  };
  auto flush = [&](int z) {  // the slab of output slice z is complete
    const float vv[1] = {acc};
    float bs[1];
    block_sum_f<kZThreads, 1>(vv, bs, sh.red);
    // kMode 0 sums u^2 = v^2 / 4 (scaling by 4 is exact)
    if (threadIdx.x == 0)
      I.partials[(long long)(z / kZSlab) * ntiles + tile] =
          (double)bs[0] * (kMode == 0 ? 4.0 : 1.0);
    acc = 0.f;
  };
  // z >= 0 here
  auto slab_end = [&](int z) { return ((z + 1) & (kZSlab - 1)) == 0 || z + 1 == z1; };
  // m slices kstart - 1 .. kend; u(m) of kstart .. kend - 1
  const int kstart = kMode == 0 ? z0 - 1 : z0;
  const int kend = kMode == 0 ? z1 + 1 : z1;
  if (warp == 0) {  // rows of m' no warp writes (outside the block's rows)
    sh.p[0][0][lane] = sh.p[1][0][lane] = 0.f;
    sh.p[0][kZRows - 1][lane] = sh.p[1][kZRows - 1][lane] = 0.f;
  }
  stage(kstart - 1);
  stage(kstart);
  stage(kstart + 1);
  asm volatile("cp.async.wait_group 2;\n" ::: "memory");  // slice kstart - 1 landed
  __syncthreads();
  ZWalkField fm, fp;
#pragma unroll
  for (int i = 0; i < kZR; i++) {
    fm.c[i] = sh.m[(kstart - 1) & 3][sy + i][lane];
    fm.s[i] = 0.f;
    fp.c[i] = fp.s[i] = 0.f;
  }
  fm.cb = sh.m[(kstart - 1) & 3][sy + kZR][lane];
  fp.cb = 0.f;
  float mp[kZR];  // m' of the thread's rows, from part A to the next step's part B
  // Step k: one barrier (slice k of m staged; the edge rows of m'(k - 2)
  // written by the other warps in the previous step), then
  //   B: the walk on m' takes m'(k - 2) (kMode 0): u(m') of slice k - 3;
  //   A: the walk on m takes slice k: u(m) and m' of slice k - 1.
  // A steady step (kS) is one whose slices (k - 1 for A, k - 3 for B) are
  // output slices of the walk, so that it needs no range tests; the steady
  // steps run in pairs, which lets the state alternate between registers
  // instead of being copied.
  auto walk_step = [&](auto steady, int k) {
    constexpr bool kS = decltype(steady)::value;
    const int zb = k - 1;  // slice whose u(m) and m' part A gives
    const long long ob = zb * plane + row0;  // its voxel at the thread's first row
    const bool a_on = kS || k <= kend;
    const bool a_out = kS || (k > kstart && zb >= z0 && zb < z1);
    // the finishing step's pre-TV image at the output voxels of slice zb,
    // loaded early so that the loads overlap the wait
    float f0[kZR];
#pragma unroll
    for (int i = 0; i < kZR; i++) {
      f0[i] = 0.f;
      if (kMode == 2 && a_out && ((rout >> i) & 1u) && ASD_IN(ob + i * D.nx, nvox))
        f0[i] = im[ob + i * D.nx];
    }
    stage(k + 2);  // slices past the walk's end are staged too (in the image or zeros)
    asm volatile("cp.async.wait_group 2;\n" ::: "memory");  // slice k landed
    __syncthreads();
    // B: m'(k - 2), written by part A of step k - 1 (kMode 0)
    if (kMode == 0 && (kS || k - 1 > kstart)) {
      const float(*ps)[32] = sh.p[k & 1];
      const float pa = ps[sy - 1][lane], pb = ps[sy + kZR][lane];
      const int zd = k - 3;  // slice whose u(m') this gives
      float u[kZR];
      if (kS || zd >= z0) {
        zfield_push<true>(fp, mp, pa, pb, u);
#pragma unroll
        for (int i = 0; i < kZR; i++)
          if ((rout >> i) & 1u) acc += u[i] * u[i];
        if (slab_end(zd)) flush(zd);
      } else {
        zfield_push<false>(fp, mp, pa, pb, u);
      }
    }
    if (!a_on) return;
    // A: slice k of m
    const float(*ms)[32] = sh.m[k & 3];
    float n[kZR], u[kZR];
#pragma unroll
    for (int i = 0; i < kZR; i++) n[i] = ms[sy + i][lane];
    const float na = ms[sy - 1][lane], nb = ms[sy + kZR][lane];
    if (!kS && k == kstart) {
      zfield_push<false>(fm, n, na, nb, u);
      return;  // the first slice: nothing else to do yet
    }
    float mprev[kZR];
#pragma unroll
    for (int i = 0; i < kZR; i++) mprev[i] = fm.c[i];
    zfield_push<true>(fm, n, na, nb, u);
    const unsigned rinz = (kS || zin(zb)) ? rin : 0u;
#pragma unroll
    for (int i = 0; i < kZR; i++) {
      const float mn = __fmaf_rn(-coef2, u[i], mprev[i]);
      const long long gi = ob + i * D.nx;
      const bool o = a_out && ((rout >> i) & 1u) && ASD_IN(gi, nvox);
      if (kMode == 0) {
        mp[i] = ((rinz >> i) & 1u) ? mn : 0.f;
        if (o) dst[gi] = mn;
      } else if (o) {
        if (kMode == 1) {
          dst[gi] = mn;
        } else {
          const float mc = mn < 0.f ? 0.f : mn;  // imgTVGradMin3D.cpp:163-170
          const float d = mc - f0[i];
          acc += d * d;
          im[gi] = mc;
          impre[gi] = mc;
        }
      }
    }
    if (kMode == 2 && a_out && slab_end(zb)) flush(zb);
    if (kMode == 0) {  // the edge rows of m'(k - 1) for the neighbouring warps
      float(*ps)[32] = sh.p[(k + 1) & 1];
      ps[sy][lane] = mp[0];
      ps[sy + kZR - 1][lane] = mp[kZR - 1];
    }
  };
  // steady steps: kMode 0 k = z0 + 3 .. z1 (A: k - 1, B: k - 3 inside
  // [z0, z1)), kMode 1 and 2 k = z0 + 1 .. z1 (A: k - 1 inside [z0, z1))
  const int ks0 = kMode == 0 ? z0 + 3 : z0 + 1, ks1 = z1;
  const int klast = kMode == 0 ? kend + 1 : kend;  // kMode 0: a last step of part B only
  int k = kstart;
#pragma unroll 1
  for (; k < ks0 && k <= klast; k++) walk_step(std::false_type(), k);
#pragma unroll 1
  for (; k + 1 <= ks1; k += 2) {
    walk_step(std::true_type(), k);
    walk_step(std::true_type(), k + 1);
  }
#pragma unroll 1
  for (; k <= klast; k++) walk_step(std::false_type(), k);
  asm volatile("cp.async.wait_group 0;\n" ::: "memory");
}

template <int kMode>
__device__ __forceinline__ void tv_zwalk_any(const Inst &I, int step, int x0, int y0, int z0,
                                             int z1, float coef, float &acc, int tile,
                                             int ntiles, ZShared &sh) {
  // 16-byte copies need 16-byte aligned rows
  const bool vec = (I.d.nx & 3) == 0 && ((unsigned long long)tv_src(I, step) & 15) == 0;
  if (vec)
    tv_zwalk<kMode, true>(I, step, x0, y0, z0, z1, coef, acc, tile, ntiles, sh);
  else
    tv_zwalk<kMode, false>(I, step, x0, y0, z0, z1, coef, acc, tile, ntiles, sh);
}

__global__ void __launch_bounds__(kZThreads, kZMinBlocks)
    k_tv_walk3d(const Inst *__restrict__ insts, int step, int slabs,
                const int *__restrict__ zmap) {
  __shared__ __align__(16) ZShared sh;
  __shared__ int s_last;
  pdl_enter();
  const Inst &I = insts[zmap ? zmap[blockIdx.z] : blockIdx.z];
  if (inst_done(I)) return;
  const int ng = I.s->ng;
  if (step >= ng) return;
  const Dims D = I.d;
  const int TXn = zwalk_tiles_x(D.nx), TYn = zwalk_tiles_y(D.ny), NS = zwalk_slabs(D.nz);
  const int ntiles = TXn * TYn;
  const int per_tile = (NS + slabs - 1) / slabs;
  const int walks = ntiles * per_tile;
  const int w = blockIdx.x;
  if (w >= walks) return;
  const int tile = w % ntiles, s0 = (w / ntiles) * slabs;
  const int x0 = (tile % TXn) * kZTX, y0 = (tile / TXn) * kZTY;
  const int z0 = s0 * kZSlab, z1 = min(D.nz, (s0 + slabs) * kZSlab);
  const bool last = step == ng - 1;
  const float coef = I.s->tv_coef_f;
  float acc = 0.f;
  if (!last)
    tv_zwalk_any<0>(I, step, x0, y0, z0, z1, coef, acc, tile, ntiles, sh);
  else if (ng == 1)
    tv_zwalk_any<1>(I, step, x0, y0, z0, z1, coef, acc, tile, ntiles, sh);
  else
    tv_zwalk_any<2>(I, step, x0, y0, z0, z1, coef, acc, tile, ntiles, sh);
  if (last && ng == 1) return;
  if (threadIdx.x == 0) {
    __threadfence();
    s_last = atomicAdd(I.counter, 1u) == (unsigned)walks - 1;
  }
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  double tot[1];
  grid_sum_final<kZThreads, 1>(I.partials, I.counter, ntiles * NS, tot);
  if (threadIdx.x == 0) {
    Scalars *s = I.s;
    if (last) {
      finish_scalars(s, tot[0]);
    } else {
      s->tv_coef = s->alpha * s->d_tv / sqrt(tot[0]);
      s->tv_coef_f = (float)s->tv_coef;
    }
  }
}

// End of an iteration for instances whose last TV step did not finish it
// (ng == 0 or ng == 1): positivity (after a TV step), dg, alpha/beta, k.
__global__ void __launch_bounds__(kThreads)
    k_finish_iter(const Inst *__restrict__ insts, const int *__restrict__ zmap) {
  pdl_enter();
  const Inst &I = insts[zmap ? zmap[blockIdx.z] : blockIdx.z];
  if (inst_done(I)) return;
  const int ng = I.s->ng;
  if (ng >= 2) return;  // finished by the last TV step
  const Dims D = I.d;
  const OwnBlock ob = own_block(tile_grid(D.nx, D.ny, D.nz, 1));
  if (ob.bid < 0) return;
  int ix, iy, iz;
  float v[1] = {0.f};
  if (tile_voxel(D.nx, D.ny, D.nz, ix, iy, iz)) {
    const unsigned i = ((unsigned)iz * D.ny + iy) * D.nx + ix;
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
  if (grid_sum<kThreads, 1>(v, I.partials, I.counter, ob.bid, ob.nblocks, tot)) {
    if (threadIdx.x == 0) finish_scalars(I.s, tot[0]);
  }
}

// Done flags of n instances (the serving queue's poll after an iteration).
__global__ void k_gather_done(const Inst *__restrict__ insts, int n, int *out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = ((volatile int *)&insts[i].s->done)[0];
}

}  // namespace

cudaError_t launch_gather_done(const Inst *insts, int n, int *out,
                               cudaStream_t st) {
  k_gather_done<<<(n + 127) / 128, 128, 0, st>>>(insts, n, out);
  return cudaGetLastError();
}

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
                               cudaStream_t st, const int *zmap) {
  const dim3 grid = group_grid(d.nx, d.ny, d.nz, batch);
  if (d.nz > 1) {
    return launch_iter(k_after_sweep<true>, grid, dim3(kThreads), st, insts, zmap);
  } else {
    // one band per walk up to a wave of walks (24 resident warps per SM at
    // 80 registers), then longer walks
    const long long units = (long long)walk_strips(d.nx) * walk_bands(d.ny);
    const long long cap = 152LL * 24;
    const long long per = (units * batch + cap - 1) / cap;
    const int bands = (int)(per < 1 ? 1 : (per > walk_bands(d.ny) ? walk_bands(d.ny) : per));
    const long long walks = (long long)walk_strips(d.nx) * ((walk_bands(d.ny) + bands - 1) / bands);
    return launch_iter(k_after_sweep_walk2d,
                       dim3((unsigned)((walks + kWalkWarps - 1) / kWalkWarps), 1, batch),
                       dim3(kWalkWarps * 32), st, insts, bands, zmap);
  }
}

int tv_walk_max(const Dims &d) {
  return d.nz > 1 ? zwalk_slabs(d.nz) : walk_bands(d.ny);
}

cudaError_t launch_tv_step(const Inst *insts, int batch, const Dims &d,
                           int step, int ng, cudaStream_t st, int walk,
                           const int *zmap) {
  (void)ng;
  const dim3 grid = group_grid(d.nx, d.ny, d.nz, batch);
  if (d.nz > 1) {
    // slabs per walk: the batch's walks within about one wave of resident
    // blocks
    const long long tiles = (long long)zwalk_tiles_x(d.nx) * zwalk_tiles_y(d.ny);
    const long long units = tiles * zwalk_slabs(d.nz);
    const long long cap = 152LL * kZMinBlocks;
    const long long per = walk > 0 ? walk : (units * batch + cap - 1) / cap;
    const int slabs = (int)(per < 1 ? 1 : (per > zwalk_slabs(d.nz) ? zwalk_slabs(d.nz) : per));
    const long long walks = tiles * ((zwalk_slabs(d.nz) + slabs - 1) / slabs);
    return launch_iter(k_tv_walk3d, dim3((unsigned)walks, 1, batch), dim3(kZThreads), st,
                       insts, step, slabs, zmap);
  } else {
    // bands per walk: the batch's walks within about one wave of 32
    // resident warps per SM; one band (16 rows) per walk for small batches,
    // which keeps a single instance's step spread over many warps
    const long long units = (long long)walk_strips(d.nx) * walk_bands(d.ny);
    const long long cap = 152LL * 32;
    const long long per = walk > 0 ? walk : (units * batch + cap - 1) / cap;
    const int bands = (int)(per < 1 ? 1 : (per > walk_bands(d.ny) ? walk_bands(d.ny) : per));
    const long long walks = (long long)walk_strips(d.nx) * ((walk_bands(d.ny) + bands - 1) / bands);
    const dim3 g2((unsigned)((walks + kWalkWarps - 1) / kWalkWarps), 1, batch);
    return launch_iter(k_tv_walk2d, g2, dim3(kWalkWarps * 32), st, insts, step, bands, zmap);
  }
}

int tv_partials_for(const Dims &d) {
  return d.nz > 1 ? zwalk_tiles_x(d.nx) * zwalk_tiles_y(d.ny) * zwalk_slabs(d.nz)
                  : walk_strips(d.nx) * walk_bands(d.ny);
}

cudaError_t launch_finish_iter(const Inst *insts, int batch, const Dims &d,
                               int ng, cudaStream_t st, const int *zmap) {
  (void)ng;
  return launch_iter(k_finish_iter, tile_grid(d.nx, d.ny, d.nz, batch), dim3(kThreads), st,
                     insts, zmap);
}

#ifdef ASDPOCS_CHECKED
ASD_CHECKED_READER(checked_take_tv)
#endif

}  // namespace asd
