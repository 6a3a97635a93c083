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
// (x, y) tiles with the slices staged in shared memory (k_tv_walk3d).  The
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
//   r = 1/sqrt(eps + dx^2 + dy^2 + dz^2)
// and the reference's four terms are
//   v = (((6c - 2(xm + ym + zm)) r + (2c - 2zp) r(+z)) + (2c - 2yp) r(+y))
//       + (2c - 2xp) r(+x):
// the denominators of its second to fourth terms are those of the +z, +y
// and +x neighbours' first terms, in the same order.
__device__ __forceinline__ float tv3_r(float dx, float dy, float dz) {
  return tv_rsqrt(__fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmaf_rn(dx, dx, tv_eps<float>()))));
}
__device__ __forceinline__ float tv3_combine(float c, float xm, float ym, float zm, float xp,
                                             float yp, float zp, float r, float rx, float ry,
                                             float rz) {
  const float c2 = __fmul_rn(2.f, c);
  const float g1 = __fmul_rn(
      __fsub_rn(__fmul_rn(6.f, c), __fmul_rn(2.f, __fadd_rn(__fadd_rn(xm, ym), zm))), r);
  const float g2 = __fmul_rn(__fsub_rn(c2, __fmul_rn(2.f, zp)), rz);
  const float g3 = __fmul_rn(__fsub_rn(c2, __fmul_rn(2.f, yp)), ry);
  const float g4 = __fmul_rn(__fsub_rn(c2, __fmul_rn(2.f, xp)), rx);
  return __fadd_rn(__fadd_rn(__fadd_rn(g1, g2), g3), g4);
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
  return tv3_combine(c, xm, ym, zm, xp, yp, zp, r, rx, ry, rz);
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
    k_after_sweep(const Inst *__restrict__ insts) {
  __shared__ Tile<1, k3D> t;
  pdl_enter();
  const Inst &I = insts[blockIdx.z];
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
    k_tv_walk2d(const Inst *__restrict__ insts, int step, int bands) {
  __shared__ float2 ring[kWalkWarps][kWalkRing * 32], ring0[kWalkWarps][kWalkRing * 32];
  pdl_enter();
  const Inst &I = insts[blockIdx.z];
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
    k_after_sweep_walk2d(const Inst *__restrict__ insts, int bands) {
  __shared__ float2 ring[kWalkWarps][4][kWalkRing * 32];
  pdl_enter();
  const Inst &I = insts[blockIdx.z];
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

// Cone-beam TV step (imgTVGradMin3D.cpp:83-170) as z walks (2.5-D
// blocking).  A block of 16 warps owns a tile of 28 x 28 output voxels in
// (x, y) and walks down z through a range of slices.  Each slice of m is
// staged with a two-voxel halo (32 x 32: lane l holds column x0 - 2 + l,
// warp w rows w and w + 16; zeros outside the image) into a ring of four
// slices by cp.async, one slice ahead.  Per slice k the block forms, on
// shrinking halo regions:
//   A  r(k) = 1/sqrt(eps + dx^2 + dy^2 + dz^2) of m       ([1, 32)^2)
//   B  v(m) of slice k - 1 from m and r (tv3_combine), and
//      m' = m - coef v(m), zero outside the image          ([1, 31)^2)
//   C  r'(k - 1) of m'                                      ([2, 31)^2)
//   D  v(m') of slice k - 2 on the tile: ||v(m')||^2, and m' written out
// so each voxel is read once and written once, with four passes of stencil
// arithmetic over slightly larger regions instead of five full stencils.
// ||v(m')||^2 (or the last step's positivity-change norm) is summed per
// tile and slab of 16 slices, and the block that finishes last sums the
// slab partials in order; walks of `slabs` consecutive slabs (host-chosen)
// give the same bits for every choice.
constexpr int kZTX = 28, kZTY = 28;                 // output tile
constexpr int kZW = kZTX + 4, kZH = kZTY + 4;       // staged slice with halo 2
constexpr int kZSlab = 16;                          // slices of a partial
constexpr int kZThreads = 512;
static_assert(kZW == 32 && kZH == 2 * (kZThreads / 32), "lane = column, two rows per warp");

__host__ __device__ __forceinline__ int zwalk_tiles_x(int nx) { return (nx + kZTX - 1) / kZTX; }
__host__ __device__ __forceinline__ int zwalk_tiles_y(int ny) { return (ny + kZTY - 1) / kZTY; }
__host__ __device__ __forceinline__ int zwalk_slabs(int nz) { return (nz + kZSlab - 1) / kZSlab; }

// kMode as in tv_walk: 0 m' and ||v(m')||^2; 1 m' only; 2 the finishing step.
template <int kMode>
__device__ __forceinline__ void tv_zwalk(const Inst &I, int step, int x0, int y0, int z0,
                                         int z1, float coef, float &acc, int tile, int ntiles,
                                         float (*sm)[kZH][kZW], float (*sr)[kZH][kZW],
                                         float (*sp)[kZH][kZW], float (*sq)[kZH][kZW],
                                         float *shf) {
  const Dims D = I.d;
  const float *src = tv_src(I, step);
  float *dst = tv_dst(I, step);
  float *const im = I.m, *const impre = I.m_pre;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const long long plane = (long long)D.nx * D.ny;
  const int gx = x0 - 2 + lane;
  const bool colin = gx >= 0 && gx < D.nx;
  int gy[2];
  bool in2[2];  // this thread's staged voxels lie inside the image in (x, y)
#pragma unroll
  for (int h = 0; h < 2; h++) {
    gy[h] = y0 - 2 + warp + 16 * h;
    in2[h] = colin && gy[h] >= 0 && gy[h] < D.ny;
  }
  auto zin = [&](int z) { return z >= 0 && z < D.nz; };
  auto stage = [&](int z) {  // slice z into ring slot z & 3
#pragma unroll
    for (int h = 0; h < 2; h++) {
      const long long gi = z * plane + (long long)gy[h] * D.nx + gx;
      const bool in = in2[h] && zin(z) && ASD_IN(gi, plane * D.nz);
      const float *g = in ? src + gi : src;
      const unsigned sa = (unsigned)__cvta_generic_to_shared(&sm[z & 3][warp + 16 * h][lane]);
      asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(sa), "l"(g),
                   "r"(in ? 4 : 0)
                   : "memory");
    }
    asm volatile("cp.async.commit_group;\n" ::: "memory");
  };
  // r of field f (previous slice fb) on [lo, hi)^2
  auto pass_r = [&](const float(*f)[kZW], const float(*fb)[kZW], float(*r)[kZW], int lo,
                    int hi) {
#pragma unroll
    for (int h = 0; h < 2; h++) {
      const int yy = warp + 16 * h;
      if (yy < lo || yy >= hi || lane < lo || lane >= hi) continue;
      const float c = f[yy][lane];
      r[yy][lane] = tv3_r(__fsub_rn(c, f[yy][lane - 1]), __fsub_rn(c, f[yy - 1][lane]),
                          __fsub_rn(c, fb[yy][lane]));
    }
  };
  auto vat = [&](const float(*fm)[kZW], const float(*f)[kZW], const float(*fp)[kZW],
                 const float(*r)[kZW], const float(*rp)[kZW], int yy) {
    return tv3_combine(f[yy][lane], f[yy][lane - 1], f[yy - 1][lane], fm[yy][lane],
                       f[yy][lane + 1], f[yy + 1][lane], fp[yy][lane], r[yy][lane],
                       r[yy][lane + 1], r[yy + 1][lane], rp[yy][lane]);
  };
  auto flush = [&](int z) {  // the slab of output slice z is complete
    const float vv[1] = {acc};
    float bs[1];
    block_sum_f<kZThreads, 1>(vv, bs, shf);
    if (threadIdx.x == 0) I.partials[(long long)(z / kZSlab) * ntiles + tile] = (double)bs[0];
    acc = 0.f;
  };
  auto ring3 = [](int z) { return (z % 3 + 3) % 3; };
  // an output voxel of this thread: tile rows and columns [2, 30)
  auto outvox = [&](int h) {
    const int yy = warp + 16 * h;
    return yy >= 2 && yy < kZH - 2 && lane >= 2 && lane < kZW - 2 && in2[h];
  };
  stage(z0 - 2);
  stage(z0 - 1);
  asm volatile("cp.async.wait_group 0;\n" ::: "memory");
  __syncthreads();
  stage(z0);
  pass_r(sm[(z0 - 1) & 3], sm[(z0 - 2) & 3], sr[(z0 - 1) & 1], 1, kZW);
  const int kend = kMode == 0 ? z1 + 1 : z1;
  for (int k = z0; k <= kend; k++) {
    // the finishing step's pre-TV image at this thread's voxels of slice
    // k - 1, loaded early so the load overlaps the wait and pass A
    float f0[2] = {0.f, 0.f};
    if (kMode == 2 && k - 1 >= z0 && k - 1 < z1) {
#pragma unroll
      for (int h = 0; h < 2; h++)
        if (outvox(h)) {
          const long long gi = (k - 1) * plane + (long long)gy[h] * D.nx + gx;
          f0[h] = ASD_IN(gi, plane * D.nz) ? im[gi] : 0.f;
        }
    }
    if (k + 1 <= kend)
      stage(k + 1);
    else
      asm volatile("cp.async.commit_group;\n" ::: "memory");
    asm volatile("cp.async.wait_group 1;\n" ::: "memory");  // slice k landed
    __syncthreads();
    // A: r(k)
    pass_r(sm[k & 3], sm[(k - 1) & 3], sr[k & 1], 1, kZW);
    __syncthreads();
    // B: v(m) and m' of slice k - 1
    const float(*m0)[kZW] = sm[(k - 2) & 3];
    const float(*m1)[kZW] = sm[(k - 1) & 3];
    const float(*m2)[kZW] = sm[k & 3];
    const float(*r1)[kZW] = sr[(k - 1) & 1];
    const float(*r2)[kZW] = sr[k & 1];
    const int zb = k - 1;
    if (kMode == 0) {
      float(*mp)[kZW] = sp[ring3(zb)];
#pragma unroll
      for (int h = 0; h < 2; h++) {
        const int yy = warp + 16 * h;
        if (yy < 1 || yy >= kZH - 1 || lane < 1 || lane >= kZW - 1) continue;
        const float v = vat(m0, m1, m2, r1, r2, yy);
        mp[yy][lane] = (in2[h] && zin(zb)) ? __fmaf_rn(-coef, v, m1[yy][lane]) : 0.f;
      }
    } else if (zb >= z0 && zb < z1) {
      // the single or finishing step: m' on the tile only
#pragma unroll
      for (int h = 0; h < 2; h++) {
        if (!outvox(h)) continue;
        const int yy = warp + 16 * h;
        const float mn = __fmaf_rn(-coef, vat(m0, m1, m2, r1, r2, yy), m1[yy][lane]);
        const long long gi = zb * plane + (long long)gy[h] * D.nx + gx;
        if (!ASD_IN(gi, plane * D.nz)) continue;
        if (kMode == 1) {
          dst[gi] = mn;
        } else {
          const float mc = mn < 0.f ? 0.f : mn;  // imgTVGradMin3D.cpp:163-170
          const float d = mc - f0[h];
          acc += d * d;
          im[gi] = mc;
          impre[gi] = mc;
        }
      }
      if (kMode == 2 && ((zb + 1) % kZSlab == 0 || zb + 1 == z1)) flush(zb);
    }
    // the next step's staging overwrites slice k - 2's ring slot
    __syncthreads();
    if (kMode != 0) continue;
    // C: r'(k - 1) (needs m' of k - 2, computed one step earlier)
    const int zc = k - 1;
    if (zc >= z0) pass_r(sp[ring3(zc)], sp[ring3(zc - 1)], sq[zc & 1], 2, kZW - 1);
    __syncthreads();
    // D: v(m') of slice k - 2 on the tile, m' written out
    const int zd = k - 2;
    if (zd >= z0) {
      const float(*p0)[kZW] = sp[ring3(zd - 1)];
      const float(*p1)[kZW] = sp[ring3(zd)];
      const float(*p2)[kZW] = sp[ring3(zd + 1)];
#pragma unroll
      for (int h = 0; h < 2; h++) {
        if (!outvox(h)) continue;
        const int yy = warp + 16 * h;
        const long long gi = zd * plane + (long long)gy[h] * D.nx + gx;
        if (ASD_IN(gi, plane * D.nz)) dst[gi] = p1[yy][lane];
        const float w = vat(p0, p1, p2, sq[zd & 1], sq[(zd + 1) & 1], yy);
        acc += w * w;
      }
      if ((zd + 1) % kZSlab == 0 || zd + 1 == z1) flush(zd);
    }
  }
  asm volatile("cp.async.wait_group 0;\n" ::: "memory");
}

__global__ void __launch_bounds__(kZThreads)
    k_tv_walk3d(const Inst *__restrict__ insts, int step, int slabs) {
  __shared__ float sm[4][kZH][kZW], sr[2][kZH][kZW], sp[3][kZH][kZW], sq[2][kZH][kZW];
  __shared__ float shf[kZThreads / 32];
  __shared__ int s_last;
  pdl_enter();
  const Inst &I = insts[blockIdx.z];
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
    tv_zwalk<0>(I, step, x0, y0, z0, z1, coef, acc, tile, ntiles, sm, sr, sp, sq, shf);
  else if (ng == 1)
    tv_zwalk<1>(I, step, x0, y0, z0, z1, coef, acc, tile, ntiles, sm, sr, sp, sq, shf);
  else
    tv_zwalk<2>(I, step, x0, y0, z0, z1, coef, acc, tile, ntiles, sm, sr, sp, sq, shf);
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
    k_finish_iter(const Inst *__restrict__ insts) {
  pdl_enter();
  const Inst &I = insts[blockIdx.z];
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
                               cudaStream_t st) {
  const dim3 grid = group_grid(d.nx, d.ny, d.nz, batch);
  if (d.nz > 1) {
    return launch_iter(k_after_sweep<true>, grid, dim3(kThreads), st, insts);
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
                       dim3(kWalkWarps * 32), st, insts, bands);
  }
}

int tv_walk_max(const Dims &d) {
  return d.nz > 1 ? zwalk_slabs(d.nz) : walk_bands(d.ny);
}

cudaError_t launch_tv_step(const Inst *insts, int batch, const Dims &d,
                           int step, int ng, cudaStream_t st, int walk) {
  (void)ng;
  const dim3 grid = group_grid(d.nx, d.ny, d.nz, batch);
  if (d.nz > 1) {
    // slabs per walk: the batch's walks within about one wave of 2 resident
    // blocks per SM (16 warps and 44 KB of slices each)
    const long long tiles = (long long)zwalk_tiles_x(d.nx) * zwalk_tiles_y(d.ny);
    const long long units = tiles * zwalk_slabs(d.nz);
    const long long cap = 152LL * 2;
    const long long per = walk > 0 ? walk : (units * batch + cap - 1) / cap;
    const int slabs = (int)(per < 1 ? 1 : (per > zwalk_slabs(d.nz) ? zwalk_slabs(d.nz) : per));
    const long long walks = tiles * ((zwalk_slabs(d.nz) + slabs - 1) / slabs);
    return launch_iter(k_tv_walk3d, dim3((unsigned)walks, 1, batch), dim3(kZThreads), st,
                       insts, step, slabs);
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
    return launch_iter(k_tv_walk2d, g2, dim3(kWalkWarps * 32), st, insts, step, bands);
  }
}

int tv_partials_for(const Dims &d) {
  return d.nz > 1 ? zwalk_tiles_x(d.nx) * zwalk_tiles_y(d.ny) * zwalk_slabs(d.nz)
                  : walk_strips(d.nx) * walk_bands(d.ny);
}

cudaError_t launch_finish_iter(const Inst *insts, int batch, const Dims &d,
                               int ng, cudaStream_t st) {
  (void)ng;
  return launch_iter(k_finish_iter, tile_grid(d.nx, d.ny, d.nz, batch), dim3(kThreads), st,
                     insts);
}

#ifdef ASDPOCS_CHECKED
ASD_CHECKED_READER(checked_take_tv)
#endif

}  // namespace asd
