// Projector kernels for sm_103a: Ax (ray-driven, one warp per ray) and Atx
// (voxel-driven, one thread per voxel), standalone and fused with the SART
// per-view update.  Compiled with -fmad=false (see projector.cuh).
//
// Atx stages the view's ray slopes in shared memory: each block first finds
// the detector window its 32x8 voxel tile projects to, computes the slopes
// of those rays once (two divisions per detector column, four per 3D ray),
// then every (voxel, bin) pair reads them instead of dividing again.
#include <algorithm>
#include <type_traits>
#include "kernels.h"
#include "projector.cuh"
#include "reduce.cuh"

namespace asd {

namespace {

constexpr int kAxWarps = 4;             // rays per Ax block
constexpr int kAtxThreads = kTileThreads;
constexpr int kTabA = 512;              // detector columns staged per block
constexpr int kTabC = 1536;             // 3D rays staged per block

__device__ __forceinline__ bool tile_voxel(const Dims &D, int &ix, int &iy,
                                           int &iz) {
  return asd::tile_voxel(D.nx, D.ny, D.nz, ix, iy, iz);
}

// Extents of an instance's volume (nx*ny*nz) and view (na*nb), for ASD_IN.
__device__ __forceinline__ long long nvox(const Dims &D) {
  return (long long)D.nx * D.ny * D.nz;
}
__device__ __forceinline__ long long nray(const Dims &D) { return (long long)D.na * D.nb; }

int atx_blocks(const Dims &d) {
  const dim3 g = tile_grid(d.nx, d.ny, d.nz, 1);
  return (int)(g.x * g.y);
}

// ------------------------------------------------------------------- Ax
// A ray's columns are dealt to kAxCols warps: lane l of warp part p takes
// columns l + 32 p, l + 32 p + 32 kAxCols, ...  The parts' lane partials are
// added in part order (through shared memory), then the lanes by the xor
// butterfly.  Every forward kernel sums a ray this way, so a ray's total
// does not depend on the kernel that computed it.  One warp per ray
// measured fastest for batches and cone beam (two: 14 % slower for a batch
// of 64 and 27 % for 256^3, 7 % faster for one 512^2 instance).
constexpr int kAxCols = 1;
constexpr int kAxBlock = kAxWarps * kAxCols * 32;  // threads per block

// This lane's partial sums of ray r over its columns (no cross-lane sum).
template <class Loader>
__device__ __forceinline__ void ax_lane_partial(const ViewGeo &G, const Dims &D,
                                                long long r, int first, Loader ld,
                                                float &ys, float &ss) {
  const int ia = (int)(r % D.na), ib = (int)(r / D.na);
  const float zd = G.z_det[ib];
  const RayMarch R = ray_setup(G, D, G.y_det[ia], zd);
  ys = 0.f;
  ss = 0.f;
  // fan beams: the loads of two columns per round; cone beams: one (its
  // three pieces per column already keep loads in flight; two measured 6 %
  // slower at 256^3)
  if (D.nz == 1 && zd == 0.0f)
    ray_columns_planar_fast<2>(R, first, 32 * kAxCols, ld, ys, ss);
  else
    ray_columns_fast<1>(R, first, 32 * kAxCols, ld, ys, ss);
}

// The block's ray totals: each warp stores its lane partials of the K values
// in sp[part][ray][k][lane]; after the barrier the part-0 warps add the parts
// in order and sum their lanes.  Every thread of the block must call it.
template <int K>
__device__ __forceinline__ void ax_combine(float (&sp)[kAxCols][kAxWarps][K][32],
                                           float (&v)[K], int part, int rw,
                                           int lane) {
  if constexpr (kAxCols == 1) {
#pragma unroll
    for (int k = 0; k < K; k++) v[k] = warp_sum(v[k]);
  } else {
#pragma unroll
    for (int k = 0; k < K; k++) sp[part][rw][k][lane] = v[k];
    __syncthreads();
    if (part == 0) {
#pragma unroll
      for (int k = 0; k < K; k++) {
        float t = sp[0][rw][k][lane];
#pragma unroll
        for (int p = 1; p < kAxCols; p++) t += sp[p][rw][k][lane];
        v[k] = warp_sum(t);
      }
    }
  }
}

__global__ void __launch_bounds__(kAxBlock)
    k_ax(const float *__restrict__ x, float *__restrict__ y,
         float *__restrict__ sr, ViewGeo G, Dims D) {
  __shared__ float sp[kAxCols][kAxWarps][2][32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int rw = warp % kAxWarps, part = warp / kAxWarps;
  const long long r = (long long)blockIdx.x * kAxWarps + rw;
  const bool in = r < (long long)D.na * D.nb;
  float v[2] = {0.f, 0.f};
  if (in)
    ax_lane_partial(G, D, r, lane + 32 * part,
                    [&](unsigned i) { return ASD_IN(i, nvox(D)) ? __ldg(x + i) : 0.f; },
                    v[0], v[1]);
  ax_combine<2>(sp, v, part, rw, lane);
  if (in && part == 0 && lane == 0 && ASD_IN(r, nray(D))) {
    y[r] = v[0] * G.scale;
    sr[r] = v[1] * G.scale;
  }
}

// Exact forward projection (siddon_setup, siddon_columns), a warp per 32
// rays: lane j sets up ray j (its FP64 arithmetic once per ray, not once per
// lane: the GPU's FP64 rate is a small fraction of its FP32 rate), then the
// warp walks the 32 rays in turn, each ray's set-up broadcast from its lane
// and its columns dealt to the lanes, summed by the butterfly; lane j keeps
// ray j's totals.
__device__ __forceinline__ DSFloat ds_shfl(DSFloat v, int src) {
  DSFloat o;
  o.hi = __shfl_sync(0xffffffffu, v.hi, src);
  o.lo = __shfl_sync(0xffffffffu, v.lo, src);
  return o;
}

__device__ __forceinline__ SidRay sid_bcast(const SidRay &R, int src) {
  SidRay o;
#pragma unroll
  for (int a = 0; a < 2; a++) {
    o.pos0[a] = ds_shfl(R.pos0[a], src);
    o.r[a] = ds_shfl(R.r[a], src);
    o.n_ax[a] = __shfl_sync(0xffffffffu, R.n_ax[a], src);
  }
  o.ua = ds_shfl(R.ua, src);
  o.ub = ds_shfl(R.ub, src);
  o.Lu = __shfl_sync(0xffffffffu, R.Lu, src);
  o.du = __shfl_sync(0xffffffffu, R.du, src);
  o.nax = __shfl_sync(0xffffffffu, R.nax, src);
  o.nu = __shfl_sync(0xffffffffu, R.nu, src);
  o.full0 = __shfl_sync(0xffffffffu, R.full0, src);
  o.full1 = __shfl_sync(0xffffffffu, R.full1, src);
  o.su = __shfl_sync(0xffffffffu, R.su, src);
  o.sv = __shfl_sync(0xffffffffu, R.sv, src);
  o.sz = __shfl_sync(0xffffffffu, R.sz, src);
  o.hit = __shfl_sync(0xffffffffu, (int)R.hit, src) != 0;
  return o;
}

// Totals of rays r0 + lane (lane < nr - r0) for the whole warp.
template <class Loader>
__device__ __forceinline__ void siddon_warp_rays(const ViewGeo &G, const Dims &D,
                                                 long long r0, long long nr, Loader ld,
                                                 float &my_y, float &my_s) {
  const int lane = threadIdx.x & 31;
  SidRay mine;
  const DSFloat z{0.f, 0.f};
  mine.pos0[0] = mine.pos0[1] = mine.r[0] = mine.r[1] = mine.ua = mine.ub = z;
  mine.Lu = 0.f;
  mine.du = mine.nax = mine.nu = mine.n_ax[0] = mine.n_ax[1] = mine.full0 = mine.full1 = 0;
  mine.su = mine.sv = mine.sz = 0u;
  mine.hit = false;
  const long long r = r0 + lane;
  if (r < nr) mine = siddon_setup(G, D, G.y_det[r % D.na], G.z_det[r / D.na]);
  const int cnt = (int)min(32LL, nr - r0);
  my_y = my_s = 0.f;
  for (int j = 0; j < cnt; j++) {
    const SidRay R = sid_bcast(mine, j);
    float ys = 0.f, ss = 0.f;
    siddon_columns(R, lane, 32, ld, ys, ss);
    ys = warp_sum(ys);
    ss = warp_sum(ss);
    if (lane == j) {
      my_y = ys;
      my_s = ss;
    }
  }
}

constexpr int kSidRays = kAxWarps * 32;  // rays per block of the exact kernels

__global__ void __launch_bounds__(kAxBlock)
    k_ax_siddon(const float *__restrict__ x, float *__restrict__ y,
                float *__restrict__ sr, ViewGeo G, Dims D) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const long long nr = (long long)D.na * D.nb;
  const long long r0 = ((long long)blockIdx.x * kAxWarps + warp) * 32;
  if (r0 >= nr) return;  // the whole warp
  float yv, sv;
  siddon_warp_rays(G, D, r0, nr,
                   [&](unsigned i) { return ASD_IN(i, nvox(D)) ? __ldg(x + i) : 0.f; }, yv, sv);
  const long long r = r0 + lane;
  if (r < nr) {
    y[r] = yv * G.scale;
    sr[r] = sv * G.scale;
  }
}

// ------------------------------------------------------------------- Atx
// Shared staging of one block: the slopes of every ray its voxels see and the
// view's values on those rays.
template <bool kPlanar>
struct AtxShared {
  static constexpr int kA = kTabA;
  static constexpr int kC = kPlanar ? kTabA : kTabC;
  float4 tabA[kA];
  float4 tabC[kPlanar ? 1 : kC];
  float ys[kC];
  int amin, amax, bmin, bmax;
};

// Footprint sum of one voxel (Ax_cone_gpu.cu:247-269) for every thread of
// the block: each block finds the detector window of its voxel tile, stages
// the window's ray slopes and view values in shared memory, and every lane of
// a warp then walks the same number of (bin) steps -- the warp's longest
// footprint -- with the face tests evaluated branch-free, so lanes seeing
// different rays do not serialise.  Each lane walks only the bins of its
// voxel's shadow (shadow_bins / shadow_bins3, inside the reference's window);
// the bins it skips have chords of exactly 0, which add nothing unless a view
// value is not finite, so a block whose window holds NaN/inf, an
// axis-parallel ray (whose reference chord is not geometric) or detector
// coordinates off the uniform grid the shadow assumes walks the whole
// window.  Pairs are accumulated in the reference's order (ib outer, ia
// inner).  A block whose window does not fit the staging arrays (extreme
// geometry) falls back to the direct per-pair computation.
// Must be called by every thread of the block.
template <bool kPlanar, class YLoad>
__device__ __forceinline__ void atx_block_sum(const ViewGeo &G, const Dims &D,
                                              bool valid, int ix, int iy,
                                              int iz, AtxShared<kPlanar> &sh,
                                              YLoad yl, float &acc,
                                              float &accl) {
  using Sh = AtxShared<kPlanar>;
  // planar kernels verify the geometry they were chosen for (z_det == 0)
  const bool planar_ok = !kPlanar || G.z_det[0] == 0.0f;
  VoxelWin w;
  w.a0 = 0;
  w.a1 = -1;
  w.b0 = 0;
  w.b1 = -1;
  if (threadIdx.x == 0) {
    sh.amin = 0x7fffffff;
    sh.amax = -1;
    sh.bmin = 0x7fffffff;
    sh.bmax = -1;
  }
  __syncthreads();
  bool has = false;
  if (valid) {
    w = voxel_window(G, D, ix, iy, iz);
    has = w.a0 <= w.a1 && w.b0 <= w.b1;
  }
  {
    // block window: warp-reduced, then one shared atomic per warp
    const int big = 0x7fffffff;
    const int a0 = __reduce_min_sync(0xffffffffu, has ? w.a0 : big);
    const int a1 = __reduce_max_sync(0xffffffffu, has ? w.a1 : -1);
    const int b0 = __reduce_min_sync(0xffffffffu, has ? w.b0 : big);
    const int b1 = __reduce_max_sync(0xffffffffu, has ? w.b1 : -1);
    if ((threadIdx.x & 31) == 0 && a1 >= 0) {
      atomicMin(&sh.amin, a0);
      atomicMax(&sh.amax, a1);
      atomicMin(&sh.bmin, b0);
      atomicMax(&sh.bmax, b1);
    }
  }
  __syncthreads();
  const int amin = sh.amin, bmin = sh.bmin;
  const int nA = sh.amax - amin + 1, nB = sh.bmax - bmin + 1;
  acc = 0.f;
  accl = 0.f;
  if (nA <= 0) return;  // no voxel of the block sees the detector
  const bool staged = planar_ok && nA <= Sh::kA && (long long)nA * nB <= Sh::kC;
  // narrowing to the pixel shadow needs finite view values and rays with
  // both in-plane components (an axis-parallel ray's reference chord ignores
  // one coordinate and is 1 for every voxel of the window)
  bool narrow = true;
  bool allx = true, ally = true;  // every ray of the window x- / y-dominant
  if (staged) {
    narrow = G.dy_det > 0.0f && (kPlanar || G.dz_det > 0.0f);
    for (int k = threadIdx.x; k < nA; k += kAtxThreads) {
      const float yd = G.y_det[amin + k];
      const float4 A = ray_tab_a(G, yd);
      narrow = narrow && A.x != 0.0f && A.y != 0.0f &&
               on_grid(yd, amin + k, D.na, G.dy_det);
      const bool xf = fabsf(A.x) > fabsf(A.y);
      allx = allx && xf;
      ally = ally && !xf;
      sh.tabA[k] = A;
    }
    allx = __syncthreads_and(allx);
    ally = __syncthreads_and(ally);
    for (int k = threadIdx.x; k < nA * nB; k += kAtxThreads) {
      const int r = kPlanar ? 0 : k / nA, c = kPlanar ? k : k - r * nA;
      const long long yi = (long long)(bmin + r) * D.na + amin + c;
      const float v = ASD_IN(yi, nray(D)) ? yl(yi) : 0.f;
      narrow = narrow && isfinite(v);
      sh.ys[k] = v;
    }
    if (!kPlanar)
      for (int k = threadIdx.x; k < nB; k += kAtxThreads)
        narrow = narrow && on_grid(G.z_det[bmin + k], bmin + k, D.nb, G.dz_det);
    narrow = __syncthreads_and(narrow);
    if (!kPlanar) {
      for (int k = threadIdx.x; k < nA * nB; k += kAtxThreads)
        sh.tabC[k] = ray_tab_c(sh.tabA[k % nA], G.z_det[bmin + k / nA]);
      __syncthreads();
    }
  }
  if (!staged) {
    if (valid) voxel_backproject(G, D, w, yl, acc, accl);
    return;
  }
  const float rx = G.cos_phi * (-G.SO) - w.xc;
  const float ry = G.sin_phi * (-G.SO) - w.yc;
  const float rz = 0.0f - w.zc;
  int lo = w.a0, hi = w.a1, blo = w.b0, bhi = w.b1;
  if (narrow && has) {
    int slo, shi, tlo, thi;
    if (kPlanar ? shadow_bins(G, D, w.xc, w.yc, slo, shi)
                : shadow_bins3(G, D, w.xc, w.yc, w.zc, slo, shi, tlo, thi)) {
      lo = max(lo, slo);
      hi = min(hi, shi);
      if (!kPlanar) {
        blo = max(blo, tlo);
        bhi = min(bhi, thi);
      }
    }
  }
  const int cntA = has && lo <= hi ? hi - lo + 1 : 0;
  const int cntB = has && blo <= bhi ? bhi - blo + 1 : 0;
  const int kA = __reduce_max_sync(0xffffffffu, cntA);
  const int kB = __reduce_max_sync(0xffffffffu, cntB);
  const int a_off = lo - amin;
  if (kPlanar && narrow && (allx || ally)) {
    // common case: no axis-parallel ray and one dominant axis for the whole
    // window; the chord needs no per-ray selection
    const int j0 = has ? a_off : 0;
    for (int ka = 0; ka < kA; ka++) {
      const bool on = ka < cntA;
      const int j = on ? j0 + ka : 0;
      const float4 A = sh.tabA[j];
      const float l = allx ? chord_planar_axis<true>(A, rx, ry)
                           : chord_planar_axis<false>(A, rx, ry);
      if (on) {
        acc += l * sh.ys[j];
        accl += l;
      }
    }
    return;
  }
  for (int kb = 0; kb < kB; kb++) {
    const bool onb = kb < cntB;
    const int ib = blo + kb;
    const float c = kPlanar ? 0.0f : G.z_det[onb ? ib : bmin] - 0.0f;
    const int row = (onb ? ib - bmin : 0) * nA + a_off;
    for (int ka = 0; ka < kA; ka++) {
      const bool on = onb && ka < cntA;
      const int j = on ? row + ka : 0;
      const float4 A = sh.tabA[on ? a_off + ka : 0];
      float l;
      if (kPlanar)
        l = chord_planar_bf(A, rx, ry, G.dz);
      else
        l = chord3_bf(A, sh.tabC[j], c, rx, ry, rz, G.dz);
      if (on) {
        acc += l * sh.ys[j];
        accl += l;
      }
    }
  }
}

template <bool kPlanar>
__global__ void __launch_bounds__(kAtxThreads, kPlanar ? 4 : 3)
    k_atx(float *__restrict__ x, const float *__restrict__ yv,
          float *__restrict__ sc, ViewGeo G, Dims D) {
  __shared__ AtxShared<kPlanar> sh;
  int ix, iy, iz;
  const bool valid = tile_voxel(D, ix, iy, iz);
  float acc, accl;
  atx_block_sum<kPlanar>(G, D, valid, ix, iy, iz, sh,
                         [&](long long i) { return ASD_IN(i, nray(D)) ? __ldg(yv + i) : 0.f; },
                         acc, accl);
  if (!valid) return;
  const unsigned idx = ((unsigned)iz * D.ny + iy) * D.nx + ix;
  if (!ASD_IN(idx, nvox(D))) return;
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

// Ray slope tables of every view (Inst::tabA) and the view flags, once per
// plan: grid (ceil(na/128), nv, instances) for the largest na and nv.
__global__ void __launch_bounds__(128)
    k_view_tables(const Inst *__restrict__ insts) {
  const Inst &I = insts[blockIdx.z];
  const Dims D = I.d;
  const int view = blockIdx.y;
  if (view >= I.nv) return;
  const int ia = blockIdx.x * 128 + threadIdx.x;
  const ViewGeo G = view_of(I, view);
  int f = 0;
  if (ia < D.na) {
    const float4 A = ray_tab_a(G, G.y_det[ia]);
    I.tabA[(long long)view * D.na + ia] = A;
    const bool xf = fabsf(A.x) > fabsf(A.y);
    f = (A.x == 0.0f || A.y == 0.0f ? kViewAxisParallel : 0) |
        (xf ? 0 : kViewNotX) | (xf ? kViewNotY : 0);
  }
  f = __reduce_or_sync(0xffffffffu, f);
  if ((threadIdx.x & 31) == 0 && f) atomicOr(I.vflags + view, f);
}

// ASD_POCS_cuda.m:117-123: [proj,sumR]=Ax(m); sumR(sumR==0)=1;
// cor0=P(:,ii)-proj; dd2+=||cor0||^2; cor=cor0./sumR.
// Also records whether every residual is finite (Scalars::cor_finite), and
// for 3D geometry writes the view's per-ray slopes ray_tab_c for the
// backward step that follows (Inst::tabc_mode: a shared table's writer does
// so even after its own iterations have ended).
template <bool k3D>
__global__ void __launch_bounds__(kAxBlock)
    k_sart_ax(const Inst *__restrict__ insts, int view, const int *__restrict__ zmap) {
  __shared__ float sp[kAxCols][kAxWarps][2][32];
  pdl_enter();
  const Inst &I = insts[zmap ? zmap[blockIdx.z] : blockIdx.z];
  if (view >= I.nv) return;
  const bool done = ((volatile int *)&I.s->done)[0] != 0;
  const bool tabc = k3D && (I.tabc_mode == kTabcShared || (!done && I.tabc_mode == kTabcOwn));
  if (done && !tabc) return;
  const Dims D = I.d;
  const long long nr = (long long)D.na * D.nb;
  const OwnBlock ob = own_block(dim3((unsigned)((nr + kAxWarps - 1) / kAxWarps), 1));
  if (ob.bid < 0) return;
  const ViewGeo G = view_of(I, view);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int rw = warp % kAxWarps, part = warp / kAxWarps;
  const long long r = (long long)blockIdx.x * kAxWarps + rw;
  if (tabc && part == 0 && lane == 0 && r < nr && ASD_IN(r, nr)) {
    const int ia = (int)(r % D.na), ib = (int)(r / D.na);
    I.tabC[r] = ray_tab_c(I.tabA[(long long)view * D.na + ia], G.z_det[ib]);
  }
  if (done) return;  // the whole instance: no reduction
  float v[2] = {0.f, 0.f};
  if (r < nr) {
    const float *m = I.m;
    ax_lane_partial(G, D, r, lane + 32 * part,
                    [&](unsigned i) { return ASD_IN(i, nvox(D)) ? m[i] : 0.f; }, v[0], v[1]);
  }
  ax_combine<2>(sp, v, part, rw, lane);
  float pt[2] = {0.f, 0.f};  // dd2, non-finite residuals
  if (r < nr && part == 0 && lane == 0) {
    const float yv = v[0] * G.scale, srv = v[1] * G.scale;
    const long long pi = (long long)view * nr + r;
    const float c0 = (ASD_IN(pi, nr * I.nv) ? sino_at(I, pi) : 0.f) - yv;
    const float cr = c0 / (srv == 0.f ? 1.f : srv);
    if (ASD_IN(r, nr)) I.cor[r * I.cor_stride] = cr;
    pt[0] = c0 * c0;
    pt[1] = isfinite(cr) ? 0.f : 1.f;
  }
  double tot[2];
  if (grid_sum<kAxBlock, 2>(pt, I.partials, I.counter, ob.bid, ob.nblocks, tot)) {
    if (threadIdx.x == 0) {
      I.s->dd2_acc += tot[0];
      I.s->cor_finite = tot[1] == 0.0;
    }
  }
}

// k_sart_ax with the exact projection (siddon_warp_rays): a warp per 32 rays,
// lane j ray j's residual, normalisation and partial sums.
template <bool k3D>
__global__ void __launch_bounds__(kAxBlock)
    k_sart_ax_exact(const Inst *__restrict__ insts, int view, const int *__restrict__ zmap) {
  pdl_enter();
  const Inst &I = insts[zmap ? zmap[blockIdx.z] : blockIdx.z];
  if (view >= I.nv) return;
  const bool done = ((volatile int *)&I.s->done)[0] != 0;
  const bool tabc = k3D && (I.tabc_mode == kTabcShared || (!done && I.tabc_mode == kTabcOwn));
  if (done && !tabc) return;
  const Dims D = I.d;
  const long long nr = (long long)D.na * D.nb;
  const OwnBlock ob = own_block(dim3((unsigned)((nr + kSidRays - 1) / kSidRays), 1));
  if (ob.bid < 0) return;
  const ViewGeo G = view_of(I, view);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const long long r0 = ((long long)blockIdx.x * kAxWarps + warp) * 32, r = r0 + lane;
  if (tabc && r < nr && ASD_IN(r, nr)) {
    const int ia = (int)(r % D.na), ib = (int)(r / D.na);
    I.tabC[r] = ray_tab_c(I.tabA[(long long)view * D.na + ia], G.z_det[ib]);
  }
  if (done) return;  // the whole instance: no reduction
  float yv = 0.f, sv = 0.f;
  if (r0 < nr) {  // warp-uniform
    const float *m = I.m;
    siddon_warp_rays(G, D, r0, nr, [&](unsigned i) { return ASD_IN(i, nvox(D)) ? m[i] : 0.f; },
                     yv, sv);
  }
  float pt[2] = {0.f, 0.f};  // dd2, non-finite residuals
  if (r < nr) {
    const float yy = yv * G.scale, srv = sv * G.scale;
    const long long pi = (long long)view * nr + r;
    const float c0 = (ASD_IN(pi, nr * I.nv) ? sino_at(I, pi) : 0.f) - yy;
    const float cr = c0 / (srv == 0.f ? 1.f : srv);
    if (ASD_IN(r, nr)) I.cor[r * I.cor_stride] = cr;
    pt[0] = c0 * c0;
    pt[1] = isfinite(cr) ? 0.f : 1.f;
  }
  double tot[2];
  if (grid_sum<kAxBlock, 2>(pt, I.partials, I.counter, ob.bid, ob.nblocks, tot)) {
    if (threadIdx.x == 0) {
      I.s->dd2_acc += tot[0];
      I.s->cor_finite = tot[1] == 0.0;
    }
  }
}

// Planar chord for a window whose rays share dominant axis AX (1: x, 2: y;
// no axis-parallel ray), or any ray (AX == 0).
template <int AX>
__device__ __forceinline__ float chord_sel(const float4 A, float rx, float ry,
                                           float dz) {
  if (AX == 1) return chord_planar_axis<true>(A, rx, ry);
  if (AX == 2) return chord_planar_axis<false>(A, rx, ry);
  return chord_planar_bf(A, rx, ry, dz);
}

// Backward step over this block's tile group (see k_sart_atx).
// ---------------------------------------------------------------------------
// Chord tables of 2-D plans.  The chords of the backward step depend on the
// geometry and the view only, so a plan computes every view's chords once
// (k_atx_chords; one table for instances sharing geometry and view angles,
// else one per instance) and its backward steps read them instead of
// repeating the window, shadow and face tests of find_l for every group and
// iteration.  Per view the table holds, for voxel vi = iy * nx + ix of the
// N = nx * ny voxels:
//   hdr[vi]          (count << 24) | first ray, 0 for no pair
//   sum[vi]          the voxel's chord sum (float bits)
//   ch[k * N + vi]   chord of pair k < count (ray first + k)
// in that order, (2 + chK) * N words per view.  The pairs, their chords and
// the chord sum are those of the narrow form of the backward steps
// (sart_atx_tiles, atx_shared_voxel), in the same order and from the same
// functions, so they give the same bits with or without the table.  Views
// with an axis-parallel ray have no table (their pairs need the full
// window); the steps also keep the direct form when a residual is not
// finite (0 * inf is not 0).
// ---------------------------------------------------------------------------
constexpr int kChordMaxSlots = 32;
// chord slots a thread loads with the table header, before it knows its count
constexpr int kChordPre = 4;

__host__ __device__ __forceinline__ size_t chord_view_words(const Dims &d, int K) {
  return (size_t)(2 + K) * (size_t)d.nx * (size_t)d.ny;
}

// Backward step over this block's tile group from the view's chord table
// (2-D, narrow form; see sart_atx_tiles): the image value, header, chord sum
// and first kChordPre chords of a voxel are loaded together, then its
// residuals (L1) in the pairs' order.
__device__ __forceinline__ void sart_atx_tiles_tab(const Inst &I, const ViewGeo &G,
                                                   const Dims &D, const int *__restrict__ tab,
                                                   int K) {
  const float beta = I.s->beta_f;
  float *m = I.m;
  const float *__restrict__ cor = I.cor;
  const size_t N = (size_t)D.nx * D.ny;
  for (int t = 0; t < kTilesPerBlock; t++) {
    int x0, y0, iz;
    if (!group_tile(D.ny, D.nz, t, x0, y0, iz)) break;
    const int ix = x0 + threadIdx.x % kTileX, iy = y0 + threadIdx.x / kTileX;
    const bool valid = ix < D.nx && iy < D.ny;
    const unsigned vi = valid ? (unsigned)iy * D.nx + ix : 0u;
    const float *__restrict__ ch = (const float *)(tab + 2 * N) + vi;
    int h = 0;
    float accl = 0.f, mv = 0.f;
    float pre[kChordPre];
#pragma unroll
    for (int k = 0; k < kChordPre; k++) pre[k] = 0.f;
    if (valid && ASD_IN(vi, N)) {
      h = __ldg(tab + vi);
      accl = __int_as_float(__ldg(tab + N + vi));
#pragma unroll
      for (int k = 0; k < kChordPre; k++)
        if (k < K) pre[k] = __ldg(ch + (size_t)k * N);  // slot k < K exists
      mv = m[vi];
    }
    const int cnt = (int)((unsigned)h >> 24), first = h & 0xffffff;
    const int kA = __reduce_max_sync(0xffffffffu, cnt);
    const long long M = nray(D);
    float acc = 0.f;
#pragma unroll
    for (int ka = 0; ka < kChordPre; ka++)
      if (ka < kA && ka < cnt && ASD_IN(first + ka, M)) acc += pre[ka] * __ldg(cor + first + ka);
    for (int ka = kChordPre; ka < kA; ka++)
      if (ka < cnt && ASD_IN(ka, K) && ASD_IN(first + ka, M))
        acc += __ldg(ch + (size_t)ka * N) * __ldg(cor + first + ka);
    if (valid && ASD_IN(vi, N)) {
      const float bp = acc * G.scale, scv = accl * G.scale;
      const float mn = mv + beta * __fdividef(bp, scv == 0.f ? 1.f : scv);
      m[vi] = mn < 0.f ? 0.f : mn;
    }
  }
}

template <bool kPlanar, int AX>
__device__ __forceinline__ void sart_atx_tiles(const Inst &I, const ViewGeo &G,
                                               const Dims &D,
                                               const float4 *__restrict__ tabA,
                                               bool narrow) {
  const float beta = I.s->beta_f;
  const bool planar_ok = !kPlanar || G.z_det[0] == 0.0f;
  float *m = I.m;
  const float *__restrict__ cor = I.cor;
  const float4 *__restrict__ tabC = I.tabC;
  const float rx0 = G.cos_phi * (-G.SO), ry0 = G.sin_phi * (-G.SO);
  for (int t = 0; t < kTilesPerBlock; t++) {
    int x0, y0, iz;
    if (!group_tile(D.ny, D.nz, t, x0, y0, iz)) break;
    const int ix = x0 + threadIdx.x % kTileX, iy = y0 + threadIdx.x / kTileX;
    const bool valid = ix < D.nx && iy < D.ny;
    float acc = 0.f, accl = 0.f;
    VoxelWin w;
    bool has = false;
    if (valid) {
      w = voxel_window(G, D, ix, iy, iz);
      has = w.a0 <= w.a1 && w.b0 <= w.b1;
    }
    if (!planar_ok) {
      // planar kernel on a geometry with z_det != 0: direct per-pair form
      if (valid)
        voxel_backproject(G, D, w,
                          [&](long long i) { return ASD_IN(i, nray(D)) ? cor[i] : 0.f; }, acc,
                          accl);
    } else {
      int lo = has ? w.a0 : 0, hi = has ? w.a1 : -1;
      int blo = has ? w.b0 : 0, bhi = has ? w.b1 : -1;
      if (narrow && has) {
        int slo, shi, tlo, thi;
        if (kPlanar ? shadow_bins(G, D, w.xc, w.yc, slo, shi)
                    : shadow_bins3(G, D, w.xc, w.yc, w.zc, slo, shi, tlo, thi)) {
          lo = max(lo, slo);
          hi = min(hi, shi);
          if (!kPlanar) {
            blo = max(blo, tlo);
            bhi = min(bhi, thi);
          }
        }
      }
      const int cntA = has && lo <= hi ? hi - lo + 1 : 0;
      const int cntB = has && blo <= bhi ? bhi - blo + 1 : 0;
      const int kA = __reduce_max_sync(0xffffffffu, cntA);
      const int kB =
          kPlanar ? (kA > 0 ? 1 : 0) : __reduce_max_sync(0xffffffffu, cntB);
      const float rx = rx0 - (has ? w.xc : 0.f), ry = ry0 - (has ? w.yc : 0.f);
      const float rz = 0.0f - (has ? w.zc : 0.f);
      if (kPlanar) {
        for (int kb = 0; kb < kB; kb++) {
          const bool onb = kb < cntB;
          for (int ka = 0; ka < kA; ka++) {
            const bool on = onb && ka < cntA;
            const int ia = on ? lo + ka : 0;
            const float4 A = ASD_IN(ia, D.na) ? __ldg(tabA + ia) : make_float4(1.f, 1.f, 1.f, 1.f);
            const float yv = on && ASD_IN(ia, nray(D)) ? __ldg(cor + ia) : 0.f;
            const float l = chord_sel<AX>(A, rx, ry, G.dz);
            if (on) {
              acc += l * yv;
              accl += l;
            }
          }
        }
      } else {
        // the voxel's (row, column) pairs as one sequence (rows outer, the
        // reference's order), so a warp walks its longest sequence rather
        // than its widest row times its tallest column
        const int cnt = cntA * cntB;
        const int kN = __reduce_max_sync(0xffffffffu, cnt);
        int ka = 0, ib = blo;
        for (int k = 0; k < kN; k++) {
          const bool on = k < cnt;
          const int ia = on ? lo + ka : 0, ibs = on ? ib : 0;
          const int r = ibs * D.na + ia;
          const bool ok = ASD_IN(ibs, D.nb) && ASD_IN(ia, D.na) && ASD_IN(r, nray(D));
          const float c = (ok ? __ldg(G.z_det + ibs) : 0.f) - 0.0f;
          const float4 A = ok ? __ldg(tabA + ia) : make_float4(1.f, 1.f, 1.f, 1.f);
          const float4 Cs = ok ? __ldg(tabC + r) : make_float4(0.f, 0.f, 0.f, 0.f);
          const float yv = on && ok ? __ldg(cor + r) : 0.f;
          const float l = AX == 0 ? chord3_bf(A, Cs, c, rx, ry, rz, G.dz)
                                  : chord3_axis<AX == 1>(A, Cs, rx, ry, rz, G.dz);
          if (on) {
            acc += l * yv;
            accl += l;
          }
          if (++ka == cntA) {
            ka = 0;
            ib++;
          }
        }
      }
    }
    const unsigned idx = ((unsigned)iz * D.ny + iy) * D.nx + ix;
    if (valid && ASD_IN(idx, nvox(D))) {
      const float bp = acc * G.scale, scv = accl * G.scale;
      const float mn = m[idx] + beta * __fdividef(bp, scv == 0.f ? 1.f : scv);
      m[idx] = mn < 0.f ? 0.f : mn;
    }
  }
}

// ASD_POCS_cuda.m:125-131: [bProj,sumC]=Atx(cor); sumC(sumC==0)=1;
// m = m + beta*(bProj./sumC); m(m<0)=0.
// Reads the view's ray tables and residuals through the L1 cache, so no
// block-wide staging or barrier is needed; each lane walks its voxel's shadow
// (or, when the view does not allow narrowing, the reference's window) in
// warp-uniform steps, pairs accumulated in the reference's order.  A view
// whose rays share one dominant in-plane axis and include no axis-parallel
// ray (the instance's view flags; a block-uniform branch) uses the
// axis-specialised chord.
template <bool kPlanar>
__global__ void __launch_bounds__(kAtxThreads, 4)
    k_sart_atx(const Inst *__restrict__ insts, int view, const int *__restrict__ zmap) {
  pdl_enter();
  const Inst &I = insts[zmap ? zmap[blockIdx.z] : blockIdx.z];
  if (view >= I.nv || ((volatile int *)&I.s->done)[0]) return;
  const Dims D = I.d;
  if (own_block(group_grid(D.nx, D.ny, D.nz, 1)).bid < 0) return;
  const ViewGeo G = view_of(I, view);
  const float4 *tabA = I.tabA + (long long)view * D.na;
  const int vf = I.vflags[view];
  const bool narrow = !(vf & kViewAxisParallel) && I.s->cor_finite &&
                      (!kPlanar || G.z_det[0] == 0.0f);
  if (kPlanar && narrow && I.chtab)
    sart_atx_tiles_tab(I, G, D, I.chtab + (size_t)view * chord_view_words(D, I.chK), I.chK);
  else if (!(vf & (kViewAxisParallel | kViewNotX)))
    sart_atx_tiles<kPlanar, 1>(I, G, D, tabA, narrow);
  else if (!(vf & (kViewAxisParallel | kViewNotY)))
    sart_atx_tiles<kPlanar, 2>(I, G, D, tabA, narrow);
  else
    sart_atx_tiles<kPlanar, 0>(I, G, D, tabA, narrow);
}

// ---------------------------------------------------------------------------
// Cone-beam backward step per voxel column (z-column form).  A thread owns a
// segment of kZSeg voxels of one (x, y) column and walks it down z.  What
// does not depend on z is computed once per segment (zcol_setup): the
// footprint window's columns and magnification, the shadow's columns and its
// corners' magnifications, and for each detector column of the shadow the
// in-plane part of the x and y face tests (col_faces, kept in shared memory,
// a thread reading only its own slots).  Each voxel then finds its rows
// (zcol_rows) and evaluates only the z parts of the face tests
// (chord3_col).  Pairs run as one sequence per voxel, rows outer (the
// reference's order), a warp walking its longest sequence; the voxels of a
// warp are 32 neighbours along x at the same z, so image reads and writes
// are coalesced.  Views that do not allow narrowing (an axis-parallel ray, a
// residual that is not finite) take the per-voxel form with the reference's
// whole window.  Columns whose shadow is wider than kZColA detector columns
// evaluate their chords from the ray tables (chord3_bf).
// Grid: (x tiles of 32, y tiles of 8 x segments, instances).
// ---------------------------------------------------------------------------
constexpr int kZSeg = 32;   // longest default segment: voxels of a column per thread
// Default segment for `voxels` voxels in a launch: the longest of 32, 16,
// 8, 4 that still gives the launch 2^21 threads (a few per SM slot).
// Measured on single volumes: 256^3 is fastest with 8 (0.566 ms against
// 0.639 with 32), 64^3 - 128^3 with 4 (64^3: 0.026 ms against 0.107).
__host__ __device__ inline int zcol_default_seg(long long voxels) {
  int seg = kZSeg;
  while (seg > 4 && voxels / seg < (1LL << 21)) seg /= 2;
  return seg;
}
constexpr int kZColA = 6;   // detector columns of a shadow kept per thread

struct ZColShared {
  float4 pts[kZColA][kAtxThreads];   // F1, F2 in-plane points
  float4 nh[kZColA][kAtxThreads];    // F1, F2 z-half terms (n1, h1, n2, h2)
  unsigned bits[kZColA][kAtxThreads];
};

// Grid of segments of `seg` voxels (a launch shape: the sums of a voxel do not
// depend on it).
__host__ __device__ inline dim3 zcol_grid(int nx, int ny, int nz, int batch,
                                          int seg = kZSeg) {
  return dim3((nx + kTileX - 1) / kTileX,
              ((ny + kTileY - 1) / kTileY) * ((nz + seg - 1) / seg), batch);
}

// This thread's column and segment [z0, z1) for an instance of sizes D;
// false when the block lies outside the instance's own grid.
__device__ __forceinline__ bool zcol_thread(const Dims &D, int seg, int &ix, int &iy,
                                            int &z0, int &z1) {
  const int ty = (D.ny + kTileY - 1) / kTileY, ns = (D.nz + seg - 1) / seg;
  if ((int)blockIdx.x * kTileX >= D.nx || (int)blockIdx.y >= ty * ns) return false;
  const int sg = blockIdx.y / ty, yt = blockIdx.y - sg * ty;
  ix = blockIdx.x * kTileX + threadIdx.x % kTileX;
  iy = yt * kTileY + threadIdx.x / kTileX;
  z0 = sg * seg;
  z1 = min(z0 + seg, D.nz);
  return true;
}

// Walks this thread's segment.  pair(r, l, on) takes the chord l of ray r
// (pairs in the reference's order; on == false for a lane past its own
// pairs), voxel(idx) ends a voxel; begin(idx) starts it (prefetches).
template <class Begin, class Pair, class Voxel>
__device__ __forceinline__ void atx_zcol_walk(const ViewGeo &G, const Dims &D,
                                              const float4 *__restrict__ tabA,
                                              const float4 *__restrict__ tabC,
                                              bool narrow, int ix, int iy, int z0, int z1,
                                              ZColShared &sh, Begin begin, Pair pair,
                                              Voxel voxel) {
  const bool valid = ix < D.nx && iy < D.ny;
  const float hz = G.dz / 2.0f;
  if (!narrow) {
    // the per-voxel form over the reference's window (no warp-wide steps)
    if (!valid) return;
    for (int iz = z0; iz < z1; iz++) {
      const unsigned idx = ((unsigned)iz * D.ny + iy) * D.nx + ix;
      if (!ASD_IN(idx, nvox(D))) continue;
      begin(idx);
      const VoxelWin w = voxel_window(G, D, ix, iy, iz);
      const float rx = G.cos_phi * (-G.SO) - w.xc, ry = G.sin_phi * (-G.SO) - w.yc;
      const float rz = 0.0f - w.zc;
      for (int ib = w.b0; ib <= w.b1; ib++) {
        const float c = (ASD_IN(ib, D.nb) ? __ldg(G.z_det + ib) : 0.f) - 0.0f;
        for (int ia = w.a0; ia <= w.a1; ia++) {
          const int r = ib * D.na + ia;
          if (!(ASD_IN(ia, D.na) && ASD_IN(r, nray(D)))) continue;
          pair(r, chord3_bf(__ldg(tabA + ia), __ldg(tabC + r), c, rx, ry, rz, G.dz), true);
        }
      }
      voxel(idx);
    }
    return;
  }
  const int t = threadIdx.x;
  ZCol col;
  int cntA = 0;
  bool wide = false;
  col.lo = 0;
  col.rx = col.ry = 0.f;
  if (valid) {
    col = zcol_setup(G, D, ix, iy, true);
    cntA = col.lo <= col.hi ? col.hi - col.lo + 1 : 0;
    wide = cntA > kZColA;
    if (!wide)
      for (int k = 0; k < cntA; k++) {
        if (!ASD_IN(col.lo + k, D.na)) continue;
        const ColFaces f = col_faces(__ldg(tabA + col.lo + k), col.rx, col.ry);
        sh.pts[k][t] = make_float4(f.p1x, f.p1y, f.p2x, f.p2y);
        sh.nh[k][t] = make_float4(f.n1, f.h1, f.n2, f.h2);
        sh.bits[k][t] = f.bits;
      }
  }
  for (int iz = z0; iz < z1; iz++) {
    const unsigned idx = ((unsigned)iz * D.ny + iy) * D.nx + ix;
    const bool vin = valid && ASD_IN(idx, nvox(D));
    if (vin) begin(idx);
    float zc = 0.f;
    int blo = 0, bhi = -1;
    const bool has = valid && zcol_rows(G, D, col, iz, zc, blo, bhi);
    const int cntB = has && blo <= bhi ? bhi - blo + 1 : 0;
    const int cnt = cntA * cntB;
    const int kN = __reduce_max_sync(0xffffffffu, cnt);
    const float rz = 0.0f - zc;
    int ka = 0, ib = blo;
    for (int k = 0; k < kN; k++) {
      const bool on = k < cnt;
      const int kk = on ? ka : 0;
      const int ia = on ? col.lo + ka : 0;
      const int r = (on ? ib : 0) * D.na + ia;
      const bool rin = ASD_IN(r, nray(D)) && ASD_IN(ia, D.na);
      const float4 Cs = rin ? __ldg(tabC + r) : make_float4(0.f, 0.f, 0.f, 0.f);
      float l;
      if (!wide) {
        const float4 p = sh.pts[kk][t], q = sh.nh[kk][t];
        const ColFaces f{p.x, p.y, p.z, p.w, q.x, q.y, q.z, q.w, sh.bits[kk][t]};
        if (f.bits & kCfMany)
          l = (f.bits & kCfXF) ? chord3_axis<true>(__ldg(tabA + ia), Cs, col.rx, col.ry, rz, G.dz)
                               : chord3_axis<false>(__ldg(tabA + ia), Cs, col.rx, col.ry, rz, G.dz);
        else
          l = chord3_col(f, Cs, col.rx, col.ry, rz, hz);
      } else {
        l = chord3_bf(__ldg(tabA + ia), Cs, 0.0f, col.rx, col.ry, rz, G.dz);
      }
      pair(r, l, on && rin);
      if (++ka == cntA) {
        ka = 0;
        ib++;
      }
    }
    if (vin) voxel(idx);
  }
}

// SART backward step of cone-beam instances (see k_sart_atx) in z columns.
__global__ void __launch_bounds__(kAtxThreads, 4)
    k_sart_atx_zcol(const Inst *__restrict__ insts, int view, int seg,
                    const int *__restrict__ zmap) {
  __shared__ ZColShared sh;
  pdl_enter();
  const Inst &I = insts[zmap ? zmap[blockIdx.z] : blockIdx.z];
  if (view >= I.nv || ((volatile int *)&I.s->done)[0]) return;
  const Dims D = I.d;
  int ix, iy, z0, z1;
  if (!zcol_thread(D, seg, ix, iy, z0, z1)) return;
  const ViewGeo G = view_of(I, view);
  const float4 *tabA = I.tabA + (long long)view * D.na;
  const bool narrow = !(I.vflags[view] & kViewAxisParallel) && I.s->cor_finite;
  const float beta = I.s->beta_f;
  float *m = I.m;
  const float *__restrict__ cor = I.cor;
  float acc = 0.f, accl = 0.f, mv = 0.f;
  atx_zcol_walk(
      G, D, tabA, I.tabC, narrow, ix, iy, z0, z1, sh,
      [&](unsigned idx) {
        mv = m[idx];
        acc = 0.f;
        accl = 0.f;
      },
      [&](int r, float l, bool on) {
        const float yv = on ? __ldg(cor + r) : 0.f;
        if (on) {
          acc += l * yv;
          accl += l;
        }
      },
      [&](unsigned idx) {
        const float bp = acc * G.scale, scv = accl * G.scale;
        const float mn = mv + beta * __fdividef(bp, scv == 0.f ? 1.f : scv);
        m[idx] = mn < 0.f ? 0.f : mn;
      });
}

// Ray tables of one view for the standalone backward step (launcher path):
// tabA[na], tabC[na*nb] and, in flag[0], whether the view forbids narrowing
// (flag[0] set unless every ray has both in-plane components, the bins lie
// on the uniform grid and every value is finite; flag[0] must be 0 before
// the launch).
__global__ void __launch_bounds__(256)
    k_view_tab3(const float *__restrict__ yv, float4 *tabA, float4 *tabC, int *flag,
                ViewGeo G, Dims D) {
  const long long nr = (long long)D.na * D.nb;
  const long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  bool ok = true;
  if (r < nr) {
    const int ia = (int)(r % D.na), ib = (int)(r / D.na);
    const float yd = G.y_det[ia], zd = G.z_det[ib];
    const float4 A = ray_tab_a(G, yd);
    if (ib == 0 && ASD_IN(ia, D.na)) tabA[ia] = A;
    if (ASD_IN(r, nr)) tabC[r] = ray_tab_c(A, zd);
    ok = A.x != 0.0f && A.y != 0.0f && on_grid(yd, ia, D.na, G.dy_det) &&
         on_grid(zd, ib, D.nb, G.dz_det) && isfinite(yv[r]) && G.dy_det > 0.0f &&
         G.dz_det > 0.0f;
  }
  if (!__all_sync(0xffffffffu, ok) && (threadIdx.x & 31) == 0) atomicOr(flag, 1);
}

// Standalone cone-beam backward step (Ax_cone_gpu.cu:214-271) in z columns,
// from the tables of k_view_tab3.
__global__ void __launch_bounds__(kAtxThreads, 4)
    k_atx_zcol(float *__restrict__ x, const float *__restrict__ yv, float *__restrict__ sc,
               const float4 *__restrict__ tabA, const float4 *__restrict__ tabC,
               const int *__restrict__ flag, ViewGeo G, Dims D, int seg) {
  __shared__ ZColShared sh;
  int ix, iy, z0, z1;
  if (!zcol_thread(D, seg, ix, iy, z0, z1)) return;
  const bool narrow = flag[0] == 0;
  float acc = 0.f, accl = 0.f;
  atx_zcol_walk(
      G, D, tabA, tabC, narrow, ix, iy, z0, z1, sh,
      [&](unsigned) {
        acc = 0.f;
        accl = 0.f;
      },
      [&](int r, float l, bool on) {
        const float v = on ? __ldg(yv + r) : 0.f;
        if (on) {
          acc += l * v;
          accl += l;
        }
      },
      [&](unsigned idx) {
        x[idx] = acc * G.scale;
        sc[idx] = accl * G.scale;
      });
}

// ---------------------------------------------------------------------------
// Shared-geometry backward step: when every instance of a plan has the same
// geometry and view angles, the chords of a (voxel, bin) pair are the same
// for all of them.  A block then handles one voxel tile for a group of
// kShareGroup instances: each lane computes the chords of its voxel's pairs
// once (kPairChunk at a time) and applies them to every instance of the
// group -- the backprojection becomes a sparse-matrix by dense-matrix
// product over the group.  Each instance accumulates its pairs in the
// reference's order, so the result is bit-identical to k_sart_atx.
// ---------------------------------------------------------------------------
constexpr int kShareGroup = kShareSlots;
// chords per round of the shared backward step's pair loop (1: 3 % faster
// than 2 for cone-beam groups, the same for fan beams)
constexpr int kPairChunk = 1;

// SART update of one voxel for the group (ASD_POCS_cuda.m:128-134):
// m += beta * (Atx(cor) * scale) / (sumC * scale), sumC == 0 -> 1, then
// positivity.  accl is the voxel's chord sum, acc[b] slot b's weighted sum.
__device__ __forceinline__ void atx_shared_apply(const ViewGeo &G, unsigned vi,
                                                 float accl, const float *acc,
                                                 unsigned active, int gn, float *m_il,
                                                 const float *s_beta) {
  const float scv = accl * G.scale;
  // the group's images, interleaved: kShareGroup / 4 float4 per voxel
  float4 *mg = (float4 *)m_il + (size_t)vi * (kShareGroup / 4);
#pragma unroll
  for (int q = 0; q < kShareGroup / 4; q++) {
    if (!((active >> (4 * q)) & 0xFu)) continue;
    float4 m4 = mg[q];
    float *mv = &m4.x;
#pragma unroll
    for (int j = 0; j < 4; j++) {
      const int b = 4 * q + j;
      if (b < gn && ((active >> b) & 1u)) {
        const float bp = acc[b] * G.scale;
        const float mn = mv[j] + s_beta[b] * __fdividef(bp, scv == 0.f ? 1.f : scv);
        mv[j] = mn < 0.f ? 0.f : mn;
      }
    }
    mg[q] = m4;
  }
}

// The voxel of this thread for the group (see k_sart_atx_shared).
template <bool kPlanar, int AX>
__device__ __forceinline__ void atx_shared_voxel(
    const ViewGeo &G, const Dims &D, const float4 *__restrict__ corg,
    const float4 *__restrict__ tabA, const float4 *__restrict__ tabC,
    bool planar_ok, bool narrow, unsigned active, int gn, float *m_il,
    const float *s_beta) {
  int ix, iy, iz;
  const bool valid = tile_voxel(D, ix, iy, iz);
  VoxelWin w;
  bool has = false;
  if (valid) {
    w = voxel_window(G, D, ix, iy, iz);
    has = w.a0 <= w.a1 && w.b0 <= w.b1;
  }
  float acc[kShareGroup];
#pragma unroll
  for (int b = 0; b < kShareGroup; b++) acc[b] = 0.f;
  float accl = 0.f;
  if (!planar_ok) {
    // planar kernel on a geometry with z_det != 0: direct per-pair form
    if (valid) {
      const float xs = G.cos_phi * (-G.SO), ys0 = G.sin_phi * (-G.SO);
      for (int ib = w.b0; ib <= w.b1; ib++)
        for (int ia = w.a0; ia <= w.a1; ia++) {
          const float yd_ = G.y_det[ia];
          const float l = chord3(xs, ys0, 0.0f, G.cos_phi * G.OD - G.sin_phi * yd_,
                                 G.sin_phi * G.OD + G.cos_phi * yd_, G.z_det[ib],
                                 G.dz, w.xc, w.yc, w.zc);
          accl += l;
          const long long r = (long long)ib * D.na + ia;
#pragma unroll
          for (int q = 0; q < kShareGroup / 4; q++) {
            if (!((active >> (4 * q)) & 0xFu)) continue;
            const float4 c4 = ASD_IN(r, nray(D)) ? __ldg(corg + r * (kShareGroup / 4) + q)
                                                 : make_float4(0.f, 0.f, 0.f, 0.f);
            acc[4 * q] += l * c4.x;
            acc[4 * q + 1] += l * c4.y;
            acc[4 * q + 2] += l * c4.z;
            acc[4 * q + 3] += l * c4.w;
          }
        }
    }
  } else {
    int lo = has ? w.a0 : 0, hi = has ? w.a1 : -1;
    int blo = has ? w.b0 : 0, bhi = has ? w.b1 : -1;
    if (narrow && has) {
      int slo, shi, tlo, thi;
      if (kPlanar ? shadow_bins(G, D, w.xc, w.yc, slo, shi)
                  : shadow_bins3(G, D, w.xc, w.yc, w.zc, slo, shi, tlo, thi)) {
        lo = max(lo, slo);
        hi = min(hi, shi);
        if (!kPlanar) {
          blo = max(blo, tlo);
          bhi = min(bhi, thi);
        }
      }
    }
    const int cntA = has && lo <= hi ? hi - lo + 1 : 0;
    const int cntB = has && blo <= bhi ? bhi - blo + 1 : 0;
    const int kA = __reduce_max_sync(0xffffffffu, cntA);
    const int kB =
        kPlanar ? (kA > 0 ? 1 : 0) : __reduce_max_sync(0xffffffffu, cntB);
    const float rx = G.cos_phi * (-G.SO) - (has ? w.xc : 0.f);
    const float ry = G.sin_phi * (-G.SO) - (has ? w.yc : 0.f);
    const float rz = 0.0f - (has ? w.zc : 0.f);
    for (int kb = 0; kb < kB; kb++) {
      const bool onb = kb < cntB;
      const int ib = blo + kb;
      const float c =
          kPlanar ? 0.0f : ((onb && ASD_IN(ib, D.nb)) ? __ldg(G.z_det + ib) : 1.0f) - 0.0f;
      const int row = onb ? ib * D.na : 0;
      for (int c0 = 0; c0 < kA; c0 += kPairChunk) {
        float l[kPairChunk];
        int idx[kPairChunk];
        bool on[kPairChunk];
#pragma unroll
        for (int j = 0; j < kPairChunk; j++) {
          const int ka = c0 + j;
          on[j] = onb && ka < cntA;
          const int ia = on[j] ? lo + ka : 0;
          idx[j] = row + ia;
          l[j] = 0.f;
          if (ka < kA) {  // warp-uniform
            const bool okr = ASD_IN(ia, D.na) && ASD_IN(row + ia, nray(D));
            const float4 A = okr ? __ldg(tabA + ia) : make_float4(1.f, 1.f, 1.f, 1.f);
            if (kPlanar)
              l[j] = chord_sel<AX>(A, rx, ry, G.dz);
            else if (AX == 0)
              l[j] = okr ? chord3_bf(A, __ldg(tabC + row + ia), c, rx, ry, rz, G.dz) : 0.f;
            else
              l[j] = okr ? chord3_axis<AX == 1>(A, __ldg(tabC + row + ia), rx, ry, rz, G.dz)
                         : 0.f;
          }
          if (on[j]) accl += l[j];
        }
#pragma unroll
        for (int j = 0; j < kPairChunk; j++) {
          if (on[j]) {
#pragma unroll
            for (int q = 0; q < kShareGroup / 4; q++) {
              // quads of the group with no running instance are skipped
              // (block-uniform); their accumulators are never read
              if (!((active >> (4 * q)) & 0xFu)) continue;
              const float4 c4 = ASD_IN(idx[j], nray(D))
                                    ? __ldg(corg + (long long)idx[j] * (kShareGroup / 4) + q)
                                    : make_float4(0.f, 0.f, 0.f, 0.f);
              acc[4 * q] += l[j] * c4.x;
              acc[4 * q + 1] += l[j] * c4.y;
              acc[4 * q + 2] += l[j] * c4.z;
              acc[4 * q + 3] += l[j] * c4.w;
            }
          }
        }
      }
    }
  }
  if (!valid) return;
  const unsigned vi = ((unsigned)iz * D.ny + iy) * D.nx + ix;
  if (!ASD_IN(vi, nvox(D))) return;
  atx_shared_apply(G, vi, accl, acc, active, gn, m_il, s_beta);
}

// Pairs of this voxel: the reference's window narrowed to the voxel's shadow.
template <int AX>
__device__ __forceinline__ void chords_voxel(const ViewGeo &G, const Dims &D,
                                             const float4 *__restrict__ tabA,
                                             bool valid, int ix, int iy, int K,
                                             int *tab, int *kmax) {
  const VoxelWin w = voxel_window(G, D, ix, iy, 0);
  const bool has = valid && w.a0 <= w.a1 && w.b0 <= w.b1;
  int lo = has ? w.a0 : 0, hi = has ? w.a1 : -1;
  if (has) {
    int slo, shi;
    if (shadow_bins(G, D, w.xc, w.yc, slo, shi)) {
      lo = max(lo, slo);
      hi = min(hi, shi);
    }
  }
  const int cnt = has && lo <= hi ? hi - lo + 1 : 0;
  if (K == 0) {  // counting pass
    const int m = __reduce_max_sync(0xffffffffu, cnt);
    if ((threadIdx.x & 31) == 0 && m > 0) atomicMax(kmax, m);
    return;
  }
  if (!valid) return;
  const size_t N = (size_t)D.nx * D.ny, vi = (size_t)iy * D.nx + ix;
  if (cnt > K) {  // cannot happen after the counting pass; the host drops the table
    atomicOr(kmax + 1, 1);
    return;
  }
  const float rx = G.cos_phi * (-G.SO) - w.xc;
  const float ry = G.sin_phi * (-G.SO) - w.yc;
  if (!ASD_IN(vi, N)) return;
  float *ch = (float *)(tab + 2 * N) + vi;
  float accl = 0.f;
  for (int ka = 0; ka < cnt; ka++) {
    if (!(ASD_IN(lo + ka, D.na) && ASD_IN(ka, K))) continue;
    const float l = chord_sel<AX>(__ldg(tabA + lo + ka), rx, ry, G.dz);
    accl += l;
    ch[(size_t)ka * N] = l;
  }
  tab[vi] = cnt ? (int)(((unsigned)cnt << 24) | (unsigned)(w.b0 * D.na + lo)) : 0;
  tab[N + vi] = __float_as_int(accl);
}

// Counting (K == 0: the largest pair count into kmax[0]) or filling pass over
// every view of the instance insts[0] (the first of instances sharing
// geometry, or one instance): grid (x tiles, y tiles, views).
__global__ void __launch_bounds__(kAtxThreads)
    k_atx_chords(const Inst *__restrict__ insts, int K, int *tabs, int *kmax) {
  const Inst &I0 = insts[0];
  const Dims D = I0.d;
  const int view = blockIdx.z;
  if (view >= I0.nv) return;
  const ViewGeo G = view_of(I0, view);
  const int vf = I0.vflags[view];
  if ((vf & kViewAxisParallel) || G.z_det[0] != 0.0f) return;  // no table
  int ix, iy, iz;
  const bool valid = tile_voxel(D, ix, iy, iz);  // the whole warp goes on
  const float4 *__restrict__ tabA = I0.tabA + (long long)view * D.na;
  int *tab = tabs ? tabs + (size_t)view * chord_view_words(D, K) : nullptr;
  if (!(vf & kViewNotX))
    chords_voxel<1>(G, D, tabA, valid, ix, iy, K, tab, kmax);
  else if (!(vf & kViewNotY))
    chords_voxel<2>(G, D, tabA, valid, ix, iy, K, tab, kmax);
  else
    chords_voxel<0>(G, D, tabA, valid, ix, iy, K, tab, kmax);
}

// The voxel of this thread for the group, from the view's chord table: the
// pairs, chords and accumulation order of atx_shared_voxel's narrow form,
// and its update (atx_shared_apply).  Everything that does not depend on the
// header -- the group's image values, the chord sum and the first
// kChordPre chord slots -- is loaded together up front, so a warp waits for
// DRAM once; the residuals it then reads are the view's few kB, in L1.
// (A kernel of its own for this path, 48 registers and 5 blocks per SM with
// the direct form out of line, measured 14 % slower: more long-scoreboard
// stalls, fewer L1 hits.)

__device__ __forceinline__ void atx_shared_voxel_tab(
    const ViewGeo &G, const Dims &D, const float4 *__restrict__ corg,
    const int *__restrict__ tab, int K, unsigned active, int gn, float *m_il,
    const float *s_beta) {
  int ix, iy, iz;
  const bool valid = tile_voxel(D, ix, iy, iz);
  const size_t N = (size_t)D.nx * D.ny;
  const unsigned vi = valid ? (unsigned)iy * D.nx + ix : 0u;
  const float *__restrict__ ch = (const float *)(tab + 2 * N) + vi;
  float4 *mg = (float4 *)m_il + (size_t)vi * (kShareGroup / 4);
  int h = 0;
  float accl = 0.f;
  float pre[kChordPre];
  float4 m4[kShareGroup / 4];
#pragma unroll
  for (int k = 0; k < kChordPre; k++) pre[k] = 0.f;
  if (valid && ASD_IN(vi, N)) {
    h = __ldg(tab + vi);
    accl = __int_as_float(__ldg(tab + N + vi));
#pragma unroll
    for (int k = 0; k < kChordPre; k++)
      if (k < K) pre[k] = __ldg(ch + (size_t)k * N);  // slot k < K exists
#pragma unroll
    for (int q = 0; q < kShareGroup / 4; q++)
      if ((active >> (4 * q)) & 0xFu) m4[q] = mg[q];
  }
  const int cnt = (int)((unsigned)h >> 24), first = h & 0xffffff;
  const int kA = __reduce_max_sync(0xffffffffu, cnt);
  float acc[kShareGroup];
#pragma unroll
  for (int b = 0; b < kShareGroup; b++) acc[b] = 0.f;
  auto pair = [&](int ka, float l) {
    const long long r = first + ka;
    if (!ASD_IN(r, nray(D))) return;
#pragma unroll
    for (int q = 0; q < kShareGroup / 4; q++) {
      if (!((active >> (4 * q)) & 0xFu)) continue;
      const float4 c4 = __ldg(corg + r * (kShareGroup / 4) + q);
      acc[4 * q] += l * c4.x;
      acc[4 * q + 1] += l * c4.y;
      acc[4 * q + 2] += l * c4.z;
      acc[4 * q + 3] += l * c4.w;
    }
  };
#pragma unroll
  for (int ka = 0; ka < kChordPre; ka++)
    if (ka < kA && ka < cnt) pair(ka, pre[ka]);
  for (int ka = kChordPre; ka < kA; ka++)
    if (ka < cnt && ASD_IN(ka, K)) pair(ka, __ldg(ch + (size_t)ka * N));
  if (!valid || !ASD_IN(vi, N)) return;
  // atx_shared_apply with the image values already loaded
  const float scv = accl * G.scale;
#pragma unroll
  for (int q = 0; q < kShareGroup / 4; q++) {
    if (!((active >> (4 * q)) & 0xFu)) continue;
    float *mv = &m4[q].x;
#pragma unroll
    for (int j = 0; j < 4; j++) {
      const int b = 4 * q + j;
      if (b < gn && ((active >> b) & 1u)) {
        const float bp = acc[b] * G.scale;
        const float mn = mv[j] + s_beta[b] * __fdividef(bp, scv == 0.f ? 1.f : scv);
        mv[j] = mn < 0.f ? 0.f : mn;
      }
    }
    mg[q] = m4[q];
  }
}

// 4 blocks per SM for fan beams; 5 for cone beams (measured 3 % faster at
// 128^3, 6 % slower for fan beams, whose extra spills cost more)
template <bool kPlanar>
__global__ void __launch_bounds__(kAtxThreads, kPlanar ? 4 : 5)
    k_sart_atx_shared(const Inst *__restrict__ insts, int batch, int view,
                      const int2 *__restrict__ gtab) {
  __shared__ float s_beta[kShareGroup];
  __shared__ unsigned s_active;
  __shared__ int s_finite;
  pdl_enter();
  const int g0 = gtab ? gtab[blockIdx.z].x : (int)blockIdx.z * kShareGroup;
  const int gn = gtab ? gtab[blockIdx.z].y : min(kShareGroup, batch - g0);
  if (threadIdx.x == 0) {
    s_active = 0u;
    s_finite = 1;
  }
  __syncthreads();
  if (threadIdx.x < gn) {
    const Inst &Ib = insts[g0 + threadIdx.x];
    const bool live = ((volatile int *)&Ib.s->done)[0] == 0;
    s_beta[threadIdx.x] = Ib.s->beta_f;
    if (live) {
      atomicOr(&s_active, 1u << threadIdx.x);
      if (!Ib.s->cor_finite) atomicAnd(&s_finite, 0);
    }
  }
  __syncthreads();
  const unsigned active = s_active;
  if (!active) return;
  const Inst &I0 = insts[g0];
  const Dims D = I0.d;  // every instance of a shared-geometry plan
  const ViewGeo G = view_of(I0, view);
  // the group's residuals, interleaved: ray r of slot b at corg[r*kShareGroup + b]
  const float4 *__restrict__ corg = (const float4 *)I0.cor;
  const float4 *__restrict__ tabA = I0.tabA + (long long)view * D.na;
  const float4 *__restrict__ tabC = I0.tabC;
  const int vf = I0.vflags[view];
  const bool planar_ok = !kPlanar || G.z_det[0] == 0.0f;
  const bool narrow = planar_ok && !(vf & kViewAxisParallel) && s_finite;
  if (kPlanar && narrow && I0.chtab)
    atx_shared_voxel_tab(G, D, corg, I0.chtab + (size_t)view * chord_view_words(D, I0.chK),
                         I0.chK, active, gn, I0.m_il, s_beta);
  else if (!(vf & (kViewAxisParallel | kViewNotX)))
    atx_shared_voxel<kPlanar, 1>(G, D, corg, tabA, tabC, planar_ok, narrow, active,
                                 gn, I0.m_il, s_beta);
  else if (!(vf & (kViewAxisParallel | kViewNotY)))
    atx_shared_voxel<kPlanar, 2>(G, D, corg, tabA, tabC, planar_ok, narrow, active,
                                 gn, I0.m_il, s_beta);
  else
    atx_shared_voxel<kPlanar, 0>(G, D, corg, tabA, tabC, planar_ok, narrow, active,
                                 gn, I0.m_il, s_beta);
}

// ---------------------------------------------------------------------------
// Shared-geometry forward step: one warp per ray for a group of kShareGroup
// instances.  The column march (cells and weights) is evaluated once per ray
// and each piece reads the group's voxel values with kShareGroup / 4 float4 loads
// from the interleaved images; every instance accumulates its pieces in the
// order of k_sart_ax and sums lanes with the same butterfly, and its block
// partials, reduction order and epilogue are those of k_sart_ax, so its
// projection, residual, dd2 and flags are bit-identical to it.
// ---------------------------------------------------------------------------
// columns per round of loads in the shared forward step: two for fan beams
// (measured 6 % faster than one); one for cone beams, whose three pieces per
// column already keep six loads in flight.  Blocks per SM: 6 for fan beams
// (72 registers, no spills), 8 for cone beams (64 registers: 10 % faster
// than 6 at 128^3).
template <bool k3D>
constexpr int kAxShareU = k3D ? 1 : 2;
// quads of a group (4 instances each) per block: one for fan beams (twice
// the warps, half the accumulators: measured 10 % faster), both for cone
// beams
template <bool k3D>
constexpr int kAxShareQ = k3D ? kShareGroup / 4 : 1;

// kU columns per round and kQ quads per block are launch shapes that a plan's
// autotuner may change (asdpocs_plan_autotune_shapes): neither changes the
// order in which an instance's pieces are added, so every shape gives the
// same bits.
template <bool k3D, int kU, int kQ>
__global__ void __launch_bounds__(kAxBlock, k3D ? 8 : 6)
    k_sart_ax_shared(const Inst *__restrict__ insts, int batch, int view,
                     const int2 *__restrict__ gtab) {
  constexpr int kQuads = kShareGroup / 4;
  pdl_enter();
  // this block: kQ of the group's quads (4 instances each), from q0
  constexpr int kS = 4 * kQ;
  __shared__ unsigned s_active;
  __shared__ float sp[kAxCols][kAxWarps][kS + 1][32];
  __shared__ float s_part[2][kAxWarps][kS];
  __shared__ int s_last[kS];
  __shared__ int s_nlast;
  const int q0 = (int)(blockIdx.z % (kQuads / kQ)) * kQ;
  const int gz = (int)(blockIdx.z / (kQuads / kQ));                  // the group
  const int g0 = gtab ? gtab[gz].x : gz * kShareGroup;
  const int gi = g0 + 4 * q0;                                        // first instance
  const int gn = min(kS, (gtab ? g0 + gtab[gz].y : batch) - gi);
  if (gn <= 0) return;
  const Inst &I0 = insts[g0];
  if (view >= I0.nv) return;
  const Dims D = I0.d;
  const long long nr = (long long)D.na * D.nb;
  const OwnBlock ob = own_block(dim3((unsigned)((nr + kAxWarps - 1) / kAxWarps), 1));
  if (ob.bid < 0) return;
  if (threadIdx.x == 0) {
    s_active = 0u;
    s_nlast = 0;
  }
  __syncthreads();
  if (threadIdx.x < gn &&
      ((volatile int *)&insts[gi + threadIdx.x].s->done)[0] == 0)
    atomicOr(&s_active, 1u << threadIdx.x);
  __syncthreads();
  const unsigned active = s_active;
  const ViewGeo G = view_of(I0, view);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int rw = warp % kAxWarps, part = warp / kAxWarps;
  const long long r = (long long)blockIdx.x * kAxWarps + rw;
  // cone beam: the plan's one ray-slope table, refreshed by group 0 every
  // view whether or not its instances still run
  if (k3D && blockIdx.z == 0 && part == 0 && lane == 0 && r < nr && ASD_IN(r, nr)) {
    const int ia = (int)(r % D.na), ib = (int)(r / D.na);
    I0.tabC[r] = ray_tab_c(I0.tabA[(long long)view * D.na + ia], G.z_det[ib]);
  }
  if (!active) return;
  float v[kS + 1];  // the instances' sums, then the weights' sum
#pragma unroll
  for (int b = 0; b <= kS; b++) v[b] = 0.f;
  const float4 *__restrict__ mg = (const float4 *)I0.m_il;
  if (r < nr) {
    const int ia = (int)(r % D.na), ib = (int)(r / D.na);
    const float zd = G.z_det[ib];
    const RayMarch R = ray_setup(G, D, G.y_det[ia], zd);
    const bool planar = D.nz == 1 && zd == 0.0f;
    // kU columns per round: their pieces first, then all their
    // (predicated) loads, then the accumulation in column and piece order
    auto march = [&](auto pieces) {
      constexpr int kP = decltype(pieces)::value;
      for (int iu0 = lane + 32 * part; iu0 < R.nu; iu0 += 32 * kAxCols * kU) {
        unsigned id[kU][kP];
        float w[kU][kP];
        bool f[kU][kP];
#pragma unroll
        for (int u = 0; u < kU; u++) {
          const int iu = iu0 + u * 32 * kAxCols;
          if constexpr (kP == 2)
            column_pieces_planar(R, iu, id[u], w[u], f[u]);
          else
            column_pieces3(R, iu, id[u], w[u], f[u]);
        }
        float4 x[kU][kP][kQ];
#pragma unroll
        for (int u = 0; u < kU; u++)
#pragma unroll
          for (int j = 0; j < kP; j++) {
            const float4 *p = mg + (size_t)id[u][j] * kQuads + q0;
            f[u][j] = f[u][j] && ASD_IN(id[u][j], nvox(D));
#pragma unroll
            for (int q = 0; q < kQ; q++)
              x[u][j][q] = (f[u][j] && ((active >> (4 * q)) & 0xFu))
                               ? __ldg(p + q)
                               : make_float4(0.f, 0.f, 0.f, 0.f);
          }
#pragma unroll
        for (int u = 0; u < kU; u++)
#pragma unroll
          for (int j = 0; j < kP; j++) {
            if (!f[u][j]) continue;
#pragma unroll
            for (int q = 0; q < kQ; q++) {
              v[4 * q] = weight_fma(w[u][j], x[u][j][q].x, v[4 * q]);
              v[4 * q + 1] = weight_fma(w[u][j], x[u][j][q].y, v[4 * q + 1]);
              v[4 * q + 2] = weight_fma(w[u][j], x[u][j][q].z, v[4 * q + 2]);
              v[4 * q + 3] = weight_fma(w[u][j], x[u][j][q].w, v[4 * q + 3]);
            }
            v[kS] += w[u][j];
          }
      }
    };
    // fan beams (nz == nb == 1: the one detector row at z = 0) are planar
    if (!k3D || planar)
      march(std::integral_constant<int, 2>());
    else if constexpr (k3D)
      march(std::integral_constant<int, 3>());
  }
  ax_combine<kS + 1>(sp, v, part, rw, lane);
  // part-0 lane b: the epilogue of k_sart_ax for instance gi + b
  float yb = 0.f;
#pragma unroll
  for (int b = 0; b < kS; b++)
    if (lane == b) yb = v[b];
  float p0 = 0.f, p1 = 0.f;
  if (part == 0 && lane < gn && ((active >> lane) & 1u) && r < nr) {
    const Inst &Ib = insts[gi + lane];
    const float yv = yb * G.scale, srv = v[kS] * G.scale;
    const long long pi = (long long)view * nr + r;
    const float c0 = (ASD_IN(pi, nr * Ib.nv) ? sino_at(Ib, pi) : 0.f) - yv;
    const float cr = c0 / (srv == 0.f ? 1.f : srv);
    if (ASD_IN(r, nr)) Ib.cor[r * Ib.cor_stride] = cr;
    p0 = c0 * c0;
    p1 = isfinite(cr) ? 0.f : 1.f;
  }
  if (part == 0 && lane < kS) {
    s_part[0][rw][lane] = p0;
    s_part[1][rw][lane] = p1;
  }
  __syncthreads();
  // per instance: the block total of k_sart_ax's block_sum_f (lane 0 of the
  // part-0 warps 0..3 the only nonzero values; combined as
  // (w0 + w2) + (w1 + w3)), its partial, its ticket
  static_assert(kAxWarps == 4, "block totals below follow block_sum_f for 4 warps");
  if (threadIdx.x < gn && ((active >> threadIdx.x) & 1u)) {
    const int b = threadIdx.x;
    const Inst &Ib = insts[gi + b];
#pragma unroll
    for (int k = 0; k < 2; k++) {
      const float t = (s_part[k][0][b] + s_part[k][2][b]) + (s_part[k][1][b] + s_part[k][3][b]);
      Ib.partials[(long long)ob.bid * 2 + k] = (double)t;
    }
    __threadfence();
    if (atomicAdd(Ib.counter, 1u) == (unsigned)ob.nblocks - 1)
      s_last[atomicAdd(&s_nlast, 1)] = b;
  }
  __syncthreads();
  const int nlast = s_nlast;
  if (nlast == 0) return;
  __threadfence();
  for (int i = 0; i < nlast; i++) {
    const Inst &Ib = insts[gi + s_last[i]];
    double tot[2];
    // the final sum of k_sart_ax's reduction (its kAxBlock threads' order)
    grid_sum_final<kAxBlock, 2>(Ib.partials, Ib.counter, ob.nblocks, tot);
    if (threadIdx.x == 0) {
      Ib.s->dd2_acc += tot[0];
      Ib.s->cor_finite = tot[1] == 0.0;
    }
  }
}

// Rounds an FP32 sinogram to FP16 / BF16 storage (round to nearest, ties to
// even: the same bits as asdpocs_store_sinogram on the host).
__global__ void __launch_bounds__(256)
    k_store_sinogram(const float *__restrict__ src, void *dst, long long n, int fmt) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    if (fmt == ASDPOCS_STORE_F16)
      ((__half *)dst)[i] = __float2half_rn(src[i]);
    else
      ((__nv_bfloat16 *)dst)[i] = __float2bfloat16_rn(src[i]);
  }
}

// Copies the running instances of each shared-geometry group between their
// own images (m) and the group's interleaved images (m_il): pack before the
// SART sweep, unpack after it.  Grid (voxel blocks, 1, groups).
__global__ void __launch_bounds__(256)
    k_group_pack(const Inst *__restrict__ insts, int batch, int unpack,
                 const int2 *__restrict__ gtab) {
  __shared__ float *s_m[kShareGroup];
  __shared__ unsigned s_active;
  pdl_enter();
  const int g0 = gtab ? gtab[blockIdx.z].x : (int)blockIdx.z * kShareGroup;
  const int gn = gtab ? gtab[blockIdx.z].y : min(kShareGroup, batch - g0);
  if (threadIdx.x == 0) s_active = 0u;
  __syncthreads();
  if (threadIdx.x < gn) {
    const Inst &Ib = insts[g0 + threadIdx.x];
    s_m[threadIdx.x] = Ib.m;
    if (((volatile int *)&Ib.s->done)[0] == 0) atomicOr(&s_active, 1u << threadIdx.x);
  }
  __syncthreads();
  const unsigned active = s_active;
  const Dims D = insts[g0].d;
  const long long n = (long long)D.nx * D.ny * D.nz;
  const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (!active || v >= n) return;
  float4 *mg = (float4 *)insts[g0].m_il + v * (kShareGroup / 4);
#pragma unroll
  for (int q = 0; q < kShareGroup / 4; q++) {
    if (!((active >> (4 * q)) & 0xFu)) continue;
    float4 x = unpack ? mg[q] : make_float4(0.f, 0.f, 0.f, 0.f);
    float *xv = &x.x;
#pragma unroll
    for (int j = 0; j < 4; j++) {
      const int b = 4 * q + j;
      if (b < gn && ((active >> b) & 1u)) {
        if (unpack)
          s_m[b][v] = xv[j];
        else
          xv[j] = s_m[b][v];
      }
    }
    if (!unpack) mg[q] = x;
  }
}

}  // namespace

cudaError_t launch_ax(const float *x, float *y, float *sr, const ViewGeo &g,
                      const Dims &d, cudaStream_t st) {
  const long long nr = (long long)d.na * d.nb;
  if (nr == 0) return cudaSuccess;
  const unsigned blocks = (unsigned)((nr + kAxWarps - 1) / kAxWarps);
  k_ax<<<blocks, kAxBlock, 0, st>>>(x, y, sr, g, d);
  return cudaGetLastError();
}

cudaError_t launch_atx(float *x, const float *y, float *sc, const ViewGeo &g,
                       const Dims &d, cudaStream_t st) {
  const dim3 grid = tile_grid(d.nx, d.ny, d.nz, 1);
  if (d.nz == 1 && d.nb == 1)
    k_atx<true><<<grid, kAtxThreads, 0, st>>>(x, y, sc, g, d);
  else
    k_atx<false><<<grid, kAtxThreads, 0, st>>>(x, y, sc, g, d);
  return cudaGetLastError();
}

cudaError_t launch_store_sinogram(const float *src, void *dst, size_t n, int fmt,
                                  cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  if (fmt == ASDPOCS_STORE_F32)
    return cudaMemcpyAsync(dst, src, n * 4, cudaMemcpyDeviceToDevice, st);
  const unsigned blocks = (unsigned)std::min<size_t>((n + 255) / 256, 152 * 64);
  k_store_sinogram<<<blocks, 256, 0, st>>>(src, dst, (long long)n, fmt);
  return cudaGetLastError();
}

size_t atx_zcol_scratch_bytes(const Dims &d) {
  const size_t a = ((size_t)d.na * sizeof(float4) + 255) & ~(size_t)255;
  const size_t c = ((size_t)d.na * d.nb * sizeof(float4) + 255) & ~(size_t)255;
  return a + c + 256;
}

cudaError_t launch_atx_zcol(float *x, const float *y, float *sc, const ViewGeo &g,
                            const Dims &d, void *scratch, cudaStream_t st) {
  char *b = (char *)scratch;
  float4 *tabA = (float4 *)b;
  float4 *tabC = (float4 *)(b + (((size_t)d.na * sizeof(float4) + 255) & ~(size_t)255));
  int *flag = (int *)(b + atx_zcol_scratch_bytes(d) - 256);
  cudaError_t e = cudaMemsetAsync(flag, 0, sizeof(int), st);
  if (e != cudaSuccess) return e;
  const long long nr = (long long)d.na * d.nb;
  k_view_tab3<<<(unsigned)((nr + 255) / 256), 256, 0, st>>>(y, tabA, tabC, flag, g, d);
  const int seg = zcol_default_seg((long long)d.nx * d.ny * d.nz);
  k_atx_zcol<<<zcol_grid(d.nx, d.ny, d.nz, 1, seg), kAtxThreads, 0, st>>>(x, y, sc, tabA,
                                                                          tabC, flag, g, d,
                                                                          seg);
  return cudaGetLastError();
}

cudaError_t launch_sart_ax(const Inst *insts, int batch, const Dims &d,
                           int view, cudaStream_t st, bool exact, const int *zmap) {
  cudaError_t e;
  const long long nr = (long long)d.na * d.nb;
  const unsigned blocks = (unsigned)((nr + kAxWarps - 1) / kAxWarps);
  const dim3 grid(blocks, 1, batch);
  const dim3 grid_ex((unsigned)((nr + kSidRays - 1) / kSidRays), 1, batch);
  const bool p3 = d.nz > 1 || d.nb > 1;
  if (exact) {
    if (p3)
      e = launch_iter(k_sart_ax_exact<true>, grid_ex, dim3(kAxBlock), st, insts, view, zmap);
    else
      e = launch_iter(k_sart_ax_exact<false>, grid_ex, dim3(kAxBlock), st, insts, view, zmap);
  } else {
    if (p3)
      e = launch_iter(k_sart_ax<true>, grid, dim3(kAxBlock), st, insts, view, zmap);
    else
      e = launch_iter(k_sart_ax<false>, grid, dim3(kAxBlock), st, insts, view, zmap);
  }
  return e;
}

cudaError_t launch_ax_siddon(const float *x, float *y, float *sr, const ViewGeo &g,
                             const Dims &d, cudaStream_t st) {
  const long long nr = (long long)d.na * d.nb;
  if (nr == 0) return cudaSuccess;
  k_ax_siddon<<<(unsigned)((nr + kSidRays - 1) / kSidRays), kAxBlock, 0, st>>>(x, y, sr, g,
                                                                                d);
  return cudaGetLastError();
}

cudaError_t launch_sart_atx(const Inst *insts, int batch, const Dims &d,
                            int view, cudaStream_t st, bool zcol, int zseg,
                            const int *zmap) {
  cudaError_t e;
  const dim3 grid = group_grid(d.nx, d.ny, d.nz, batch);
  zseg = zseg > 0 ? zseg : zcol_default_seg((long long)d.nx * d.ny * d.nz * batch);
  if (d.nz > 1 && zcol)
    e = launch_iter(k_sart_atx_zcol, zcol_grid(d.nx, d.ny, d.nz, batch, zseg),
                    dim3(kAtxThreads), st, insts, view, zseg, zmap);
  else if (d.nz > 1 || d.nb > 1)
    e = launch_iter(k_sart_atx<false>, grid, dim3(kAtxThreads), st, insts, view, zmap);
  else
    e = launch_iter(k_sart_atx<true>, grid, dim3(kAtxThreads), st, insts, view, zmap);
  return e;
}

cudaError_t launch_sart_atx_shared(const Inst *insts, int batch,
                                   const Dims &d, int view, cudaStream_t st,
                                   const int2 *gtab, int ngroups) {
  cudaError_t e;
  dim3 grid = tile_grid(d.nx, d.ny, d.nz, 1);
  grid.z = gtab ? ngroups : (batch + kShareGroup - 1) / kShareGroup;
  if (d.nz > 1 || d.nb > 1)
    e = launch_iter(k_sart_atx_shared<false>, grid, dim3(kAtxThreads), st, insts, batch,
                    view, gtab);
  else
    e = launch_iter(k_sart_atx_shared<true>, grid, dim3(kAtxThreads), st, insts, batch,
                    view, gtab);
  return e;
}

template <bool k3D, int kU, int kQ>
static cudaError_t sart_ax_shared_as(const Inst *insts, int batch, unsigned blocks,
                                     unsigned groups, int view, cudaStream_t st,
                                     const int2 *gtab) {
  return launch_iter(k_sart_ax_shared<k3D, kU, kQ>,
                     dim3(blocks, 1, groups * (kShareGroup / 4 / kQ)), dim3(kAxBlock), st,
                     insts, batch, view, gtab);
}

template <bool k3D>
static cudaError_t sart_ax_shared_shape(const Inst *insts, int batch, unsigned blocks,
                                        unsigned groups, int view, cudaStream_t st, int u,
                                        int q, const int2 *gtab) {
  u = u ? u : kAxShareU<k3D>;
  q = q ? q : kAxShareQ<k3D>;
  if (u == 1 && q == 1)
    return sart_ax_shared_as<k3D, 1, 1>(insts, batch, blocks, groups, view, st, gtab);
  if (u == 2 && q == 1)
    return sart_ax_shared_as<k3D, 2, 1>(insts, batch, blocks, groups, view, st, gtab);
  if (u == 1 && q == 2)
    return sart_ax_shared_as<k3D, 1, 2>(insts, batch, blocks, groups, view, st, gtab);
  if (u == 2 && q == 2)
    return sart_ax_shared_as<k3D, 2, 2>(insts, batch, blocks, groups, view, st, gtab);
  return cudaErrorInvalidValue;
}

cudaError_t launch_sart_ax_shared(const Inst *insts, int batch, const Dims &d,
                                  int view, cudaStream_t st, int u, int q,
                                  const int2 *gtab, int ngroups) {
  const long long nr = (long long)d.na * d.nb;
  const unsigned blocks = (unsigned)((nr + kAxWarps - 1) / kAxWarps);
  const unsigned groups =
      gtab ? (unsigned)ngroups : (unsigned)((batch + kShareGroup - 1) / kShareGroup);
  if (d.nz > 1 || d.nb > 1)
    return sart_ax_shared_shape<true>(insts, batch, blocks, groups, view, st, u, q, gtab);
  return sart_ax_shared_shape<false>(insts, batch, blocks, groups, view, st, u, q, gtab);
}

cudaError_t launch_group_pack(const Inst *insts, int batch, const Dims &d,
                              int unpack, cudaStream_t st, const int2 *gtab, int ngroups) {
  cudaError_t e;
  const long long n = (long long)d.nx * d.ny * d.nz;
  const dim3 grid((unsigned)((n + 255) / 256), 1,
                  gtab ? ngroups : (batch + kShareGroup - 1) / kShareGroup);
  e = launch_iter(k_group_pack, grid, dim3(256), st, insts, batch, unpack, gtab);
  return e;
}

cudaError_t launch_atx_chords(const Inst *insts, const Dims &d, int nv, int K,
                              int *tabs, int *kmax, cudaStream_t st) {
  if (K < 0 || K > kChordMaxSlots || (K > 0 && !tabs) || d.nz != 1 || d.nb != 1)
    return cudaErrorInvalidValue;
  dim3 grid = tile_grid(d.nx, d.ny, 1, nv);
  k_atx_chords<<<grid, kAtxThreads, 0, st>>>(insts, K, tabs, kmax);
  return cudaGetLastError();
}

size_t atx_chord_words(const Dims &d, int nv, int K) {
  return chord_view_words(d, K) * (size_t)nv;
}

int atx_chord_max_slots() { return kChordMaxSlots; }

cudaError_t launch_view_tables(const Inst *insts, int batch, const Dims &d,
                               int nv, cudaStream_t st) {
  k_view_tables<<<dim3((d.na + 127) / 128, nv, batch), 128, 0, st>>>(insts);
  return cudaGetLastError();
}

#ifdef ASDPOCS_CHECKED
ASD_CHECKED_READER(checked_take_proj)
#endif

int reduce_blocks_for(const Dims &d) {
  const long long nr = (long long)d.na * d.nb;
  const long long ax = (nr + kAxWarps - 1) / kAxWarps;
  const long long at = atx_blocks(d);
  return (int)(ax > at ? ax : at);
}

}  // namespace asd
