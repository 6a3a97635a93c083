// Device math of the ray-driven projector (Ax) and the voxel-driven
// backprojector (Atx).
//
// Parity contract: every float operation below is an IEEE single-precision
// operation in the same order as the reference expressions
// (src/AxAtx/Ax_cone_gpu.cu), and the translation units that include this
// file are compiled with -fmad=false, so nothing is contracted into a fused
// multiply-add.  Division and square root are the IEEE-rounded ones
// (-prec-div/-prec-sqrt default).  Per-ray/per-view quantities are hoisted
// out of the inner loops only where the hoisted value is bit-identical to
// the one the reference recomputes.
#pragma once
#include <math.h>
#include <string.h>

#include "common.cuh"

// Host+device: the same code also runs on the CPU in the host-side test of
// the device math (tests/device_math).
#define ASD_HD __host__ __device__ __forceinline__

namespace asd {

// a/b through the hardware reciprocal (within 2 ulp) in device code; the
// IEEE quotient in the host build of this header.
ASD_HD float fast_div(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fdividef(a, b);
#else
  return a / b;
#endif
}

// Forward-step weights and sums (never a branch decision): the hardware
// square root (sqrt.approx, within 2^-22 relative) and fused multiply-adds
// in device code; the IEEE square root and fmaf in the host build.
ASD_HD float weight_sqrt(float x) {
#ifdef __CUDA_ARCH__
  float r;
  asm("sqrt.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
#else
  return sqrtf(x);
#endif
}
ASD_HD float weight_fma(float a, float b, float c) {
#ifdef __CUDA_ARCH__
  return __fmaf_rn(a, b, c);
#else
  return fmaf(a, b, c);
#endif
}

// ---------------------------------------------------------------------------
// Ax: partial sums of one ray over the columns iu = first, first+step, ...
// (Ax_cone_gpu.cu:339-776).
//
// The ray is marched along its driving axis u (x when |dx|>|dy|, :372, else
// y, :573).  In each column it spans [v1,v2] across the in-plane transverse
// axis v and [w1,w2] in z (sorted by slope sign, :377-394).  The column
// length l (:402) is split at the v-crossing (fraction rv from v1) and at the
// z-crossing (fraction rz from w1); pieces are the overlaps of [0,rv],[rv,1]
// with [0,rz],[rz,1], added in position order.  The reference enumerates
// these overlaps as 16 explicit cases (:398-570); rows / slices that fall
// outside the volume lose their pieces under the same range tests
// (cy2==0 keeps only the upper row, cy2==ny only the lower one, ...).
// Indices the reference would read out of bounds (|slope|>1 in z, which it
// does not support) are skipped instead.
// ---------------------------------------------------------------------------
struct RayMarch {
  float us, vs, slope1, slope2, len2, dz2sq, dz;
  float lfac;  // (len2+dz2sq)/len2: column length factor (fast weights)
  int nu, nv, nz, nu2, nv2, nz2;
  unsigned su, sv, sz;  // memory strides of u, v and z (volumes < 2^31 voxels)
};

ASD_HD RayMarch ray_setup(const ViewGeo &G, const Dims &D,
                                              float ydet, float zdet) {
  RayMarch R;
  const float x1 = G.cos_phi * (-G.SO);
  const float y1 = G.sin_phi * (-G.SO);
  const float z1 = 0.0f;
  const float x2 = G.cos_phi * G.OD - G.sin_phi * ydet;
  const float y2 = G.sin_phi * G.OD + G.cos_phi * ydet;
  const float z2 = zdet;
  const bool xdrive = fabsf(x1 - x2) > fabsf(y1 - y2);
  const float du = xdrive ? (x2 - x1) : (y2 - y1);
  const float dv = xdrive ? (y2 - y1) : (x2 - x1);
  R.us = xdrive ? x1 : y1;
  R.vs = xdrive ? y1 : x1;
  R.slope1 = dv / du;
  R.slope2 = (z2 - z1) / du;
  R.len2 = (x1 - x2) * (x1 - x2) + (y1 - y2) * (y1 - y2);
  R.dz2sq = (z1 - z2) * (z1 - z2);
  R.dz = G.dz;
  R.nu = xdrive ? D.nx : D.ny;
  R.nv = xdrive ? D.ny : D.nx;
  R.nz = D.nz;
  R.nu2 = R.nu / 2;
  R.nv2 = R.nv / 2;
  R.nz2 = D.nz / 2;
  R.su = xdrive ? 1u : (unsigned)D.nx;
  R.sv = xdrive ? (unsigned)D.nx : 1u;
  R.sz = (unsigned)D.nx * (unsigned)D.ny;
  R.lfac = (R.len2 + R.dz2sq) / R.len2;
  return R;
}

// Adds the contributions of columns first, first+step, ... to (ys, ss).
// kExact = true evaluates every weight with the reference's expressions
// (bit-identical per column).  kExact = false (the kernels) keeps every
// branch decision identical -- cell indices and split tests use the same
// float expressions -- but forms the weights without IEEE divisions or
// square roots: the column length as sqrt(fma(d, d, 1) * lfac) (lfac =
// (len2+dz2sq)/len2 per ray) through the hardware square root and the split
// fractions through the hardware reciprocal, each within 2 ulp of the
// reference's value, and adds weight * voxel to the ray sum with one fused
// multiply-add.
template <bool kExact = true, class Loader>
ASD_HD void ray_columns(const RayMarch &R, int first,
                                            int step, Loader ld, float &ys,
                                            float &ss) {
  for (int iu = first; iu < R.nu; iu += step) {
    const float uu1 = (float)(iu - R.nu2);
    const float uu2 = uu1 + 1;
    float v1, v2, w1, w2;
    if (R.slope1 >= 0) {
      v1 = R.vs + R.slope1 * (uu1 - R.us) + R.nv2;
      v2 = R.vs + R.slope1 * (uu2 - R.us) + R.nv2;
    } else {
      v1 = R.vs + R.slope1 * (uu2 - R.us) + R.nv2;
      v2 = R.vs + R.slope1 * (uu1 - R.us) + R.nv2;
    }
    const int cv1 = (int)floorf(v1), cv2 = (int)floorf(v2);
    {
      const float q1 = 0.0f + R.slope2 * ((R.slope2 >= 0 ? uu1 : uu2) - R.us);
      const float q2 = 0.0f + R.slope2 * ((R.slope2 >= 0 ? uu2 : uu1) - R.us);
      // q/dz: with dz == 1 (every gateway call) the division is the identity
      w1 = (kExact || R.dz != 1.0f ? q1 / R.dz : q1) + R.nz2;
      w2 = (kExact || R.dz != 1.0f ? q2 / R.dz : q2) + R.nz2;
    }
    const int cz1 = (int)floorf(w1), cz2 = (int)floorf(w2);
    const bool vsplit = cv1 != cv2, zsplit = cz1 != cz2;
    bool vlo, vhi, zlo, zhi;
    if (!vsplit) {
      vlo = cv1 >= 0 && cv1 <= R.nv - 1;
      vhi = false;
    } else if (cv2 > 0 && cv2 < R.nv) {
      vlo = vhi = true;
    } else {
      vlo = cv2 == R.nv;
      vhi = cv2 == 0;
    }
    if (!zsplit) {
      zlo = cz1 >= 0 && cz1 <= R.nz - 1;
      zhi = false;
    } else if (cz2 > 0 && cz2 < R.nz) {
      zlo = zhi = true;
    } else {
      zlo = cz2 == R.nz;
      zhi = cz2 == 0;
    }
    vlo = vlo && cv1 >= 0 && cv1 < R.nv;
    vhi = vhi && cv2 >= 0 && cv2 < R.nv;
    zlo = zlo && cz1 >= 0 && cz1 < R.nz;
    zhi = zhi && cz2 >= 0 && cz2 < R.nz;
    if (!(vlo || vhi) || !(zlo || zhi)) continue;

    const float d = v2 - v1;
    const float l = kExact ? sqrtf((d * d + 1) * (R.len2 + R.dz2sq) / R.len2)
                           : weight_sqrt(weight_fma(d, d, 1.f) * R.lfac);
    const unsigned base = (unsigned)iu * R.su;
    const unsigned ilo = base + (unsigned)cv1 * R.sv;
    const unsigned ihi = base + (unsigned)cv2 * R.sv;
    const unsigned zl = (unsigned)cz1 * R.sz, zh = (unsigned)cz2 * R.sz;
#define ASD_PIECE(w, idx)                                   \
  do {                                                      \
    const float w_ = (w);                                   \
    ys = kExact ? ys + w_ * ld(idx) : weight_fma(w_, ld(idx), ys); \
    ss += w_;                                               \
  } while (0)
    if (!vsplit && !zsplit) {
      ASD_PIECE(l, ilo + zl);
    } else if (!vsplit) {
      const float rz = kExact ? (cz2 - w1) / (w2 - w1) : fast_div(cz2 - w1, w2 - w1);
      if (zlo) ASD_PIECE(rz * l, ilo + zl);
      if (zhi) ASD_PIECE((1 - rz) * l, ilo + zh);
    } else if (!zsplit) {
      const float rv = kExact ? (cv2 - v1) / d : fast_div(cv2 - v1, d);
      if (vlo) ASD_PIECE(rv * l, ilo + zl);
      if (vhi) ASD_PIECE((1 - rv) * l, ihi + zl);
    } else {
      const float rv = kExact ? (cv2 - v1) / d : fast_div(cv2 - v1, d);
      const float rz = kExact ? (cz2 - w1) / (w2 - w1) : fast_div(cz2 - w1, w2 - w1);
      if (rv > rz) {
        if (vlo && zlo) ASD_PIECE(rz * l, ilo + zl);
        if (vlo && zhi) ASD_PIECE((rv - rz) * l, ilo + zh);
        if (vhi && zhi) ASD_PIECE((1 - rv) * l, ihi + zh);
      } else {
        if (vlo && zlo) ASD_PIECE(rv * l, ilo + zl);
        if (vhi && zlo) ASD_PIECE((rz - rv) * l, ihi + zl);
        if (vhi && zhi) ASD_PIECE((1 - rz) * l, ihi + zh);
      }
    }
#undef ASD_PIECE
  }
}

// The kernels' form of ray_columns<false> (same cells, weights and
// accumulation order, so bit-identical to it): each column yields at most
// three pieces in position order (A, B, C) with their validity, evaluated
// without control flow; a group of U columns is evaluated first, its
// predicated loads are issued together, then the pieces are accumulated in
// order, so a lane keeps up to 3U loads in flight.
// The pieces of column iu for ray_columns_fast: at most three, in position
// order (A, B, C), with their validity, evaluated without control flow.
ASD_HD void column_pieces3(const RayMarch &R, int iu, unsigned (&id)[3],
                           float (&w)[3], bool (&f)[3]) {
  const bool pos1 = R.slope1 >= 0, pos2 = R.slope2 >= 0;
  const bool zdiv = R.dz != 1.0f;
  const float uu1 = (float)(iu - R.nu2);
  const float uu2 = uu1 + 1;
  const float ua = pos1 ? uu1 : uu2, ub = pos1 ? uu2 : uu1;
  const float v1 = R.vs + R.slope1 * (ua - R.us) + R.nv2;
  const float v2 = R.vs + R.slope1 * (ub - R.us) + R.nv2;
  const int cv1 = (int)floorf(v1), cv2 = (int)floorf(v2);
  const float q1 = 0.0f + R.slope2 * ((pos2 ? uu1 : uu2) - R.us);
  const float q2 = 0.0f + R.slope2 * ((pos2 ? uu2 : uu1) - R.us);
  const float w1 = (zdiv ? q1 / R.dz : q1) + R.nz2;
  const float w2 = (zdiv ? q2 / R.dz : q2) + R.nz2;
  const int cz1 = (int)floorf(w1), cz2 = (int)floorf(w2);
  const bool vs = cv1 != cv2, zs = cz1 != cz2;
  const bool vmid = cv2 > 0 && cv2 < R.nv, zmid = cz2 > 0 && cz2 < R.nz;
  const bool in = iu < R.nu;
  const bool vlo = in && (vs ? (vmid || cv2 == R.nv) : (cv1 >= 0 && cv1 <= R.nv - 1)) &&
                   cv1 >= 0 && cv1 < R.nv;
  const bool vhi = in && vs && (vmid || cv2 == 0) && cv2 >= 0 && cv2 < R.nv;
  const bool zlo = (zs ? (zmid || cz2 == R.nz) : (cz1 >= 0 && cz1 <= R.nz - 1)) &&
                   cz1 >= 0 && cz1 < R.nz;
  const bool zhi = zs && (zmid || cz2 == 0) && cz2 >= 0 && cz2 < R.nz;
  const float d = v2 - v1;
  const float l = weight_sqrt(weight_fma(d, d, 1.f) * R.lfac);
  const float rv = fast_div(cv2 - v1, d);
  const float rz = fast_div(cz2 - w1, w2 - w1);
  const unsigned base = (unsigned)iu * R.su;
  const unsigned ilo = base + (unsigned)cv1 * R.sv;
  const unsigned ihi = base + (unsigned)cv2 * R.sv;
  const unsigned zl = (unsigned)cz1 * R.sz, zh = (unsigned)cz2 * R.sz;
  const bool vfirst = !(rv > rz);  // both split: the v crossing comes first
  // piece A: from the column entry
  w[0] = !vs ? (zs ? rz * l : l) : (!zs ? rv * l : (vfirst ? rv : rz) * l);
  id[0] = ilo + zl;
  f[0] = vlo && zlo;
  // piece B
  w[1] = !vs ? (1 - rz) * l : (!zs ? (1 - rv) * l : (vfirst ? (rz - rv) : (rv - rz)) * l);
  id[1] = !vs ? ilo + zh : (!zs ? ihi + zl : (vfirst ? ihi + zl : ilo + zh));
  f[1] = !vs ? (zs && vlo && zhi)
             : (!zs ? (vhi && zlo) : (vfirst ? (vhi && zlo) : (vlo && zhi)));
  // piece C (both split)
  w[2] = (vfirst ? (1 - rz) : (1 - rv)) * l;
  id[2] = ihi + zh;
  f[2] = vs && zs && vhi && zhi;
}

// The kernels' form of ray_columns<false> (same cells, weights and
// accumulation order, so bit-identical to it): a group of U columns'
// pieces is evaluated first, its predicated loads are issued together, then
// the pieces are accumulated in order, so a lane keeps up to 3U loads in
// flight.
template <int U = 2, class Loader>
ASD_HD void ray_columns_fast(const RayMarch &R, int first, int step, Loader ld,
                             float &ys, float &ss) {
  for (int iu0 = first; iu0 < R.nu; iu0 += U * step) {
    float w[U][3], x[U][3];
    unsigned id[U][3];
    bool f[U][3];
#pragma unroll
    for (int k = 0; k < U; k++) column_pieces3(R, iu0 + k * step, id[k], w[k], f[k]);
#pragma unroll
    for (int k = 0; k < U; k++)
#pragma unroll
      for (int j = 0; j < 3; j++) x[k][j] = f[k][j] ? ld(id[k][j]) : 0.f;
#pragma unroll
    for (int k = 0; k < U; k++)
#pragma unroll
      for (int j = 0; j < 3; j++)
        if (f[k][j]) {
          ys = weight_fma(w[k][j], x[k][j], ys);
          ss += w[k][j];
        }
  }
}

// Planar case of ray_columns (nz == 1 and the ray in the plane z = 0, i.e.
// z_det == 0): slope2 is +-0, so every column has w1 = w2 = 0, slice 0 and
// len2 + dz2sq == len2; the z tests are dropped.  Bit-identical to the
// generic march for these rays.
template <bool kExact = true, class Loader>
ASD_HD void ray_columns_planar(const RayMarch &R, int first,
                                                   int step, Loader ld,
                                                   float &ys, float &ss) {
  for (int iu = first; iu < R.nu; iu += step) {
    const float uu1 = (float)(iu - R.nu2);
    const float uu2 = uu1 + 1;
    float v1, v2;
    if (R.slope1 >= 0) {
      v1 = R.vs + R.slope1 * (uu1 - R.us) + R.nv2;
      v2 = R.vs + R.slope1 * (uu2 - R.us) + R.nv2;
    } else {
      v1 = R.vs + R.slope1 * (uu2 - R.us) + R.nv2;
      v2 = R.vs + R.slope1 * (uu1 - R.us) + R.nv2;
    }
    const int cv1 = (int)floorf(v1), cv2 = (int)floorf(v2);
    const unsigned base = (unsigned)iu * R.su;
    const float d = v2 - v1;
    if (cv1 == cv2) {
      if (cv1 < 0 || cv1 > R.nv - 1) continue;
      const float l = kExact ? sqrtf((d * d + 1) * R.len2 / R.len2)
                             : weight_sqrt(weight_fma(d, d, 1.f));
      const float w = l;
      const float x = ld(base + (unsigned)cv1 * R.sv);
      ys = kExact ? ys + w * x : weight_fma(w, x, ys);
      ss += w;
    } else {
      bool vlo, vhi;
      if (cv2 > 0 && cv2 < R.nv) {
        vlo = vhi = true;
      } else {
        vlo = cv2 == R.nv;
        vhi = cv2 == 0;
      }
      vlo = vlo && cv1 >= 0 && cv1 < R.nv;
      vhi = vhi && cv2 >= 0 && cv2 < R.nv;
      if (!(vlo || vhi)) continue;
      const float l = kExact ? sqrtf((d * d + 1) * R.len2 / R.len2)
                             : weight_sqrt(weight_fma(d, d, 1.f));
      const float rv = kExact ? (cv2 - v1) / d : fast_div(cv2 - v1, d);
      if (vlo) {
        const float w = rv * l;
        const float x = ld(base + (unsigned)cv1 * R.sv);
        ys = kExact ? ys + w * x : weight_fma(w, x, ys);
        ss += w;
      }
      if (vhi) {
        const float w = (1 - rv) * l;
        const float x = ld(base + (unsigned)cv2 * R.sv);
        ys = kExact ? ys + w * x : weight_fma(w, x, ys);
        ss += w;
      }
    }
  }
}

// The kernels' form of ray_columns_planar<false>: the same cells, weights
// and accumulation order, computed without control flow.  Each column yields
// at most two pieces (lower and upper row) with their validity; a group of
// U columns is evaluated first, then its (predicated) loads are issued
// together, then the pieces are accumulated in order -- so a lane keeps 2U
// loads in flight instead of waiting on each column in turn.
// The pieces of column iu for ray_columns_planar_fast: the lower and the
// upper row, with their validity, evaluated without control flow.
ASD_HD void column_pieces_planar(const RayMarch &R, int iu, unsigned (&id)[2],
                                 float (&w)[2], bool (&f)[2]) {
  const bool pos = R.slope1 >= 0;
  const float uu1 = (float)(iu - R.nu2);
  const float uu2 = uu1 + 1;
  const float ua = pos ? uu1 : uu2, ub = pos ? uu2 : uu1;
  const float v1 = R.vs + R.slope1 * (ua - R.us) + R.nv2;
  const float v2 = R.vs + R.slope1 * (ub - R.us) + R.nv2;
  const int cv1 = (int)floorf(v1), cv2 = (int)floorf(v2);
  const bool split = cv1 != cv2;
  const bool mid = cv2 > 0 && cv2 < R.nv;
  const bool in = iu < R.nu;
  f[0] = in && cv1 >= 0 && cv1 < R.nv && (split ? (mid || cv2 == R.nv) : true);
  f[1] = in && split && cv2 >= 0 && cv2 < R.nv && (mid || cv2 == 0);
  const float d = v2 - v1;
  const float l = weight_sqrt(weight_fma(d, d, 1.f));
  const float rv = fast_div(cv2 - v1, d);
  w[0] = split ? rv * l : l;
  w[1] = (1 - rv) * l;
  const unsigned base = (unsigned)iu * R.su;
  id[0] = base + (unsigned)cv1 * R.sv;
  id[1] = base + (unsigned)cv2 * R.sv;
}

// The kernels' form of ray_columns_planar<false>: the same cells, weights
// and accumulation order, computed without control flow.  A group of U
// columns is evaluated first, then its (predicated) loads are issued
// together, then the pieces are accumulated in order -- so a lane keeps 2U
// loads in flight instead of waiting on each column in turn.
template <int U = 4, class Loader>
ASD_HD void ray_columns_planar_fast(const RayMarch &R, int first, int step,
                                    Loader ld, float &ys, float &ss) {
  for (int iu0 = first; iu0 < R.nu; iu0 += U * step) {
    float w[U][2], x[U][2];
    unsigned id[U][2];
    bool f[U][2];
#pragma unroll
    for (int k = 0; k < U; k++) column_pieces_planar(R, iu0 + k * step, id[k], w[k], f[k]);
#pragma unroll
    for (int k = 0; k < U; k++)
#pragma unroll
      for (int j = 0; j < 2; j++) x[k][j] = f[k][j] ? ld(id[k][j]) : 0.f;
#pragma unroll
    for (int k = 0; k < U; k++)
#pragma unroll
      for (int j = 0; j < 2; j++)
        if (f[k][j]) {
          ys = weight_fma(w[k][j], x[k][j], ys);
          ss += w[k][j];
        }
  }
}

// ---------------------------------------------------------------------------
// Exact forward projection (Siddon's method): the intersection length of the
// ray with every voxel it crosses, not the reference's column march (whose
// 3-D splits approximate them; its 2-D march is already exact).  The ray runs
// from the source to the bin centre in voxel units; the volume spans
// [-(n/2), n - n/2) along x and y and [-(nz/2), nz - nz/2) * dz along z.
// The lanes of a warp share the ray's columns along its dominant in-plane
// axis u.  Per ray (FP64, as an FP64 Siddon reference computes it): the
// in-volume parameter range and, for the other axes, their position (in
// cells) at the start of each column as a line in the column index.  Per
// lane the positions at its columns' starts advance in double-single FP32
// pairs (two-sum), so the loop has no FP64 arithmetic; inside a column
// everything is FP32 in a local coordinate s in [0, 1] along u: the planes
// of the other axes are crossed at (m - f) / k, the segments between
// crossings lie in the cell of their midpoint, and a segment's length is
// its s-extent times the ray's length per unit of u.  The two columns where
// the ray enters and leaves the volume clip s in FP64.  Lengths and sums are
// FP32.  Fan beams (nz == nb == 1) are traced in the plane (two axes).
// ---------------------------------------------------------------------------
// A value as an unevaluated sum hi + lo of two floats (about 48 bits).
struct DSFloat {
  float hi, lo;
};

ASD_HD DSFloat ds_from(double x) {
  DSFloat r;
  r.hi = (float)x;
  r.lo = (float)(x - (double)r.hi);
  return r;
}

// a * k for a small integer k (|k| < 2^16): the high product's rounding error
// recovered exactly by a fused multiply-add.
ASD_HD DSFloat ds_mul_int(DSFloat a, int k) {
  const float kf = (float)k;
  const float p = a.hi * kf;
#ifdef __CUDA_ARCH__
  const float e = __fmaf_rn(a.hi, kf, -p);
#else
  const float e = fmaf(a.hi, kf, -p);
#endif
  DSFloat r;
  const float t = e + a.lo * kf;
  r.hi = p + t;
  r.lo = t - (r.hi - p);
  return r;
}

// a + b, both double-single (Knuth's two-sum on the high parts, then one
// renormalisation); exact to about 2^-44 relative.
ASD_HD DSFloat ds_add(DSFloat a, DSFloat b) {
  const float s = a.hi + b.hi;
  const float bb = s - a.hi;
  const float e = (a.hi - (s - bb)) + (b.hi - bb);
  const float t = (a.lo + b.lo) + e;
  DSFloat r;
  r.hi = s + t;
  r.lo = t - (r.hi - s);
  return r;
}

struct SidRay {
  // the dominant in-plane axis u and the other axes (in-plane, then z):
  // positions in cells along the ray as lines in the u cell coordinate,
  // pos_k(u) = pos0[k] + u * r[k] (double-single); the in-volume u range
  // [ua, ub] and the columns [full0, full1) wholly inside it
  DSFloat pos0[2], r[2], ua, ub;
  float Lu;   // ray length per cell of u
  int du, nax, nu, n_ax[2], full0, full1;
  unsigned su, sv, sz;  // memory strides of u, the other in-plane axis and z
  bool hit;
};

ASD_HD SidRay siddon_setup(const ViewGeo &G, const Dims &D, float ydet, float zdet) {
  SidRay s;
  const bool planar = D.nz == 1 && D.nb == 1;
  s.nax = planar ? 1 : 2;
  const double p0[3] = {(double)G.cos_phi * -(double)G.SO, (double)G.sin_phi * -(double)G.SO,
                        0.0};
  const double p1[3] = {(double)G.cos_phi * G.OD - (double)G.sin_phi * ydet,
                        (double)G.sin_phi * G.OD + (double)G.cos_phi * ydet,
                        planar ? 0.0 : (double)zdet};
  const double d0 = p1[0] - p0[0], d1 = p1[1] - p0[1], d2 = planar ? 0.0 : p1[2] - p0[2];
  const bool yu = fabs(d0) < fabs(d1);
  s.du = yu ? 1 : 0;
  const double du = yu ? d1 : d0, p0u = yu ? p0[1] : p0[0];
  const double lou = (double)(0 - (yu ? D.ny : D.nx) / 2);
  s.nu = yu ? D.ny : D.nx;
  s.hit = du != 0.0;
  const double rdu = s.hit ? 1.0 / du : 0.0;
  // t (0 at the source, 1 at the bin) as a line in u: the ray segment
  const double ut0 = p0u - lou, ut1 = p0u + du - lou;
  double ua = fmax(0.0, fmin(ut0, ut1)), ub = fmin((double)s.nu, fmax(ut0, ut1));
  const double dk[2] = {yu ? d0 : d1, d2};
  const double p0k[2] = {yu ? p0[0] : p0[1], 0.0};
  const double lok[2] = {(double)(0 - (yu ? D.nx : D.ny) / 2), (double)(0 - D.nz / 2) * G.dz};
  const double hk[2] = {1.0, G.dz};
  s.n_ax[0] = yu ? D.nx : D.ny;
  s.n_ax[1] = D.nz;
  double pos0d[2] = {0.0, 0.0}, rd[2] = {0.0, 0.0};
#pragma unroll
  for (int a = 0; a < 2; a++) {
    if (a >= s.nax || !s.hit) continue;
    double r = dk[a] * rdu, q = (p0k[a] + (lou - p0u) * r - lok[a]);
    if (hk[a] != 1.0) {
      r /= hk[a];
      q /= hk[a];
    }
    pos0d[a] = q;
    rd[a] = r;
    // where the line leaves [0, n] of this axis
    if (r != 0.0) {
      const double ir = 1.0 / r;
      const double e0 = (0.0 - q) * ir, e1 = ((double)s.n_ax[a] - q) * ir;
      ua = fmax(ua, fmin(e0, e1));
      ub = fmin(ub, fmax(e0, e1));
    } else if (q < 0.0 || q > (double)s.n_ax[a]) {
      s.hit = false;
    }
  }
#pragma unroll
  for (int a = 0; a < 2; a++) {
    s.pos0[a] = ds_from(pos0d[a]);
    s.r[a] = ds_from(rd[a]);
  }
  s.hit = s.hit && ub > ua;
  s.ua = ds_from(s.hit ? ua : 0.0);
  s.ub = ds_from(s.hit ? ub : 0.0);
  s.full0 = s.hit ? (int)ceil(ua) : 0;
  s.full1 = s.hit ? (int)floor(ub) : 0;
  // the length per cell of u, in FP32 (a relative error of ~1e-7)
  const float fd0 = (float)d0, fd1 = (float)d1, fd2 = (float)d2;
  s.Lu = sqrtf(fd0 * fd0 + fd1 * fd1 + fd2 * fd2) / fabsf((float)du);
  const unsigned nx = (unsigned)D.nx;
  s.su = yu ? nx : 1u;
  s.sv = yu ? 1u : nx;
  s.sz = nx * (unsigned)D.ny;
  return s;
}

// Adds the exact segments of columns first, first + step, ... of ray R's
// dominant axis to (ys, ss): ys += l * x[voxel], ss += l, l in FP32.
template <class Loader>
ASD_HD void siddon_columns(const SidRay &R, int first, int step, Loader ld, float &ys,
                           float &ss) {
  if (!R.hit || first >= R.nu) return;
  const int nax = R.nax;
  const int full0 = R.full0, full1 = R.full1;  // columns [full0, full1) wholly inside
  DSFloat pos[2], inc[2];
  float kf[2], ikf[2];
#pragma unroll
  for (int a = 0; a < 2; a++) {
    pos[a].hi = pos[a].lo = inc[a].hi = inc[a].lo = 0.f;
    kf[a] = ikf[a] = 0.f;
    if (a < nax) {
      pos[a] = ds_add(R.pos0[a], ds_mul_int(R.r[a], first));
      inc[a] = ds_mul_int(R.r[a], step);
      kf[a] = R.r[a].hi;
      ikf[a] = kf[a] != 0.f ? 1.0f / kf[a] : 0.f;
    }
  }
  const float Lu = R.Lu;
  const unsigned su = R.su, sv = R.sv, sz = R.sz;
  const int guard_max = 2 * (R.nu + R.n_ax[0] + R.n_ax[1]) + 8;
  for (int iu = first; iu < R.nu; iu += step) {
    // the column's in-volume s range
    float s0 = 0.f, s1 = 1.f;
    if (iu < full0 || iu + 1 > full1) {  // the ray enters or leaves here
      s0 = fmaxf(0.f, (R.ua.hi - (float)iu) + R.ua.lo);
      s1 = fminf(1.f, (R.ub.hi - (float)iu) + R.ub.lo);
    }
    // cells and fractions at s = 0, the next plane crossed after s0
    int cell[2] = {0, 0}, m[2] = {0, 0}, sg[2] = {0, 0};
    float f[2] = {0.f, 0.f}, sn[2] = {3.0e38f, 3.0e38f};
#pragma unroll
    for (int a = 0; a < 2; a++) {
      if (a >= nax) continue;
      const float c = floorf(pos[a].hi);
      float fr = (pos[a].hi - c) + pos[a].lo;
      int ci = (int)c;
      if (fr >= 1.f) {
        fr -= 1.f;
        ci += 1;
      } else if (fr < 0.f) {
        fr += 1.f;
        ci -= 1;
      }
      cell[a] = ci;
      f[a] = fr;
      if (kf[a] != 0.f) {
        sg[a] = kf[a] > 0.f ? 1 : -1;
        const float pp = fr + s0 * kf[a];
        int mm = sg[a] > 0 ? (int)floorf(pp) + 1 : (int)ceilf(pp) - 1;
        float t = ((float)mm - fr) * ikf[a];
        for (int g = 0; g < 2 && t <= s0; g++) {  // rounding: plane at or behind s0
          mm += sg[a];
          t = ((float)mm - fr) * ikf[a];
        }
        m[a] = mm;
        sn[a] = t;
      }
      pos[a] = ds_add(pos[a], inc[a]);
    }
    // merge walk over the crossings inside [s0, s1]
    float s = s0;
    for (int guard = 0; s < s1 && guard < guard_max; guard++) {
      const float t = fminf(s1, fminf(sn[0], sn[1]));
      if (t > s) {
        const float mid = 0.5f * (s + t);
        bool in = true;
        unsigned idx = (unsigned)iu * su;
#pragma unroll
        for (int a = 0; a < 2; a++) {
          if (a >= nax) continue;
          const int c = cell[a] + (int)floorf(f[a] + mid * kf[a]);
          in = in && c >= 0 && c < R.n_ax[a];
          idx += (unsigned)c * (a == 0 ? sv : sz);
        }
        if (in) {
          const float l = (t - s) * Lu;
          ys += l * ld(idx);
          ss += l;
        }
      }
#pragma unroll
      for (int a = 0; a < 2; a++)
        if (a < nax && sn[a] == t) {
          m[a] += sg[a];
          sn[a] = ((float)m[a] - f[a]) * ikf[a];
        }
      s = t;
    }
  }
}

// Warp-wide sum; the xor butterfly leaves bit-identical totals in every lane
// (IEEE addition is commutative).
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// ---------------------------------------------------------------------------
// Atx: chord length of a line through one voxel (find_l / find_l_3d,
// Ax_cone_gpu.cu:16-209).  The line starts at the source; (rx,ry,rz) is the
// source minus the voxel centre.  Faces normal to the dominant in-plane axis
// are tested first (x,y,z when |a|>|b|, else y,x,z), each pair lower face
// then upper face; the first two boundary points found define the chord.
// Comparisons with NaN/inf (c == 0 in 2D) are false, as in the reference.
// ---------------------------------------------------------------------------
struct Hits {
  int n;
  float p0x, p0y, p0z, p1x, p1y, p1z;
};

ASD_HD void add_hit(Hits &h, float a, float b, float c) {
  if (h.n == 0) {
    h.p0x = a;
    h.p0y = b;
    h.p0z = c;
    h.n = 1;
  } else if (h.n == 1) {
    h.p1x = a;
    h.p1y = b;
    h.p1z = c;
    h.n = 2;
  }
}

// find_l: line (p1,q1)->(p2,q2) and a (dp x dq) box centred at (pc,qc).
ASD_HD float chord2(float p1, float q1, float p2, float q2,
                                        float dp, float dq, float pc,
                                        float qc) {
  const float a = p2 - p1, b = q2 - q1;
  const float hp = dp / 2.0f, hq = dq / 2.0f;
  if (a == 0) return fabsf(p1 - pc) <= hp ? dq : 0.0f;
  if (b == 0) return fabsf(q1 - qc) <= hq ? dp : 0.0f;
  const float rp = p1 - pc, rq = q1 - qc;
  Hits h;
  h.n = 0;
  const bool pfirst = fabsf(a) > fabsf(b);
#pragma unroll
  for (int pass = 0; pass < 2; pass++) {
    if (h.n >= 2) break;
    if ((pass == 0) == pfirst) {
      const float s = b / a;
      const float t = s * (-rp) + rq, u = s * hp;
      if (fabsf(t - u) <= hq) add_hit(h, -hp, t - u, 0.f);
      if (fabsf(t + u) <= hq) add_hit(h, hp, t + u, 0.f);
    } else {
      const float s = a / b;
      const float t = s * (-rq) + rp, u = s * hq;
      if (fabsf(t - u) <= hp) add_hit(h, t - u, -hq, 0.f);
      if (fabsf(t + u) <= hp) add_hit(h, t + u, hq, 0.f);
    }
  }
  if (h.n < 2) return 0.0f;
  const float e0 = h.p1x - h.p0x, e1 = h.p1y - h.p0y;
  return sqrtf(e0 * e0 + e1 * e1);
}

// find_l_3d with unit x/y voxel size and z size dz.
ASD_HD float chord3(float x1, float y1, float z1, float x2,
                                        float y2, float z2, float dz, float xc,
                                        float yc, float zc) {
  const float a = x2 - x1, b = y2 - y1, c = z2 - z1;
  const float hx = 1.0f / 2.0f, hy = 1.0f / 2.0f, hz = dz / 2.0f;
  if (a == 0) return chord2(y1, z1, y2, z2, 1.0f, dz, yc, zc);
  if (b == 0) return chord2(x1, z1, x2, z2, 1.0f, dz, xc, zc);
  const float rx = x1 - xc, ry = y1 - yc, rz = z1 - zc;
  const bool xfirst = fabsf(a) > fabsf(b);
  Hits h;
  h.n = 0;
#pragma unroll
  for (int pass = 0; pass < 3; pass++) {
    if (h.n >= 2) break;
    const int axis = pass == 2 ? 2 : (((pass == 0) == xfirst) ? 0 : 1);
    if (axis == 0) {
      float s = b / a;
      const float t0 = s * (-rx) + ry, u0 = s * hx;
      s = c / a;
      const float t1 = s * (-rx) + rz, u1 = s * hx;
      if (fabsf(t0 - u0) <= hy && fabsf(t1 - u1) <= hz)
        add_hit(h, -hx, t0 - u0, t1 - u1);
      if (fabsf(t0 + u0) <= hy && fabsf(t1 + u1) <= hz)
        add_hit(h, hx, t0 + u0, t1 + u1);
    } else if (axis == 1) {
      float s = a / b;
      const float t0 = s * (-ry) + rx, u0 = s * hy;
      s = c / b;
      const float t1 = s * (-ry) + rz, u1 = s * hy;
      if (fabsf(t0 - u0) <= hx && fabsf(t1 - u1) <= hz)
        add_hit(h, t0 - u0, -hy, t1 - u1);
      if (fabsf(t0 + u0) <= hx && fabsf(t1 + u1) <= hz)
        add_hit(h, t0 + u0, hy, t1 + u1);
    } else {
      float s = a / c;
      const float t0 = s * (-rz) + rx, u0 = s * hz;
      s = b / c;
      const float t1 = s * (-rz) + ry, u1 = s * hz;
      if (fabsf(t0 - u0) <= hx && fabsf(t1 - u1) <= hy)
        add_hit(h, t0 - u0, t1 - u1, -hz);
      if (fabsf(t0 + u0) <= hx && fabsf(t1 + u1) <= hy)
        add_hit(h, t0 + u0, t1 + u1, hz);
    }
  }
  if (h.n < 2) return 0.0f;
  const float e0 = h.p1x - h.p0x, e1 = h.p1y - h.p0y, e2 = h.p1z - h.p0z;
  return sqrtf(e0 * e0 + e1 * e1 + e2 * e2);
}

// Per-voxel footprint of Atx (Ax_cone_gpu.cu:230-253).
struct VoxelWin {
  float xc, yc, zc;
  int a0, a1, b0, b1;
};

ASD_HD VoxelWin voxel_window(const ViewGeo &G,
                                                 const Dims &D, int ix, int iy,
                                                 int iz) {
  VoxelWin w;
  const float SD = G.SD;   // SO + OD
  const int na2 = D.na / 2, nb2 = D.nb / 2;
  const int nx2 = D.nx / 2, ny2 = D.ny / 2, nz2 = D.nz / 2;
  const float d = G.dwin;  // sqrtf((1 + dz*dz)/2)
  // (float)(i + 0.5 - n2) is evaluated in double by the reference; for
  // |i - n2| < 2^22 the float form below is the same exactly-representable
  // value and avoids FP64 arithmetic (slow on this GPU).
  w.zc = ((float)(iz - nz2) + 0.5f) * G.dz;
  w.yc = (float)(iy - ny2) + 0.5f;
  w.xc = (float)(ix - nx2) + 0.5f;
  const float xr = G.cos_phi * w.xc + G.sin_phi * w.yc;
  const float yr = -G.sin_phi * w.xc + G.cos_phi * w.yc;
  float t = SD / ((xr + G.SO) * G.dy_det);
  const int amax = (int)floorf((yr + 1) * t + na2);
  const int amin = (int)floorf((yr - 1) * t + na2);
  // same expression with dz_det (== dy_det in every gateway call, where the
  // division need not be repeated)
  if (G.dz_det != G.dy_det) t = SD / ((xr + G.SO) * G.dz_det);
  const int bmax = (int)floorf((w.zc + d) * t + nb2);
  const int bmin = (int)floorf((w.zc - d) * t + nb2);
  w.a0 = amin > 0 ? amin : 0;
  w.a1 = amax < D.na - 1 ? amax : D.na - 1;
  w.b0 = bmin > 0 ? bmin : 0;
  w.b1 = bmax < D.nb - 1 ? bmax : D.nb - 1;
  return w;
}

// ---------------------------------------------------------------------------
// Shadows.  A ray that misses a voxel box by more than the rounding of the
// face tests of find_l / find_l_3d (about 1e-4 voxel widths at these
// distances) has no face hit, so its chord is exactly 0.  On a detector with
// uniform bins (y_det[i] = (i - na/2 + 0.5) * dy_det, z_det likewise, as every
// gateway call has) the rays that can meet the box are those whose bin
// centres lie inside the bounding rectangle of the projections of the box's
// corners; the functions below return that rectangle widened by 0.05 bin
// (0.02-0.05 voxel widths at the voxel in these geometries), so every bin they
// drop has a chord of exactly 0 -- provided no ray is axis-parallel (the
// reference's chord ignores one coordinate there) and the view values are
// finite (0 * inf is not 0).  The column of a point depends on its in-plane
// position only, so the columns come from the four corners of the pixel; the
// rows from all eight corners.  They return false (no narrowing) when a
// corner is not in front of the source.
// ---------------------------------------------------------------------------
ASD_HD float hd_rcp(float x) {
#ifdef __CUDA_ARCH__
  return __frcp_rn(x);
#else
  return 1.0f / x;
#endif
}

// Detector coordinate v of bin i on the uniform grid (i - n/2 + 0.5) * pitch,
// to 1e-3 bin (the shadows' 0.05-bin margin absorbs that).
ASD_HD bool on_grid(float v, int i, int n, float pitch) {
  return fabsf(v - ((float)i - n * 0.5f + 0.5f) * pitch) <= 1e-3f * pitch;
}

ASD_HD bool shadow_bins(const ViewGeo &G, const Dims &D, float xc, float yc,
                        int &lo, int &hi) {
  const float xr = G.cos_phi * xc + G.sin_phi * yc;
  const float yr = -G.sin_phi * xc + G.cos_phi * yc;
  const float hc = 0.5f * G.cos_phi, hs = 0.5f * G.sin_phi;
  const float inv_det = hd_rcp(G.dy_det);
  const float off = D.na * 0.5f - 0.5f;
  float fmin = 3.0e38f, fmax = -3.0e38f;
  bool ok = true;
#pragma unroll
  for (int k = 0; k < 4; k++) {
    const float ex = (k & 1) ? 1.f : -1.f, ey = (k & 2) ? 1.f : -1.f;
    const float px = xr + ex * hc + ey * hs;  // rotated corner
    const float py = yr - ex * hs + ey * hc;
    const float den = px + G.SO;
    ok = ok && den > 1e-3f;
    const float f = fast_div(py * G.SD, den) * inv_det + off;
    fmin = fminf(fmin, f);
    fmax = fmaxf(fmax, f);
  }
  lo = (int)ceilf(fmin - 0.05f);
  hi = (int)floorf(fmax + 0.05f);
  return ok;
}

ASD_HD bool shadow_bins3(const ViewGeo &G, const Dims &D, float xc, float yc,
                         float zc, int &alo, int &ahi, int &blo, int &bhi) {
  const float xr = G.cos_phi * xc + G.sin_phi * yc;
  const float yr = -G.sin_phi * xc + G.cos_phi * yc;
  const float hc = 0.5f * G.cos_phi, hs = 0.5f * G.sin_phi;
  const float inv_a = hd_rcp(G.dy_det), inv_b = hd_rcp(G.dz_det);
  const float offa = D.na * 0.5f - 0.5f, offb = D.nb * 0.5f - 0.5f;
  const float hz = 0.5f * G.dz;
  const float zlo = (zc - hz) * inv_b, zhi = (zc + hz) * inv_b;
  float umin = 3.0e38f, umax = -3.0e38f, vmin = 3.0e38f, vmax = -3.0e38f;
  bool ok = true;
#pragma unroll
  for (int k = 0; k < 4; k++) {
    const float ex = (k & 1) ? 1.f : -1.f, ey = (k & 2) ? 1.f : -1.f;
    const float px = xr + ex * hc + ey * hs;
    const float py = yr - ex * hs + ey * hc;
    const float den = px + G.SO;
    ok = ok && den > 1e-3f;
    const float q = fast_div(G.SD, den);  // magnification at this corner
    const float u = py * q * inv_a + offa;
    const float v0 = zlo * q + offb, v1 = zhi * q + offb;
    umin = fminf(umin, u);
    umax = fmaxf(umax, u);
    vmin = fminf(vmin, fminf(v0, v1));
    vmax = fmaxf(vmax, fmaxf(v0, v1));
  }
  alo = (int)ceilf(umin - 0.05f);
  ahi = (int)floorf(umax + 0.05f);
  blo = (int)ceilf(vmin - 0.05f);
  bhi = (int)floorf(vmax + 0.05f);
  return ok;
}

// Sums l*y and l over the voxel's footprint (reference loop order: ib outer,
// ia inner; Ax_cone_gpu.cu:255-269).
template <class YLoad>
ASD_HD void voxel_backproject(const ViewGeo &G,
                                                  const Dims &D,
                                                  const VoxelWin &w, YLoad yl,
                                                  float &acc, float &accl) {
  const float xs = G.cos_phi * (-G.SO), ys = G.sin_phi * (-G.SO), zs = 0.0f;
  for (int ib = w.b0; ib <= w.b1; ib++) {
    const float zd = G.z_det[ib];
    for (int ia = w.a0; ia <= w.a1; ia++) {
      const float yd_ = G.y_det[ia];
      const float xd = G.cos_phi * G.OD - G.sin_phi * yd_;
      const float ydd = G.sin_phi * G.OD + G.cos_phi * yd_;
      const float l = chord3(xs, ys, zs, xd, ydd, zd, G.dz, w.xc, w.yc, w.zc);
      acc += l * yl((long long)ib * D.na + ia);
      accl += l;
    }
  }
}

// ---------------------------------------------------------------------------
// Per-view ray tables for Atx.  The slopes find_l_3d divides out for every
// (voxel, bin) pair depend on the ray only; they are computed once per ray
// with the same float operations and reused:
//   RayA (per detector column ia):  a = x2-x1, b = y2-y1, b/a, a/b
//   RayC (per ray (ia, ib), 3D):    c/a, c/b, a/c, b/c  with c = z2 - z1
// ---------------------------------------------------------------------------
ASD_HD float4 ray_tab_a(const ViewGeo &G, float ydet) {
  const float x1 = G.cos_phi * (-G.SO), y1 = G.sin_phi * (-G.SO);
  const float x2 = G.cos_phi * G.OD - G.sin_phi * ydet;
  const float y2 = G.sin_phi * G.OD + G.cos_phi * ydet;
  const float a = x2 - x1, b = y2 - y1;
  return make_float4(a, b, b / a, a / b);
}

ASD_HD float4 ray_tab_c(const float4 A, float zdet) {
  const float c = zdet - 0.0f;
  return make_float4(c / A.x, c / A.y, A.x / c, A.y / c);
}

// find_l on line direction (a, b) with precomputed b/a, a/b, relative start
// (rp, rq) = start - box centre, half sizes (hp, hq), full sizes (dp, dq).
ASD_HD float chord2_rel(float a, float b, float sba,
                                            float sab, float rp, float rq,
                                            float hp, float hq, float dp,
                                            float dq) {
  if (a == 0) return fabsf(rp) <= hp ? dq : 0.0f;
  if (b == 0) return fabsf(rq) <= hq ? dp : 0.0f;
  Hits h;
  h.n = 0;
  const bool pfirst = fabsf(a) > fabsf(b);
#pragma unroll
  for (int pass = 0; pass < 2; pass++) {
    if (h.n >= 2) break;
    if ((pass == 0) == pfirst) {
      const float t = sba * (-rp) + rq, u = sba * hp;
      if (fabsf(t - u) <= hq) add_hit(h, -hp, t - u, 0.f);
      if (fabsf(t + u) <= hq) add_hit(h, hp, t + u, 0.f);
    } else {
      const float t = sab * (-rq) + rp, u = sab * hq;
      if (fabsf(t - u) <= hp) add_hit(h, t - u, -hq, 0.f);
      if (fabsf(t + u) <= hp) add_hit(h, t + u, hq, 0.f);
    }
  }
  if (h.n < 2) return 0.0f;
  const float e0 = h.p1x - h.p0x, e1 = h.p1y - h.p0y;
  return sqrtf(e0 * e0 + e1 * e1);
}

// find_l_3d from the tables; (rx, ry, rz) = source - voxel centre.
ASD_HD float chord3_tab(const float4 A, const float4 Cs,
                                           float c, float rx, float ry,
                                           float rz, float dz) {
  const float a = A.x, b = A.y;
  const float hx = 0.5f, hy = 0.5f, hz = dz / 2.0f;
  if (a == 0) return chord2_rel(b, c, Cs.y, Cs.w, ry, rz, 0.5f, hz, 1.0f, dz);
  if (b == 0) return chord2_rel(a, c, Cs.x, Cs.z, rx, rz, 0.5f, hz, 1.0f, dz);
  const bool xfirst = fabsf(a) > fabsf(b);
  Hits h;
  h.n = 0;
#pragma unroll
  for (int pass = 0; pass < 3; pass++) {
    if (h.n >= 2) break;
    const int axis = pass == 2 ? 2 : (((pass == 0) == xfirst) ? 0 : 1);
    if (axis == 0) {
      const float t0 = A.z * (-rx) + ry, u0 = A.z * hx;
      const float t1 = Cs.x * (-rx) + rz, u1 = Cs.x * hx;
      if (fabsf(t0 - u0) <= hy && fabsf(t1 - u1) <= hz)
        add_hit(h, -hx, t0 - u0, t1 - u1);
      if (fabsf(t0 + u0) <= hy && fabsf(t1 + u1) <= hz)
        add_hit(h, hx, t0 + u0, t1 + u1);
    } else if (axis == 1) {
      const float t0 = A.w * (-ry) + rx, u0 = A.w * hy;
      const float t1 = Cs.y * (-ry) + rz, u1 = Cs.y * hy;
      if (fabsf(t0 - u0) <= hx && fabsf(t1 - u1) <= hz)
        add_hit(h, t0 - u0, -hy, t1 - u1);
      if (fabsf(t0 + u0) <= hx && fabsf(t1 + u1) <= hz)
        add_hit(h, t0 + u0, hy, t1 + u1);
    } else {
      const float t0 = Cs.z * (-rz) + rx, u0 = Cs.z * hz;
      const float t1 = Cs.w * (-rz) + ry, u1 = Cs.w * hz;
      if (fabsf(t0 - u0) <= hx && fabsf(t1 - u1) <= hy)
        add_hit(h, t0 - u0, t1 - u1, -hz);
      if (fabsf(t0 + u0) <= hx && fabsf(t1 + u1) <= hy)
        add_hit(h, t0 + u0, t1 + u1, hz);
    }
  }
  if (h.n < 2) return 0.0f;
  const float e0 = h.p1x - h.p0x, e1 = h.p1y - h.p0y, e2 = h.p1z - h.p0z;
  return sqrtf(e0 * e0 + e1 * e1 + e2 * e2);
}

// find_l_3d for a planar geometry (nz == 1, nb == 1, z_det == 0): c == 0, the
// z tests of the x/y faces always pass (|rz| == dz/2), the z faces never
// match (their slopes are infinite) and every hit has z == rz, so the chord
// is the in-plane one.  Lines with a == 0 or b == 0 fall back to the (y,z) or
// (x,z) chord, which is the full voxel width (1) in this geometry.
ASD_HD float chord_planar(const float4 A, float rx,
                                             float ry, float dz) {
  const float a = A.x, b = A.y;
  if (a == 0) return b == 0 ? (fabsf(ry) <= 0.5f ? dz : 0.0f) : 1.0f;
  if (b == 0) return 1.0f;
  Hits h;
  h.n = 0;
  const bool xfirst = fabsf(a) > fabsf(b);
#pragma unroll
  for (int pass = 0; pass < 2; pass++) {
    if (h.n >= 2) break;
    if ((pass == 0) == xfirst) {
      const float t = A.z * (-rx) + ry, u = A.z * 0.5f;
      if (fabsf(t - u) <= 0.5f) add_hit(h, -0.5f, t - u, 0.f);
      if (fabsf(t + u) <= 0.5f) add_hit(h, 0.5f, t + u, 0.f);
    } else {
      const float t = A.w * (-ry) + rx, u = A.w * 0.5f;
      if (fabsf(t - u) <= 0.5f) add_hit(h, t - u, -0.5f, 0.f);
      if (fabsf(t + u) <= 0.5f) add_hit(h, t + u, 0.5f, 0.f);
    }
  }
  if (h.n < 2) return 0.0f;
  const float e0 = h.p1x - h.p0x, e1 = h.p1y - h.p0y;
  return sqrtf(e0 * e0 + e1 * e1);
}

// ---------------------------------------------------------------------------
// Branch-free forms for the kernels.  The reference tests the faces in a
// fixed order and keeps the first two points that pass; evaluating every
// candidate (the tests have no side effects) and selecting the first two
// valid ones in that order gives the same chord, without the divergent
// early exits that serialise a warp whose lanes see different rays.
// ---------------------------------------------------------------------------
// The reference's "first two face hits in face order", chosen from the last
// face to the first: a hit face becomes the first point and pushes the
// previous first to second, so after all six faces p0, p1 are the first two
// hits in order -- six selects per face and no ordering counter (n counts
// the hits).  Measured 1.6 % faster than taking the faces in order with a
// counter on the cone-beam backward step.
struct Pick2Rev {
  int n;
  float p0x, p0y, p0z, p1x, p1y, p1z;
  ASD_HD void put(bool f, float x, float y, float z) {
    p1x = f ? p0x : p1x;
    p1y = f ? p0y : p1y;
    p1z = f ? p0z : p1z;
    p0x = f ? x : p0x;
    p0y = f ? y : p0y;
    p0z = f ? z : p0z;
    n += f ? 1 : 0;
  }
};

// chord_planar without divergent control flow (same result).  The faces are
// relabelled so the dominant in-plane axis comes first ("primary", tested
// first by the reference) and the other second; the chord is then
//   both primary faces hit -> primary-  to primary+,
//   one primary face hit   -> that point to the first secondary face hit,
//   none                   -> secondary- to secondary+,
// which is the reference's "first two hits" rule for a convex pixel.  Every
// point coordinate is the same float expression as in the reference, and the
// squared length is a sum of the same two terms (in swapped order when y is
// primary, which does not change an IEEE sum).
ASD_HD float chord_planar_bf(const float4 A, float rx, float ry, float dz) {
  const float a = A.x, b = A.y;
  const bool xfirst = fabsf(a) > fabsf(b);
  const float s1 = xfirst ? A.z : A.w, s2 = xfirst ? A.w : A.z;
  const float r1 = xfirst ? rx : ry, r2 = xfirst ? ry : rx;
  const float t1 = s1 * (-r1) + r2, u1 = s1 * 0.5f;
  const float t2 = s2 * (-r2) + r1, u2 = s2 * 0.5f;
  const float pm = t1 - u1, pp = t1 + u1;  // primary faces, at -0.5 / +0.5
  const float sm = t2 - u2, sp = t2 + u2;  // secondary faces
  const bool fpm = fabsf(pm) <= 0.5f, fpp = fabsf(pp) <= 0.5f;
  const bool fsm = fabsf(sm) <= 0.5f, fsp = fabsf(sp) <= 0.5f;
  float e1, e2;
  bool ok;
  if (fpm && fpp) {
    e1 = 1.0f;  // 0.5 - (-0.5)
    e2 = pp - pm;
    ok = true;
  } else if (fpm || fpp) {
    const float p0a = fpm ? -0.5f : 0.5f, p0b = fpm ? pm : pp;
    const float q1a = fsm ? sm : sp, q1b = fsm ? -0.5f : 0.5f;
    e1 = q1a - p0a;
    e2 = q1b - p0b;
    ok = fsm || fsp;
  } else {
    e1 = sp - sm;
    e2 = 1.0f;
    ok = fsm && fsp;
  }
  const float l = ok ? sqrtf(e1 * e1 + e2 * e2) : 0.0f;
  if (a == 0) return b == 0 ? (fabsf(ry) <= 0.5f ? dz : 0.0f) : 1.0f;
  if (b == 0) return 1.0f;
  return l;
}

// chord_planar_bf for a ray known to have a != 0, b != 0 and the given
// dominant axis (XF: |a| > |b|): the same expressions without the selects.
template <bool XF>
ASD_HD float chord_planar_axis(const float4 A, float rx, float ry) {
  const float s1 = XF ? A.z : A.w, s2 = XF ? A.w : A.z;
  const float r1 = XF ? rx : ry, r2 = XF ? ry : rx;
  const float t1 = s1 * (-r1) + r2, u1 = s1 * 0.5f;
  const float t2 = s2 * (-r2) + r1, u2 = s2 * 0.5f;
  const float pm = t1 - u1, pp = t1 + u1;
  const float sm = t2 - u2, sp = t2 + u2;
  const bool fpm = fabsf(pm) <= 0.5f, fpp = fabsf(pp) <= 0.5f;
  const bool fsm = fabsf(sm) <= 0.5f, fsp = fabsf(sp) <= 0.5f;
  float e1, e2;
  bool ok;
  if (fpm && fpp) {
    e1 = 1.0f;
    e2 = pp - pm;
    ok = true;
  } else if (fpm || fpp) {
    const float p0a = fpm ? -0.5f : 0.5f, p0b = fpm ? pm : pp;
    const float q1a = fsm ? sm : sp, q1b = fsm ? -0.5f : 0.5f;
    e1 = q1a - p0a;
    e2 = q1b - p0b;
    ok = fsm || fsp;
  } else {
    e1 = sp - sm;
    e2 = 1.0f;
    ok = fsm && fsp;
  }
  return ok ? sqrtf(e1 * e1 + e2 * e2) : 0.0f;
}

// chord3_tab without divergent control flow in the common case (the a == 0
// or b == 0 fallbacks keep their branch; they need an axis-aligned ray).
ASD_HD float chord3_bf(const float4 A, const float4 Cs, float c, float rx,
                       float ry, float rz, float dz) {
  const float a = A.x, b = A.y;
  const float hz = dz / 2.0f;
  if (a == 0) return chord2_rel(b, c, Cs.y, Cs.w, ry, rz, 0.5f, hz, 1.0f, dz);
  if (b == 0) return chord2_rel(a, c, Cs.x, Cs.z, rx, rz, 0.5f, hz, 1.0f, dz);
  // x faces
  const float xt0 = A.z * (-rx) + ry, xu0 = A.z * 0.5f;
  const float xt1 = Cs.x * (-rx) + rz, xu1 = Cs.x * 0.5f;
  const float xmy = xt0 - xu0, xmz = xt1 - xu1, xpy = xt0 + xu0, xpz = xt1 + xu1;
  const bool fxm = fabsf(xmy) <= 0.5f && fabsf(xmz) <= hz;
  const bool fxp = fabsf(xpy) <= 0.5f && fabsf(xpz) <= hz;
  // y faces
  const float yt0 = A.w * (-ry) + rx, yu0 = A.w * 0.5f;
  const float yt1 = Cs.y * (-ry) + rz, yu1 = Cs.y * 0.5f;
  const float ymx = yt0 - yu0, ymz = yt1 - yu1, ypx = yt0 + yu0, ypz = yt1 + yu1;
  const bool fym = fabsf(ymx) <= 0.5f && fabsf(ymz) <= hz;
  const bool fyp = fabsf(ypx) <= 0.5f && fabsf(ypz) <= hz;
  // z faces
  const float zt0 = Cs.z * (-rz) + rx, zu0 = Cs.z * hz;
  const float zt1 = Cs.w * (-rz) + ry, zu1 = Cs.w * hz;
  const float zmx = zt0 - zu0, zmy = zt1 - zu1, zpx = zt0 + zu0, zpy = zt1 + zu1;
  const bool fzm = fabsf(zmx) <= 0.5f && fabsf(zmy) <= 0.5f;
  const bool fzp = fabsf(zpx) <= 0.5f && fabsf(zpy) <= 0.5f;
  const bool xfirst = fabsf(a) > fabsf(b);
  // faces in the reference's order (x-, x+, y-, y+ or y-, y+, x-, x+; then
  // z-, z+), taken from the last
  Pick2Rev p;
  p.n = 0;
  p.p0x = p.p0y = p.p0z = p.p1x = p.p1y = p.p1z = 0.f;
  p.put(fzp, zpx, zpy, hz);
  p.put(fzm, zmx, zmy, -hz);
  if (xfirst) {
    p.put(fyp, ypx, 0.5f, ypz);
    p.put(fym, ymx, -0.5f, ymz);
    p.put(fxp, 0.5f, xpy, xpz);
    p.put(fxm, -0.5f, xmy, xmz);
  } else {
    p.put(fxp, 0.5f, xpy, xpz);
    p.put(fxm, -0.5f, xmy, xmz);
    p.put(fyp, ypx, 0.5f, ypz);
    p.put(fym, ymx, -0.5f, ymz);
  }
  if (p.n < 2) return 0.0f;
  const float e0 = p.p1x - p.p0x, e1 = p.p1y - p.p0y, e2 = p.p1z - p.p0z;
  return sqrtf(e0 * e0 + e1 * e1 + e2 * e2);
}

// chord3_bf for a ray known to have a != 0, b != 0 and the given dominant
// in-plane axis (XF: |a| > |b|): the same expressions, face order fixed.
template <bool XF>
ASD_HD float chord3_axis(const float4 A, const float4 Cs, float rx, float ry,
                         float rz, float dz) {
  const float hz = dz / 2.0f;
  const float xt0 = A.z * (-rx) + ry, xu0 = A.z * 0.5f;
  const float xt1 = Cs.x * (-rx) + rz, xu1 = Cs.x * 0.5f;
  const float xmy = xt0 - xu0, xmz = xt1 - xu1, xpy = xt0 + xu0, xpz = xt1 + xu1;
  const bool fxm = fabsf(xmy) <= 0.5f && fabsf(xmz) <= hz;
  const bool fxp = fabsf(xpy) <= 0.5f && fabsf(xpz) <= hz;
  const float yt0 = A.w * (-ry) + rx, yu0 = A.w * 0.5f;
  const float yt1 = Cs.y * (-ry) + rz, yu1 = Cs.y * 0.5f;
  const float ymx = yt0 - yu0, ymz = yt1 - yu1, ypx = yt0 + yu0, ypz = yt1 + yu1;
  const bool fym = fabsf(ymx) <= 0.5f && fabsf(ymz) <= hz;
  const bool fyp = fabsf(ypx) <= 0.5f && fabsf(ypz) <= hz;
  const float zt0 = Cs.z * (-rz) + rx, zu0 = Cs.z * hz;
  const float zt1 = Cs.w * (-rz) + ry, zu1 = Cs.w * hz;
  const float zmx = zt0 - zu0, zmy = zt1 - zu1, zpx = zt0 + zu0, zpy = zt1 + zu1;
  const bool fzm = fabsf(zmx) <= 0.5f && fabsf(zmy) <= 0.5f;
  const bool fzp = fabsf(zpx) <= 0.5f && fabsf(zpy) <= 0.5f;
  // faces in the reference's order (x-, x+, y-, y+ or y-, y+, x-, x+; then
  // z-, z+), taken from the last
  Pick2Rev p;
  p.n = 0;
  p.p0x = p.p0y = p.p0z = p.p1x = p.p1y = p.p1z = 0.f;
  p.put(fzp, zpx, zpy, hz);
  p.put(fzm, zmx, zmy, -hz);
  if (XF) {
    p.put(fyp, ypx, 0.5f, ypz);
    p.put(fym, ymx, -0.5f, ymz);
    p.put(fxp, 0.5f, xpy, xpz);
    p.put(fxm, -0.5f, xmy, xmz);
  } else {
    p.put(fxp, 0.5f, xpy, xpz);
    p.put(fxm, -0.5f, xmy, xmz);
    p.put(fyp, ypx, 0.5f, ypz);
    p.put(fym, ymx, -0.5f, ymz);
  }
  if (p.n < 2) return 0.0f;
  const float e0 = p.p1x - p.p0x, e1 = p.p1y - p.p0y, e2 = p.p1z - p.p0z;
  return sqrtf(e0 * e0 + e1 * e1 + e2 * e2);
}

// ---------------------------------------------------------------------------
// Cone-beam backward step per voxel column (z-column form).
//
// For a voxel column (ix, iy) and a detector column ia, the x and y face
// tests of find_l_3d (Ax_cone_gpu.cu:120-209) split into an in-plane part --
// the face point's in-plane coordinate t0 -/+ u0 and its |.| <= 1/2 test,
// which depend on the ray's in-plane slopes and the column only -- and a z
// part, t1 -/+ u1 and its |.| <= dz/2 test, which depends on the voxel's z.
// ColFaces keeps the in-plane part of one (column, detector column): the
// first two x/y faces, in the reference's face order, whose in-plane test
// passes.  Faces whose in-plane test fails can never be hits, so a voxel's
// hits are, in order, F1 and F2 (if their z tests pass), then the z- and z+
// faces: chord3_col takes the first two of those four, which is the
// reference's first-two-hits rule.  When three or four in-plane tests pass
// (a ray through a column corner, to within rounding) the column keeps
// kCfMany and its pairs use chord3_axis.  Every face value is the reference
// expression, rounded as there, so the chord is find_l_3d's bit for bit.
// Requires a != 0 and b != 0 (no axis-parallel ray).
// ---------------------------------------------------------------------------
constexpr unsigned kCfV1 = 1u, kCfV2 = 2u;    // F1 / F2 exists
constexpr unsigned kCfY1 = 4u, kCfY2 = 8u;    // F1 / F2 is a y face
constexpr unsigned kCfU1 = 16u, kCfU2 = 32u;  // F1 / F2 is an upper face
constexpr unsigned kCfMany = 64u;             // three or more in-plane hits
constexpr unsigned kCfXF = 128u;              // |a| > |b| (x faces first)

struct ColFaces {
  float p1x, p1y, p2x, p2y;  // in-plane coordinates of F1 and F2
  // z halves of F1 and F2: z = s * n + rz + s * h with s = c/a (x faces) or
  // c/b (y faces), n = -rx or -ry (NaN when the face does not exist, so its
  // z test fails by itself) and h = -1/2 (lower face) or +1/2 (upper face)
  float n1, h1, n2, h2;
  unsigned bits;
};

ASD_HD float __int_as_float_hd(int i) {
#ifdef __CUDA_ARCH__
  return __int_as_float(i);
#else
  float f;
  memcpy(&f, &i, 4);
  return f;
#endif
}

// In-plane part of the x/y face tests of ray A (ray_tab_a) for the voxel
// column whose centre is the source minus (rx, ry).
ASD_HD ColFaces col_faces(const float4 A, float rx, float ry) {
  const float xt0 = A.z * (-rx) + ry, xu0 = A.z * 0.5f;
  const float xmy = xt0 - xu0, xpy = xt0 + xu0;
  const float yt0 = A.w * (-ry) + rx, yu0 = A.w * 0.5f;
  const float ymx = yt0 - yu0, ypx = yt0 + yu0;
  const bool fxm = fabsf(xmy) <= 0.5f, fxp = fabsf(xpy) <= 0.5f;
  const bool fym = fabsf(ymx) <= 0.5f, fyp = fabsf(ypx) <= 0.5f;
  const bool xf = fabsf(A.x) > fabsf(A.y);
  // the four faces in the reference's order, each (pass, x, y, bits)
  const bool pass[4] = {xf ? fxm : fym, xf ? fxp : fyp, xf ? fym : fxm, xf ? fyp : fxp};
  const float px[4] = {xf ? -0.5f : ymx, xf ? 0.5f : ypx, xf ? ymx : -0.5f, xf ? ypx : 0.5f};
  const float py[4] = {xf ? xmy : -0.5f, xf ? xpy : 0.5f, xf ? -0.5f : xmy, xf ? 0.5f : xpy};
  // face k: bit 0 = upper, bit 1 = y face
  const unsigned kind[4] = {xf ? 0u : 2u, xf ? 1u : 3u, xf ? 2u : 0u, xf ? 3u : 1u};
  ColFaces f;
  f.p1x = f.p1y = f.p2x = f.p2y = 0.f;
  unsigned k1 = 0, k2 = 0;
  int n = 0;
  // taken from the last face to the first: a passing face becomes F1 and
  // pushes the previous F1 to F2
#pragma unroll
  for (int k = 3; k >= 0; k--) {
    const bool p = pass[k];
    f.p2x = p ? f.p1x : f.p2x;
    f.p2y = p ? f.p1y : f.p2y;
    k2 = p ? k1 : k2;
    f.p1x = p ? px[k] : f.p1x;
    f.p1y = p ? py[k] : f.p1y;
    k1 = p ? kind[k] : k1;
    n += p ? 1 : 0;
  }
  f.bits = (n >= 1 ? kCfV1 : 0u) | (n >= 2 ? kCfV2 : 0u) | ((k1 & 2u) ? kCfY1 : 0u) |
           ((k2 & 2u) ? kCfY2 : 0u) | ((k1 & 1u) ? kCfU1 : 0u) | ((k2 & 1u) ? kCfU2 : 0u) |
           (n > 2 ? kCfMany : 0u) | (xf ? kCfXF : 0u);
  const float nan = __int_as_float_hd(0x7fc00000);
  f.n1 = n >= 1 ? -((k1 & 2u) ? ry : rx) : nan;
  f.n2 = n >= 2 ? -((k2 & 2u) ? ry : rx) : nan;
  f.h1 = (k1 & 1u) ? 0.5f : -0.5f;
  f.h2 = (k2 & 1u) ? 0.5f : -0.5f;
  return f;
}

// find_l_3d of ray (A, Cs) and the voxel at (rx, ry, rz) from the source,
// given the column's ColFaces f (without kCfMany).  hz = dz / 2.
ASD_HD float chord3_col(const ColFaces &f, const float4 Cs, float rx, float ry,
                        float rz, float hz) {
  const unsigned bits = f.bits;
  // z parts of F1 and F2: t -/+ u with t = s * (-r) + rz, u = s * (1/2),
  // s = c/a (x faces) or c/b (y faces); s * (-1/2) is -(s * (1/2)) exactly
  // and t + (-u) is t - u, so these are the reference's values
  const float c1 = (bits & kCfY1) ? Cs.y : Cs.x;
  const float z1 = (c1 * f.n1 + rz) + c1 * f.h1;
  const float c2 = (bits & kCfY2) ? Cs.y : Cs.x;
  const float z2 = (c2 * f.n2 + rz) + c2 * f.h2;
  const bool h1 = fabsf(z1) <= hz;  // false for a missing face (NaN)
  const bool h2 = fabsf(z2) <= hz;
  // z faces
  const float zt0 = Cs.z * (-rz) + rx, zu0 = Cs.z * hz;
  const float zt1 = Cs.w * (-rz) + ry, zu1 = Cs.w * hz;
  const float zmx = zt0 - zu0, zmy = zt1 - zu1, zpx = zt0 + zu0, zpy = zt1 + zu1;
  const bool fzm = fabsf(zmx) <= 0.5f && fabsf(zmy) <= 0.5f;
  const bool fzp = fabsf(zpx) <= 0.5f && fabsf(zpy) <= 0.5f;
  const int n = (h1 ? 1 : 0) + (h2 ? 1 : 0) + (fzm ? 1 : 0) + (fzp ? 1 : 0);
  // first z hit
  const float qx = fzm ? zmx : zpx, qy = fzm ? zmy : zpy, qz = fzm ? -hz : hz;
  // first hit: F1, else F2, else the first z hit
  const float ax = h1 ? f.p1x : (h2 ? f.p2x : qx);
  const float ay = h1 ? f.p1y : (h2 ? f.p2y : qy);
  const float az = h1 ? z1 : (h2 ? z2 : qz);
  // second hit: F2 after F1; the first z hit after one face; z+ after z-
  const bool both = h1 && h2, one = h1 != h2;
  const float bx = both ? f.p2x : (one ? qx : zpx);
  const float by = both ? f.p2y : (one ? qy : zpy);
  const float bz = both ? z2 : (one ? qz : hz);
  const float e0 = bx - ax, e1 = by - ay, e2 = bz - az;
  return n >= 2 ? sqrtf(e0 * e0 + e1 * e1 + e2 * e2) : 0.0f;
}

// Per-column part of the footprint (voxel_window's columns and its
// magnification, shadow_bins3's columns and its corners' magnifications);
// zcol_rows then gives each voxel's rows.  Same expressions as voxel_window
// and shadow_bins3, so the same pairs.
struct ZCol {
  float xc, yc, rx, ry, ta, tb;
  float q[4];      // magnification at the four corners (shadow rows)
  int a0, a1;      // window columns (clamped)
  int lo, hi;      // window columns narrowed to the shadow
  bool ok;         // every corner in front of the source (shadow usable)
};

ASD_HD ZCol zcol_setup(const ViewGeo &G, const Dims &D, int ix, int iy, bool narrow) {
  ZCol c;
  const int na2 = D.na / 2, nx2 = D.nx / 2, ny2 = D.ny / 2;
  c.yc = (float)(iy - ny2) + 0.5f;
  c.xc = (float)(ix - nx2) + 0.5f;
  const float xr = G.cos_phi * c.xc + G.sin_phi * c.yc;
  const float yr = -G.sin_phi * c.xc + G.cos_phi * c.yc;
  c.ta = G.SD / ((xr + G.SO) * G.dy_det);
  c.tb = G.dz_det != G.dy_det ? G.SD / ((xr + G.SO) * G.dz_det) : c.ta;
  const int amax = (int)floorf((yr + 1) * c.ta + na2);
  const int amin = (int)floorf((yr - 1) * c.ta + na2);
  c.a0 = amin > 0 ? amin : 0;
  c.a1 = amax < D.na - 1 ? amax : D.na - 1;
  const float hc = 0.5f * G.cos_phi, hs = 0.5f * G.sin_phi;
  const float inv_a = hd_rcp(G.dy_det);
  const float offa = D.na * 0.5f - 0.5f;
  float umin = 3.0e38f, umax = -3.0e38f;
  bool ok = true;
#pragma unroll
  for (int k = 0; k < 4; k++) {
    const float ex = (k & 1) ? 1.f : -1.f, ey = (k & 2) ? 1.f : -1.f;
    const float px = xr + ex * hc + ey * hs;
    const float py = yr - ex * hs + ey * hc;
    const float den = px + G.SO;
    ok = ok && den > 1e-3f;
    c.q[k] = fast_div(G.SD, den);
    const float u = py * c.q[k] * inv_a + offa;
    umin = fminf(umin, u);
    umax = fmaxf(umax, u);
  }
  c.ok = narrow && ok;
  c.lo = c.a0;
  c.hi = c.a1;
  if (c.ok) {
    const int alo = (int)ceilf(umin - 0.05f), ahi = (int)floorf(umax + 0.05f);
    c.lo = c.lo > alo ? c.lo : alo;
    c.hi = c.hi < ahi ? c.hi : ahi;
  }
  c.rx = G.cos_phi * (-G.SO) - c.xc;
  c.ry = G.sin_phi * (-G.SO) - c.yc;
  return c;
}

// Rows [blo, bhi] of voxel iz of column c (the window's rows narrowed to the
// shadow's); false when the reference's window is empty.
ASD_HD bool zcol_rows(const ViewGeo &G, const Dims &D, const ZCol &c, int iz, float &zc,
                      int &blo, int &bhi) {
  const int nb2 = D.nb / 2, nz2 = D.nz / 2;
  zc = ((float)(iz - nz2) + 0.5f) * G.dz;
  const int bmax = (int)floorf((zc + G.dwin) * c.tb + nb2);
  const int bmin = (int)floorf((zc - G.dwin) * c.tb + nb2);
  blo = bmin > 0 ? bmin : 0;
  bhi = bmax < D.nb - 1 ? bmax : D.nb - 1;
  const bool has = c.a0 <= c.a1 && blo <= bhi;
  if (has && c.ok) {
    const float hz = 0.5f * G.dz;
    const float inv_b = hd_rcp(G.dz_det);
    const float offb = D.nb * 0.5f - 0.5f;
    const float zlo = (zc - hz) * inv_b, zhi = (zc + hz) * inv_b;
    float vmin = 3.0e38f, vmax = -3.0e38f;
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const float v0 = zlo * c.q[k] + offb, v1 = zhi * c.q[k] + offb;
      vmin = fminf(vmin, fminf(v0, v1));
      vmax = fmaxf(vmax, fmaxf(v0, v1));
    }
    const int tlo = (int)ceilf(vmin - 0.05f), thi = (int)floorf(vmax + 0.05f);
    blo = blo > tlo ? blo : tlo;
    bhi = bhi < thi ? bhi : thi;
  }
  return has;
}

}  // namespace asd
