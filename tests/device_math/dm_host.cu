// Host build of the projector device math (csrc/projector.cuh) -- TEST
// INFRASTRUCTURE.  The same __host__ __device__ functions the kernels call
// run here on the CPU, so the CPU test suite can check the kernels' float
// logic bit for bit against the oracle without a GPU:
//   dm_ax   -- Ax with the columns of a ray split over `lanes` partial sums
//              combined by the same xor butterfly as the warp reduction,
//              with the reference's weight expressions (exact=1) or the
//              kernels' division-free ones (exact=0: the kernels' grouped
//              form, exact=2: the per-column form it must match);
//   dm_atx  -- Atx through the staged ray tables and the branch-free chords
//              (ray_tab_a / ray_tab_c, chord_planar_bf / chord3_bf) as the
//              kernels run it (staged=1), the same restricted to each voxel's
//              shadow (shadow_bins / shadow_bins3) under the kernels'
//              conditions (staged=2), or the direct per-pair form.
// Compiled with -ffp-contract=off so the host compiler fuses nothing.
#include <string.h>

#include <vector>

#include "../../asd_pocs_mex_cuda_demo_gb300/csrc/projector.cuh"

using namespace asd;

static ViewGeo geo(float c, float s, const float *yd, const float *zd, float SO,
                   float OD, float scale, float ddy, float ddz, float dz) {
  return with_constants(ViewGeo{c, s, SO, OD, scale, ddy, ddz, dz, yd, zd});
}

extern "C" void dm_ax(const float *x, float *y, float *sr, float c, float s,
                      const float *yd, const float *zd, float SO, float OD,
                      float scale, float dz, int nx, int ny, int nz, int na,
                      int nb, int lanes, int exact) {
  const ViewGeo G = geo(c, s, yd, zd, SO, OD, scale, 0.f, 0.f, dz);
  const Dims D{nx, ny, nz, na, nb};
  std::vector<float> py(lanes), ps(lanes);
  for (long long r = 0; r < (long long)na * nb; r++) {
    const int ia = (int)(r % na), ib = (int)(r / na);
    const RayMarch R = ray_setup(G, D, yd[ia], zd[ib]);
    const bool planar = nz == 1 && zd[ib] == 0.0f;
    py.assign(lanes, 0.f);
    ps.assign(lanes, 0.f);
    for (int l = 0; l < lanes; l++) {
      float a = 0.f, b = 0.f;
      auto ld = [&](long long i) { return x[i]; };
      if (planar && exact == 1)
        ray_columns_planar<true>(R, l, lanes, ld, a, b);
      else if (planar && exact == 2)
        ray_columns_planar<false>(R, l, lanes, ld, a, b);
      else if (planar)
        ray_columns_planar_fast(R, l, lanes, ld, a, b);
      else if (exact == 1)
        ray_columns<true>(R, l, lanes, ld, a, b);
      else if (exact == 2)
        ray_columns<false>(R, l, lanes, ld, a, b);
      else
        ray_columns_fast<2>(R, l, lanes, ld, a, b);
      py[l] = a;
      ps[l] = b;
    }
    // more than 32 partials: kAxCols warps share the ray's columns; their
    // lane partials are added in part order before the lanes are summed
    if (lanes > 32) {
      for (int l = 0; l < 32; l++)
        for (int q = 1; q < lanes / 32; q++) {
          py[l] += py[l + 32 * q];
          ps[l] += ps[l + 32 * q];
        }
      py.resize(32);
      ps.resize(32);
    }
    const int nl = lanes > 32 ? 32 : lanes;
    // xor butterfly (warp_sum): every lane ends with the same total
    for (int o = nl / 2; o > 0; o >>= 1) {
      std::vector<float> ny_(py), ns_(ps);
      for (int l = 0; l < nl; l++) {
        ny_[l] = py[l] + py[l ^ o];
        ns_[l] = ps[l] + ps[l ^ o];
      }
      py.swap(ny_);
      ps.swap(ns_);
    }
    y[r] = py[0] * G.scale;
    sr[r] = ps[0] * G.scale;
  }
}

extern "C" void dm_atx(float *x, const float *yv, float *sc, float c, float s,
                       const float *yd, const float *zd, float SO, float OD,
                       float scale, float ddy, float ddz, float dz, int nx,
                       int ny, int nz, int na, int nb, int staged) {
  const ViewGeo G = geo(c, s, yd, zd, SO, OD, scale, ddy, ddz, dz);
  const Dims D{nx, ny, nz, na, nb};
  const bool planar = nz == 1 && nb == 1 && zd[0] == 0.0f;
  std::vector<float4> tA(na), tC(planar ? 0 : (size_t)na * nb);
  for (int ia = 0; ia < na; ia++) tA[ia] = ray_tab_a(G, yd[ia]);
  if (!planar)
    for (long long k = 0; k < (long long)na * nb; k++)
      tC[k] = ray_tab_c(tA[k % na], zd[k / na]);
  // the kernels narrow to the shadow only for views with no axis-parallel
  // ray, finite values and bins on the uniform grid
  bool narrow = staged == 2 && ddy > 0.0f && (planar || ddz > 0.0f);
  for (int ia = 0; ia < na; ia++)
    narrow = narrow && tA[ia].x != 0.0f && tA[ia].y != 0.0f &&
             on_grid(yd[ia], ia, na, ddy);
  for (int ib = 0; ib < nb && !planar; ib++)
    narrow = narrow && on_grid(zd[ib], ib, nb, ddz);
  for (long long k = 0; k < (long long)na * nb; k++)
    narrow = narrow && isfinite(yv[k]);
  for (int iz = 0; iz < nz; iz++)
    for (int iy = 0; iy < ny; iy++)
      for (int ix = 0; ix < nx; ix++) {
        const VoxelWin w = voxel_window(G, D, ix, iy, iz);
        float acc = 0.f, accl = 0.f;
        if (!staged) {
          voxel_backproject(G, D, w, [&](long long i) { return yv[i]; }, acc,
                            accl);
        } else {
          const float rx = G.cos_phi * (-G.SO) - w.xc;
          const float ry = G.sin_phi * (-G.SO) - w.yc;
          const float rz = 0.0f - w.zc;
          int a0 = w.a0, a1 = w.a1, b0 = w.b0, b1 = w.b1;
          if (narrow) {
            int slo, shi, tlo, thi;
            if (planar ? shadow_bins(G, D, w.xc, w.yc, slo, shi)
                       : shadow_bins3(G, D, w.xc, w.yc, w.zc, slo, shi, tlo, thi)) {
              a0 = a0 > slo ? a0 : slo;
              a1 = a1 < shi ? a1 : shi;
              if (!planar) {
                b0 = b0 > tlo ? b0 : tlo;
                b1 = b1 < thi ? b1 : thi;
              }
            }
          }
          for (int ib = b0; ib <= b1; ib++) {
            const float cc = zd[ib] - 0.0f;
            for (int ia = a0; ia <= a1; ia++) {
              const long long k = (long long)ib * na + ia;
              float l;
              if (planar && tA[ia].x != 0.0f && tA[ia].y != 0.0f)
                l = fabsf(tA[ia].x) > fabsf(tA[ia].y)
                        ? chord_planar_axis<true>(tA[ia], rx, ry)
                        : chord_planar_axis<false>(tA[ia], rx, ry);
              else if (planar)
                l = chord_planar_bf(tA[ia], rx, ry, dz);
              else
                l = chord3_bf(tA[ia], tC[k], cc, rx, ry, rz, dz);
              acc += l * yv[k];
              accl += l;
            }
          }
        }
        const long long idx = ((long long)iz * ny + iy) * nx + ix;
        x[idx] = acc * scale;
        sc[idx] = accl * scale;
      }
}
