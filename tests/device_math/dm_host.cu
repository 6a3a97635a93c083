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
//              conditions (staged=2), or the direct per-pair form;
//   dm_chord_count / dm_atx_table -- the 2-D chord tables' layout, filled
//              and read back;
//   dm_atx3_zcol -- the cone-beam backward step walked down voxel columns,
//              as the z-column kernel runs it;
//   dm_ax_siddon -- the exact (Siddon) forward projection, its columns split
//              over `lanes` partial sums combined by the warp butterfly.
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

// Chord tables of the 2-D backward step, as k_atx_chords lays them out for
// one view -- header (count << 24 | first ray), chord sum, then K slot
// planes of N chords -- from the same window, shadow and chord functions,
// the chord function picked per view (every ray x-dominant, every ray
// y-dominant, or the general form) as the kernels pick it.  dm_chord_count
// returns the view's largest pair count, 0 when the view has an
// axis-parallel ray (no table); dm_atx_table builds the table with K slots
// and replays it the way the backward steps read it (pairs of a voxel in
// slot order), giving Atx and its chord sums; it returns 0, or -1 when a
// voxel has more than K pairs.
namespace {
struct PlanarView {
  ViewGeo G;
  Dims D;
  std::vector<float4> tA;
  int ax = -1;  // 1: x-dominant rays, 2: y-dominant, 0: mixed; -1: no table
};

PlanarView planar_view(float c, float s, const float *yd, const float *zd, float SO,
                       float OD, float scale, float ddy, int nx, int ny, int na) {
  PlanarView v{geo(c, s, yd, zd, SO, OD, scale, ddy, ddy, 1.0f), Dims{nx, ny, 1, na, 1},
               std::vector<float4>(na), -1};
  bool par = false, allx = true, ally = true;
  for (int ia = 0; ia < na; ia++) {
    const float4 A = ray_tab_a(v.G, yd[ia]);
    v.tA[ia] = A;
    par = par || A.x == 0.0f || A.y == 0.0f;
    const bool xf = fabsf(A.x) > fabsf(A.y);
    allx = allx && xf;
    ally = ally && !xf;
  }
  if (!par && zd[0] == 0.0f) v.ax = allx ? 1 : (ally ? 2 : 0);
  return v;
}

// The pairs of voxel (ix, iy): first ray and count, as chords_voxel finds them.
void voxel_pairs(const PlanarView &v, int ix, int iy, int &first, int &cnt, float &rx,
                 float &ry) {
  const VoxelWin w = voxel_window(v.G, v.D, ix, iy, 0);
  const bool has = w.a0 <= w.a1 && w.b0 <= w.b1;
  int lo = has ? w.a0 : 0, hi = has ? w.a1 : -1;
  if (has) {
    int slo, shi;
    if (shadow_bins(v.G, v.D, w.xc, w.yc, slo, shi)) {
      lo = lo > slo ? lo : slo;
      hi = hi < shi ? hi : shi;
    }
  }
  cnt = has && lo <= hi ? hi - lo + 1 : 0;
  first = has ? w.b0 * v.D.na + lo : 0;
  rx = v.G.cos_phi * (-v.G.SO) - w.xc;
  ry = v.G.sin_phi * (-v.G.SO) - w.yc;
}

float view_chord(const PlanarView &v, int ia, float rx, float ry) {
  const float4 A = v.tA[ia];
  if (v.ax == 1) return chord_planar_axis<true>(A, rx, ry);
  if (v.ax == 2) return chord_planar_axis<false>(A, rx, ry);
  return chord_planar_bf(A, rx, ry, v.G.dz);
}
}  // namespace

extern "C" int dm_chord_count(float c, float s, const float *yd, float SO, float OD,
                              float ddy, int nx, int ny, int na) {
  const float zd0 = 0.0f;
  const PlanarView v = planar_view(c, s, yd, &zd0, SO, OD, 1.0f, ddy, nx, ny, na);
  if (v.ax < 0) return 0;
  int K = 0;
  for (int iy = 0; iy < ny; iy++)
    for (int ix = 0; ix < nx; ix++) {
      int first, cnt;
      float rx, ry;
      voxel_pairs(v, ix, iy, first, cnt, rx, ry);
      K = cnt > K ? cnt : K;
    }
  return K;
}

extern "C" int dm_atx_table(float *x, const float *yv, float *sc, float c, float s,
                            const float *yd, float SO, float OD, float scale, float ddy,
                            int nx, int ny, int na, int K) {
  const float zd0 = 0.0f;
  const PlanarView v = planar_view(c, s, yd, &zd0, SO, OD, scale, ddy, nx, ny, na);
  const size_t N = (size_t)nx * ny;
  std::vector<int> tab((size_t)(2 + K) * N, 0);
  float *ch = (float *)(tab.data() + 2 * N);
  for (int iy = 0; iy < ny; iy++)  // the filling pass
    for (int ix = 0; ix < nx; ix++) {
      const size_t vi = (size_t)iy * nx + ix;
      int first, cnt;
      float rx, ry;
      voxel_pairs(v, ix, iy, first, cnt, rx, ry);
      if (cnt > K) return -1;
      float accl = 0.f;
      for (int k = 0; k < cnt; k++) {
        const float l = view_chord(v, first + k, rx, ry);
        accl += l;
        ch[(size_t)k * N + vi] = l;
      }
      tab[vi] = cnt ? (int)(((unsigned)cnt << 24) | (unsigned)first) : 0;
      memcpy(&tab[N + vi], &accl, 4);
    }
  for (size_t vi = 0; vi < N; vi++) {  // the backward step's reading
    const int h = tab[vi];
    const int cnt = (int)((unsigned)h >> 24), first = h & 0xffffff;
    float acc = 0.f, accl;
    memcpy(&accl, &tab[N + vi], 4);
    for (int k = 0; k < cnt; k++) acc += ch[(size_t)k * N + vi] * yv[first + k];
    x[vi] = acc * scale;
    sc[vi] = accl * scale;
  }
  return 0;
}

// dm_atx3_zcol -- the cone-beam backward step walked down each (x, y) voxel
// column as the z-column kernel runs it: the window's and shadow's columns,
// the corners' magnifications and, for every detector column of the shadow,
// the in-plane part of the x and y face tests (col_faces) once per column;
// each voxel then needs its rows (zcol_rows) and the z parts of the face
// tests (chord3_col).  Columns with three or more in-plane hits use
// chord3_axis.  Narrowing conditions as dm_atx (staged=2); views that do not
// allow narrowing take the per-voxel form.
extern "C" void dm_atx3_zcol(float *x, const float *yv, float *sc, float c, float s,
                             const float *yd, const float *zd, float SO, float OD,
                             float scale, float ddy, float ddz, float dz, int nx, int ny,
                             int nz, int na, int nb) {
  const ViewGeo G = geo(c, s, yd, zd, SO, OD, scale, ddy, ddz, dz);
  const Dims D{nx, ny, nz, na, nb};
  std::vector<float4> tA(na), tC((size_t)na * nb);
  for (int ia = 0; ia < na; ia++) tA[ia] = ray_tab_a(G, yd[ia]);
  for (long long k = 0; k < (long long)na * nb; k++) tC[k] = ray_tab_c(tA[k % na], zd[k / na]);
  bool narrow = ddy > 0.0f && ddz > 0.0f;
  for (int ia = 0; ia < na; ia++)
    narrow = narrow && tA[ia].x != 0.0f && tA[ia].y != 0.0f && on_grid(yd[ia], ia, na, ddy);
  for (int ib = 0; ib < nb; ib++) narrow = narrow && on_grid(zd[ib], ib, nb, ddz);
  for (long long k = 0; k < (long long)na * nb; k++) narrow = narrow && isfinite(yv[k]);
  if (!narrow) {
    dm_atx(x, yv, sc, c, s, yd, zd, SO, OD, scale, ddy, ddz, dz, nx, ny, nz, na, nb, 1);
    return;
  }
  const float hz = dz / 2.0f;
  std::vector<ColFaces> cf(na);
  for (int iy = 0; iy < ny; iy++)
    for (int ix = 0; ix < nx; ix++) {
      const ZCol col = zcol_setup(G, D, ix, iy, true);
      const int cntA = col.lo <= col.hi ? col.hi - col.lo + 1 : 0;
      for (int k = 0; k < cntA; k++) cf[k] = col_faces(tA[col.lo + k], col.rx, col.ry);
      for (int iz = 0; iz < nz; iz++) {
        float zc;
        int blo, bhi;
        const bool has = zcol_rows(G, D, col, iz, zc, blo, bhi);
        const int cntB = has && blo <= bhi ? bhi - blo + 1 : 0;
        const float rz = 0.0f - zc;
        float acc = 0.f, accl = 0.f;
        for (int kb = 0; kb < (has ? cntB : 0); kb++)
          for (int ka = 0; ka < cntA; ka++) {
            const long long r = (long long)(blo + kb) * na + col.lo + ka;
            const ColFaces &f = cf[ka];
            float l;
            if (f.bits & kCfMany)
              l = (f.bits & kCfXF) ? chord3_axis<true>(tA[col.lo + ka], tC[r], col.rx, col.ry, rz, dz)
                                   : chord3_axis<false>(tA[col.lo + ka], tC[r], col.rx, col.ry, rz, dz);
            else
              l = chord3_col(f, tC[r], col.rx, col.ry, rz, hz);
            acc += l * yv[r];
            accl += l;
          }
        const long long idx = ((long long)iz * ny + iy) * nx + ix;
        x[idx] = acc * scale;
        sc[idx] = accl * scale;
      }
    }
}

extern "C" void dm_ax_siddon(const float *x, float *y, float *sr, float c, float s,
                             const float *yd, const float *zd, float SO, float OD,
                             float scale, float dz, int nx, int ny, int nz, int na, int nb,
                             int lanes) {
  const ViewGeo G = geo(c, s, yd, zd, SO, OD, scale, 0.f, 0.f, dz);
  const Dims D{nx, ny, nz, na, nb};
  std::vector<float> py(lanes), ps(lanes);
  for (long long r = 0; r < (long long)na * nb; r++) {
    const SidRay R = siddon_setup(G, D, yd[r % na], zd[r / na]);
    for (int l = 0; l < lanes; l++) {
      float a = 0.f, b = 0.f;
      siddon_columns(R, l, lanes, [&](unsigned i) { return x[i]; }, a, b);
      py[l] = a;
      ps[l] = b;
    }
    for (int o = lanes / 2; o > 0; o >>= 1) {
      std::vector<float> ny_(py), ns_(ps);
      for (int l = 0; l < lanes; l++) {
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
