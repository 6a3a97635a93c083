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
//   dm_atx3_zcol -- the cone-beam backward step walked down voxel columns
//              (the form planned for the cone-beam kernel).
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

// dm_atx3_zcol -- the cone-beam backward step as a walk down each (x, y)
// voxel column, the form planned for the cone-beam kernel: what does not
// depend on z is computed once per column -- the window's columns and its
// magnification (one division), the shadow's columns and the four corners'
// magnifications (four divisions), and for every detector column of the
// shadow the in-plane parts of the x and y face tests -- and each voxel of
// the column then needs its rows (multiply-adds) and the z parts of the face
// tests.  The expressions are those of voxel_window, shadow_bins3 and
// chord3_bf, split where they do not depend on z, so the result must be the
// per-voxel form's bit for bit.  Narrowing conditions as dm_atx (staged=2).
namespace {
struct InPlane3 {
  float xmy, xpy, ymx, ypx;
  bool ixm, ixp, iym, iyp;
};

InPlane3 inplane3(const float4 A, float rx, float ry) {
  InPlane3 p;
  const float xt0 = A.z * (-rx) + ry, xu0 = A.z * 0.5f;
  p.xmy = xt0 - xu0;
  p.xpy = xt0 + xu0;
  p.ixm = fabsf(p.xmy) <= 0.5f;
  p.ixp = fabsf(p.xpy) <= 0.5f;
  const float yt0 = A.w * (-ry) + rx, yu0 = A.w * 0.5f;
  p.ymx = yt0 - yu0;
  p.ypx = yt0 + yu0;
  p.iym = fabsf(p.ymx) <= 0.5f;
  p.iyp = fabsf(p.ypx) <= 0.5f;
  return p;
}

// chord3_bf for a ray with a != 0 and b != 0, from its in-plane parts.
float chord3_z(const float4 A, const InPlane3 &p, const float4 Cs, float rx, float ry,
               float rz, float dz) {
  const float hz = dz / 2.0f;
  const float xt1 = Cs.x * (-rx) + rz, xu1 = Cs.x * 0.5f;
  const float xmz = xt1 - xu1, xpz = xt1 + xu1;
  const bool fxm = p.ixm && fabsf(xmz) <= hz;
  const bool fxp = p.ixp && fabsf(xpz) <= hz;
  const float yt1 = Cs.y * (-ry) + rz, yu1 = Cs.y * 0.5f;
  const float ymz = yt1 - yu1, ypz = yt1 + yu1;
  const bool fym = p.iym && fabsf(ymz) <= hz;
  const bool fyp = p.iyp && fabsf(ypz) <= hz;
  const float zt0 = Cs.z * (-rz) + rx, zu0 = Cs.z * hz;
  const float zt1 = Cs.w * (-rz) + ry, zu1 = Cs.w * hz;
  const float zmx = zt0 - zu0, zmy = zt1 - zu1, zpx = zt0 + zu0, zpy = zt1 + zu1;
  const bool fzm = fabsf(zmx) <= 0.5f && fabsf(zmy) <= 0.5f;
  const bool fzp = fabsf(zpx) <= 0.5f && fabsf(zpy) <= 0.5f;
  Pick2Rev q;
  q.n = 0;
  q.p0x = q.p0y = q.p0z = q.p1x = q.p1y = q.p1z = 0.f;
  q.put(fzp, zpx, zpy, hz);
  q.put(fzm, zmx, zmy, -hz);
  if (fabsf(A.x) > fabsf(A.y)) {
    q.put(fyp, p.ypx, 0.5f, ypz);
    q.put(fym, p.ymx, -0.5f, ymz);
    q.put(fxp, 0.5f, p.xpy, xpz);
    q.put(fxm, -0.5f, p.xmy, xmz);
  } else {
    q.put(fxp, 0.5f, p.xpy, xpz);
    q.put(fxm, -0.5f, p.xmy, xmz);
    q.put(fyp, p.ypx, 0.5f, ypz);
    q.put(fym, p.ymx, -0.5f, ymz);
  }
  if (q.n < 2) return 0.0f;
  const float e0 = q.p1x - q.p0x, e1 = q.p1y - q.p0y, e2 = q.p1z - q.p0z;
  return sqrtf(e0 * e0 + e1 * e1 + e2 * e2);
}
}  // namespace

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
  const int na2 = na / 2, nb2 = nb / 2, nx2 = nx / 2, ny2 = ny / 2, nz2 = nz / 2;
  const float hz = 0.5f * G.dz;
  const float inv_a = hd_rcp(G.dy_det), inv_b = hd_rcp(G.dz_det);
  const float offa = na * 0.5f - 0.5f, offb = nb * 0.5f - 0.5f;
  std::vector<InPlane3> ip(na);
  for (int iy = 0; iy < ny; iy++)
    for (int ix = 0; ix < nx; ix++) {
      // ---- once per column: voxel_window's columns and magnification
      const float yc = (float)(iy - ny2) + 0.5f, xc = (float)(ix - nx2) + 0.5f;
      const float xr = G.cos_phi * xc + G.sin_phi * yc;
      const float yr = -G.sin_phi * xc + G.cos_phi * yc;
      const float ta = G.SD / ((xr + G.SO) * G.dy_det);
      const float tb = G.dz_det != G.dy_det ? G.SD / ((xr + G.SO) * G.dz_det) : ta;
      const int amax = (int)floorf((yr + 1) * ta + na2);
      const int amin = (int)floorf((yr - 1) * ta + na2);
      const int a0 = amin > 0 ? amin : 0, a1 = amax < na - 1 ? amax : na - 1;
      // shadow_bins3's columns and its corners' magnifications
      const float hc = 0.5f * G.cos_phi, hs = 0.5f * G.sin_phi;
      float q[4], umin = 3.0e38f, umax = -3.0e38f;
      bool ok = true;
      for (int k = 0; k < 4; k++) {
        const float ex = (k & 1) ? 1.f : -1.f, ey = (k & 2) ? 1.f : -1.f;
        const float px = xr + ex * hc + ey * hs;
        const float py = yr - ex * hs + ey * hc;
        const float den = px + G.SO;
        ok = ok && den > 1e-3f;
        q[k] = fast_div(G.SD, den);
        const float u = py * q[k] * inv_a + offa;
        umin = fminf(umin, u);
        umax = fmaxf(umax, u);
      }
      int lo = a0, hi = a1;
      const bool nar = narrow && ok;
      if (nar) {
        const int alo = (int)ceilf(umin - 0.05f), ahi = (int)floorf(umax + 0.05f);
        lo = lo > alo ? lo : alo;
        hi = hi < ahi ? hi : ahi;
      }
      const float rx = G.cos_phi * (-G.SO) - xc;
      const float ry = G.sin_phi * (-G.SO) - yc;
      for (int ia = lo; ia <= hi; ia++) ip[ia] = inplane3(tA[ia], rx, ry);
      // ---- per voxel of the column: rows and the z parts
      for (int iz = 0; iz < nz; iz++) {
        const float zc = ((float)(iz - nz2) + 0.5f) * G.dz;
        const int bmax = (int)floorf((zc + G.dwin) * tb + nb2);
        const int bmin = (int)floorf((zc - G.dwin) * tb + nb2);
        int blo = bmin > 0 ? bmin : 0, bhi = bmax < nb - 1 ? bmax : nb - 1;
        float acc = 0.f, accl = 0.f;
        const bool has = a0 <= a1 && blo <= bhi;
        if (has && nar) {
          const float zlo = (zc - hz) * inv_b, zhi = (zc + hz) * inv_b;
          float vmin = 3.0e38f, vmax = -3.0e38f;
          for (int k = 0; k < 4; k++) {
            const float v0 = zlo * q[k] + offb, v1 = zhi * q[k] + offb;
            vmin = fminf(vmin, fminf(v0, v1));
            vmax = fmaxf(vmax, fmaxf(v0, v1));
          }
          const int tlo = (int)ceilf(vmin - 0.05f), thi = (int)floorf(vmax + 0.05f);
          blo = blo > tlo ? blo : tlo;
          bhi = bhi < thi ? bhi : thi;
        }
        const float rz = 0.0f - zc;
        if (has)
          for (int ib = blo; ib <= bhi; ib++) {
            const float cc = zd[ib] - 0.0f;
            for (int ia = lo; ia <= hi; ia++) {
              const long long k = (long long)ib * na + ia;
              const float4 A = tA[ia];
              const float l = (A.x != 0.0f && A.y != 0.0f)
                                  ? chord3_z(A, ip[ia], tC[k], rx, ry, rz, dz)
                                  : chord3_bf(A, tC[k], cc, rx, ry, rz, dz);
              acc += l * yv[k];
              accl += l;
            }
          }
        const long long idx = ((long long)iz * ny + iy) * nx + ix;
        x[idx] = acc * scale;
        sc[idx] = accl * scale;
      }
    }
}
