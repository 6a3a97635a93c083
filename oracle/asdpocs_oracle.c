/*
 * CPU oracle for the ASD-POCS hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py (cpu_baseline and the
 * reference arm) load this code, and only as the checker / CPU baseline.
 * The product library (asd_pocs_mex_cuda_demo_gb300) never links it.
 *
 * Each function restates one piece of the reference (file:line cited on the
 * function).  Float expressions follow the reference's operation order, and
 * the file is compiled with -ffp-contract=off so no multiply-add is fused.
 * The restatement is pinned against the reference's own code built for the
 * host (oracle/build_ref.sh) by tests/test_oracle_vs_reference.py and against
 * the committed golden vectors in tests/golden/.
 */
#include "asdpocs_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------------ */
/* Forward projection (Ax_cone_gpu.cu:339-776)                               */
/* ------------------------------------------------------------------------ */

/* Accumulate one weighted voxel into the ray sums (the reference adds
 * `w*x[idx]` to y and `w` to sr in place, in traversal order). */
static inline void acc_piece(float w, const float *x, long idx, float *ys,
                             float *ss) {
  *ys += w * x[idx];
  *ss += w;
}

/*
 * One ray of Ax.  The ray is marched column by column along its driving axis
 * u (x when |dx|>|dy|, Ax_cone_gpu.cu:372; else y, :573).  In each column the
 * ray spans [v1,v2] in the in-plane transverse axis and [w1,w2] in z
 * (sorted by the sign of the slope, :377-394).  The column length l (:402)
 * is split at the (at most one) v-crossing, fraction rv measured from v1, and
 * the (at most one) z-crossing, fraction rz measured from w1; the pieces are
 * the overlaps of [0,rv],[rv,1] with [0,rz],[rz,1] (:398-570 enumerate these
 * 16 cases explicitly).  Rows/slices outside the volume drop their pieces
 * exactly as the reference's range tests do (cy2==0 keeps only the upper row,
 * cy2==n keeps only the lower one, ...).
 */
static void ax_ray(const float *x, float *yout, float *srout, float cos_phi,
                   float sin_phi, float ydet, float zdet, float SO, float OD,
                   float dz, int nx, int ny, int nz, float scale) {
  const int nx2 = nx / 2, ny2 = ny / 2, nz2 = nz / 2;
  const float x1 = cos_phi * (-SO);
  const float y1 = sin_phi * (-SO);
  const float z1 = 0.0f;
  const float x2 = cos_phi * OD - sin_phi * ydet;
  const float y2 = sin_phi * OD + cos_phi * ydet;
  const float z2 = zdet;
  float ys = 0.0f, ss = 0.0f;

  const int xdrive = fabsf(x1 - x2) > fabsf(y1 - y2);
  /* u: driving axis, v: in-plane transverse axis */
  const float us = xdrive ? x1 : y1;
  const float vs = xdrive ? y1 : x1;
  const float du = xdrive ? (x2 - x1) : (y2 - y1);
  const float dv = xdrive ? (y2 - y1) : (x2 - x1);
  const float slope1 = dv / du;
  const float slope2 = (z2 - z1) / du;
  const int nu = xdrive ? nx : ny;
  const int nv = xdrive ? ny : nx;
  const int nu2 = xdrive ? nx2 : ny2;
  const int nv2 = xdrive ? ny2 : nx2;
  const long su = xdrive ? 1 : nx; /* memory stride of u */
  const long sv = xdrive ? nx : 1; /* memory stride of v */
  const long sz = (long)nx * ny;
  const float len2 = (x1 - x2) * (x1 - x2) + (y1 - y2) * (y1 - y2);
  const float dz2sq = (z1 - z2) * (z1 - z2);

  for (int iu = 0; iu < nu; iu++) {
    const float uu1 = (float)(iu - nu2);
    const float uu2 = uu1 + 1;
    float v1, v2, w1, w2;
    if (slope1 >= 0) {
      v1 = vs + slope1 * (uu1 - us) + nv2;
      v2 = vs + slope1 * (uu2 - us) + nv2;
    } else {
      v1 = vs + slope1 * (uu2 - us) + nv2;
      v2 = vs + slope1 * (uu1 - us) + nv2;
    }
    const int cv1 = (int)floorf(v1), cv2 = (int)floorf(v2);
    if (slope2 >= 0) {
      w1 = (z1 + slope2 * (uu1 - us)) / dz + nz2;
      w2 = (z1 + slope2 * (uu2 - us)) / dz + nz2;
    } else {
      w1 = (z1 + slope2 * (uu2 - us)) / dz + nz2;
      w2 = (z1 + slope2 * (uu1 - us)) / dz + nz2;
    }
    const int cz1 = (int)floorf(w1), cz2 = (int)floorf(w2);

    /* which rows / slices may receive pieces (reference range tests) */
    int vlo, vhi, zlo, zhi;
    const int vsplit = cv1 != cv2, zsplit = cz1 != cz2;
    if (!vsplit) {
      vlo = cv1 >= 0 && cv1 <= nv - 1;
      vhi = 0;
    } else if (cv2 > 0 && cv2 < nv) {
      vlo = vhi = 1;
    } else {
      vlo = cv2 == nv;
      vhi = cv2 == 0;
    }
    if (!zsplit) {
      zlo = cz1 >= 0 && cz1 <= nz - 1;
      zhi = 0;
    } else if (cz2 > 0 && cz2 < nz) {
      zlo = zhi = 1;
    } else {
      zlo = cz2 == nz;
      zhi = cz2 == 0;
    }
    /* Guard against indices the reference would read out of bounds
     * (|slope|>1 cases it does not support): such pieces are skipped. */
    vlo = vlo && cv1 >= 0 && cv1 < nv;
    vhi = vhi && cv2 >= 0 && cv2 < nv;
    zlo = zlo && cz1 >= 0 && cz1 < nz;
    zhi = zhi && cz2 >= 0 && cz2 < nz;
    if (!(vlo || vhi) || !(zlo || zhi)) continue;

    const float d = v2 - v1;
    const float l = sqrtf((d * d + 1) * (len2 + dz2sq) / len2);
    const long base = (long)iu * su;
    const long ilo = base + (long)cv1 * sv, ihi = base + (long)cv2 * sv;
    const long zl = (long)cz1 * sz, zh = (long)cz2 * sz;

    if (!vsplit && !zsplit) {
      acc_piece(l, x, ilo + zl, &ys, &ss);
    } else if (!vsplit) {
      const float rz = (cz2 - w1) / (w2 - w1);
      if (zlo) acc_piece(rz * l, x, ilo + zl, &ys, &ss);
      if (zhi) acc_piece((1 - rz) * l, x, ilo + zh, &ys, &ss);
    } else if (!zsplit) {
      const float rv = (cv2 - v1) / d;
      if (vlo) acc_piece(rv * l, x, ilo + zl, &ys, &ss);
      if (vhi) acc_piece((1 - rv) * l, x, ihi + zl, &ys, &ss);
    } else {
      const float rv = (cv2 - v1) / d;
      const float rz = (cz2 - w1) / (w2 - w1);
      if (rv > rz) {
        if (vlo && zlo) acc_piece(rz * l, x, ilo + zl, &ys, &ss);
        if (vlo && zhi) acc_piece((rv - rz) * l, x, ilo + zh, &ys, &ss);
        if (vhi && zhi) acc_piece((1 - rv) * l, x, ihi + zh, &ys, &ss);
      } else {
        if (vlo && zlo) acc_piece(rv * l, x, ilo + zl, &ys, &ss);
        if (vhi && zlo) acc_piece((rz - rv) * l, x, ihi + zl, &ys, &ss);
        if (vhi && zhi) acc_piece((1 - rz) * l, x, ihi + zh, &ys, &ss);
      }
    }
  }
  *yout = ys * scale;
  *srout = ss * scale;
}

void orc_ax(const float *x, float *y, float *sr, float cos_phi, float sin_phi,
            const float *y_det, const float *z_det, float SO, float OD,
            float scale, float dz, int nx, int ny, int nz, int na, int nb,
            int nthreads) {
  const long nrays = (long)na * nb;
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthreads)
#endif
  for (long r = 0; r < nrays; r++) {
    const int ia = (int)(r % na), ib = (int)(r / na);
    ax_ray(x, &y[r], &sr[r], cos_phi, sin_phi, y_det[ia], z_det[ib], SO, OD,
           dz, nx, ny, nz, scale);
  }
  (void)nthreads;
}

/* ------------------------------------------------------------------------ */
/* Intersection length of a line with one voxel (Ax_cone_gpu.cu:16-209)      */
/* ------------------------------------------------------------------------ */

/* Up to two boundary points where the line meets the box, recorded in the
 * order the reference tests the faces. */
typedef struct {
  int n;
  float p[2][3];
} hits_t;

static inline void hit(hits_t *h, float a, float b, float c) {
  if (h->n < 2) {
    h->p[h->n][0] = a;
    h->p[h->n][1] = b;
    h->p[h->n][2] = c;
    h->n++;
  }
}

/* 2D (find_l, :16-117): line (p1,q1)->(p2,q2), box of size (dp,dq) centred
 * at (pc,qc).  Faces normal to the dominant axis are tested first, each pair
 * lower face then upper face; the first two hits define the chord. */
static float chord2(float p1, float q1, float p2, float q2, float dp,
                    float dq, float pc, float qc) {
  const float a = p2 - p1, b = q2 - q1;
  const float hp = dp / 2.0f, hq = dq / 2.0f;
  if (a == 0) return fabsf(p1 - pc) <= hp ? dq : 0.0f;
  if (b == 0) return fabsf(q1 - qc) <= hq ? dp : 0.0f;
  const float rp = p1 - pc, rq = q1 - qc;
  hits_t h;
  h.n = 0;
  for (int pass = 0; pass < 2 && h.n < 2; pass++) {
    const int pfaces = (fabsf(a) > fabsf(b)) == (pass == 0);
    if (pfaces) { /* faces p = -hp, +hp */
      const float s = b / a;
      const float t = s * (-rp) + rq, u = s * hp;
      if (fabsf(t - u) <= hq) hit(&h, -hp, t - u, 0);
      if (fabsf(t + u) <= hq) hit(&h, hp, t + u, 0);
    } else { /* faces q = -hq, +hq */
      const float s = a / b;
      const float t = s * (-rq) + rp, u = s * hq;
      if (fabsf(t - u) <= hp) hit(&h, t - u, -hq, 0);
      if (fabsf(t + u) <= hp) hit(&h, t + u, hq, 0);
    }
  }
  if (h.n < 2) return 0.0f;
  const float e0 = h.p[1][0] - h.p[0][0], e1 = h.p[1][1] - h.p[0][1];
  return sqrtf(e0 * e0 + e1 * e1);
}

/* 3D (find_l_3d, :120-209).  Unit x/y voxel size, z size dz.  Lines with no
 * x (or y) extent fall back to the 2D chord in the (y,z) (or (x,z)) plane.
 * Face order: x,y,z when |a|>|b|, else y,x,z. */
static float chord3(float x1, float y1, float z1, float x2, float y2,
                    float z2, float dz, float xc, float yc, float zc) {
  const float a = x2 - x1, b = y2 - y1, c = z2 - z1;
  const float hx = 1.0f / 2.0f, hy = 1.0f / 2.0f, hz = dz / 2.0f;
  if (a == 0) return chord2(y1, z1, y2, z2, 1.0f, dz, yc, zc);
  if (b == 0) return chord2(x1, z1, x2, z2, 1.0f, dz, xc, zc);
  const float rx = x1 - xc, ry = y1 - yc, rz = z1 - zc;
  const int xfirst = fabsf(a) > fabsf(b);
  hits_t h;
  h.n = 0;
  for (int pass = 0; pass < 3 && h.n < 2; pass++) {
    const int axis = pass == 2 ? 2 : ((pass == 0) == xfirst ? 0 : 1);
    if (axis == 0) {
      float s = b / a;
      const float t0 = s * (-rx) + ry, u0 = s * hx;
      s = c / a;
      const float t1 = s * (-rx) + rz, u1 = s * hx;
      if (fabsf(t0 - u0) <= hy && fabsf(t1 - u1) <= hz)
        hit(&h, -hx, t0 - u0, t1 - u1);
      if (fabsf(t0 + u0) <= hy && fabsf(t1 + u1) <= hz)
        hit(&h, hx, t0 + u0, t1 + u1);
    } else if (axis == 1) {
      float s = a / b;
      const float t0 = s * (-ry) + rx, u0 = s * hy;
      s = c / b;
      const float t1 = s * (-ry) + rz, u1 = s * hy;
      if (fabsf(t0 - u0) <= hx && fabsf(t1 - u1) <= hz)
        hit(&h, t0 - u0, -hy, t1 - u1);
      if (fabsf(t0 + u0) <= hx && fabsf(t1 + u1) <= hz)
        hit(&h, t0 + u0, hy, t1 + u1);
    } else {
      float s = a / c;
      const float t0 = s * (-rz) + rx, u0 = s * hz;
      s = b / c;
      const float t1 = s * (-rz) + ry, u1 = s * hz;
      if (fabsf(t0 - u0) <= hx && fabsf(t1 - u1) <= hy)
        hit(&h, t0 - u0, t1 - u1, -hz);
      if (fabsf(t0 + u0) <= hx && fabsf(t1 + u1) <= hy)
        hit(&h, t0 + u0, t1 + u1, hz);
    }
  }
  if (h.n < 2) return 0.0f;
  const float e0 = h.p[1][0] - h.p[0][0], e1 = h.p[1][1] - h.p[0][1],
              e2 = h.p[1][2] - h.p[0][2];
  return sqrtf(e0 * e0 + e1 * e1 + e2 * e2);
}

/* ------------------------------------------------------------------------ */
/* Backprojection (Ax_cone_gpu.cu:214-331)                                   */
/* ------------------------------------------------------------------------ */

void orc_atx(float *x, const float *y, float *sc, float cos_phi, float sin_phi,
             const float *y_det, const float *z_det, float SO, float OD,
             float scale, float dy_det, float dz_det, float dz, int nx, int ny,
             int nz, int na, int nb, int nthreads) {
  const long N = (long)nx * ny * nz;
  const float SD = SO + OD;
  const int na2 = na / 2, nb2 = nb / 2;
  const int nx2 = nx / 2, ny2 = ny / 2, nz2 = nz / 2;
  const float d = sqrtf((1 + dz * dz) / 2);
  const float xs = cos_phi * (-SO), ys = sin_phi * (-SO), zs = 0.0f;
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(static) num_threads(nthreads)
#endif
  for (long idx = 0; idx < N; idx++) {
    const int ix = (int)(idx % nx);
    const long iyz = idx / nx;
    const int iy = (int)(iyz % ny), iz = (int)(iyz / ny);
    const float zc = (float)(iz + 0.5 - nz2) * dz;
    const float yc = (float)(iy + 0.5 - ny2);
    const float xc = (float)(ix + 0.5 - nx2);
    const float xr = cos_phi * xc + sin_phi * yc;
    const float yr = -sin_phi * xc + cos_phi * yc;
    float t = SD / ((xr + SO) * dy_det);
    const int amax = (int)floorf((yr + 1) * t + na2);
    const int amin = (int)floorf((yr - 1) * t + na2);
    t = SD / ((xr + SO) * dz_det);
    const int bmax = (int)floorf((zc + d) * t + nb2);
    const int bmin = (int)floorf((zc - d) * t + nb2);
    float acc = 0.0f, accl = 0.0f;
    const int b0 = bmin > 0 ? bmin : 0, b1 = bmax < nb - 1 ? bmax : nb - 1;
    const int a0 = amin > 0 ? amin : 0, a1 = amax < na - 1 ? amax : na - 1;
    for (int ib = b0; ib <= b1; ib++) {
      for (int ia = a0; ia <= a1; ia++) {
        const float xd = cos_phi * OD - sin_phi * y_det[ia];
        const float yd = sin_phi * OD + cos_phi * y_det[ia];
        const float l = chord3(xs, ys, zs, xd, yd, z_det[ib], dz, xc, yc, zc);
        acc += l * y[(long)ib * na + ia];
        accl += l;
      }
    }
    x[idx] = acc * scale;
    sc[idx] = accl * scale;
  }
  (void)nthreads;
}

/* ------------------------------------------------------------------------ */
/* Gateway geometry (Ax_main_test.cpp:138-161, Atx_main_test.cpp:149-172)    */
/* ------------------------------------------------------------------------ */

void orc_gateway_geometry(double phi, double SO_mm, double OD_mm,
                          double vxlsize, double detsize, int na, int nb,
                          float *cos_phi, float *sin_phi, float *SO, float *OD,
                          float *scale, float *det, float *y_det,
                          float *z_det) {
  /* the gateway reads every para field as float, then takes cos/sin of the
   * float angle, and divides lengths by the voxel size in float */
  const float phif = (float)phi;
  const float sc = (float)vxlsize;
  *cos_phi = cosf(phif);
  *sin_phi = sinf(phif);
  *scale = sc;
  *SO = (float)SO_mm / sc;
  *OD = (float)OD_mm / sc;
  *det = (float)detsize / sc;
  for (int i = 0; i < na; i++)
    y_det[i] = (float)(((double)(float)i - (double)(float)na / 2.0 + 0.5) *
                       (double)*det);
  for (int i = 0; i < nb; i++)
    z_det[i] = (float)(((double)(float)i - (double)(float)nb / 2.0 + 0.5) *
                       (double)*det);
}

/* ------------------------------------------------------------------------ */
/* TV steepest descent (imgTVGradMin.cpp:56-119, imgTVGradMin3D.cpp:75-170)  */
/* ------------------------------------------------------------------------ */

static double sq(double v) { return v * v; }

int orc_tv2d(const double *img_in, double *img_out, int rowN, int colN,
             double alpha, int nTVIter, int pos, const double *img_old) {
  const long N = (long)rowN * colN;
  const long W = rowN + 2;
  double *u = (double *)calloc((size_t)(rowN + 2) * (colN + 2), sizeof(double));
  double *v = (double *)malloc((size_t)N * sizeof(double));
  memcpy(img_out, img_in, (size_t)N * sizeof(double));
  double d = 0;
  for (long i = 0; i < N; i++) d += sq(img_out[i] - (img_old ? img_old[i] : 0));
  d = sqrt(d);
  const double eps = 1e-8;
  for (int it = 0; it < nTVIter; it++) {
    /* zero-bordered copy, x (row index r) fastest */
    for (int c = 0; c < colN; c++)
      memcpy(&u[1 + (c + 1) * W], &img_out[(long)c * rowN],
             (size_t)rowN * sizeof(double));
    double norm = 0;
    long k = 0;
    for (int c = 1; c <= colN; c++) {
      for (int r = 1; r <= rowN; r++, k++) {
        const double c0 = u[r + c * W];
        const double xm = u[r - 1 + c * W], ym = u[r + (c - 1) * W];
        const double xp = u[r + 1 + c * W], yp = u[r + (c + 1) * W];
        const double xpym = u[r + 1 + (c - 1) * W];
        const double xmyp = u[r - 1 + (c + 1) * W];
        const double g1 = ((c0 - xm) + (c0 - ym)) /
                          sqrt(eps + sq(c0 - xm) + sq(c0 - ym));
        const double g2 = -(xp - c0) / sqrt(eps + sq(xp - c0) + sq(xp - xpym));
        const double g3 = -(yp - c0) / sqrt(eps + sq(yp - c0) + sq(yp - xmyp));
        v[k] = g1 + g2 + g3;
        norm += v[k] * v[k];
      }
    }
    norm = sqrt(norm);
    for (long i = 0; i < N; i++) img_out[i] -= alpha * d * v[i] / norm;
  }
  if (pos == 1 && nTVIter > 0)
    for (long i = 0; i < N; i++)
      if (img_out[i] < 0) img_out[i] = 0;
  free(u);
  free(v);
  return 0;
}

int orc_tv3d(const double *img_in, double *img_out, int Nx, int Ny, int Nz,
             double alpha, int nTVIter, int pos, const double *img_old,
             int nthreads) {
  const long N = (long)Nx * Ny * Nz;
  /* zero-bordered copy in image order (x fastest); the reference stores its
   * padded copy with y fastest, which does not change any value */
  const long PX = Nx + 2, PY = Ny + 2;
  const long SX = 1, SY = PX, SZ = PX * PY;
  double *u = (double *)calloc((size_t)PX * PY * (Nz + 2), sizeof(double));
  double *v = (double *)malloc((size_t)N * sizeof(double));
  memcpy(img_out, img_in, (size_t)N * sizeof(double));
  double d = 0;
  for (long i = 0; i < N; i++) d += sq(img_out[i] - (img_old ? img_old[i] : 0));
  d = sqrt(d);
  const double eps = 1e-8;
  (void)nthreads;
  for (int it = 0; it < nTVIter; it++) {
    for (int z = 0; z < Nz; z++)
      for (int y = 0; y < Ny; y++)
        memcpy(&u[1 + (y + 1) * SY + (z + 1) * SZ],
               &img_out[(long)y * Nx + (long)z * Nx * Ny],
               (size_t)Nx * sizeof(double));
#ifdef _OPENMP
    int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
#pragma omp parallel for schedule(static) num_threads(nt)
#endif
    for (int z = 1; z <= Nz; z++) {
      for (int y = 1; y <= Ny; y++) {
        for (int x = 1; x <= Nx; x++) {
          const long p = x * SX + y * SY + z * SZ;
          const double c0 = u[p];
          const double xm = u[p - SX], ym = u[p - SY], zm = u[p - SZ];
          const double xp = u[p + SX], yp = u[p + SY], zp = u[p + SZ];
          const double xm_zp = u[p - SX + SZ], ym_zp = u[p - SY + SZ];
          const double xm_yp = u[p - SX + SY], yp_zm = u[p + SY - SZ];
          const double xp_ym = u[p + SX - SY], xp_zm = u[p + SX - SZ];
          const double g1 = (6 * c0 - 2 * (xm + ym + zm)) /
                            sqrt(eps + sq(c0 - xm) + sq(c0 - ym) + sq(c0 - zm));
          const double g2 = (2 * c0 - 2 * zp) /
                            sqrt(eps + sq(zp - xm_zp) + sq(zp - ym_zp) +
                                 sq(zp - c0));
          const double g3 = (2 * c0 - 2 * yp) /
                            sqrt(eps + sq(yp - xm_yp) + sq(yp - c0) +
                                 sq(yp - yp_zm));
          const double g4 = (2 * c0 - 2 * xp) /
                            sqrt(eps + sq(xp - c0) + sq(xp - xp_ym) +
                                 sq(xp - xp_zm));
          v[(x - 1) + (long)(y - 1) * Nx + (long)(z - 1) * Nx * Ny] =
              g1 + g2 + g3 + g4;
        }
      }
    }
    double norm = 0;
    for (long i = 0; i < N; i++) norm += v[i] * v[i];
    norm = sqrt(norm);
    for (long i = 0; i < N; i++) img_out[i] -= alpha * d * v[i] / norm;
  }
  if (pos == 1 && nTVIter > 0)
    for (long i = 0; i < N; i++)
      if (img_out[i] < 0) img_out[i] = 0;
  free(u);
  free(v);
  return 0;
}

int orc_tv_any(const double *img_in, double *img_out, int nx, int ny, int nz,
               double alpha, int nTVIter, int pos, const double *img_old,
               int nthreads) {
  if (nz >= 2)
    return orc_tv3d(img_in, img_out, nx, ny, nz, alpha, nTVIter, pos, img_old,
                    nthreads);
  return orc_tv2d(img_in, img_out, nx, ny, alpha, nTVIter, pos, img_old);
}

/* ------------------------------------------------------------------------ */
/* Exact FP64 Siddon (test oracle for intersection lengths)                  */
/* ------------------------------------------------------------------------ */

static int cmp_d(const void *a, const void *b) {
  const double x = *(const double *)a, y = *(const double *)b;
  return (x > y) - (x < y);
}

/* Visit every (voxel, length) of one ray in FP64.  Grid planes: x = i-nx/2,
 * y = j-ny/2 (integer halves), z = (k-nz/2)*dz.  Planar rays ignore z. */
typedef void (*visit_fn)(void *ctx, long idx, double len);

static void siddon_ray(double xs, double ys, double zs, double xd, double yd,
                       double zd, double dz, int nx, int ny, int nz,
                       int planar, double *buf, visit_fn f, void *ctx) {
  const double P0[3] = {xs, ys, zs}, P1[3] = {xd, yd, zd};
  const double lo[3] = {(double)(0 - nx / 2), (double)(0 - ny / 2),
                        (double)(0 - nz / 2) * dz};
  const int n[3] = {nx, ny, nz};
  const double h[3] = {1.0, 1.0, dz};
  const int naxes = planar ? 2 : 3;
  double amin = 0.0, amax = 1.0;
  for (int k = 0; k < naxes; k++) {
    const double dk = P1[k] - P0[k];
    const double b0 = lo[k], b1 = lo[k] + n[k] * h[k];
    if (dk == 0) {
      if (P0[k] < b0 || P0[k] > b1) return;
      continue;
    }
    double t0 = (b0 - P0[k]) / dk, t1 = (b1 - P0[k]) / dk;
    if (t0 > t1) {
      const double t = t0;
      t0 = t1;
      t1 = t;
    }
    if (t0 > amin) amin = t0;
    if (t1 < amax) amax = t1;
  }
  if (amax <= amin) return;
  int m = 0;
  buf[m++] = amin;
  buf[m++] = amax;
  for (int k = 0; k < naxes; k++) {
    const double dk = P1[k] - P0[k];
    if (dk == 0) continue;
    for (int i = 0; i <= n[k]; i++) {
      const double t = (lo[k] + i * h[k] - P0[k]) / dk;
      if (t > amin && t < amax) buf[m++] = t;
    }
  }
  qsort(buf, (size_t)m, sizeof(double), cmp_d);
  double L = 0;
  for (int k = 0; k < naxes; k++) L += (P1[k] - P0[k]) * (P1[k] - P0[k]);
  L = sqrt(L);
  for (int i = 0; i + 1 < m; i++) {
    const double t0 = buf[i], t1 = buf[i + 1];
    if (t1 <= t0) continue;
    const double tm = 0.5 * (t0 + t1);
    int c[3] = {0, 0, 0};
    int ok = 1;
    for (int k = 0; k < naxes; k++) {
      c[k] = (int)floor((P0[k] + tm * (P1[k] - P0[k]) - lo[k]) / h[k]);
      if (c[k] < 0 || c[k] >= n[k]) ok = 0;
    }
    if (!ok) continue;
    const long idx = (long)c[2] * nx * ny + (long)c[1] * nx + c[0];
    f(ctx, idx, (t1 - t0) * L);
  }
}

typedef struct {
  const float *x;
  double y, s;
} fwd_ctx;
static void fwd_visit(void *vc, long idx, double len) {
  fwd_ctx *c = (fwd_ctx *)vc;
  c->y += len * (double)c->x[idx];
  c->s += len;
}
typedef struct {
  double *x, *sc;
  double yv;
} bwd_ctx;
static void bwd_visit(void *vc, long idx, double len) {
  bwd_ctx *c = (bwd_ctx *)vc;
  c->x[idx] += len * c->yv;
  c->sc[idx] += len;
}
typedef struct {
  long long n;
} cnt_ctx;
static void cnt_visit(void *vc, long idx, double len) {
  (void)idx;
  if (len > 0) ((cnt_ctx *)vc)->n++;
}

static void ray_ends(float cos_phi, float sin_phi, float SO, float OD,
                     float yd, float zd, double *P) {
  P[0] = (double)cos_phi * -(double)SO;
  P[1] = (double)sin_phi * -(double)SO;
  P[2] = 0.0;
  P[3] = (double)cos_phi * OD - (double)sin_phi * yd;
  P[4] = (double)sin_phi * OD + (double)cos_phi * yd;
  P[5] = zd;
}

void orc_siddon_ax_f64(const float *x, double *y, double *sr, float cos_phi,
                       float sin_phi, const float *y_det, const float *z_det,
                       float SO, float OD, float scale, float dz, int nx, int ny,
                       int nz, int na, int nb) {
  const int planar = nz == 1 && nb == 1;
  double *buf = (double *)malloc(sizeof(double) * (size_t)(nx + ny + nz + 8));
  for (int ib = 0; ib < nb; ib++)
    for (int ia = 0; ia < na; ia++) {
      double P[6];
      ray_ends(cos_phi, sin_phi, SO, OD, y_det[ia], z_det[ib], P);
      fwd_ctx c = {x, 0, 0};
      siddon_ray(P[0], P[1], planar ? 0 : P[2], P[3], P[4], planar ? 0 : P[5],
                 dz, nx, ny, nz, planar, buf, fwd_visit, &c);
      y[(long)ib * na + ia] = c.y * scale;
      sr[(long)ib * na + ia] = c.s * scale;
    }
  free(buf);
}

void orc_siddon_atx_f64(double *x, const double *y, double *sc, float cos_phi,
                        float sin_phi, const float *y_det, const float *z_det,
                        float SO, float OD, float scale, float dz, int nx,
                        int ny, int nz, int na, int nb) {
  const int planar = nz == 1 && nb == 1;
  const long N = (long)nx * ny * nz;
  memset(x, 0, sizeof(double) * (size_t)N);
  memset(sc, 0, sizeof(double) * (size_t)N);
  double *buf = (double *)malloc(sizeof(double) * (size_t)(nx + ny + nz + 8));
  for (int ib = 0; ib < nb; ib++)
    for (int ia = 0; ia < na; ia++) {
      double P[6];
      ray_ends(cos_phi, sin_phi, SO, OD, y_det[ia], z_det[ib], P);
      bwd_ctx c = {x, sc, y[(long)ib * na + ia]};
      siddon_ray(P[0], P[1], planar ? 0 : P[2], P[3], P[4], planar ? 0 : P[5],
                 dz, nx, ny, nz, planar, buf, bwd_visit, &c);
    }
  for (long i = 0; i < N; i++) {
    x[i] *= scale;
    sc[i] *= scale;
  }
  free(buf);
}

long long orc_siddon_nnz(float cos_phi, float sin_phi, const float *y_det,
                         const float *z_det, float SO, float OD, float dz,
                         int nx, int ny, int nz, int na, int nb) {
  const int planar = nz == 1 && nb == 1;
  double *buf = (double *)malloc(sizeof(double) * (size_t)(nx + ny + nz + 8));
  cnt_ctx c = {0};
  for (int ib = 0; ib < nb; ib++)
    for (int ia = 0; ia < na; ia++) {
      double P[6];
      ray_ends(cos_phi, sin_phi, SO, OD, y_det[ia], z_det[ib], P);
      siddon_ray(P[0], P[1], planar ? 0 : P[2], P[3], P[4], planar ? 0 : P[5],
                 dz, nx, ny, nz, planar, buf, cnt_visit, &c);
    }
  free(buf);
  return c.n;
}

/* The FP64 Siddon projection in the driver's forward-projector form (FP32
 * outputs): the oracle of the library's exact forward mode. */
void orc_ax_siddon_for_driver(const float *x, float *y, float *sr, float c, float s,
                              const float *yd, const float *zd, float SO, float OD,
                              float sc, float dz, int nx, int ny, int nz, int na, int nb,
                              int nt) {
  (void)nt;
  const long M = (long)na * nb;
  double *yy = (double *)malloc(sizeof(double) * (size_t)M);
  double *ss = (double *)malloc(sizeof(double) * (size_t)M);
  orc_siddon_ax_f64(x, yy, ss, c, s, yd, zd, SO, OD, sc, dz, nx, ny, nz, na, nb);
  for (long i = 0; i < M; i++) {
    y[i] = (float)yy[i];
    sr[i] = (float)ss[i];
  }
  free(yy);
  free(ss);
}

/* ------------------------------------------------------------------------ */
/* ASD-POCS driver (ASD_POCS_cuda.m:97-182), FP64 image state                 */
/* ------------------------------------------------------------------------ */

static void orc_ax_default(const float *x, float *y, float *sr, float c,
                           float s, const float *yd, const float *zd, float SO,
                           float OD, float sc, float dz, int nx, int ny,
                           int nz, int na, int nb, int nt) {
  orc_ax(x, y, sr, c, s, yd, zd, SO, OD, sc, dz, nx, ny, nz, na, nb, nt);
}
static void orc_atx_default(float *x, const float *y, float *scv, float c,
                            float s, const float *yd, const float *zd,
                            float SO, float OD, float sc, float ddy,
                            float ddz, float dz, int nx, int ny, int nz,
                            int na, int nb, int nt) {
  orc_atx(x, y, scv, c, s, yd, zd, SO, OD, sc, ddy, ddz, dz, nx, ny, nz, na,
          nb, nt);
}

/* One SART sweep over all views (ASD_POCS_cuda.m:110-134 ==
 * SART_cuda_inline.m:63-87).  m is updated in place; returns dd2. */
static double sart_sweep(const double *P, const double *phi_vec,
                         const orc_asd_params *p, double beta, double *m,
                         float *mf, float *proj, float *sumR, float *cor,
                         float *bproj, float *sumC, float *ydet, float *zdet,
                         int nthreads, orc_ax_fn ax, orc_atx_fn atx) {
  const long N = (long)p->nx * p->ny * p->nz;
  const long M = (long)p->na * p->nb;
  double dd2 = 0;
  for (int ii = 0; ii < p->nv; ii++) {
    /* theta_i = phi_vec(ii)/180*pi; para.phi = -1*theta_i */
    const double theta = phi_vec[ii] / 180.0 * 3.14159265358979323846;
    float c, s, SO, OD, scale, det;
    orc_gateway_geometry(-1 * theta, p->SO, p->OD, p->vxlsize, p->detsize,
                         p->na, p->nb, &c, &s, &SO, &OD, &scale, &det, ydet,
                         zdet);
    for (long i = 0; i < N; i++) mf[i] = (float)m[i];
    ax(mf, proj, sumR, c, s, ydet, zdet, SO, OD, scale, 1.0f, p->nx, p->ny,
       p->nz, p->na, p->nb, nthreads);
    double n2 = 0;
    const double *Pv = P + (long)ii * M;
    for (long r = 0; r < M; r++) {
      const double sr = sumR[r] == 0 ? 1.0 : (double)sumR[r];
      const double c0 = Pv[r] - (double)proj[r];
      n2 += c0 * c0;
      cor[r] = (float)(c0 / sr);
    }
    dd2 += n2;
    atx(bproj, cor, sumC, c, s, ydet, zdet, SO, OD, scale, det, det, 1.0f,
        p->nx, p->ny, p->nz, p->na, p->nb, nthreads);
    for (long i = 0; i < N; i++) {
      const double scv = sumC[i] == 0 ? 1.0 : (double)sumC[i];
      double v = m[i] + beta * ((double)bproj[i] / scv);
      m[i] = v < 0 ? 0 : v;
    }
  }
  return dd2;
}

static double dnorm(const double *a, const double *b, long n) {
  double s = 0;
  for (long i = 0; i < n; i++) s += (a[i] - b[i]) * (a[i] - b[i]);
  return sqrt(s);
}

static int tv_default(const double *in, double *out, int nx, int ny, int nz,
                      double alpha, int n, int pos, const double *old,
                      int nthreads) {
  return orc_tv_any(in, out, nx, ny, nz, alpha, n, pos, old, nthreads);
}

int orc_asdpocs_with(const double *P, const double *phi_vec,
                     const orc_asd_params *p, const double *m0,
                     const double *I0, double *m_res, double *rmse,
                     orc_asd_out *out, int nthreads, orc_ax_fn ax,
                     orc_atx_fn atx, orc_tv_fn tv) {
  const long N = (long)p->nx * p->ny * p->nz;
  const long M = (long)p->na * p->nb;
  double *m = (double *)calloc((size_t)N, sizeof(double));
  double *m_pre = (double *)malloc(sizeof(double) * (size_t)N);
  double *m_k1 = (double *)malloc(sizeof(double) * (size_t)N);
  double *f0 = (double *)malloc(sizeof(double) * (size_t)N);
  float *mf = (float *)malloc(sizeof(float) * (size_t)N);
  float *bproj = (float *)malloc(sizeof(float) * (size_t)N);
  float *sumC = (float *)malloc(sizeof(float) * (size_t)N);
  float *proj = (float *)malloc(sizeof(float) * (size_t)M);
  float *sumR = (float *)malloc(sizeof(float) * (size_t)M);
  float *cor = (float *)malloc(sizeof(float) * (size_t)M);
  float *ydet = (float *)malloc(sizeof(float) * (size_t)p->na);
  float *zdet = (float *)malloc(sizeof(float) * (size_t)p->nb);
  if (!ax) ax = orc_ax_default;
  if (!atx) atx = orc_atx_default;
  if (!tv) tv = tv_default;
  if (m0) memcpy(m, m0, sizeof(double) * (size_t)N);
  double alpha = p->alpha, beta = p->beta, dd2 = 0;
  int k;
  for (k = 1; k <= p->maxnumIter; k++) {
    memcpy(m_pre, m, sizeof(double) * (size_t)N);
    dd2 = sart_sweep(P, phi_vec, p, beta, m, mf, proj, sumR, cor, bproj, sumC,
                     ydet, zdet, nthreads, ax, atx);
    const double dd = sqrt(dd2);
    memcpy(m_res, m, sizeof(double) * (size_t)N);
    if (I0 && rmse) {
      double s = 0;
      for (long i = 0; i < N; i++) s += (m[i] - I0[i]) * (m[i] - I0[i]);
      rmse[k - 1] = sqrt(s / (double)N);
    }
    const double dp = dnorm(m, m_pre, N);
    if (dp / (double)N <= p->stopRelChg) break;
    if (k == 1) memcpy(m_k1, m_pre, sizeof(double) * (size_t)N);
    memcpy(f0, m, sizeof(double) * (size_t)N);
    tv(f0, m, p->nx, p->ny, p->nz, alpha, p->ng, 1, m_k1, nthreads);
    const double dg = dnorm(m, f0, N);
    if (dg > p->r_max * dp && dd > p->epsilon) alpha = alpha * p->alpha_red;
    beta = beta * p->beta_red;
  }
  if (k > p->maxnumIter) k = p->maxnumIter;
  if (out) {
    out->iterations = k;
    out->dataTolerance = dd2;
    out->alpha = alpha;
    out->beta = beta;
  }
  free(m);
  free(m_pre);
  free(m_k1);
  free(f0);
  free(mf);
  free(bproj);
  free(sumC);
  free(proj);
  free(sumR);
  free(cor);
  free(ydet);
  free(zdet);
  return 0;
}

int orc_asdpocs(const double *P, const double *phi_vec, const orc_asd_params *p,
                const double *m0, const double *I0, double *m_res, double *rmse,
                orc_asd_out *out, int nthreads) {
  return orc_asdpocs_with(P, phi_vec, p, m0, I0, m_res, rmse, out, nthreads,
                          0, 0, 0);
}

int orc_sart(const double *P, const double *phi_vec, const orc_asd_params *p,
             double lambda, const double *m0, double *m_out, double *datatol,
             int nthreads) {
  const long N = (long)p->nx * p->ny * p->nz;
  const long M = (long)p->na * p->nb;
  float *mf = (float *)malloc(sizeof(float) * (size_t)N);
  float *bproj = (float *)malloc(sizeof(float) * (size_t)N);
  float *sumC = (float *)malloc(sizeof(float) * (size_t)N);
  float *proj = (float *)malloc(sizeof(float) * (size_t)M);
  float *sumR = (float *)malloc(sizeof(float) * (size_t)M);
  float *cor = (float *)malloc(sizeof(float) * (size_t)M);
  float *ydet = (float *)malloc(sizeof(float) * (size_t)p->na);
  float *zdet = (float *)malloc(sizeof(float) * (size_t)p->nb);
  if (m0)
    memcpy(m_out, m0, sizeof(double) * (size_t)N);
  else
    memset(m_out, 0, sizeof(double) * (size_t)N);
  const double dt =
      sart_sweep(P, phi_vec, p, lambda, m_out, mf, proj, sumR, cor, bproj,
                 sumC, ydet, zdet, nthreads, orc_ax_default, orc_atx_default);
  if (datatol) *datatol = dt;
  free(mf);
  free(bproj);
  free(sumC);
  free(proj);
  free(sumR);
  free(cor);
  free(ydet);
  free(zdet);
  return 0;
}
