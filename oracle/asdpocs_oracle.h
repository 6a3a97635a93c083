/*
 * CPU oracle for the ASD-POCS hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * This is a plain-C restatement of the reference's projector, TV and
 * ASD-POCS driver semantics, used by tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference legs of bench.py as the checker.  The product
 * library never links, loads or calls it.
 *
 * Parity pin: the restatement is checked against the reference's own
 * src/AxAtx and src/tvmin code built for the host (oracle/build_ref.sh) and
 * against golden vectors produced by that build (tests/golden/).
 *
 * Float semantics: compiled with -ffp-contract=off so every float operation
 * is rounded exactly as written (no fused multiply-add), in the same order as
 * the reference expressions.
 */
#ifndef ASDPOCS_ORACLE_H
#define ASDPOCS_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Ax_cone_gpu.cu:339-776 -- ray-driven projection of one view. */
void orc_ax(const float *x, float *y, float *sr, float cos_phi, float sin_phi,
            const float *y_det, const float *z_det, float SO, float OD,
            float scale, float dz, int nx, int ny, int nz, int na, int nb,
            int nthreads);

/* Ax_cone_gpu.cu:214-331 -- voxel-driven backprojection of one view
 * (x, sc are outputs, y is the input view). */
void orc_atx(float *x, const float *y, float *sc, float cos_phi, float sin_phi,
             const float *y_det, const float *z_det, float SO, float OD,
             float scale, float dy_det, float dz_det, float dz, int nx, int ny,
             int nz, int na, int nb, int nthreads);

/* imgTVGradMin.cpp:16-140 (2D) and imgTVGradMin3D.cpp:18-189 (3D).
 * img_old may be NULL (zeros).  Returns 0. */
int orc_tv2d(const double *img_in, double *img_out, int rowN, int colN,
             double alpha, int nTVIter, int pos, const double *img_old);
int orc_tv3d(const double *img_in, double *img_out, int Nx, int Ny, int Nz,
             double alpha, int nTVIter, int pos, const double *img_old,
             int nthreads);

/* Ax_main_test.cpp:138-161 / Atx_main_test.cpp:149-172: conversion of the
 * para struct to the launcher arguments (voxel units, detector coordinates). */
void orc_gateway_geometry(double phi, double SO_mm, double OD_mm,
                          double vxlsize, double detsize, int na, int nb,
                          float *cos_phi, float *sin_phi, float *SO, float *OD,
                          float *scale, float *det, float *y_det, float *z_det);

/* Exact line/voxel intersection (Siddon, FP64).  Planar (nz==1 && nb==1) rays
 * are intersected with the pixel grid only; otherwise with the voxel grid. */
void orc_siddon_ax_f64(const float *x, double *y, double *sr, float cos_phi,
                       float sin_phi, const float *y_det, const float *z_det,
                       float SO, float OD, float scale, float dz, int nx, int ny,
                       int nz, int na, int nb);
void orc_siddon_atx_f64(double *x, const double *y, double *sc, float cos_phi,
                        float sin_phi, const float *y_det, const float *z_det,
                        float SO, float OD, float scale, float dz, int nx,
                        int ny, int nz, int na, int nb);
/* Number of (ray, voxel) pairs with positive exact intersection length. */
long long orc_siddon_nnz(float cos_phi, float sin_phi, const float *y_det,
                         const float *z_det, float SO, float OD, float dz,
                         int nx, int ny, int nz, int na, int nb);

/* ASD_POCS_cuda.m:20-182 with FP64 image state, as in MATLAB. */
typedef struct {
  int nx, ny, nz, na, nb, nv;
  double SO, OD, vxlsize, detsize; /* mm, as in the para struct */
  int maxnumIter, ng;
  double alpha, alpha_red, beta, beta_red, r_max, epsilon, stopRelChg;
} orc_asd_params;

typedef struct {
  int iterations;       /* out.IterationNum */
  double dataTolerance; /* out.dataTolerance (dd2 of the last sweep) */
  double alpha, beta;   /* out.alpha / out.beta */
} orc_asd_out;

/* Pluggable projector/TV implementations, so the same driver runs either the
 * oracle's own restatement or the reference's host-built code. */
typedef void (*orc_ax_fn)(const float *, float *, float *, float, float,
                          const float *, const float *, float, float, float,
                          float, int, int, int, int, int, int);
typedef void (*orc_atx_fn)(float *, const float *, float *, float, float,
                           const float *, const float *, float, float, float,
                           float, float, float, int, int, int, int, int, int);
typedef int (*orc_tv_fn)(const double *, double *, int, int, int, double, int,
                         int, const double *, int);

/* P: (na*nb) x nv column-major; phi_vec in degrees; m0 may be NULL (zeros);
 * I0 may be NULL (no RMSE); rmse (length maxnumIter) may be NULL.
 * m_res receives the post-SART, pre-TV image of the last iteration. */
int orc_asdpocs(const double *P, const double *phi_vec, const orc_asd_params *p,
                const double *m0, const double *I0, double *m_res, double *rmse,
                orc_asd_out *out, int nthreads);
int orc_asdpocs_with(const double *P, const double *phi_vec,
                     const orc_asd_params *p, const double *m0,
                     const double *I0, double *m_res, double *rmse,
                     orc_asd_out *out, int nthreads, orc_ax_fn ax,
                     orc_atx_fn atx, orc_tv_fn tv);

/* SART_cuda_inline.m:17-108: one sweep with relaxation lambda. */
int orc_sart(const double *P, const double *phi_vec, const orc_asd_params *p,
             double lambda, const double *m0, double *m_out, double *datatol,
             int nthreads);

/* Unified TV entry point used by the driver: nz==1 -> 2D, else 3D. */
int orc_tv_any(const double *img_in, double *img_out, int nx, int ny, int nz,
               double alpha, int nTVIter, int pos, const double *img_old,
               int nthreads);

#ifdef __cplusplus
}
#endif
#endif
