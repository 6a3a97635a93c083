/*
 * asdpocs_gb300 -- C ABI of the GB300 (sm_103a) ASD-POCS hot path.
 *
 * Drop-in boundary for the reference's projector / TV / ASD-POCS path
 * (imagereconstruction/ASD_POCS_mex_cuda_demo).  Every entry point is plain C:
 * pointers, sizes and scalars only.
 *
 * Layouts (identical to the reference):
 *   volume   x-fastest, idx = iz*ny*nx + iy*nx + ix   (Ax_cone_gpu.cu:237),
 *            i.e. a MATLAB column-major [nx,ny,nz] array;
 *   view     na*nb values, ia fastest, id = ib*na + ia   (Ax_cone_gpu.cu:360);
 *   sinogram (na*nb) x nv column-major: view ii is contiguous
 *            (ASD_POCS_cuda.m:121, P(:,ii)).
 * Geometry at the launcher level is in voxel units (SO, OD, detector
 * coordinates divided by the voxel size; Ax_main_test.cpp:141-161).
 *
 * Error behaviour: functions returning int return ASDPOCS_OK (0) or an
 * asdpocs_status code; asdpocs_last_error() gives the message of the last
 * failure on the calling thread.  The two launcher drop-ins keep the
 * reference's void signatures; failures there are reported through
 * asdpocs_last_status()/asdpocs_last_error().
 */
#ifndef ASDPOCS_GB300_H
#define ASDPOCS_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  ASDPOCS_OK = 0,
  ASDPOCS_ERR_ARG = 1,     /* bad argument / size mismatch (mexErrMsgTxt)  */
  ASDPOCS_ERR_CUDA = 2,    /* CUDA runtime error                           */
  ASDPOCS_ERR_NOMEM = 3,   /* device allocation failed / over HBM budget   */
  ASDPOCS_ERR_STATE = 4,   /* call not valid in the object's current state */
  ASDPOCS_ERR_TIMEOUT = 5, /* a bounded device-side wait gave up           */
  ASDPOCS_ERR_NODEV = 6    /* no CUDA device                               */
} asdpocs_status;

/* Message / status of the last failed call on this thread ("" / 0 if none). */
const char *asdpocs_last_error(void);
int asdpocs_last_status(void);
/* Library version string. */
const char *asdpocs_version(void);

/* Bounds-checked build only (libasdpocs_gb300_checked.so, compiled with
 * ASDPOCS_CHECKED; no counterpart in the reference, which checks nothing):
 * the number of out-of-range volume, sinogram, residual and table indices
 * the projector and TV kernels met since the last call (each such access
 * was skipped), and the first one with its extent in first[0], first[1].
 * Synchronises the device; clears the counts.  The normal build returns
 * ASDPOCS_ERR_STATE. */
int asdpocs_checked_errors(unsigned long long *count, long long first[2]);

/* ------------------------------------------------------------------ */
/* Launcher drop-ins: identical signatures to the reference            */
/* ------------------------------------------------------------------ */

/* Replaces Ax_cone_mf_gpu_new (src/AxAtx/Ax_cone_gpu.cu:778-805).
 * Host pointers; synchronous.  X: nx*ny*nz volume (input); y, sr: na*nb
 * projection and ray sums (outputs); y_det[na], z_det[nb] detector
 * coordinates; SO, OD in voxel units; scale = voxel size. */
void Ax_cone_mf_gpu_new(float *X, float *y, float *sr, float cos_phi,
                        float sin_phi, float *y_det, float *z_det, float SO,
                        float OD, float scale, float dz, int nx, int ny, int nz,
                        int na, int nb);

/* Replaces Atx_cone_mf_gpu_new (src/AxAtx/Ax_cone_gpu.cu:299-331).
 * Host pointers; synchronous.  Note the reference's naming: X (nx*ny*nz)
 * and sc are OUTPUTS, y (na*nb) is the input view. */
void Atx_cone_mf_gpu_new(float *X, float *y, float *sc, float cos_phi,
                         float sin_phi, float *y_det, float *z_det, float SO,
                         float OD, float scale, float dy_det, float dz_det,
                         float dz, int nx, int ny, int nz, int na, int nb);

/* ------------------------------------------------------------------ */
/* Device-pointer variants (no copies; enqueued on `stream`)           */
/* ------------------------------------------------------------------ */

/* Same computation as Ax_cone_mf_gpu_new on device buffers.  stream is a
 * cudaStream_t (NULL = legacy default stream).  Asynchronous. */
int asdpocs_ax_device(const float *x_d, float *y_d, float *sr_d, float cos_phi,
                      float sin_phi, const float *y_det_d,
                      const float *z_det_d, float SO, float OD, float scale,
                      float dz, int nx, int ny, int nz, int na, int nb,
                      void *stream);

/* Exact forward projection (no counterpart in the reference, whose 3-D
 * column march approximates the voxel chords): Siddon's method, the length
 * of the ray inside every voxel it crosses, with FP64 plane-crossing
 * parameters, FP32 lengths and FP32 sums.  Same arguments and outputs as
 * Ax_cone_mf_gpu_new (host buffers, synchronous) / asdpocs_ax_device (device
 * buffers, asynchronous on `stream`).  In 2-D it agrees with the reference
 * march to FP32 rounding. */
int asdpocs_ax_siddon(const float *X, float *y, float *sr, float cos_phi,
                      float sin_phi, const float *y_det, const float *z_det,
                      float SO, float OD, float scale, float dz, int nx, int ny,
                      int nz, int na, int nb);
int asdpocs_ax_siddon_device(const float *x_d, float *y_d, float *sr_d, float cos_phi,
                             float sin_phi, const float *y_det_d, const float *z_det_d,
                             float SO, float OD, float scale, float dz, int nx, int ny,
                             int nz, int na, int nb, void *stream);

/* Same computation as Atx_cone_mf_gpu_new on device buffers (x_d, sc_d
 * outputs, y_d input).  Asynchronous. */
int asdpocs_atx_device(float *x_d, const float *y_d, float *sc_d,
                       float cos_phi, float sin_phi, const float *y_det_d,
                       const float *z_det_d, float SO, float OD, float scale,
                       float dy_det, float dz_det, float dz, int nx, int ny,
                       int nz, int na, int nb, void *stream);

/* Adjoint consistency of one view's projector pair, the launcher-level
 * arguments as above (all pointers on the host): dots[0] = <A x, y> and
 * dots[1] = <x, A^T y>, both accumulated in FP64 on the GPU in a fixed
 * order.  A and A^T carry the same `scale`, so the two agree to the FP32
 * rounding of the projections.  Synchronous. */
int asdpocs_adjoint_check(const float *X, const float *y, float cos_phi, float sin_phi,
                          const float *y_det, const float *z_det, float SO, float OD,
                          float scale, float dy_det, float dz_det, float dz, int nx,
                          int ny, int nz, int na, int nb, double dots[2]);

/* ------------------------------------------------------------------ */
/* mex-level entry points (the para struct as a C struct)              */
/* ------------------------------------------------------------------ */

/* The fields the gateways read (Ax_main_test.cpp:48-126); lengths in mm,
 * phi in radians (scalar). */
typedef struct {
  double SO, OD, vxlsize, detsize, phi;
  int nx, ny, nz, na, nb;
} asdpocs_para;

/* [y,sr] = Ax_cone_gpu(single X, para)   (Ax_main_test.cpp:19-164).
 * numel_X is checked against nx*ny*nz ("Error size of input argument X!").
 * Host pointers; y, sr have na*nb elements. */
int Ax_cone_gpu(const float *X, long long numel_X, const asdpocs_para *para,
                float *y, float *sr);

/* [x,sc] = Atx_cone_gpu(single Y, para)  (Atx_main_test.cpp:20-176).
 * numel_Y is checked against na*nb.  x, sc have nx*ny*nz elements. */
int Atx_cone_gpu(const float *Y, long long numel_Y, const asdpocs_para *para,
                 float *x, float *sc);

/* The adjoint check (asdpocs_adjoint_check) of the view described by para:
 * dots[0] = <Ax_cone_gpu(X), Y>, dots[1] = <X, Atx_cone_gpu(Y)>, FP64 on the
 * GPU.  numel checks as above. */
int asdpocs_adjoint_check_para(const float *X, long long numel_X, const float *Y,
                               long long numel_Y, const asdpocs_para *para,
                               double dots[2]);

/* I2 = imgTVGradMin(I, alpha, nTVIter, pos[, I0])   (imgTVGradMin.cpp:16-140)
 * I: rowN x colN double, column-major; img_old may be NULL (zeros).
 * Computed on the GPU in FP64. */
int imgTVGradMin(const double *img, double *img_out, int rowN, int colN,
                 double alpha, int nTVIter, int pos, const double *img_old);

/* I2 = imgTVGradMin3D(I, alpha, nTVIter, pos[, I0]) (imgTVGradMin3D.cpp:18-189)
 * I: Nx x Ny x Nz double, column-major.  FP64 on the GPU. */
int imgTVGradMin3D(const double *img, double *img_out, int Nx, int Ny, int Nz,
                   double alpha, int nTVIter, int pos, const double *img_old);

/* FP32 device variants of the TV minimisation (in place on img_d). */
int asdpocs_tv_device(float *img_d, const float *img_old_d, int nx, int ny,
                      int nz, double alpha, int nTVIter, int pos, void *stream);

/* Allocation-free form of asdpocs_tv_device (no counterpart in the
 * reference).  For callers that cannot call cudaMalloc -- an external
 * allocator that owns device memory, a fixed memory budget, or a real-time
 * loop that must not stall on an allocation: the work images and reduction
 * scratch live in a fixed array of about 8.5 MB that every GPU loading the
 * library holds until exit.  Images are limited to nx*ny*nz <= 1,048,576
 * voxels, to 65,536 tiles of 32 x 8 voxels and to 65,535 tile rows
 * (ceil(ny/8) * nz); others are rejected with ASDPOCS_ERR_ARG.  Asynchronous on
 * `stream`; the first call on a device looks up the array's address and
 * should come before any stream capture.  All calls share the array, so
 * calls that overlap on the GPU race. */
int asdpocs_tv_device_noalloc(float *img_d, const float *img_old_d, int nx,
                              int ny, int nz, double alpha, int nTVIter,
                              int pos, void *stream);

/* ------------------------------------------------------------------ */
/* ASD-POCS reconstruction jobs (device resident)                      */
/* ------------------------------------------------------------------ */

/* Device storage of a job's sinogram (asdpocs_options.sino_storage).  The
 * reference keeps P in double and passes single-precision views to the GPU
 * (Ax_main_test.cpp:45); here it is stored once on the device in FP32 or, to
 * halve its bytes, rounded to nearest (ties to even) to FP16 or BF16.  Every
 * read widens it to FP32; ray sums, residuals and images stay FP32 and the
 * step-control scalars FP64. */
enum {
  ASDPOCS_STORE_F32 = 0,
  ASDPOCS_STORE_F16 = 1, /* 11-bit significand, range 6e-5 .. 65504 */
  ASDPOCS_STORE_BF16 = 2 /* 8-bit significand, FP32's range        */
};

/* Forward projection of the SART steps (asdpocs_options.ax_mode): the
 * reference's column march (Ax_cone_gpu.cu:339-776) or the exact Siddon
 * projection of asdpocs_ax_siddon (no counterpart in the reference). */
enum { ASDPOCS_AX_REFERENCE = 0, ASDPOCS_AX_EXACT = 1 };

/* Option set of ASD_POCS_cuda.m:20-96 (defaults via asdpocs_options_default),
 * plus the sinogram storage and the forward mode (no counterpart in the
 * reference).  The instances of one plan share one ax_mode; the serving
 * queue runs ASDPOCS_AX_REFERENCE jobs only. */
typedef struct {
  int maxnumIter;       /* 5      */
  int numOfgradients;   /* ng, 20 */
  double alpha;         /* 0.02   */
  double alpha_red;     /* 0.95   */
  double beta;          /* 1      */
  double beta_red;      /* 0.995  */
  double r_max;         /* 0.95   */
  double epsilon;       /* eps    */
  double stopRelChg;    /* eps    */
  int sino_storage;     /* ASDPOCS_STORE_F32 */
  int ax_mode;          /* ASDPOCS_AX_REFERENCE */
} asdpocs_options;
void asdpocs_options_default(asdpocs_options *opt);

/* Rounds n FP32 values to the sinogram storage `storage` (2 bytes each for
 * FP16 / BF16, 4 for FP32), as the plans and the serving queue store them:
 * round to nearest, ties to even; NaN stays NaN, overflow gives inf. */
int asdpocs_store_sinogram(const float *in, void *out, unsigned long long n,
                           int storage);

/* Per-reconstruction outputs (the `out` struct of ASD_POCS_cuda.m:173-180). */
typedef struct {
  int IterationNum;
  double dataTolerance; /* dd2 of the last SART sweep */
  double alpha, beta;
  double dp, dg;        /* last ||m-m_pre||, ||m_TV - m_SART|| */
} asdpocs_stats;

/* Geometry of one reconstruction instance (the para struct minus phi). */
typedef struct {
  int nx, ny, nz, na, nb, nv;
  double SO, OD, vxlsize, detsize; /* mm */
} asdpocs_geometry;

typedef struct asdpocs_plan_s *asdpocs_plan;

/* Create a plan for `batch` reconstructions (the batch descriptor: one
 * geometry, angle list and option set per instance).  geom[i] and opt[i] are
 * per instance and may differ in every field, sizes included, except that
 * the instances are all 2-D (nz == nb == 1), all single-slice with nb > 1,
 * or all 3-D (nz > 1).  phi_vec_deg holds the instances' angle lists one
 * after the other (geom[0].nv values, then geom[1].nv, ...).  Each step of
 * the iteration is one launch per sub-batch (up to eight, on their own
 * streams); instances with equal sizes, geometry and angles run as groups
 * that share the projector work, and a view's launches cover only the
 * instances that have that view.  An instance gives the same result, bit
 * for bit, alone or in any batch.  All device memory is allocated here;
 * hbm_budget_bytes (0 = no limit) rejects plans that would exceed it. */
int asdpocs_plan_create(asdpocs_plan *plan, int batch,
                        const asdpocs_geometry *geom,
                        const double *phi_vec_deg,
                        const asdpocs_options *opt,
                        unsigned long long hbm_budget_bytes, void *stream);
int asdpocs_plan_destroy(asdpocs_plan plan);
/* How asdpocs_plan_create would run these instances, computed on the host
 * without a GPU (same arguments, checks and messages): group_of[i] is the
 * group of instances sharing geometry that instance i runs in (-1: it runs
 * through the per-instance kernels), sub_of[i] its sub-batch (one stream
 * each); either pointer may be NULL.  Returns the number of sub-batches, or
 * minus the status (ASDPOCS_ERR_*) of the error asdpocs_plan_create would
 * report.  Replaces nothing in the reference, which runs one
 * reconstruction at a time (ASD_POCS_cuda.m:103-171). */
int asdpocs_plan_layout(int batch, const asdpocs_geometry *geom,
                        const double *phi_vec_deg, const asdpocs_options *opt,
                        int *group_of, int *sub_of);
/* Device bytes held by the plan. */
unsigned long long asdpocs_plan_bytes(asdpocs_plan plan);

/* Load instance data.  `where`: 0 = host pointer (copied on the plan's
 * stream), 1 = device pointer.  P: (na*nb) x nv float sinogram, rounded to
 * the instance's sino_storage; m0 / I0: nx*ny*nz (NULL = zeros / no RMSE);
 * sizes are the instance's own. */
int asdpocs_plan_set_sinogram(asdpocs_plan plan, int inst, const float *P,
                              int where);
int asdpocs_plan_set_initial(asdpocs_plan plan, int inst, const float *m0,
                             int where);
int asdpocs_plan_set_reference(asdpocs_plan plan, int inst, const float *I0,
                               int where);
/* Reset iteration state (alpha, beta, k) of every instance to the options. */
int asdpocs_plan_reset(asdpocs_plan plan);

/* Run the ASD-POCS iterations of every instance (asynchronous on the plan's
 * stream).  use_graph != 0 captures one iteration into a CUDA graph once
 * and replays it. */
int asdpocs_plan_run(asdpocs_plan plan, int use_graph);
/* Wait for the plan's stream. */
int asdpocs_plan_sync(asdpocs_plan plan);

/* Results: m_res (post-SART image of the last iteration, nx*ny*nz floats),
 * per-iteration RMSE (maxnumIter doubles, if a reference image was set) and
 * the stats.  `where` as above; host copies synchronise the stream. */
int asdpocs_plan_get_image(asdpocs_plan plan, int inst, float *m, int where);
int asdpocs_plan_get_stats(asdpocs_plan plan, int inst, asdpocs_stats *st,
                           double *rmse);
/* Device pointer of an instance's sinogram / result image (for zero-copy
 * pipelines).  The sinogram pointer exists only for FP32 storage (NULL with
 * ASDPOCS_ERR_STATE otherwise: load FP16 / BF16 sinograms through
 * asdpocs_plan_set_sinogram, which rounds them). */
float *asdpocs_plan_sinogram_ptr(asdpocs_plan plan, int inst);
float *asdpocs_plan_image_ptr(asdpocs_plan plan, int inst);

/* Autotuner for the TV step's work partition: the walk length in bands of
 * 16 rows per column walk (2-D) or slabs of 16 slices per z walk (3-D).
 * Times `reps` TV steps per candidate (the batch-size rule, then 1, 2, 4,
 * ... up to a whole image) on the plan's stream -- steps 0, 1, ..., ng - 2,
 * 1, ..., each reading the previous one's output as in an iteration -- and
 * keeps the fastest for later runs.  Every walk length gives the same bits
 * (the norm is summed per band or slab in a fixed order).  The timed steps
 * read the image and write only work buffers and the step size, so the
 * reconstruction state is unchanged: call it after asdpocs_plan_reset()
 * and before a run.  *walk (may be NULL) receives the
 * choice (0: the batch-size rule), *ms (may be NULL) its time per step.
 * Plans with fewer than two TV steps per iteration keep the rule. */
int asdpocs_plan_autotune(asdpocs_plan plan, int reps, int *walk, double *ms);

/* Launch shapes of a plan's kernels (no counterpart in the reference).  No
 * shape changes any result bit; they only change how the work is laid out
 * over the GPU.  0 selects the built-in default. */
typedef struct {
  int tv_walk;         /* TV step: bands (2-D) or slabs (3-D) per walk */
  int ax_cols;         /* shared-geometry forward step: columns of loads per round, 1 or 2 */
  int ax_quads;        /* ... and quads of 4 instances per block, 1 or 2 */
  int zcol_segment;    /* cone-beam backward step: voxels per column segment, 8 .. 64 */
  int pdl;             /* programmatic dependent launches: -1 auto (plans on one stream),
                        * 0 off, 1 on */
  double iteration_ms; /* autotune: one iteration with the chosen shapes (device time) */
} asdpocs_shapes;

/* Autotuner for every launch shape of the plan: each shape that applies to
 * the plan's kind is timed over its candidates on the plan's own data (the
 * TV walk by its steps, the cone-beam column segment by the backward step,
 * the shared forward step's shape and programmatic launches by whole
 * iterations, where concurrent sub-batches overlap as in a run) and the
 * fastest kept.  Ends with asdpocs_plan_reset (the reconstruction state goes
 * back to its start). */
int asdpocs_plan_autotune_shapes(asdpocs_plan plan, int reps, asdpocs_shapes *out);
/* The plan's current shapes, or set them (0 = default; pdl -1 = auto). */
int asdpocs_plan_get_shapes(asdpocs_plan plan, asdpocs_shapes *out);
int asdpocs_plan_set_shapes(asdpocs_plan plan, const asdpocs_shapes *s);
/* Pins the TV walk length (0: the batch-size rule; larger values are
 * clipped to a whole image). */
int asdpocs_plan_set_tv_walk(asdpocs_plan plan, int walk);

/* Number of sub-batches the plan runs concurrently, each on its own stream
 * with its own captured iteration (2 once the batch holds 16 instances,
 * else 1); asdpocs_plan_run orders them after the plan's stream and the
 * plan's stream after them.  Every launch of an iteration is issued once
 * per sub-batch. */
int asdpocs_plan_streams(asdpocs_plan plan);

/* Chord slots per voxel of the plan's backward-step chord tables (the
 * largest over its instances' tables), 0 when it has none.  A plan of 2-D
 * instances computes the chords of every (voxel, ray) pair of every view
 * once -- one table for instances sharing geometry and view angles, else one
 * per instance -- at creation, and its backward steps read them (2 + slots
 * words per voxel and view, counted in asdpocs_plan_bytes; results are the
 * same bits as without them).  The tables stay within half the free device
 * memory and what is left of hbm_budget_bytes; instances whose tables do not
 * fit, or whose voxels have more than 32 pairs, compute the chords in every
 * step, and so does every plan when ASDPOCS_NO_CHORD_TABLE is set at
 * creation.
 * Replaces nothing in the reference, whose Atx_cone_mf_gpu_new
 * (Ax_cone_gpu.cu:299-331) recomputes the chords in every call. */
int asdpocs_plan_chord_slots(asdpocs_plan plan);

/* Profiling hook: average device time (ms, CUDA events on the plan's
 * stream) of `reps` back-to-back launches of one phase kernel for the whole
 * batch.  phase: 0 = SART forward step (Ax + residual), 1 = SART backward
 * step (Atx + update; each timed launch follows its view's untimed
 * forward step, whose residuals and tables it reads), both at `reps` views
 * spread evenly over the scan, 2 = one TV step (the steps that do not end
 * the iteration),
 * 3 = end-of-sweep scalars.  The launches modify the plan's state: call
 * asdpocs_plan_reset() before the next run. */
int asdpocs_plan_time_phase(asdpocs_plan plan, int phase, int reps,
                            double *avg_ms);

/* One-call equivalent of [m_res,out] = ASD_POCS_cuda(P, para): host buffers,
 * FP64 in/out as in MATLAB (P: (na*nb) x nv, column-major; phi_vec in
 * degrees; m0 / I0 may be NULL; rmse may be NULL). */
int ASD_POCS_cuda(const double *P, const double *phi_vec_deg,
                  const asdpocs_geometry *geom, const asdpocs_options *opt,
                  const double *m0, const double *I0, double *m_res,
                  double *rmse, asdpocs_stats *out);

/* m = SART_cuda_inline(P, para): one SART sweep with relaxation lambda
 * (SART_cuda_inline.m:17-108). */
int SART_cuda_inline(const double *P, const double *phi_vec_deg,
                     const asdpocs_geometry *geom, double lambda,
                     const double *m0, double *m_out, double *dataTolerance);

/* ---------------------------------------------------------------------
 * Device-side synthetic inputs (utilities/phantom3d.m semantics), so
 * benchmark and serving inputs need no host round trip.
 * --------------------------------------------------------------------- */

/* vol_d[nx*ny*nz] (x fastest) = scale * the sum of the amplitudes of the
 * ellipsoids containing each voxel's point on phantom3d.m's grid (n = the
 * largest dimension, points in [-1, 1]; voxel (r, c, k) at x = g[c],
 * y = g[r], z = g[k]).  ellipsoids: n_ellipsoids rows of 16 doubles --
 * amplitude, semi-axes a, b, c, centre x0, y0, z0, then the 3 x 3 rotation
 * row-major (q = R p) -- at most 32 rows.  FP64 with one rounding per
 * operation, so the host restatement gives the same volume bit for bit.
 * Asynchronous on `stream`. */
int asdpocs_phantom_device(float *vol_d, int nx, int ny, int nz,
                           const double *ellipsoids, int n_ellipsoids,
                           double scale, void *stream);

/* out_d[i] = -ln(max(k, 1) / I0) with k ~ Poisson(I0 * exp(-p_d[i])), from
 * a counter-based generator keyed by `seed` (the value of element i depends
 * on seed and i only).  out_d may equal p_d.  Asynchronous on `stream`. */
int asdpocs_poisson_noise_device(const float *p_d, float *out_d, long long n,
                                 double I0, unsigned long long seed,
                                 void *stream);

/* ---------------------------------------------------------------------
 * Serving queue (no counterpart in the reference, whose drivers run one
 * reconstruction at a time).  Jobs of any geometry, view count and
 * iteration budget are submitted at any time.  A worker thread admits them
 * into free slots of device-resident lanes -- one lane per scan protocol
 * (identical sizes, geometry and view angles), each on its own CUDA stream,
 * its backward step computing each chord once for a group of its jobs --
 * when the HBM budget has room, runs one ASD-POCS iteration of every job of
 * a lane per launch sequence (a replayed CUDA graph), retires jobs as they
 * finish and admits waiting ones in their place, so jobs that arrive while
 * others run join them on the device.  Each job's result is bit-identical
 * to the same job run alone in a plan.  The budget counts the jobs' state.
 * A lane also holds its protocol's geometry tables and its slots'
 * interleaved images (4 bytes per voxel and slot; a lane gets as many slots,
 * in groups of 8, as fit in an eighth of the budget, at least 8) until the
 * server is destroyed; a 2-D lane also holds its protocol's backward-step
 * chord tables (see asdpocs_plan_chord_slots), every lane's together within
 * a quarter of the budget.  All calls are thread-safe.
 * --------------------------------------------------------------------- */
typedef struct asdpocs_server_s *asdpocs_server;

typedef struct {
  int slots_per_lane;                  /* concurrent jobs per lane (32)   */
  unsigned long long hbm_budget_bytes; /* device bytes for job state;
                                          0 = half the free memory       */
  int inflight;                        /* iterations queued ahead per
                                          lane (2)                        */
} asdpocs_server_config;
void asdpocs_server_config_default(asdpocs_server_config *cfg);

enum {
  ASDPOCS_JOB_QUEUED = 0,
  ASDPOCS_JOB_RUNNING = 1,
  ASDPOCS_JOB_DONE = 2,
  ASDPOCS_JOB_FAILED = 3,
  ASDPOCS_JOB_CANCELLED = 4
};

/* Times of a finished job (host steady clock, milliseconds). */
typedef struct {
  double queued_ms; /* submission to admission  */
  double run_ms;    /* admission to result ready */
  double total_ms;  /* submission to result ready (the job's latency) */
} asdpocs_job_times;

/* Start the worker on the calling thread's current device (cfg NULL =
 * defaults). */
int asdpocs_server_create(asdpocs_server *server,
                          const asdpocs_server_config *cfg);
/* Queue a job: geometry, geom->nv view angles (degrees), options (NULL =
 * defaults), sinogram P ((na*nb) x nv floats, host), optional initial image
 * m0 and reference image I0 (nx*ny*nz floats, host; NULL = zeros / no
 * RMSE).  The data are copied before the call returns.  A job larger than
 * the whole HBM budget is rejected with ASDPOCS_ERR_NOMEM. */
int asdpocs_server_submit(asdpocs_server server, const asdpocs_geometry *geom,
                          const double *phi_vec_deg, const asdpocs_options *opt,
                          const float *P, const float *m0, const float *I0,
                          long long *job);
/* Current state of a job (ASDPOCS_JOB_*). */
int asdpocs_server_poll(asdpocs_server server, long long job, int *state);
/* Cancel a job (no counterpart in the reference, which runs one
 * reconstruction per call).  A queued job leaves its queue; a running job
 * leaves its slot at the end of the iteration in flight, its device memory
 * returned in stream order, without touching the jobs that share its
 * launches.  Returns ASDPOCS_ERR_STATE for a job that has finished or is
 * already copying out its results.  A cancelled job must still be released
 * with asdpocs_server_wait, which then returns ASDPOCS_ERR_STATE. */
int asdpocs_server_cancel(asdpocs_server server, long long job);
/* Wait for a job and take its results (image nx*ny*nz floats, stats, the
 * per-iteration RMSE if a reference was given, times); any output may be
 * NULL.  The job is released: a second wait on it is an error. */
int asdpocs_server_wait(asdpocs_server server, long long job, float *m_res,
                        asdpocs_stats *st, double *rmse,
                        asdpocs_job_times *times);
/* Device bytes held by admitted jobs now, and the peak so far. */
int asdpocs_server_memory(asdpocs_server server, unsigned long long *in_use,
                          unsigned long long *peak);
/* Stop the worker (jobs not yet finished fail) and release everything. */
int asdpocs_server_destroy(asdpocs_server server);

#ifdef __cplusplus
}
#endif
#endif
