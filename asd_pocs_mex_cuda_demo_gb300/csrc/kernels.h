// Launch wrappers of the device kernels (internal interface between the
// kernel translation units and the host library).
#pragma once
#include "common.cuh"

namespace asd {

// ---- projectors (kernels_proj.cu) ----
// Ax of one view: y, sr (na*nb) from x.
cudaError_t launch_ax(const float *x, float *y, float *sr, const ViewGeo &g,
                      const Dims &d, cudaStream_t st);
// Exact Ax of one view (Siddon's method: FP64 crossing parameters, FP32
// lengths and sums) instead of the reference's column march.
cudaError_t launch_ax_siddon(const float *x, float *y, float *sr, const ViewGeo &g,
                             const Dims &d, cudaStream_t st);
// Atx of one view: x, sc (nx*ny*nz) from y.
cudaError_t launch_atx(float *x, const float *y, float *sc, const ViewGeo &g,
                       const Dims &d, cudaStream_t st);

// Atx of one cone-beam view (nz > 1) walked down voxel columns, bit-identical
// to launch_atx; `scratch` holds the view's ray tables
// (atx_zcol_scratch_bytes(d) bytes, 256-byte aligned).
size_t atx_zcol_scratch_bytes(const Dims &d);
cudaError_t launch_atx_zcol(float *x, const float *y, float *sc, const ViewGeo &g,
                            const Dims &d, void *scratch, cudaStream_t st);

#ifdef ASDPOCS_CHECKED
// Bounds-checked builds: read and clear the out-of-range counts (and the
// first bad index with its extent) of the projector and TV kernels.
cudaError_t checked_take_proj(unsigned long long *count, long long *first);
cudaError_t checked_take_tv(unsigned long long *count, long long *first);
#endif

// Stores n FP32 sinogram values (device) as `fmt` (ASDPOCS_STORE_*) at dst.
cudaError_t launch_store_sinogram(const float *src, void *dst, size_t n, int fmt,
                                  cudaStream_t st);

// Batched launches take the plan's largest sizes `d` (each field the
// maximum over its instances) for the grid; every instance reads its own
// sizes from Inst::d, and instances of one plan are all planar (nz == nb ==
// 1) or all not.
//
// Fused SART steps of view `view` for `batch` instances (ASD_POCS_cuda.m:
// 116-131); instances with fewer views skip.  sart_ax: Ax of m, residual
// against P, dd2 accumulation, row normalisation -> cor.  sart_atx: Atx of
// cor, column normalisation, update m += beta*bp/sumC, positivity.
// `exact`: the forward step uses the exact projection (launch_ax_siddon).
// `zmap` (device, `batch` entries; null: 0 .. batch - 1): the instances of
// `insts` the launch covers, grid slice z running instance zmap[z]; `d` must
// hold the largest sizes among them.
cudaError_t launch_sart_ax(const Inst *insts, int batch, const Dims &d,
                           int view, cudaStream_t st, bool exact = false,
                           const int *zmap = nullptr);
// Cone beams (nz > 1) walk voxel columns (k_sart_atx_zcol) in segments of
// `zseg` voxels (0: the default) unless `zcol` is false (the per-voxel form;
// bit-identical).  `zmap` as for launch_sart_ax.
cudaError_t launch_sart_atx(const Inst *insts, int batch, const Dims &d,
                            int view, cudaStream_t st, bool zcol = true, int zseg = 0,
                            const int *zmap = nullptr);

// ---- TV and scalars (kernels_tv.cu) ----
// FP64 / FP32 TV minimisation on device buffers (reference semantics).
cudaError_t tv_minimize_f64(double *img, const double *img_old, double *work_a,
                            double *work_b, double *scal, double *partials,
                            unsigned *counter, int nx, int ny, int nz,
                            double alpha, int n_iter, int pos, cudaStream_t st);
cudaError_t tv_minimize_f32(float *img, const float *img_old, float *work_a,
                            float *work_b, double *scal, double *partials,
                            unsigned *counter, int nx, int ny, int nz,
                            double alpha, int n_iter, int pos, cudaStream_t st);

// Per-iteration ASD-POCS steps for a batch (ASD_POCS_cuda.m:137-170).
cudaError_t launch_iter_begin(const Inst *insts, int batch, cudaStream_t st);
// `zmap` (device, `batch` entries; null: 0 .. batch - 1): the instances of
// `insts` a launch covers, as for launch_sart_ax.
cudaError_t launch_after_sweep(const Inst *insts, int batch, const Dims &d,
                               cudaStream_t st, const int *zmap = nullptr);
// `walk`: bands (2-D) or slabs (3-D) per walk of the TV step; 0 picks it
// from the batch size.  Results do not depend on it.
cudaError_t launch_tv_step(const Inst *insts, int batch, const Dims &d,
                           int step, int ng, cudaStream_t st, int walk = 0,
                           const int *zmap = nullptr);
// Largest useful `walk` for images of size d (the bands or slabs of one).
int tv_walk_max(const Dims &d);
cudaError_t launch_finish_iter(const Inst *insts, int batch, const Dims &d,
                               int ng, cudaStream_t st, const int *zmap = nullptr);

int reduce_blocks_for(const Dims &d);
// Strips x bands of the 2-D walks (the TV steps keep one partial for each,
// the end of the sweep four), or tiles x slabs of the cone-beam TV step.
int tv_partials_for(const Dims &d);

// Copies Inst::s->done of n instances into the device array out[n].
cudaError_t launch_gather_done(const Inst *insts, int n, int *out,
                               cudaStream_t st);

// Backward step for a batch whose instances share geometry and view angles:
// chords computed once per voxel and applied to groups of instances (read
// from the plan's chord tables, Inst::chtab, where it has them).
// `gtab` (device, `ngroups` entries; null: groups of kShareSlots
// consecutive instances): the launch's groups as (first instance, count),
// each group's instances sharing geometry and view angles; groups of
// different sizes may share a launch, `d` holding the largest sizes.
cudaError_t launch_sart_atx_shared(const Inst *insts, int batch,
                                   const Dims &d, int view, cudaStream_t st,
                                   const int2 *gtab = nullptr, int ngroups = 0);

// Forward step for a batch whose instances share geometry and view angles:
// the column march evaluated once per ray for groups of instances whose
// images are interleaved (Inst::m_il) during the sweep.
// `u` columns of loads per round and `q` quads of instances per block (1 or
// 2 each; 0: the defaults, 2 x 1 for fan beams, 1 x 2 for cone beams) are
// launch shapes that do not change results.
// `gtab`, `ngroups` as for launch_sart_atx_shared.
cudaError_t launch_sart_ax_shared(const Inst *insts, int batch, const Dims &d,
                                  int view, cudaStream_t st, int u = 0, int q = 0,
                                  const int2 *gtab = nullptr, int ngroups = 0);
// Copies the running instances' images into (unpack = 0) or out of
// (unpack = 1) their group's interleaved images (`gtab`, `ngroups` as for
// launch_sart_atx_shared).
cudaError_t launch_group_pack(const Inst *insts, int batch, const Dims &d,
                              int unpack, cudaStream_t st, const int2 *gtab = nullptr,
                              int ngroups = 0);

// Backward-step chord tables (Inst::chtab) of the 2-D instance insts[0]
// (and of the instances sharing its geometry), whose view tables must be
// built.  K == 0
// counts: the largest number of pairs of a voxel goes to kmax[0] (zeroed
// first).  K > 0 fills `tabs` (atx_chord_words(d, nv, K) ints) and sets
// kmax[1] if a voxel has more than K pairs.
cudaError_t launch_atx_chords(const Inst *insts, const Dims &d, int nv, int K,
                              int *tabs, int *kmax, cudaStream_t st);
size_t atx_chord_words(const Dims &d, int nv, int K);
int atx_chord_max_slots();

// Ray slope tables and flags of every view (Inst::tabA, Inst::vflags, which
// must be zeroed first), computed once per plan.
cudaError_t launch_view_tables(const Inst *insts, int batch, const Dims &d,
                               int nv, cudaStream_t st);

}  // namespace asd
