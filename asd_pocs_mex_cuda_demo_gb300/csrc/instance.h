// Device state of one reconstruction instance (internal): shared by the
// batched plans and the serving queue.
#pragma once
#include <vector>
#include "kernels.h"

namespace asd {

// Byte offsets of an instance's buffers inside its block of device memory
// (each 256-byte aligned), at the instance's own sizes; `bytes` is the
// block's size.
struct InstLayout {
  size_t P, m, m_pre, m_res, m_k1, I0, tvb, tvc, cor, m_il, ydet, zdet, trig,
      rmse, part, cnt, scal, tabA, tabC, vflags, bytes;
  int p_fmt;  // sinogram storage (ASDPOCS_STORE_*)
};

// Kind of an instance: 0 = 2-D fan beam (nz == nb == 1), 1 = one slice with
// detector rows (nz == 1, nb > 1), 2 = cone beam (nz > 1).  Instances that
// run in one launch share a kind (their kernels are templated on it).
int instance_kind(const asdpocs_geometry &g);

// Sizes and counts of `g` checked (status and message set on failure).
int check_instance(const asdpocs_geometry &g, const asdpocs_options &o);

// Parts of an instance's block: its state (sinogram, images, scalars,
// reduction scratch) and its geometry (detector coordinates, view angles,
// ray tables, residual buffer).  Instances that share geometry can keep one
// geometry part between them.
constexpr int kLayoutState = 1, kLayoutGeometry = 2;

// Layout of the parts `parts` of an instance (absent parts take no bytes);
// cor_floats is the length of its residual buffer (na*nb, or kShareSlots
// times that for the first instance of a shared group) and il_floats that of
// the interleaved images of a shared group (kShareSlots*N for the group's
// first instance, else 0).
// sino_storage: the sinogram's storage (ASDPOCS_STORE_*, 2 or 4 bytes a value).
InstLayout layout_instance(const asdpocs_geometry &g, int max_iter,
                           size_t cor_floats,
                           int parts = kLayoutState | kLayoutGeometry,
                           size_t il_floats = 0, int sino_storage = ASDPOCS_STORE_F32);

// Host copy of a job's sinogram in its storage: n FP32 values rounded as
// asdpocs_store_sinogram does, into out (n * sino_elem_bytes(fmt) bytes).
void store_sinogram_host(const float *in, void *out, size_t n, int fmt);

// Points I's state pointers at the block `b` laid out as `o`.
void bind_state(Inst &I, char *b, const InstLayout &o);

// Points I's geometry at the block `b` laid out as `o` (own residual buffer,
// stride 1, own ray-slope table) and uploads the detector coordinates and
// view cosines/sines on `st` (the host staging is released when the call
// returns).
cudaError_t bind_geometry(Inst &I, char *b, const InstLayout &o,
                          const asdpocs_geometry &g, const double *phi_deg,
                          cudaStream_t st);

// Both of the above for a block holding both parts.
cudaError_t bind_instance(Inst &I, char *b, const InstLayout &o,
                          const asdpocs_geometry &g, const double *phi_deg,
                          cudaStream_t st);

// Scalars of an instance before its first iteration (ASD_POCS_cuda.m:34-96
// defaults already applied to `o`).
Scalars initial_scalars(const asdpocs_options &o, bool has_ref);

// Enqueues the start state of an instance on `st`: m, m_pre, m_res = m_k1,
// a zero reduction ticket and the scalars (copied from `s`, which must stay
// valid until the copy has run unless it is pageable host memory).
cudaError_t reset_instance(const Inst &I, const Scalars &s, cudaStream_t st);

// Enqueues one ASD-POCS iteration of `batch` instances on `st` (grids for
// the largest sizes `d`, nv views, ng TV steps): per view the SART forward
// and backward steps, the end-of-sweep scalars, the TV steps and the end of
// the iteration.  `shared`: the instances share geometry and angles and sit
// in groups with interleaved images (Inst::m_il), packed before the sweep
// and unpacked after it.
// `finish`: some instance may run fewer than two TV steps, so the
// end-of-iteration kernel is needed (otherwise the last TV step ends every
// instance's iteration and the launch is skipped).
// How the kernels of an iteration are launched.  Every field but `exact`
// is a launch shape that leaves every result bit unchanged (what
// asdpocs_plan_autotune_shapes may pick); `exact` selects the exact forward
// projection (a mode: different results).
struct IterShape {
  int tv_walk = 0;          // TV walk length (0: the batch-size rule)
  bool zcol = true;         // cone beams: z-column backward step (else per voxel)
  int zseg = 0;             //   its segment length in voxels (0: the default)
  int ax_u = 0, ax_q = 0;   // shared forward step: columns of loads per round,
                            //   quads of instances per block (0: the defaults)
  bool pdl = false;         // programmatic dependent launches (work alone on
                            //   its stream)
  bool exact = false;       // forward steps: exact projection (launch_sart_ax)
};
// Instances of one launch with different view counts: for each run of
// views [v0, v1), the instances that have those views (a device list of
// `count` indices into the launch's instances) and their largest sizes, so
// that the projector steps of those views cover only them.
// Launches of the shared-geometry kernels with group tables list the
// groups instead (gtab: `count` groups as (first instance, count)).
struct ViewSet {
  int v0 = 0, v1 = 0, count = 0;
  Dims d{};
  const int *zmap = nullptr;
  const int2 *gtab = nullptr;
  size_t zoff = 0;  // position of the list in its plan's index buffers
};
// `zall` (device, `batch` entries; null: 0 .. batch - 1): the instances of
// d_inst the iteration runs.  `sets`: runs of views in order covering
// [0, nv) (null or empty: every instance of zall in every view, at sizes d).
// `gall` (shared only; device, `ngroups` entries; null: groups of
// kShareSlots consecutive instances): the groups of instances sharing
// geometry, as (first instance, count).
cudaError_t enqueue_iteration(const Inst *d_inst, int batch, const Dims &d,
                              int nv, int ng, bool shared, cudaStream_t st,
                              const IterShape &shape = IterShape(), bool finish = true,
                              const std::vector<ViewSet> *sets = nullptr,
                              const int *zall = nullptr, const int2 *gall = nullptr,
                              int ngroups = 0);

// Backward-step chord tables (Inst::chtab) of instances sharing 2-D geometry
// and view angles, from d_inst[0], whose view tables are built: a counting
// pass for the slots per voxel, then a filling pass, synchronous on `st`.
// Leaves *tab_out null (and returns cudaSuccess) when the instances are not
// 2-D, a voxel has more than 32 pairs, the tables would take more than
// max_bytes, or the allocation fails; the caller then computes chords in
// every step.  The caller frees *tab_out (cudaFree) and sets the
// descriptors' chtab and chK.
cudaError_t build_chord_tables(const Inst *d_inst, const Dims &d, int nv,
                               size_t max_bytes, cudaStream_t st, int **tab_out,
                               int *K_out, size_t *bytes_out);

}  // namespace asd
