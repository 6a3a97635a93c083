// Shared definitions of the asdpocs_gb300 library (internal).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/asdpocs_gb300.h"

namespace asd {

// ---------------------------------------------------------------------------
// Error reporting (thread-local last error, as returned by asdpocs_last_error)
// ---------------------------------------------------------------------------
int set_error(int status, const char *fmt, ...);
void clear_error();
int cuda_status(cudaError_t e, const char *what);

#define ASD_CUDA(call)                                         \
  do {                                                         \
    cudaError_t e_ = (call);                                   \
    if (e_ != cudaSuccess) return ::asd::cuda_status(e_, #call); \
  } while (0)

// ---------------------------------------------------------------------------
// Geometry (launcher level: voxel units, as passed to Ax_cone_mf_gpu_new)
// ---------------------------------------------------------------------------
struct Dims {
  int nx, ny, nz, na, nb;
};

struct ViewGeo {
  float cos_phi, sin_phi;
  float SO, OD, scale;
  float dy_det, dz_det, dz;
  const float *y_det;  // device, na
  const float *z_det;  // device, nb
  // per-view constants of the backprojector footprint, with_constants()
  float SD;    // SO + OD
  float dwin;  // sqrtf((1 + dz*dz)/2), the footprint half-height
};

// Fills the derived constants with the reference's float expressions
// (Ax_cone_gpu.cu:230,233).
__host__ __device__ inline ViewGeo with_constants(ViewGeo g) {
  g.SD = g.SO + g.OD;
  g.dwin = sqrtf((1 + g.dz * g.dz) / 2);
  return g;
}

// ---------------------------------------------------------------------------
// Per-instance state of a batched ASD-POCS plan (device resident)
// ---------------------------------------------------------------------------
struct Scalars {
  // ASD-POCS step control (ASD_POCS_cuda.m:137-170), FP64 on the device
  double alpha, beta;
  double alpha_red, beta_red, r_max, epsilon, stopRelChg;
  double dd2_acc;   // running ||P - Ax||^2 over the current sweep
  double dd2;       // dd2 of the last complete sweep (out.dataTolerance)
  double dp;        // ||m - m_pre|| of the last sweep
  double d_tv;      // ||m - m_k1|| at TV entry (imgTVGradMin.cpp:57-60)
  double tv_coef;   // alpha*d/||v|| of the current TV step
  float tv_coef_f;  // FP32 copies read by the per-voxel kernels
  float beta_f;
  double dg;        // ||m_TV - m_SART||
  int k;            // 1-based iteration about to run / running
  int done;         // stop criterion met or maxnumIter reached
  int iterations;   // out.IterationNum
  int maxIter, ng;
  int has_ref;      // I0 present
  int pad;
};

struct Inst {
  ViewGeo g;                 // geometry (cos/sin filled per view from trig)
  const float2 *trig;        // [nv] (cos_phi, sin_phi) per view
  const float *P;            // sinogram, view-major, na*nb*nv
  float *m;                  // current image (A)
  float *m_pre;              // image at sweep start
  float *m_res;              // post-SART snapshot (returned image)
  float *m_k1;               // TV distance reference (m0)
  float *I0;                 // reference image or nullptr
  float *tv_b, *tv_c;        // TV ping-pong buffers
  float *cor;                // correction of the current view, na*nb
  double *rmse;              // [maxIter]
  double *partials;          // reduction partials [blocks * 3]
  unsigned *counter;         // reduction ticket
  Scalars *s;
};

constexpr int kMaxPartials = 1 << 22;  // blocks per reduction (sanity bound)
constexpr int kMaxReduceK = 3;          // values reduced together

}  // namespace asd
