// Host side of the asdpocs_gb300 C ABI: launcher drop-ins, mex-level entry
// points, TV entry points and the device-resident ASD-POCS plans.
#include <limits.h>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <mutex>
#include <new>
#include <numeric>
#include <vector>

#include "instance.h"

namespace asd {

// ------------------------------------------------------------------ errors
static thread_local int g_status = 0;
static thread_local char g_msg[512] = "";

int set_error(int status, const char *fmt, ...) {
  g_status = status;
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_msg, sizeof g_msg, fmt, ap);
  va_end(ap);
  return status;
}
void clear_error() {
  g_status = 0;
  g_msg[0] = 0;
}
int cuda_status(cudaError_t e, const char *what) {
  const int st = (e == cudaErrorMemoryAllocation) ? ASDPOCS_ERR_NOMEM
                 : (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver)
                     ? ASDPOCS_ERR_NODEV
                     : ASDPOCS_ERR_CUDA;
  return set_error(st, "%s: %s", what, cudaGetErrorString(e));
}

// ------------------------------------------------ gateway geometry helpers
// Ax_main_test.cpp:138-161 / Atx_main_test.cpp:149-172: every para field is
// read as float; cos/sin of the float angle; lengths divided by the voxel
// size in float; detector coordinates (i - n/2 + 0.5)*det evaluated in
// double and rounded to float; dz = 1.
struct GatewayGeo {
  float cos_phi, sin_phi, SO, OD, scale, det;
  std::vector<float> y_det, z_det;
};

static void gateway_geometry(double phi, double SO, double OD, double vxl,
                             double detsize, int na, int nb, GatewayGeo &g) {
  const float phif = (float)phi;
  g.scale = (float)vxl;
  g.cos_phi = cosf(phif);
  g.sin_phi = sinf(phif);
  g.SO = (float)SO / g.scale;
  g.OD = (float)OD / g.scale;
  g.det = (float)detsize / g.scale;
  g.y_det.resize(na);
  g.z_det.resize(nb);
  for (int i = 0; i < na; i++)
    g.y_det[i] = (float)(((double)(float)i - (double)(float)na / 2.0 + 0.5) *
                         (double)g.det);
  for (int i = 0; i < nb; i++)
    g.z_det[i] = (float)(((double)(float)i - (double)(float)nb / 2.0 + 0.5) *
                         (double)g.det);
}

// angle of view ii as the driver passes it: para.phi = -phi_vec(ii)/180*pi
// (ASD_POCS_cuda.m:111,116), then read as float by the gateway.
static float2 view_trig(double phi_deg) {
  const double theta = phi_deg / 180.0 * 3.14159265358979323846;
  const float phif = (float)(-1 * theta);
  return make_float2(cosf(phif), sinf(phif));
}

// ------------------------------------- workspace of the host-pointer calls
// Grow-only device buffers reused by the synchronous drop-ins, so a call
// does not pay cudaMalloc/cudaFree (the reference allocates five buffers per
// call, Ax_cone_gpu.cu:787-804).  One workspace per device, serialised.
struct Workspace {
  std::mutex mu;
  void *buf = nullptr;
  size_t cap = 0;
  cudaStream_t st = nullptr;
};
static Workspace g_ws[64];

static int ws_acquire(Workspace *&w, size_t bytes) {
  int dev = 0;
  ASD_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return set_error(ASDPOCS_ERR_NODEV, "device id");
  w = &g_ws[dev];
  if (!w->st) ASD_CUDA(cudaStreamCreateWithFlags(&w->st, cudaStreamNonBlocking));
  if (bytes > w->cap) {
    if (w->buf) cudaFree(w->buf);
    w->buf = nullptr;
    w->cap = 0;
    ASD_CUDA(cudaMalloc(&w->buf, bytes));
    w->cap = bytes;
  }
  return 0;
}

static inline size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

// The TV entry points' image limit: its tile grid must launch (see tile_rows).
static int check_tv_dims(int nx, int ny, int nz) {
  if (nx <= 0 || ny <= 0 || nz <= 0)
    return set_error(ASDPOCS_ERR_ARG, "bad image dimensions");
  if (tile_rows(ny, nz) > kMaxGridRows)
    return set_error(ASDPOCS_ERR_ARG,
                     "image of %d x %d x %d needs %lld tile rows (ceil(ny/8)*nz), over "
                     "the limit of %lld",
                     nx, ny, nz, tile_rows(ny, nz), kMaxGridRows);
  return 0;
}

static int check_dims(int nx, int ny, int nz, int na, int nb) {
  if (nx <= 0 || ny <= 0 || nz <= 0 || na <= 0 || nb <= 0)
    return set_error(ASDPOCS_ERR_ARG,
                     "dimensions must be positive (nx=%d ny=%d nz=%d na=%d nb=%d)",
                     nx, ny, nz, na, nb);
  if ((long long)nx * ny * nz > (1LL << 34) || (long long)na * nb > (1LL << 31))
    return set_error(ASDPOCS_ERR_ARG, "dimensions too large");
  return 0;
}

}  // namespace asd

using namespace asd;

// ======================================================================
extern "C" {

const char *asdpocs_last_error(void) { return g_msg; }
int asdpocs_last_status(void) { return g_status; }
const char *asdpocs_version(void) {
#ifdef ASDPOCS_CHECKED
  return "asdpocs_gb300 0.2 (sm_103a, bounds-checked)";
#else
  return "asdpocs_gb300 0.2 (sm_103a)";
#endif
}

int asdpocs_checked_errors(unsigned long long *count, long long first[2]) {
  clear_error();
  if (!count || !first) return set_error(ASDPOCS_ERR_ARG, "null pointer");
#ifdef ASDPOCS_CHECKED
  ASD_CUDA(cudaDeviceSynchronize());
  unsigned long long cp = 0, ct = 0;
  long long fp[2] = {0, 0}, ft[2] = {0, 0};
  ASD_CUDA(checked_take_proj(&cp, fp));
  ASD_CUDA(checked_take_tv(&ct, ft));
  *count = cp + ct;
  first[0] = cp ? fp[0] : ft[0];
  first[1] = cp ? fp[1] : ft[1];
  return 0;
#else
  *count = 0;
  first[0] = first[1] = 0;
  return set_error(ASDPOCS_ERR_STATE,
                   "not a bounds-checked build (libasdpocs_gb300_checked.so has the checks)");
#endif
}

// ------------------------------------------------------------ projectors
static int ax_device(const float *x_d, float *y_d, float *sr_d, float cos_phi,
                     float sin_phi, const float *y_det_d, const float *z_det_d, float SO,
                     float OD, float scale, float dz, int nx, int ny, int nz, int na,
                     int nb, void *stream, bool exact) {
  clear_error();
  if (int e = check_dims(nx, ny, nz, na, nb)) return e;
  if (!x_d || !y_d || !sr_d || !y_det_d || !z_det_d)
    return set_error(ASDPOCS_ERR_ARG, "null pointer");
  const ViewGeo g = with_constants(
      ViewGeo{cos_phi, sin_phi, SO, OD, scale, 0.f, 0.f, dz, y_det_d, z_det_d});
  Dims d{nx, ny, nz, na, nb};
  if (exact)
    ASD_CUDA(launch_ax_siddon(x_d, y_d, sr_d, g, d, (cudaStream_t)stream));
  else
    ASD_CUDA(launch_ax(x_d, y_d, sr_d, g, d, (cudaStream_t)stream));
  return 0;
}

int asdpocs_ax_device(const float *x_d, float *y_d, float *sr_d, float cos_phi,
                      float sin_phi, const float *y_det_d,
                      const float *z_det_d, float SO, float OD, float scale,
                      float dz, int nx, int ny, int nz, int na, int nb,
                      void *stream) {
  return ax_device(x_d, y_d, sr_d, cos_phi, sin_phi, y_det_d, z_det_d, SO, OD, scale, dz, nx,
                   ny, nz, na, nb, stream, false);
}

int asdpocs_ax_siddon_device(const float *x_d, float *y_d, float *sr_d, float cos_phi,
                             float sin_phi, const float *y_det_d, const float *z_det_d,
                             float SO, float OD, float scale, float dz, int nx, int ny,
                             int nz, int na, int nb, void *stream) {
  return ax_device(x_d, y_d, sr_d, cos_phi, sin_phi, y_det_d, z_det_d, SO, OD, scale, dz, nx,
                   ny, nz, na, nb, stream, true);
}

int asdpocs_atx_device(float *x_d, const float *y_d, float *sc_d,
                       float cos_phi, float sin_phi, const float *y_det_d,
                       const float *z_det_d, float SO, float OD, float scale,
                       float dy_det, float dz_det, float dz, int nx, int ny,
                       int nz, int na, int nb, void *stream) {
  clear_error();
  if (int e = check_dims(nx, ny, nz, na, nb)) return e;
  if (!x_d || !y_d || !sc_d || !y_det_d || !z_det_d)
    return set_error(ASDPOCS_ERR_ARG, "null pointer");
  const ViewGeo g = with_constants(ViewGeo{cos_phi, sin_phi, SO, OD, scale,
                                           dy_det, dz_det, dz, y_det_d, z_det_d});
  Dims d{nx, ny, nz, na, nb};
  ASD_CUDA(launch_atx(x_d, y_d, sc_d, g, d, (cudaStream_t)stream));
  return 0;
}

static int ax_host(const float *X, float *y, float *sr, float cos_phi,
                   float sin_phi, const float *y_det, const float *z_det,
                   float SO, float OD, float scale, float dz, int nx, int ny,
                   int nz, int na, int nb, bool exact = false) {
  clear_error();
  if (int e = check_dims(nx, ny, nz, na, nb)) return e;
  if (!X || !y || !sr || !y_det || !z_det)
    return set_error(ASDPOCS_ERR_ARG, "null pointer");
  const size_t N = (size_t)nx * ny * nz, M = (size_t)na * nb;
  const size_t oX = 0, oY = align256(N * 4), oS = oY + align256(M * 4),
               oA = oS + align256(M * 4), oB = oA + align256((size_t)na * 4),
               tot = oB + align256((size_t)nb * 4);
  Workspace *w;
  if (int e = ws_acquire(w, tot)) return e;
  std::lock_guard<std::mutex> lk(w->mu);
  char *b = (char *)w->buf;
  ASD_CUDA(cudaMemcpyAsync(b + oX, X, N * 4, cudaMemcpyHostToDevice, w->st));
  ASD_CUDA(cudaMemcpyAsync(b + oA, y_det, (size_t)na * 4, cudaMemcpyHostToDevice, w->st));
  ASD_CUDA(cudaMemcpyAsync(b + oB, z_det, (size_t)nb * 4, cudaMemcpyHostToDevice, w->st));
  const ViewGeo g = with_constants(ViewGeo{cos_phi, sin_phi, SO, OD, scale, 0.f,
                                           0.f, dz, (const float *)(b + oA),
                                           (const float *)(b + oB)});
  Dims d{nx, ny, nz, na, nb};
  if (exact)
    ASD_CUDA(launch_ax_siddon((const float *)(b + oX), (float *)(b + oY), (float *)(b + oS), g,
                              d, w->st));
  else
    ASD_CUDA(launch_ax((const float *)(b + oX), (float *)(b + oY), (float *)(b + oS), g, d,
                       w->st));
  ASD_CUDA(cudaMemcpyAsync(y, b + oY, M * 4, cudaMemcpyDeviceToHost, w->st));
  ASD_CUDA(cudaMemcpyAsync(sr, b + oS, M * 4, cudaMemcpyDeviceToHost, w->st));
  ASD_CUDA(cudaStreamSynchronize(w->st));
  return 0;
}

}  // extern "C"

namespace asd {
namespace {

constexpr int kDotThreads = 256, kDotBlocks = 152 * 4;

// FP64 partial dot products of a and b, one per block, each over a fixed
// grid-stride subset and summed in a fixed order.
__global__ void __launch_bounds__(kDotThreads)
    k_dot_f64(const float *__restrict__ a, const float *__restrict__ b, long long n,
              double *__restrict__ partials) {
  __shared__ double sh[kDotThreads / 32];
  double s = 0.0;
  for (long long i = (long long)blockIdx.x * kDotThreads + threadIdx.x; i < n;
       i += (long long)kDotBlocks * kDotThreads)
    s += (double)a[i] * (double)b[i];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < kDotThreads / 32; w++) t += sh[w];
    partials[blockIdx.x] = t;
  }
}

// out = the block partials summed in block order (one thread)
__global__ void k_sum_f64(const double *__restrict__ partials, int n, double *out) {
  double t = 0.0;
  for (int i = 0; i < n; i++) t += partials[i];
  *out = t;
}

}  // namespace
}  // namespace asd

namespace asd {

cudaError_t build_chord_tables(const Inst *d_inst, const Dims &d, int nv,
                               size_t max_bytes, cudaStream_t st, int **tab_out,
                               int *K_out, size_t *bytes_out) {
  *tab_out = nullptr;
  *K_out = 0;
  *bytes_out = 0;
  if (d.nz != 1 || d.nb != 1 || (long long)d.na >= (1LL << 24) || nv > 65535)
    return cudaSuccess;
  int *kmax = nullptr;
  if (cudaMalloc(&kmax, 2 * sizeof(int)) != cudaSuccess) {
    cudaGetLastError();  // out of memory is not sticky: go on without tables
    return cudaSuccess;
  }
  int hk[2] = {0, 0};
  cudaError_t e = cudaMemsetAsync(kmax, 0, sizeof(hk), st);
  if (e == cudaSuccess) e = launch_atx_chords(d_inst, d, nv, 0, nullptr, kmax, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(hk, kmax, sizeof(hk), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  const int K = hk[0];
  const size_t bytes = atx_chord_words(d, nv, K) * sizeof(int);
  int *tab = nullptr;
  if (e == cudaSuccess && K > 0 && K <= atx_chord_max_slots() && bytes <= max_bytes &&
      cudaMalloc(&tab, bytes) != cudaSuccess) {
    cudaGetLastError();
    tab = nullptr;
  }
  if (tab) {
    e = launch_atx_chords(d_inst, d, nv, K, tab, kmax, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(hk, kmax, sizeof(hk), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e == cudaSuccess && hk[1] == 0) {
      *tab_out = tab;
      *K_out = K;
      *bytes_out = bytes;
      tab = nullptr;
    }
  }
  if (tab) cudaFree(tab);
  cudaFree(kmax);
  return e;
}

}  // namespace asd

extern "C" {

int asdpocs_adjoint_check(const float *X, const float *yv, float cos_phi, float sin_phi,
                          const float *y_det, const float *z_det, float SO, float OD,
                          float scale, float dy_det, float dz_det, float dz, int nx,
                          int ny, int nz, int na, int nb, double dots[2]) {
  clear_error();
  if (int e = check_dims(nx, ny, nz, na, nb)) return e;
  if (!X || !yv || !y_det || !z_det || !dots)
    return set_error(ASDPOCS_ERR_ARG, "null pointer");
  const size_t N = (size_t)nx * ny * nz, M = (size_t)na * nb;
  const size_t oX = 0, oY = oX + align256(N * 4), oAx = oY + align256(M * 4),
               oSr = oAx + align256(M * 4), oAty = oSr + align256(M * 4),
               oSc = oAty + align256(N * 4), oA = oSc + align256(N * 4),
               oB = oA + align256((size_t)na * 4), oP = oB + align256((size_t)nb * 4),
               oD = oP + align256((size_t)kDotBlocks * 8), tot = oD + 256;
  Workspace *w;
  if (int e = ws_acquire(w, tot)) return e;
  std::lock_guard<std::mutex> lk(w->mu);
  char *b = (char *)w->buf;
  ASD_CUDA(cudaMemcpyAsync(b + oX, X, N * 4, cudaMemcpyHostToDevice, w->st));
  ASD_CUDA(cudaMemcpyAsync(b + oY, yv, M * 4, cudaMemcpyHostToDevice, w->st));
  ASD_CUDA(cudaMemcpyAsync(b + oA, y_det, (size_t)na * 4, cudaMemcpyHostToDevice, w->st));
  ASD_CUDA(cudaMemcpyAsync(b + oB, z_det, (size_t)nb * 4, cudaMemcpyHostToDevice, w->st));
  const ViewGeo g = with_constants(ViewGeo{cos_phi, sin_phi, SO, OD, scale, dy_det, dz_det,
                                           dz, (const float *)(b + oA),
                                           (const float *)(b + oB)});
  const Dims d{nx, ny, nz, na, nb};
  ASD_CUDA(launch_ax((const float *)(b + oX), (float *)(b + oAx), (float *)(b + oSr), g, d,
                     w->st));
  ASD_CUDA(launch_atx((float *)(b + oAty), (const float *)(b + oY), (float *)(b + oSc), g, d,
                      w->st));
  double *part = (double *)(b + oP), *dd = (double *)(b + oD);
  k_dot_f64<<<kDotBlocks, kDotThreads, 0, w->st>>>((const float *)(b + oAx),
                                                   (const float *)(b + oY), (long long)M,
                                                   part);
  k_sum_f64<<<1, 1, 0, w->st>>>(part, kDotBlocks, dd);
  k_dot_f64<<<kDotBlocks, kDotThreads, 0, w->st>>>((const float *)(b + oX),
                                                   (const float *)(b + oAty), (long long)N,
                                                   part);
  k_sum_f64<<<1, 1, 0, w->st>>>(part, kDotBlocks, dd + 1);
  ASD_CUDA(cudaGetLastError());
  ASD_CUDA(cudaMemcpyAsync(dots, dd, 16, cudaMemcpyDeviceToHost, w->st));
  ASD_CUDA(cudaStreamSynchronize(w->st));
  return 0;
}

static int atx_host(float *X, const float *yv, float *sc, float cos_phi,
                    float sin_phi, const float *y_det, const float *z_det,
                    float SO, float OD, float scale, float dy_det, float dz_det,
                    float dz, int nx, int ny, int nz, int na, int nb) {
  clear_error();
  if (int e = check_dims(nx, ny, nz, na, nb)) return e;
  if (!X || !yv || !sc || !y_det || !z_det)
    return set_error(ASDPOCS_ERR_ARG, "null pointer");
  const size_t N = (size_t)nx * ny * nz, M = (size_t)na * nb;
  const Dims d{nx, ny, nz, na, nb};
  // cone beams: the view's ray tables for the z-column backward step
  const size_t zs = nz > 1 ? atx_zcol_scratch_bytes(d) : 0;
  const size_t oX = 0, oS = align256(N * 4), oY = oS + align256(N * 4),
               oA = oY + align256(M * 4), oB = oA + align256((size_t)na * 4),
               oT = oB + align256((size_t)nb * 4), tot = oT + zs;
  Workspace *w;
  if (int e = ws_acquire(w, tot)) return e;
  std::lock_guard<std::mutex> lk(w->mu);
  char *b = (char *)w->buf;
  ASD_CUDA(cudaMemcpyAsync(b + oY, yv, M * 4, cudaMemcpyHostToDevice, w->st));
  ASD_CUDA(cudaMemcpyAsync(b + oA, y_det, (size_t)na * 4, cudaMemcpyHostToDevice, w->st));
  ASD_CUDA(cudaMemcpyAsync(b + oB, z_det, (size_t)nb * 4, cudaMemcpyHostToDevice, w->st));
  const ViewGeo g = with_constants(ViewGeo{cos_phi, sin_phi, SO, OD, scale,
                                           dy_det, dz_det, dz, (const float *)(b + oA),
                                           (const float *)(b + oB)});
  if (nz > 1)
    ASD_CUDA(launch_atx_zcol((float *)(b + oX), (const float *)(b + oY), (float *)(b + oS), g,
                             d, b + oT, w->st));
  else
    ASD_CUDA(launch_atx((float *)(b + oX), (const float *)(b + oY), (float *)(b + oS), g, d,
                        w->st));
  ASD_CUDA(cudaMemcpyAsync(X, b + oX, N * 4, cudaMemcpyDeviceToHost, w->st));
  ASD_CUDA(cudaMemcpyAsync(sc, b + oS, N * 4, cudaMemcpyDeviceToHost, w->st));
  ASD_CUDA(cudaStreamSynchronize(w->st));
  return 0;
}

void Ax_cone_mf_gpu_new(float *X, float *y, float *sr, float cos_phi,
                        float sin_phi, float *y_det, float *z_det, float SO,
                        float OD, float scale, float dz, int nx, int ny, int nz,
                        int na, int nb) {
  ax_host(X, y, sr, cos_phi, sin_phi, y_det, z_det, SO, OD, scale, dz, nx, ny,
          nz, na, nb);
}

int asdpocs_ax_siddon(const float *X, float *y, float *sr, float cos_phi,
                      float sin_phi, const float *y_det, const float *z_det,
                      float SO, float OD, float scale, float dz, int nx, int ny,
                      int nz, int na, int nb) {
  return ax_host(X, y, sr, cos_phi, sin_phi, y_det, z_det, SO, OD, scale, dz, nx, ny, nz,
                 na, nb, true);
}

void Atx_cone_mf_gpu_new(float *X, float *y, float *sc, float cos_phi,
                         float sin_phi, float *y_det, float *z_det, float SO,
                         float OD, float scale, float dy_det, float dz_det,
                         float dz, int nx, int ny, int nz, int na, int nb) {
  atx_host(X, y, sc, cos_phi, sin_phi, y_det, z_det, SO, OD, scale, dy_det,
           dz_det, dz, nx, ny, nz, na, nb);
}

// ------------------------------------------------------ mex-level calls
static int check_para(const asdpocs_para *p) {
  if (!p) return set_error(ASDPOCS_ERR_ARG, "Error usage! (para is NULL)");
  return check_dims(p->nx, p->ny, p->nz, p->na, p->nb);
}

int Ax_cone_gpu(const float *X, long long numel_X, const asdpocs_para *para,
                float *y, float *sr) {
  clear_error();
  if (int e = check_para(para)) return e;
  if (numel_X != (long long)para->nx * para->ny * para->nz)
    return set_error(ASDPOCS_ERR_ARG, "Error size of input argument X!");
  GatewayGeo g;
  gateway_geometry(para->phi, para->SO, para->OD, para->vxlsize, para->detsize,
                   para->na, para->nb, g);
  return ax_host(X, y, sr, g.cos_phi, g.sin_phi, g.y_det.data(), g.z_det.data(),
                 g.SO, g.OD, g.scale, 1.0f, para->nx, para->ny, para->nz,
                 para->na, para->nb);
}

int asdpocs_adjoint_check_para(const float *X, long long numel_X, const float *Y,
                               long long numel_Y, const asdpocs_para *para,
                               double dots[2]) {
  clear_error();
  if (int e = check_para(para)) return e;
  if (numel_X != (long long)para->nx * para->ny * para->nz)
    return set_error(ASDPOCS_ERR_ARG, "Error size of input argument X!");
  if (numel_Y != (long long)para->na * para->nb)
    return set_error(ASDPOCS_ERR_ARG, "Error size of input argument Y!");
  GatewayGeo g;
  gateway_geometry(para->phi, para->SO, para->OD, para->vxlsize, para->detsize,
                   para->na, para->nb, g);
  return asdpocs_adjoint_check(X, Y, g.cos_phi, g.sin_phi, g.y_det.data(), g.z_det.data(),
                               g.SO, g.OD, g.scale, g.det, g.det, 1.0f, para->nx,
                               para->ny, para->nz, para->na, para->nb, dots);
}

int Atx_cone_gpu(const float *Y, long long numel_Y, const asdpocs_para *para,
                 float *x, float *sc) {
  clear_error();
  if (int e = check_para(para)) return e;
  if (numel_Y != (long long)para->na * para->nb)
    return set_error(ASDPOCS_ERR_ARG, "Error size of input argument Y!");
  GatewayGeo g;
  gateway_geometry(para->phi, para->SO, para->OD, para->vxlsize, para->detsize,
                   para->na, para->nb, g);
  return atx_host(x, Y, sc, g.cos_phi, g.sin_phi, g.y_det.data(),
                  g.z_det.data(), g.SO, g.OD, g.scale, g.det, g.det, 1.0f,
                  para->nx, para->ny, para->nz, para->na, para->nb);
}

}  // extern "C"

// ------------------------------------------------------------------- TV
template <class T>
static int tv_host(const T *img, T *out, int nx, int ny, int nz, double alpha,
                   int n, int pos, const T *old) {
  clear_error();
  if (!img || !out) return set_error(ASDPOCS_ERR_ARG, "null pointer");
  if (int e = check_tv_dims(nx, ny, nz)) return e;
  const size_t N = (size_t)nx * ny * nz;
  const size_t tiles = (size_t)((nx + 31) / 32) * ((ny + 7) / 8) * nz;
  const size_t oI = 0, oO = align256(N * sizeof(T)), oA = oO + align256(N * sizeof(T)),
               oB = oA + align256(N * sizeof(T)), oS = oB + align256(N * sizeof(T)),
               oP = oS + 256, oC = oP + align256(tiles * sizeof(double) * 3),
               tot = oC + 256;
  Workspace *w;
  if (int e = ws_acquire(w, tot)) return e;
  std::lock_guard<std::mutex> lk(w->mu);
  char *b = (char *)w->buf;
  ASD_CUDA(cudaMemsetAsync(b + oC, 0, 256, w->st));
  ASD_CUDA(cudaMemcpyAsync(b + oI, img, N * sizeof(T), cudaMemcpyHostToDevice, w->st));
  if (old)
    ASD_CUDA(cudaMemcpyAsync(b + oO, old, N * sizeof(T), cudaMemcpyHostToDevice, w->st));
  cudaError_t e;
  if (sizeof(T) == 8)
    e = tv_minimize_f64((double *)(b + oI), old ? (const double *)(b + oO) : nullptr,
                        (double *)(b + oA), (double *)(b + oB), (double *)(b + oS),
                        (double *)(b + oP), (unsigned *)(b + oC), nx, ny, nz, alpha,
                        n, pos, w->st);
  else
    e = tv_minimize_f32((float *)(b + oI), old ? (const float *)(b + oO) : nullptr,
                        (float *)(b + oA), (float *)(b + oB), (double *)(b + oS),
                        (double *)(b + oP), (unsigned *)(b + oC), nx, ny, nz, alpha,
                        n, pos, w->st);
  ASD_CUDA(e);
  ASD_CUDA(cudaMemcpyAsync(out, b + oI, N * sizeof(T), cudaMemcpyDeviceToHost, w->st));
  ASD_CUDA(cudaStreamSynchronize(w->st));
  return 0;
}

extern "C" {

int imgTVGradMin(const double *img, double *img_out, int rowN, int colN,
                 double alpha, int nTVIter, int pos, const double *img_old) {
  return tv_host<double>(img, img_out, rowN, colN, 1, alpha, nTVIter, pos,
                         img_old);
}

int imgTVGradMin3D(const double *img, double *img_out, int Nx, int Ny, int Nz,
                   double alpha, int nTVIter, int pos, const double *img_old) {
  if (Nz < 1) return set_error(ASDPOCS_ERR_ARG, "bad image dimensions");
  if (Nz < 2) {
    // MATLAB drops a trailing singleton dimension, so the reference never
    // sees Nz == 1 in a valid call (it would read past the dimension array,
    // imgTVGradMin3D.cpp:44-46).  Such calls are rejected.
    return set_error(ASDPOCS_ERR_ARG,
                     "imgTVGradMin3D expects a 3-D image (Nz >= 2)");
  }
  return tv_host<double>(img, img_out, Nx, Ny, Nz, alpha, nTVIter, pos,
                         img_old);
}

int asdpocs_tv_device(float *img_d, const float *img_old_d, int nx, int ny,
                      int nz, double alpha, int nTVIter, int pos,
                      void *stream) {
  clear_error();
  if (!img_d) return set_error(ASDPOCS_ERR_ARG, "null pointer");
  if (int e = check_tv_dims(nx, ny, nz)) return e;
  const size_t N = (size_t)nx * ny * nz;
  const size_t tiles = (size_t)((nx + 31) / 32) * ((ny + 7) / 8) * nz;
  const size_t oA = 0, oB = align256(N * 4), oS = oB + align256(N * 4),
               oP = oS + 256, oC = oP + align256(tiles * sizeof(double) * 3),
               tot = oC + 256;
  Workspace *w;
  if (int e = ws_acquire(w, tot)) return e;
  std::lock_guard<std::mutex> lk(w->mu);
  char *b = (char *)w->buf;
  cudaStream_t st = (cudaStream_t)stream;
  ASD_CUDA(cudaMemsetAsync(b + oC, 0, 256, st));
  ASD_CUDA(tv_minimize_f32(img_d, img_old_d, (float *)(b + oA), (float *)(b + oB),
                           (double *)(b + oS), (double *)(b + oP),
                           (unsigned *)(b + oC), nx, ny, nz, alpha, nTVIter, pos,
                           st));
  // the workspace is reused by the next call: finish before releasing it
  ASD_CUDA(cudaStreamSynchronize(st));
  return 0;
}

void asdpocs_options_default(asdpocs_options *o) {
  if (!o) return;
  o->maxnumIter = 5;
  o->numOfgradients = 20;
  o->alpha = 0.02;
  o->alpha_red = 0.95;
  o->beta = 1.0;
  o->beta_red = 0.995;
  o->r_max = 0.95;
  o->epsilon = 2.220446049250313e-16;
  o->stopRelChg = 2.220446049250313e-16;
  o->sino_storage = ASDPOCS_STORE_F32;
  o->ax_mode = ASDPOCS_AX_REFERENCE;
}

int asdpocs_store_sinogram(const float *in, void *out, unsigned long long n, int storage) {
  clear_error();
  if (n && (!in || !out)) return set_error(ASDPOCS_ERR_ARG, "null pointer");
  if (storage < ASDPOCS_STORE_F32 || storage > ASDPOCS_STORE_BF16)
    return set_error(ASDPOCS_ERR_ARG, "unknown sinogram storage %d", storage);
  store_sinogram_host(in, out, (size_t)n, storage);
  return 0;
}

}  // extern "C"

// ======================================================================
// Plans: batched, device-resident ASD-POCS
// ======================================================================
namespace asd {
// A plan's batch runs as one or two sub-batches, each on its own stream with
// its own captured iteration, so that the forward, backward and TV kernels
// of one sub-batch overlap those of the other (each kernel alone leaves the
// GPU partly idle: it is bound by latency, not by a unit's throughput).
// Instances never read each other's state, so results do not change.
struct SubBatch {
  int first = 0, count = 0;  // instances [first, first + count)
  // plans of uneven instances: the sub-batch's instances (any of the plan's,
  // in order) and their device list in the plan's arena (null: the range
  // above)
  std::vector<int> members;
  std::vector<int> units;  // the groups (mixed plans) or instances dealt to it
  const int *zall = nullptr;
  // runs the shared-geometry kernels: over [first, first + count) in groups
  // of kShareSlots, or (mixed plans) over the groups of groups_host (first
  // position in d_inst, count) with their device list gall
  bool shared = false;
  std::vector<int2> groups_host;
  const int2 *gall = nullptr;
  std::vector<int2> gtab_host;  // mixed plans: the view sets' group lists
  Dims d{};                  // largest sizes of these instances
  int nv = 0, max_ng = 0, min_ng = 0;
  // instances of different view counts: the runs of views and who has them
  // (lists in the plan's arena), and the lists on the host
  std::vector<ViewSet> sets;
  std::vector<int> zmap_host;
  cudaStream_t st = nullptr;  // the plan's stream when there is one sub-batch
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaEvent_t done = nullptr;
};
}  // namespace asd

struct asdpocs_plan_s {
  int device = 0;
  cudaStream_t st = nullptr;
  bool own_stream = false;
  int batch = 0;
  Dims d{};    // largest sizes over the instances (grids of the launches)
  int nv = 0;  // largest number of views
  int max_iter = 0, max_ng = 0, min_ng = 0;
  std::vector<asdpocs_geometry> geom;
  std::vector<asdpocs_options> opt;
  std::vector<Inst> h_inst;
  std::vector<int> has_ref;
  bool shared = false;  // all instances share sizes, geometry and angles
  // 2-D instances of several geometries that run as groups of instances
  // sharing geometry (the shared-geometry kernels with group tables): the
  // groups (instance indices) and each instance's position in d_inst, where
  // every group is contiguous
  bool mixed = false;
  std::vector<std::vector<int>> groups;
  std::vector<int> gclass;  // each group's geometry (groups of one geometry share it)
  std::vector<int> slot;
  std::vector<Inst> h_dev;  // mixed plans: the descriptors in d_inst order
  std::vector<size_t> phi_off;  // each instance's first angle in phi_vec_deg
  bool zcol = true;     // cone beams: z-column backward step (else per voxel)
  bool exact = false;   // forward steps: exact Siddon projection (ax_mode)
  int tv_walk = 0;      // TV walk length (0: from the batch size)
  int zseg = 0;         // z-column segment length (0: the default)
  int ax_u = 0, ax_q = 0;  // shared forward step's shape (0: the defaults)
  int pdl = -1;         // programmatic dependent launches: -1 = when the plan
                        // runs on one stream, 0 = off, 1 = on
  Inst *d_inst = nullptr;
  void *arena = nullptr;
  size_t bytes = 0;
  std::vector<asd::SubBatch> subs;
  cudaEvent_t fork = nullptr;  // orders the sub-batches after the plan's stream
  int *chtab = nullptr;        // backward-step chord tables (2-D shared plans)
  int chK = 0;                 // their slots per voxel and view (the largest
                               // over the instances' own tables)
  std::vector<int *> inst_tabs;  // instances' own tables (2-D, geometry apart)
  unsigned long long budget = 0;  // HBM budget of the plan (0: none)
};

namespace asd {

int instance_kind(const asdpocs_geometry &g) {
  return g.nz > 1 ? 2 : (g.nb > 1 ? 1 : 0);
}

// FP32 to FP16, round to nearest with ties to even (IEEE 754 binary16).
static uint16_t f32_to_f16(float f) {
  uint32_t x;
  memcpy(&x, &f, 4);
  const uint32_t sign = (x >> 16) & 0x8000u;
  const uint32_t ax = x & 0x7fffffffu;
  if (ax > 0x7f800000u) return (uint16_t)(sign | 0x7e00u | ((ax >> 13) & 0x3ffu));  // NaN
  if (ax >= 0x477ff000u) return (uint16_t)(sign | 0x7c00u);  // rounds to inf (or is inf)
  if (ax >= 0x38800000u) {  // normal half: rebias the exponent, round 13 bits
    const uint32_t m = ax - 0x38000000u;  // exponent 127 -> 15
    const uint32_t r = (m >> 13) + (((m >> 12) & 1u) & (((m & 0xfffu) != 0) | ((m >> 13) & 1u)));
    return (uint16_t)(sign | r);
  }
  if (ax < 0x33000000u) return (uint16_t)sign;  // below half the smallest subnormal
  // subnormal half: value = mant * 2^-24 with the implicit bit restored
  const uint32_t e = ax >> 23;              // 102 .. 112
  const uint32_t mant = (ax & 0x7fffffu) | 0x800000u;
  const uint32_t shift = 126 - e;           // bits dropped: 14 .. 24
  const uint32_t q = mant >> shift, rem = mant & ((1u << shift) - 1u), half = 1u << (shift - 1);
  const uint32_t r = q + ((rem > half) || (rem == half && (q & 1u)) ? 1u : 0u);
  return (uint16_t)(sign | r);
}

// FP32 to BF16, round to nearest with ties to even; NaN stays NaN.
static uint16_t f32_to_bf16(float f) {
  uint32_t x;
  memcpy(&x, &f, 4);
  if ((x & 0x7fffffffu) > 0x7f800000u) return (uint16_t)((x >> 16) | 0x40u);
  const uint32_t r = x + 0x7fffu + ((x >> 16) & 1u);
  return (uint16_t)(r >> 16);
}

void store_sinogram_host(const float *in, void *out, size_t n, int fmt) {
  if (fmt == ASDPOCS_STORE_F32) {
    memcpy(out, in, n * 4);
    return;
  }
  uint16_t *o = (uint16_t *)out;
  if (fmt == ASDPOCS_STORE_F16)
    for (size_t i = 0; i < n; i++) o[i] = f32_to_f16(in[i]);
  else
    for (size_t i = 0; i < n; i++) o[i] = f32_to_bf16(in[i]);
}

int check_instance(const asdpocs_geometry &g, const asdpocs_options &o) {
  if (int e = check_dims(g.nx, g.ny, g.nz, g.na, g.nb)) return e;
  if (o.sino_storage < ASDPOCS_STORE_F32 || o.sino_storage > ASDPOCS_STORE_BF16)
    return set_error(ASDPOCS_ERR_ARG, "unknown sinogram storage %d", o.sino_storage);
  if (o.ax_mode != ASDPOCS_AX_REFERENCE && o.ax_mode != ASDPOCS_AX_EXACT)
    return set_error(ASDPOCS_ERR_ARG, "unknown forward mode %d", o.ax_mode);
  if (g.nv <= 0) return set_error(ASDPOCS_ERR_ARG, "nv must be positive");
  if (o.maxnumIter < 0 || o.numOfgradients < 0)
    return set_error(ASDPOCS_ERR_ARG, "negative iteration counts");
  return 0;
}

InstLayout layout_instance(const asdpocs_geometry &g, int max_iter,
                           size_t cor_floats, int parts, size_t il_floats,
                           int sino_storage) {
  const Dims d{g.nx, g.ny, g.nz, g.na, g.nb};
  const size_t N = (size_t)g.nx * g.ny * g.nz;
  const size_t M = (size_t)g.na * g.nb;
  const bool st = parts & kLayoutState, geo = parts & kLayoutGeometry;
  const size_t per_img = st ? align256(N * 4) : 0;
  const size_t nblk = (size_t)reduce_blocks_for(d);
  const bool proj3d = g.nz > 1 || g.nb > 1;
  InstLayout o;
  size_t off = 0;
  o.p_fmt = sino_storage;
  o.P = off; off += st ? align256(M * g.nv * sino_elem_bytes(sino_storage)) : 0;
  o.m = off; off += per_img;
  o.m_pre = off; off += per_img;
  o.m_res = off; off += per_img;
  o.m_k1 = off; off += per_img;
  o.I0 = off; off += per_img;
  o.tvb = off; off += per_img;
  o.tvc = off; off += per_img;
  o.rmse = off; off += st ? align256((size_t)(max_iter + 1) * 8) : 0;
  // block partials of the projector and tile kernels; the 2-D walks keep four
  // values per strip and band
  const size_t nparts = std::max(nblk * kMaxReduceK, (size_t)tv_partials_for(d) * 4);
  o.part = off; off += st ? align256(nparts * 8) : 0;
  o.cnt = off; off += st ? 256 : 0;
  o.scal = off; off += st ? align256(sizeof(Scalars)) : 0;
  o.cor = off; off += geo ? align256(cor_floats * 4) : 0;
  o.m_il = off; off += geo ? align256(il_floats * 4) : 0;
  o.tabA = off; off += geo ? align256((size_t)g.na * g.nv * 16) : 0;
  o.vflags = off; off += geo ? align256((size_t)g.nv * 4) : 0;
  o.tabC = off; off += geo ? align256(proj3d ? M * 16 : 16) : 0;
  o.ydet = off; off += geo ? align256((size_t)g.na * 4) : 0;
  o.zdet = off; off += geo ? align256((size_t)g.nb * 4) : 0;
  o.trig = off; off += geo ? align256((size_t)g.nv * 8) : 0;
  o.bytes = off;
  return o;
}

void bind_state(Inst &I, char *b, const InstLayout &o) {
  I.P = (const void *)(b + o.P);
  I.p_fmt = o.p_fmt;
  I.m = (float *)(b + o.m);
  I.m_pre = (float *)(b + o.m_pre);
  I.m_res = (float *)(b + o.m_res);
  I.m_k1 = (float *)(b + o.m_k1);
  I.I0 = (float *)(b + o.I0);
  I.tv_b = (float *)(b + o.tvb);
  I.tv_c = (float *)(b + o.tvc);
  I.rmse = (double *)(b + o.rmse);
  I.partials = (double *)(b + o.part);
  I.counter = (unsigned *)(b + o.cnt);
  I.s = (Scalars *)(b + o.scal);
}

cudaError_t bind_geometry(Inst &I, char *b, const InstLayout &o,
                          const asdpocs_geometry &g, const double *phi_deg,
                          cudaStream_t st) {
  I.d = Dims{g.nx, g.ny, g.nz, g.na, g.nb};
  I.nv = g.nv;
  GatewayGeo gg;
  gateway_geometry(0.0, g.SO, g.OD, g.vxlsize, g.detsize, g.na, g.nb, gg);
  I.g = with_constants(ViewGeo{0.f, 0.f, gg.SO, gg.OD, gg.scale, gg.det, gg.det,
                               1.0f, (const float *)(b + o.ydet),
                               (const float *)(b + o.zdet)});
  std::vector<float2> trig(g.nv);
  for (int v = 0; v < g.nv; v++) trig[v] = view_trig(phi_deg[v]);
  I.trig = (const float2 *)(b + o.trig);
  I.cor = (float *)(b + o.cor);
  I.cor_stride = 1;
  I.m_il = nullptr;
  I.tabA = (float4 *)(b + o.tabA);
  I.vflags = (int *)(b + o.vflags);
  I.tabC = (float4 *)(b + o.tabC);
  I.tabc_mode = kTabcOwn;
  I.chtab = nullptr;
  I.chK = 0;
  // pageable sources: staged before each call returns
  cudaError_t e = cudaMemcpyAsync(b + o.ydet, gg.y_det.data(), (size_t)g.na * 4,
                                  cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(b + o.zdet, gg.z_det.data(), (size_t)g.nb * 4,
                        cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(b + o.trig, trig.data(), (size_t)g.nv * 8,
                        cudaMemcpyHostToDevice, st);
  return e;
}

cudaError_t bind_instance(Inst &I, char *b, const InstLayout &o,
                          const asdpocs_geometry &g, const double *phi_deg,
                          cudaStream_t st) {
  bind_state(I, b, o);
  return bind_geometry(I, b, o, g, phi_deg, st);
}

Scalars initial_scalars(const asdpocs_options &o, bool has_ref) {
  Scalars s;
  memset(&s, 0, sizeof s);
  s.alpha = o.alpha;
  s.beta = o.beta;
  s.beta_f = (float)o.beta;
  s.alpha_red = o.alpha_red;
  s.beta_red = o.beta_red;
  s.r_max = o.r_max;
  s.epsilon = o.epsilon;
  s.stopRelChg = o.stopRelChg;
  s.k = 1;
  s.maxIter = o.maxnumIter;
  s.ng = o.numOfgradients;
  s.done = o.maxnumIter <= 0;
  s.has_ref = has_ref;
  return s;
}

cudaError_t reset_instance(const Inst &I, const Scalars &s, cudaStream_t st) {
  const size_t bytes = (size_t)I.d.nx * I.d.ny * I.d.nz * 4;
  cudaError_t e = cudaMemcpyAsync(I.m, I.m_k1, bytes, cudaMemcpyDeviceToDevice, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(I.m_pre, I.m_k1, bytes, cudaMemcpyDeviceToDevice, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(I.m_res, I.m_k1, bytes, cudaMemcpyDeviceToDevice, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(I.counter, 0, 256, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(I.s, &s, sizeof s, cudaMemcpyHostToDevice, st);
  return e;
}

}  // namespace asd

namespace asd {

cudaError_t enqueue_iteration(const Inst *d_inst, int batch, const Dims &d,
                              int nv, int ng, bool shared, cudaStream_t st,
                              const IterShape &sh, bool finish,
                              const std::vector<ViewSet> *sets, const int *zall,
                              const int2 *gall, int ngroups) {
  const PdlScope scope(sh.pdl);
  cudaError_t e = cudaSuccess;
  if (shared) e = launch_group_pack(d_inst, batch, d, 0, st, gall, ngroups);
  const bool by_set = sets && !sets->empty();
  size_t si = 0;
  for (int v = 0; v < nv && e == cudaSuccess; v++) {
    int vb = batch, vg = ngroups;
    Dims vd = d;
    const int *zmap = zall;
    const int2 *gtab = gall;
    if (by_set) {
      while (si + 1 < sets->size() && v >= (*sets)[si].v1) si++;
      const ViewSet &S = (*sets)[si];
      vb = vg = S.count;
      vd = S.d;
      zmap = S.zmap;
      gtab = S.gtab;
      if (S.count == 0) continue;
    }
    if (shared) {
      e = launch_sart_ax_shared(d_inst, batch, vd, v, st, sh.ax_u, sh.ax_q, gtab, vg);
      if (e == cudaSuccess) e = launch_sart_atx_shared(d_inst, batch, vd, v, st, gtab, vg);
      continue;
    }
    e = launch_sart_ax(d_inst, vb, vd, v, st, sh.exact, zmap);
    if (e == cudaSuccess) e = launch_sart_atx(d_inst, vb, vd, v, st, sh.zcol, sh.zseg, zmap);
  }
  if (shared && e == cudaSuccess) e = launch_group_pack(d_inst, batch, d, 1, st, gall, ngroups);
  if (e == cudaSuccess) e = launch_after_sweep(d_inst, batch, d, st, zall);
  for (int s = 0; s < ng && e == cudaSuccess; s++)
    e = launch_tv_step(d_inst, batch, d, s, ng, st, sh.tv_walk, zall);
  if (e == cudaSuccess && finish) e = launch_finish_iter(d_inst, batch, d, ng, st, zall);
  return e;
}

// The launch shapes of the plan's iterations.
static IterShape plan_shape(asdpocs_plan p) {
  IterShape sh;
  sh.tv_walk = p->tv_walk;
  sh.zcol = p->zcol;
  sh.zseg = p->zseg;
  sh.ax_u = p->ax_u;
  sh.ax_q = p->ax_q;
  sh.pdl = p->pdl < 0 ? p->subs.size() == 1 : p->pdl == 1;
  sh.exact = p->exact;
  return sh;
}

// One iteration of sub-batch s on its stream.
static int plan_enqueue_sub(asdpocs_plan p, const SubBatch &s) {
  const bool listed = !s.members.empty();
  ASD_CUDA(enqueue_iteration(listed ? p->d_inst : p->d_inst + s.first,
                             listed ? (int)s.members.size() : s.count, s.d, s.nv, s.max_ng,
                             s.shared, s.st, plan_shape(p), s.min_ng < 2, &s.sets, s.zall,
                             s.gall, (int)s.groups_host.size()));
  return 0;
}

// Splits the batch into up to kMaxSubBatches sub-batches of whole groups
// (kShareSlots instances), at least kSubGroups groups each; a single
// sub-batch runs on the plan's stream.  Sizes, view and TV-step counts per
// sub-batch.
constexpr int kMaxSubBatches = 2, kSubGroups = 1;
// Plans of instances that differ in view count or size run as up to
// kUnevenSubBatches sub-batches on their own streams: the later views of the
// instances with the most views are small launches bound by latency, which
// overlap only across streams.  The units dealt are the plan's groups of
// instances sharing geometry (mixed plans) or its instances.  Units of the
// same sizes go to the same sub-batches (a launch's grid is sized for its
// largest unit, so that mixed sizes leave blocks idle): each class of sizes
// gets sub-batches in proportion to its work (views x voxels), and its units
// are dealt by decreasing work to its sub-batch with the least work so far.
// With more classes than sub-batches every unit is dealt that way over all
// of them.
constexpr int kUnevenSubBatches = 8;
static bool plan_uneven(asdpocs_plan p) {
  if (p->shared) return false;
  const asdpocs_geometry &g0 = p->geom[0];
  for (int i = 1; i < p->batch; i++) {
    const asdpocs_geometry &g = p->geom[i];
    if (g.nv != g0.nv || g.nx != g0.nx || g.ny != g0.ny || g.nz != g0.nz || g.na != g0.na ||
        g.nb != g0.nb)
      return true;
  }
  return false;
}
static bool same_sizes(const asdpocs_geometry &g, const asdpocs_geometry &h) {
  return g.nx == h.nx && g.ny == h.ny && g.nz == h.nz && g.na == h.na && g.nb == h.nb;
}
// Units 0 .. n-1 (work[u], an instance of each in rep[u]) dealt to at most
// nsub bins as described above.
static std::vector<std::vector<int>> deal_units(asdpocs_plan p, const std::vector<double> &work,
                                                const std::vector<int> &rep, int nsub) {
  const int n = (int)work.size();
  std::vector<std::vector<int>> cls;  // classes of equal sizes, in order of first appearance
  for (int u = 0; u < n; u++) {
    size_t c = 0;
    while (c < cls.size() && !same_sizes(p->geom[rep[u]], p->geom[rep[cls[c][0]]])) c++;
    if (c == cls.size()) cls.emplace_back();
    cls[c].push_back(u);
  }
  if ((int)cls.size() > nsub) {  // more classes than sub-batches: one class
    cls.assign(1, std::vector<int>(n));
    std::iota(cls[0].begin(), cls[0].end(), 0);
  }
  // bins per class: one each, the rest one at a time to the class with the
  // most work per bin (while it has units to spare)
  std::vector<double> cw(cls.size(), 0.0);
  std::vector<int> cn(cls.size(), 1);
  for (size_t c = 0; c < cls.size(); c++)
    for (int u : cls[c]) cw[c] += work[u];
  for (int left = nsub - (int)cls.size(); left > 0; left--) {
    int best = -1;
    for (size_t c = 0; c < cls.size(); c++)
      if (cn[c] < (int)cls[c].size() && (best < 0 || cw[c] / cn[c] > cw[best] / cn[best]))
        best = (int)c;
    if (best < 0) break;
    cn[best]++;
  }
  std::vector<std::vector<int>> bins;
  for (size_t c = 0; c < cls.size(); c++) {
    std::vector<int> ord = cls[c];
    std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) { return work[a] > work[b]; });
    const size_t b0 = bins.size();
    bins.resize(b0 + cn[c]);
    std::vector<double> load(cn[c], 0.0);
    for (int u : ord) {
      const int k = (int)(std::min_element(load.begin(), load.end()) - load.begin());
      load[k] += work[u];
      bins[b0 + k].push_back(u);
    }
  }
  for (auto &b : bins) std::sort(b.begin(), b.end());
  return bins;
}
static void sub_add(SubBatch &s, asdpocs_plan p, int i) {
  const asdpocs_geometry &g = p->geom[i];
  s.d.nx = std::max(s.d.nx, g.nx);
  s.d.ny = std::max(s.d.ny, g.ny);
  s.d.nz = std::max(s.d.nz, g.nz);
  s.d.na = std::max(s.d.na, g.na);
  s.d.nb = std::max(s.d.nb, g.nb);
  s.nv = std::max(s.nv, g.nv);
  const int ng = p->opt[i].numOfgradients;
  s.max_ng = std::max(s.max_ng, ng);
  s.min_ng = std::min(s.min_ng, ng);
}
// The sub-batches' instances, sizes and counts (host only; plan_make_subs
// adds their streams).
static void plan_deal(asdpocs_plan p) {
  if (p->mixed || plan_uneven(p)) {
    // units: the groups (mixed plans) or the instances
    const int n = p->mixed ? (int)p->groups.size() : p->batch;
    std::vector<double> work(n);
    std::vector<int> rep(n);
    for (int u = 0; u < n; u++) {
      rep[u] = p->mixed ? p->groups[u][0] : u;
      const asdpocs_geometry &g = p->geom[rep[u]];
      // a group's march is shared; its instances' loads and sums are not
      const double per = p->mixed ? 1.0 + 0.25 * (double)p->groups[u].size() : 1.0;
      work[u] = (double)g.nv * g.nx * g.ny * g.nz * per;
    }
    const std::vector<std::vector<int>> bins =
        deal_units(p, work, rep, std::min(kUnevenSubBatches, n));
    const int total = (int)bins.size();
    p->subs.assign(total, SubBatch{});
    for (int k = 0; k < total; k++) {
      SubBatch &s = p->subs[k];
      s.shared = p->mixed;
      s.min_ng = INT_MAX;
      for (int u : bins[k]) {
        s.units.push_back(u);
        if (p->mixed) {
          const std::vector<int> &grp = p->groups[u];
          s.groups_host.push_back(make_int2(p->slot[grp[0]], (int)grp.size()));
          for (int i : grp) {
            s.members.push_back(p->slot[i]);
            sub_add(s, p, i);
          }
        } else {
          s.members.push_back(u);
          sub_add(s, p, u);
        }
      }
      std::sort(s.members.begin(), s.members.end());
    }
    return;
  }
  // whole groups per sub-batch, at least kSubGroups of them
  const int groups = (p->batch + kShareSlots - 1) / kShareSlots;
  const int want = std::max(1, std::min(kMaxSubBatches, groups / kSubGroups));
  const int per = (groups + want - 1) / want * kShareSlots;  // instances per sub-batch
  const int nsub = (p->batch + per - 1) / per;
  p->subs.assign(nsub, SubBatch{});
  for (int k = 0; k < nsub; k++) {
    SubBatch &s = p->subs[k];
    s.shared = p->shared;
    s.first = k * per;
    s.count = std::min(p->batch, (k + 1) * per) - s.first;
    for (int i = s.first; i < s.first + s.count; i++) {
      const asdpocs_geometry &g = p->geom[i];
      s.d.nx = std::max(s.d.nx, g.nx);
      s.d.ny = std::max(s.d.ny, g.ny);
      s.d.nz = std::max(s.d.nz, g.nz);
      s.d.na = std::max(s.d.na, g.na);
      s.d.nb = std::max(s.d.nb, g.nb);
      s.nv = std::max(s.nv, g.nv);
      const int ng = p->opt[i].numOfgradients;
      s.max_ng = std::max(s.max_ng, ng);
      s.min_ng = i == s.first ? ng : std::min(s.min_ng, ng);
    }
  }
}
// Streams of the sub-batches: a single one runs on the plan's stream.
static int plan_make_subs(asdpocs_plan p) {
  plan_deal(p);
  const bool multi = p->subs.size() > 1;
  for (SubBatch &s : p->subs) {
    if (!multi) {
      s.st = p->st;
    } else {
      ASD_CUDA(cudaStreamCreateWithFlags(&s.st, cudaStreamNonBlocking));
      ASD_CUDA(cudaEventCreateWithFlags(&s.done, cudaEventDisableTiming));
    }
  }
  if (multi) ASD_CUDA(cudaEventCreateWithFlags(&p->fork, cudaEventDisableTiming));
  return 0;
}

// Instances of one sub-batch with different view counts (plans without
// shared geometry): views [0, nv) cut at each distinct view count, and for
// each run the instances that still have views there, at their largest
// sizes -- so that the projector steps of the later views launch only those
// instances' blocks.  Every instance keeps its own grid positions, so its
// results are the same bits.
static void plan_view_sets(asdpocs_plan p) {
  if (p->shared) return;
  for (SubBatch &s : p->subs) {
    s.sets.clear();
    s.zmap_host.clear();
    s.gtab_host.clear();
    // units: the sub-batch's groups (mixed plans) or instances
    std::vector<int> who = s.units;
    const bool listed = !who.empty();
    if (!listed)
      for (int i = s.first; i < s.first + s.count; i++) who.push_back(i);
    auto rep_of = [&](int u) { return s.shared && listed ? p->groups[u][0] : u; };
    std::vector<int> cuts;
    for (int u : who) cuts.push_back(p->geom[rep_of(u)].nv);
    std::sort(cuts.begin(), cuts.end());
    cuts.erase(std::unique(cuts.begin(), cuts.end()), cuts.end());
    if (cuts.size() < 2) continue;  // every instance has every view
    int v0 = 0;
    for (int t : cuts) {
      ViewSet S;
      S.v0 = v0;
      S.v1 = t;
      S.zoff = s.shared ? s.gtab_host.size() : s.zmap_host.size();
      for (int u : who) {
        const int r = rep_of(u);
        const asdpocs_geometry &g = p->geom[r];
        if (g.nv <= v0) continue;
        if (s.shared)
          s.gtab_host.push_back(make_int2(p->slot[r], (int)p->groups[u].size()));
        else
          s.zmap_host.push_back(listed ? u : u - s.first);
        S.count++;
        S.d.nx = std::max(S.d.nx, g.nx);
        S.d.ny = std::max(S.d.ny, g.ny);
        S.d.nz = std::max(S.d.nz, g.nz);
        S.d.na = std::max(S.d.na, g.na);
        S.d.nb = std::max(S.d.nb, g.nb);
      }
      s.sets.push_back(S);
      v0 = t;
    }
  }
}

// First instance of the sub-batch holding instance i.
static int plan_sub_first(asdpocs_plan p, int i) {
  int f = 0;
  for (const SubBatch &s : p->subs)
    if (i >= s.first) f = s.first;
  return f;
}

}  // namespace asd

namespace asd {
// The host part of a plan: checks, per-instance options, and how the
// instances run (shared geometry, groups of a mixed plan, exact mode).  No
// GPU call; *out is a new plan, or null with the status set.
static int plan_describe(asdpocs_plan *out, int batch, const asdpocs_geometry *geom,
                         const double *phi_vec_deg, const asdpocs_options *opt) {
  if (!out || !geom || !phi_vec_deg || batch <= 0)
    return set_error(ASDPOCS_ERR_ARG, "bad plan arguments");
  *out = nullptr;
  const asdpocs_geometry &g0 = geom[0];
  Dims dmax{0, 0, 0, 0, 0};
  int nv_max = 0;
  std::vector<size_t> phi_off(batch);
  size_t phi_n = 0;
  asdpocs_options dflt;
  asdpocs_options_default(&dflt);
  for (int i = 0; i < batch; i++) {
    const asdpocs_geometry &gi = geom[i];
    if (int e = check_instance(gi, opt ? opt[i] : dflt)) return e;
    if (instance_kind(gi) != instance_kind(g0))
      return set_error(ASDPOCS_ERR_ARG,
                       "instances of one plan must be all 2-D (nz == nb == 1), "
                       "all single-slice, or all 3-D");
    dmax.nx = std::max(dmax.nx, gi.nx);
    dmax.ny = std::max(dmax.ny, gi.ny);
    dmax.nz = std::max(dmax.nz, gi.nz);
    dmax.na = std::max(dmax.na, gi.na);
    dmax.nb = std::max(dmax.nb, gi.nb);
    nv_max = std::max(nv_max, gi.nv);
    phi_off[i] = phi_n;
    phi_n += (size_t)gi.nv;
  }
  asdpocs_plan p = new (std::nothrow) asdpocs_plan_s;
  if (!p) return set_error(ASDPOCS_ERR_NOMEM, "host allocation");
  p->batch = batch;
  p->d = dmax;
  p->nv = nv_max;
  p->geom.assign(geom, geom + batch);
  p->phi_off = phi_off;
  p->opt.resize(batch);
  for (int i = 0; i < batch; i++) {
    p->opt[i] = opt ? opt[i] : dflt;
    if (p->opt[i].maxnumIter > p->max_iter) p->max_iter = p->opt[i].maxnumIter;
    if (p->opt[i].numOfgradients > p->max_ng)
      p->max_ng = p->opt[i].numOfgradients;
    if (i == 0 || p->opt[i].numOfgradients < p->min_ng)
      p->min_ng = p->opt[i].numOfgradients;
  }
  p->has_ref.assign(batch, 0);
  // instances with identical sizes, geometry and view angles share the
  // projector coefficients of every view
  auto same_geometry = [&](int i, int j) {
    const asdpocs_geometry &gi = geom[i], &gj = geom[j];
    return gi.nx == gj.nx && gi.ny == gj.ny && gi.nz == gj.nz && gi.na == gj.na &&
           gi.nb == gj.nb && gi.nv == gj.nv && gi.SO == gj.SO && gi.OD == gj.OD &&
           gi.vxlsize == gj.vxlsize && gi.detsize == gj.detsize &&
           memcmp(phi_vec_deg + phi_off[j], phi_vec_deg + phi_off[i],
                  sizeof(double) * (size_t)gj.nv) == 0;
  };
  p->shared = batch > 1;
  for (int i = 1; i < batch && p->shared; i++) p->shared = same_geometry(i, 0);
  // forward mode: one per plan; the shared-geometry forward step runs the
  // reference's march only, so exact plans run every instance on its own
  for (int i = 0; i < batch; i++)
    if (p->opt[i].ax_mode != p->opt[0].ax_mode) {
      delete p;
      return set_error(ASDPOCS_ERR_ARG,
                       "the instances of a plan must share one forward mode (ax_mode)");
    }
  p->exact = p->opt[0].ax_mode == ASDPOCS_AX_EXACT;
  if (p->exact) p->shared = false;
  if (getenv("ASDPOCS_NO_SHARED_GEOMETRY")) p->shared = false;
  // 2-D instances of several geometries: groups of up to kShareSlots
  // instances of one geometry (in instance order), laid out one after the
  // other in d_inst, when some instances share their geometry
  if (!p->shared && !p->exact && batch > 1 && !getenv("ASDPOCS_NO_SHARED_GEOMETRY")) {
    bool planar = true;
    for (int i = 0; i < batch; i++) planar = planar && geom[i].nz == 1 && geom[i].nb == 1;
    if (planar) {
      std::vector<int> cls(batch, -1), reps;
      for (int i = 0; i < batch; i++) {
        for (size_t c = 0; c < reps.size() && cls[i] < 0; c++)
          if (same_geometry(i, reps[c])) cls[i] = (int)c;
        if (cls[i] < 0) {
          cls[i] = (int)reps.size();
          reps.push_back(i);
        }
      }
      for (size_t c = 0; c < reps.size(); c++) {
        std::vector<int> cur;
        for (int i = 0; i < batch; i++) {
          if (cls[i] != (int)c) continue;
          cur.push_back(i);
          if ((int)cur.size() == kShareSlots) {
            p->groups.push_back(cur);
            p->gclass.push_back((int)c);
            cur.clear();
          }
        }
        if (!cur.empty()) {
          p->groups.push_back(cur);
          p->gclass.push_back((int)c);
        }
      }
      p->mixed = p->groups.size() < (size_t)batch;  // else no instance shares
      if (p->mixed) {
        p->slot.assign(batch, 0);
        int k = 0;
        for (const auto &g : p->groups)
          for (int i : g) p->slot[i] = k++;
      } else {
        p->groups.clear();
        p->gclass.clear();
      }
    }
  }
  // ASDPOCS_CONE_ATX=voxel: the per-voxel form of the cone-beam backward step
  // (same results; kept for comparison)
  {
    const char *f = getenv("ASDPOCS_CONE_ATX");
    p->zcol = !(f && strcmp(f, "voxel") == 0);
  }
  *out = p;
  return 0;
}

}  // namespace asd

extern "C" {


// The instances' descriptors to d_inst (mixed plans: in group order).
static cudaError_t plan_upload(asdpocs_plan p) {
  const Inst *src = p->h_inst.data();
  if (p->mixed) {
    p->h_dev.resize(p->batch);
    for (int i = 0; i < p->batch; i++) p->h_dev[p->slot[i]] = p->h_inst[i];
    src = p->h_dev.data();
  }
  return cudaMemcpyAsync(p->d_inst, src, sizeof(Inst) * p->batch, cudaMemcpyHostToDevice,
                         p->st);
}

// Device bytes the plan's chord tables may take: half the free memory, and
// what is left of the plan's HBM budget.
static cudaError_t plan_chord_room(asdpocs_plan p, size_t &room) {
  size_t free_b = 0, total_b = 0;
  const cudaError_t e = cudaMemGetInfo(&free_b, &total_b);
  room = free_b / 2;
  if (p->budget)
    room = std::min(room, p->budget > p->bytes ? (size_t)(p->budget - p->bytes) : (size_t)0);
  return e;
}

// The chord tables of a plan of one instance or of instances sharing
// geometry (see build_chord_tables); every instance's descriptor points at
// them.
static cudaError_t plan_chord_tables(asdpocs_plan p) {
  size_t room = 0;
  if (cudaError_t e0 = plan_chord_room(p, room)) return e0;
  int *tab = nullptr, K = 0;
  size_t bytes = 0;
  cudaError_t e = build_chord_tables(p->d_inst, p->d, p->nv, room, p->st, &tab, &K, &bytes);
  if (!tab) return e;
  p->chtab = tab;  // freed with the plan
  p->chK = K;
  p->bytes += bytes;
  for (Inst &I : p->h_inst) {
    I.chtab = tab;
    I.chK = K;
  }
  e = plan_upload(p);
  if (e == cudaSuccess) e = cudaStreamSynchronize(p->st);
  return e;
}

// Mixed plans: a table per geometry (the group's first instance, shared by
// the groups of that geometry), in group order, while they fit.
static cudaError_t plan_group_chord_tables(asdpocs_plan p) {
  size_t room = 0;
  cudaError_t e = plan_chord_room(p, room);
  if (e != cudaSuccess) return e;
  std::vector<int *> made(p->groups.size(), nullptr);
  std::vector<int> madeK(p->groups.size(), 0);
  bool any = false;
  for (size_t k = 0; k < p->groups.size() && e == cudaSuccess; k++) {
    const int r = p->groups[k][0];
    int *tab = nullptr, K = 0;
    // a group of a geometry that already has its table
    for (size_t j = 0; j < k && !tab; j++)
      if (made[j] && p->gclass[j] == p->gclass[k]) {
        tab = made[j];
        K = madeK[j];
      }
    if (!tab) {
      const asdpocs_geometry &g = p->geom[r];
      size_t bytes = 0;
      e = build_chord_tables(p->d_inst + p->slot[r], Dims{g.nx, g.ny, g.nz, g.na, g.nb}, g.nv,
                             room, p->st, &tab, &K, &bytes);
      if (!tab) continue;
      p->inst_tabs.push_back(tab);  // freed with the plan
      p->bytes += bytes;
      room -= bytes;
    }
    made[k] = tab;
    madeK[k] = K;
    p->chK = std::max(p->chK, K);
    for (int i : p->groups[k]) {
      p->h_inst[i].chtab = tab;
      p->h_inst[i].chK = K;
    }
    any = true;
  }
  if (e == cudaSuccess && any) e = plan_upload(p);
  if (e == cudaSuccess) e = cudaStreamSynchronize(p->st);
  return e;
}

// Instances of different 2-D geometry: a table per instance, in instance
// order, while they fit (plan_chord_room); the instances left without one
// compute their chords in every step.
static cudaError_t plan_instance_chord_tables(asdpocs_plan p) {
  size_t room = 0;
  cudaError_t e = plan_chord_room(p, room);
  if (e != cudaSuccess) return e;
  bool any = false;
  for (int i = 0; i < p->batch && e == cudaSuccess; i++) {
    const asdpocs_geometry &g = p->geom[i];
    int *tab = nullptr, K = 0;
    size_t bytes = 0;
    e = build_chord_tables(p->d_inst + i, Dims{g.nx, g.ny, g.nz, g.na, g.nb}, g.nv, room,
                           p->st, &tab, &K, &bytes);
    if (!tab) continue;
    p->inst_tabs.push_back(tab);  // freed with the plan
    p->chK = std::max(p->chK, K);
    p->bytes += bytes;
    room -= bytes;
    p->h_inst[i].chtab = tab;
    p->h_inst[i].chK = K;
    any = true;
  }
  if (e == cudaSuccess && any) {
    e = plan_upload(p);
    if (e == cudaSuccess) e = cudaStreamSynchronize(p->st);
  }
  return e;
}

int asdpocs_plan_create(asdpocs_plan *out, int batch,
                        const asdpocs_geometry *geom,
                        const double *phi_vec_deg, const asdpocs_options *opt,
                        unsigned long long hbm_budget_bytes, void *stream) {
  clear_error();
  if (out) *out = nullptr;
  asdpocs_plan p = nullptr;
  if (int rc = plan_describe(&p, batch, geom, phi_vec_deg, opt)) return rc;
  p->budget = hbm_budget_bytes;
  cudaGetDevice(&p->device);
  if (stream) {
    p->st = (cudaStream_t)stream;
  } else {
    cudaError_t e = cudaStreamCreateWithFlags(&p->st, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
      delete p;
      return cuda_status(e, "cudaStreamCreate");
    }
    p->own_stream = true;
  }
  if (int rc = plan_make_subs(p)) {
    asdpocs_plan_destroy(p);
    return rc;
  }
  plan_view_sets(p);
  // mixed plans: the first instance of each instance's group
  std::vector<int> group_first(batch, -1);
  for (const auto &g : p->groups)
    for (int i : g) group_first[i] = g[0];
  // ---- arena: each instance's block at its own sizes ----
  std::vector<InstLayout> lay(batch);
  std::vector<size_t> base(batch);
  size_t off = 0;
  for (int i = 0; i < batch; i++) {
    const size_t M = (size_t)geom[i].na * geom[i].nb;
    // shared-geometry groups interleave their residuals in the buffer of
    // the group's first instance (kShareSlots values per ray)
    const bool first = p->shared ? i % kShareSlots == 0 : p->mixed && group_first[i] == i;
    const size_t N = (size_t)geom[i].nx * geom[i].ny * geom[i].nz;
    lay[i] = layout_instance(geom[i], p->opt[i].maxnumIter, first ? M * kShareSlots : M,
                             kLayoutState | kLayoutGeometry, first ? N * kShareSlots : 0,
                             p->opt[i].sino_storage);
    base[i] = off;
    off += lay[i].bytes;
  }
  const size_t inst_off = off;
  off += align256(sizeof(Inst) * batch);
  const size_t zmap_off = off;  // the sub-batches' instance and group lists
  size_t zints = 0, zpairs = 0;
  for (const SubBatch &s : p->subs) {
    zints += s.zmap_host.size() + s.members.size();
    zpairs += s.groups_host.size() + s.gtab_host.size();
  }
  off += align256(zints * sizeof(int));
  const size_t gtab_off = off;
  off += align256(zpairs * sizeof(int2));
  p->bytes = off;
  if (hbm_budget_bytes && off > hbm_budget_bytes) {
    if (p->own_stream) cudaStreamDestroy(p->st);
    delete p;
    return set_error(ASDPOCS_ERR_NOMEM,
                     "plan needs %zu bytes, over the HBM budget of %llu", off,
                     hbm_budget_bytes);
  }
  cudaError_t e = cudaMalloc(&p->arena, off);
  if (e != cudaSuccess) {
    if (p->own_stream) cudaStreamDestroy(p->st);
    delete p;
    return cuda_status(e, "cudaMalloc(plan)");
  }
  char *b = (char *)p->arena;
  e = cudaMemsetAsync(b, 0, off, p->st);
  p->h_inst.resize(batch);
  for (int i = 0; i < batch && e == cudaSuccess; i++) {
    Inst &I = p->h_inst[i];
    e = bind_instance(I, b + base[i], lay[i], geom[i], phi_vec_deg + p->phi_off[i], p->st);
    if (p->mixed) {
      const int g = group_first[i];
      I.cor = (float *)(b + base[g] + lay[g].cor) + (p->slot[i] - p->slot[g]);
      I.cor_stride = kShareSlots;
      I.m_il = (float *)(b + base[g] + lay[g].m_il);
    }
    if (p->shared) {
      const int g = i - i % kShareSlots;
      I.cor = (float *)(b + base[g] + lay[g].cor) + i % kShareSlots;
      I.cor_stride = kShareSlots;
      I.m_il = (float *)(b + base[g] + lay[g].m_il);
      // one ray-slope table per sub-batch: its first instance refreshes it
      // every view (the sub-batches run different views at a time)
      const int f = plan_sub_first(p, i);
      I.tabC = (float4 *)(b + base[f] + lay[f].tabC);
      I.tabc_mode = i == f ? kTabcShared : kTabcNone;
    }
  }
  p->d_inst = (Inst *)(b + inst_off);
  if (e == cudaSuccess) e = plan_upload(p);
  {
    int *dz = (int *)(b + zmap_off);
    for (SubBatch &s : p->subs) {
      if (!s.members.empty()) {
        s.zall = dz;
        if (e == cudaSuccess)
          e = cudaMemcpyAsync(dz, s.members.data(), s.members.size() * sizeof(int),
                              cudaMemcpyHostToDevice, p->st);
        dz += s.members.size();
      }
      if (s.zmap_host.empty()) continue;
      for (ViewSet &S : s.sets) S.zmap = dz + S.zoff;
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(dz, s.zmap_host.data(), s.zmap_host.size() * sizeof(int),
                            cudaMemcpyHostToDevice, p->st);
      dz += s.zmap_host.size();
    }
    int2 *dg = (int2 *)(b + gtab_off);
    for (SubBatch &s : p->subs) {
      if (!s.groups_host.empty()) {
        s.gall = dg;
        if (e == cudaSuccess)
          e = cudaMemcpyAsync(dg, s.groups_host.data(), s.groups_host.size() * sizeof(int2),
                              cudaMemcpyHostToDevice, p->st);
        dg += s.groups_host.size();
      }
      if (s.gtab_host.empty()) continue;
      for (ViewSet &S : s.sets) S.gtab = dg + S.zoff;
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(dg, s.gtab_host.data(), s.gtab_host.size() * sizeof(int2),
                            cudaMemcpyHostToDevice, p->st);
      dg += s.gtab_host.size();
    }
  }
  if (e == cudaSuccess) e = launch_view_tables(p->d_inst, batch, p->d, p->nv, p->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(p->st);
  if (e == cudaSuccess && !getenv("ASDPOCS_NO_CHORD_TABLE"))
    e = p->shared || batch == 1 ? plan_chord_tables(p)
        : p->mixed              ? plan_group_chord_tables(p)
                                : plan_instance_chord_tables(p);
  if (e != cudaSuccess) {
    asdpocs_plan_destroy(p);
    return cuda_status(e, "plan setup");
  }
  *out = p;
  return asdpocs_plan_reset(p);
}

int asdpocs_plan_layout(int batch, const asdpocs_geometry *geom, const double *phi_vec_deg,
                        const asdpocs_options *opt, int *group_of, int *sub_of) {
  clear_error();
  asdpocs_plan p = nullptr;
  if (int rc = plan_describe(&p, batch, geom, phi_vec_deg, opt)) return -rc;
  plan_deal(p);
  std::vector<int> user(batch);  // instance at each position of d_inst
  for (int i = 0; i < batch; i++) user[p->mixed ? p->slot[i] : i] = i;
  for (int i = 0; i < batch; i++) {
    if (group_of) group_of[i] = -1;
    if (sub_of) sub_of[i] = -1;
  }
  if (group_of) {
    if (p->shared)
      for (int i = 0; i < batch; i++) group_of[i] = i / kShareSlots;
    for (size_t k = 0; k < p->groups.size(); k++)
      for (int i : p->groups[k]) group_of[i] = (int)k;
  }
  if (sub_of)
    for (size_t k = 0; k < p->subs.size(); k++) {
      const SubBatch &s = p->subs[k];
      if (!s.members.empty())
        for (int pos : s.members) sub_of[user[pos]] = (int)k;
      else
        for (int i = s.first; i < s.first + s.count; i++) sub_of[i] = (int)k;
    }
  const int n = (int)p->subs.size();
  delete p;
  return n;
}

int asdpocs_plan_destroy(asdpocs_plan p) {
  if (!p) return 0;
  for (SubBatch &s : p->subs) {
    if (s.exec) cudaGraphExecDestroy(s.exec);
    if (s.graph) cudaGraphDestroy(s.graph);
    if (s.st && s.st != p->st) {
      cudaStreamSynchronize(s.st);
      cudaStreamDestroy(s.st);
    }
    if (s.done) cudaEventDestroy(s.done);
  }
  if (p->fork) cudaEventDestroy(p->fork);
  if (p->st) cudaStreamSynchronize(p->st);
  if (p->arena) cudaFree(p->arena);
  if (p->chtab) cudaFree(p->chtab);
  for (int *t : p->inst_tabs) cudaFree(t);
  if (p->own_stream && p->st) cudaStreamDestroy(p->st);
  delete p;
  return 0;
}

unsigned long long asdpocs_plan_bytes(asdpocs_plan p) {
  return p ? (unsigned long long)p->bytes : 0ULL;
}

// bytes of one image of instance `inst`
static size_t inst_bytes(asdpocs_plan p, int inst) {
  const Dims &d = p->h_inst[inst].d;
  return (size_t)d.nx * d.ny * d.nz * 4;
}

static int plan_check(asdpocs_plan p, int inst) {
  if (!p) return set_error(ASDPOCS_ERR_ARG, "null plan");
  if (inst < 0 || inst >= p->batch)
    return set_error(ASDPOCS_ERR_ARG, "instance %d out of range", inst);
  return 0;
}

static int plan_put(asdpocs_plan p, void *dst, const void *src, size_t bytes,
                    int where) {
  if (!src) {
    ASD_CUDA(cudaMemsetAsync(dst, 0, bytes, p->st));
  } else {
    ASD_CUDA(cudaMemcpyAsync(dst, src, bytes,
                             where ? cudaMemcpyDeviceToDevice
                                   : cudaMemcpyHostToDevice,
                             p->st));
    if (!where) ASD_CUDA(cudaStreamSynchronize(p->st));
  }
  return 0;
}

int asdpocs_plan_set_sinogram(asdpocs_plan p, int inst, const float *P,
                              int where) {
  clear_error();
  if (int e = plan_check(p, inst)) return e;
  if (!P) return set_error(ASDPOCS_ERR_ARG, "null sinogram");
  const Inst &I = p->h_inst[inst];
  const size_t n = (size_t)I.d.na * I.d.nb * I.nv;
  if (I.p_fmt == ASDPOCS_STORE_F32) return plan_put(p, (void *)I.P, P, n * 4, where);
  // FP16 / BF16 storage: rounded on the device from a device sinogram, on
  // the host from a host one (the same bits either way)
  if (where) {
    ASD_CUDA(launch_store_sinogram(P, (void *)I.P, n, I.p_fmt, p->st));
    return 0;
  }
  std::vector<uint16_t> h(n);
  store_sinogram_host(P, h.data(), n, I.p_fmt);
  return plan_put(p, (void *)I.P, h.data(), n * 2, 0);
}

int asdpocs_plan_set_initial(asdpocs_plan p, int inst, const float *m0,
                             int where) {
  clear_error();
  if (int e = plan_check(p, inst)) return e;
  return plan_put(p, p->h_inst[inst].m_k1, m0, inst_bytes(p, inst), where);
}

int asdpocs_plan_set_reference(asdpocs_plan p, int inst, const float *I0,
                               int where) {
  clear_error();
  if (int e = plan_check(p, inst)) return e;
  p->has_ref[inst] = I0 != nullptr;
  return plan_put(p, p->h_inst[inst].I0, I0, inst_bytes(p, inst), where);
}

int asdpocs_plan_reset(asdpocs_plan p) {
  clear_error();
  if (!p) return set_error(ASDPOCS_ERR_ARG, "null plan");
  for (int i = 0; i < p->batch; i++)
    ASD_CUDA(reset_instance(p->h_inst[i], initial_scalars(p->opt[i], p->has_ref[i]),
                            p->st));
  ASD_CUDA(cudaStreamSynchronize(p->st));
  return 0;
}

}  // extern "C"

namespace asd {
// Enqueues `iters` iterations of every sub-batch (through the captured
// graphs when use_graph, capturing them first if needed), ordered after the
// work queued on the plan's stream and before what follows it.
static int plan_iterations(asdpocs_plan p, int iters, bool use_graph) {
  if (use_graph) {
    for (SubBatch &s : p->subs) {
      if (s.exec) continue;
      ASD_CUDA(cudaStreamBeginCapture(s.st, cudaStreamCaptureModeThreadLocal));
      const int rc = plan_enqueue_sub(p, s);
      cudaGraph_t g = nullptr;
      const cudaError_t e = cudaStreamEndCapture(s.st, &g);
      if (rc) {
        if (g) cudaGraphDestroy(g);
        return rc;
      }
      ASD_CUDA(e);
      s.graph = g;
      ASD_CUDA(cudaGraphInstantiate(&s.exec, s.graph, 0));
    }
  }
  const bool multi = p->subs.size() > 1;
  if (multi) {  // the sub-batches start after the work queued on the plan's stream
    ASD_CUDA(cudaEventRecord(p->fork, p->st));
    for (SubBatch &s : p->subs) ASD_CUDA(cudaStreamWaitEvent(s.st, p->fork, 0));
  }
  for (int k = 0; k < iters; k++)
    for (SubBatch &s : p->subs) {
      if (use_graph)
        ASD_CUDA(cudaGraphLaunch(s.exec, s.st));
      else if (int rc = plan_enqueue_sub(p, s))
        return rc;
    }
  if (multi) {  // and the plan's stream continues after both
    for (SubBatch &s : p->subs) {
      ASD_CUDA(cudaEventRecord(s.done, s.st));
      ASD_CUDA(cudaStreamWaitEvent(p->st, s.done, 0));
    }
  }
  return 0;
}
}  // namespace asd

extern "C" {

int asdpocs_plan_run(asdpocs_plan p, int use_graph) {
  clear_error();
  if (!p) return set_error(ASDPOCS_ERR_ARG, "null plan");
  if (p->max_iter <= 0) return 0;
  return plan_iterations(p, p->max_iter, use_graph != 0);
}

int asdpocs_plan_sync(asdpocs_plan p) {
  clear_error();
  if (!p) return set_error(ASDPOCS_ERR_ARG, "null plan");
  ASD_CUDA(cudaStreamSynchronize(p->st));
  return 0;
}

int asdpocs_plan_get_image(asdpocs_plan p, int inst, float *m, int where) {
  clear_error();
  if (int e = plan_check(p, inst)) return e;
  if (!m) return set_error(ASDPOCS_ERR_ARG, "null output");
  ASD_CUDA(cudaMemcpyAsync(m, p->h_inst[inst].m_res, inst_bytes(p, inst),
                           where ? cudaMemcpyDeviceToDevice
                                 : cudaMemcpyDeviceToHost,
                           p->st));
  if (!where) ASD_CUDA(cudaStreamSynchronize(p->st));
  return 0;
}

int asdpocs_plan_get_stats(asdpocs_plan p, int inst, asdpocs_stats *st,
                           double *rmse) {
  clear_error();
  if (int e = plan_check(p, inst)) return e;
  Scalars s;
  ASD_CUDA(cudaMemcpyAsync(&s, p->h_inst[inst].s, sizeof s,
                           cudaMemcpyDeviceToHost, p->st));
  if (rmse && p->opt[inst].maxnumIter > 0)
    ASD_CUDA(cudaMemcpyAsync(rmse, p->h_inst[inst].rmse,
                             (size_t)p->opt[inst].maxnumIter * 8,
                             cudaMemcpyDeviceToHost, p->st));
  ASD_CUDA(cudaStreamSynchronize(p->st));
  if (st) {
    st->IterationNum = s.iterations;
    st->dataTolerance = s.dd2;
    st->alpha = s.alpha;
    st->beta = s.beta;
    st->dp = s.dp;
    st->dg = s.dg;
  }
  return 0;
}

float *asdpocs_plan_sinogram_ptr(asdpocs_plan p, int inst) {
  if (p && inst >= 0 && inst < p->batch && p->h_inst[inst].p_fmt != ASDPOCS_STORE_F32) {
    set_error(ASDPOCS_ERR_STATE,
              "instance %d stores its sinogram in 16 bits: load it with "
              "asdpocs_plan_set_sinogram",
              inst);
    return nullptr;
  }
  if (plan_check(p, inst)) return nullptr;
  return (float *)p->h_inst[inst].P;
}

float *asdpocs_plan_image_ptr(asdpocs_plan p, int inst) {
  if (plan_check(p, inst)) return nullptr;
  return p->h_inst[inst].m_res;
}

int asdpocs_plan_time_phase(asdpocs_plan p, int phase, int reps,
                            double *avg_ms) {
  clear_error();
  if (!p || !avg_ms || reps <= 0 || phase < 0 || phase > 3)
    return set_error(ASDPOCS_ERR_ARG, "bad profiling arguments");
  cudaEvent_t e0, e1;
  ASD_CUDA(cudaEventCreate(&e0));
  ASD_CUDA(cudaEventCreate(&e1));
  const IterShape sh = plan_shape(p);
  const PdlScope scope(sh.pdl);  // launched as in the plan's iteration
  const int ng = p->max_ng > 0 ? p->max_ng : 1;
  // projector steps: views spread evenly over the scan (a view's cost
  // depends on its angle)
  auto view_of_rep = [&](int i) { return (int)(((long long)i * p->nv / reps) % p->nv); };
  // mixed plans: each sub-batch's groups in turn
  auto ax = [&](int v) {
    if (p->mixed) {
      cudaError_t e = cudaSuccess;
      for (const SubBatch &s : p->subs)
        if (e == cudaSuccess)
          e = launch_sart_ax_shared(p->d_inst, 0, s.d, v, p->st, sh.ax_u, sh.ax_q, s.gall,
                                    (int)s.groups_host.size());
      return e;
    }
    return p->shared ? launch_sart_ax_shared(p->d_inst, p->batch, p->d, v, p->st, sh.ax_u,
                                             sh.ax_q)
                     : launch_sart_ax(p->d_inst, p->batch, p->d, v, p->st, sh.exact);
  };
  auto atx = [&](int v) {
    if (p->mixed) {
      cudaError_t e = cudaSuccess;
      for (const SubBatch &s : p->subs)
        if (e == cudaSuccess)
          e = launch_sart_atx_shared(p->d_inst, 0, s.d, v, p->st, s.gall,
                                     (int)s.groups_host.size());
      return e;
    }
    return p->shared ? launch_sart_atx_shared(p->d_inst, p->batch, p->d, v, p->st)
                     : launch_sart_atx(p->d_inst, p->batch, p->d, v, p->st, sh.zcol, sh.zseg);
  };
  auto launch = [&](int i) -> cudaError_t {
    switch (phase) {
      case 0: return ax(view_of_rep(i));
      // the TV steps that do not end the iteration (the last one would
      // advance the iteration count and, at maxIter, stop the instances, so
      // that later launches had nothing to do)
      case 2: return launch_tv_step(p->d_inst, p->batch, p->d,
                                    ng > 2 ? 1 + i % (ng - 2) : 0, ng, p->st, p->tv_walk);
      default: return launch_after_sweep(p->d_inst, p->batch, p->d, p->st);
    }
  };
  cudaError_t e = cudaSuccess;
  float ms = 0.f;
  if (phase == 1) {
    // the backward step reads what the forward step of its view leaves (the
    // residuals, the ray-slope table, their finiteness), and its cost
    // depends on it: each timed launch follows its view's untimed forward
    // step
    for (int i = 0; i < reps && e == cudaSuccess; i++) {
      const int v = view_of_rep(i);
      e = ax(v);
      if (e == cudaSuccess) e = cudaEventRecord(e0, p->st);
      if (e == cudaSuccess) e = atx(v);
      if (e == cudaSuccess) e = cudaEventRecord(e1, p->st);
      if (e == cudaSuccess) e = cudaEventSynchronize(e1);
      float t = 0.f;
      if (e == cudaSuccess) e = cudaEventElapsedTime(&t, e0, e1);
      ms += t;
    }
  } else {
    e = launch(0);  // warm-up
    if (e == cudaSuccess) e = cudaEventRecord(e0, p->st);
    for (int i = 0; i < reps && e == cudaSuccess; i++) e = launch(i);
    if (e == cudaSuccess) e = cudaEventRecord(e1, p->st);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  ASD_CUDA(e);
  *avg_ms = (double)ms / reps;
  return 0;
}

static void plan_drop_graph(asdpocs_plan p) {
  for (SubBatch &s : p->subs) {
    if (s.exec) cudaGraphExecDestroy(s.exec);
    if (s.graph) cudaGraphDestroy(s.graph);
    s.exec = nullptr;
    s.graph = nullptr;
  }
}

int asdpocs_plan_streams(asdpocs_plan p) { return p ? (int)p->subs.size() : 0; }

int asdpocs_plan_chord_slots(asdpocs_plan p) { return p ? p->chK : 0; }

int asdpocs_plan_set_tv_walk(asdpocs_plan p, int walk) {
  clear_error();
  if (!p || walk < 0) return set_error(ASDPOCS_ERR_ARG, "bad walk length");
  if (walk != p->tv_walk) plan_drop_graph(p);  // the captured launches change
  p->tv_walk = walk;
  return 0;
}

int asdpocs_plan_autotune(asdpocs_plan p, int reps, int *walk, double *ms) {
  clear_error();
  if (!p || reps <= 0) return set_error(ASDPOCS_ERR_ARG, "bad autotune arguments");
  if (p->max_ng < 2) {
    if (walk) *walk = p->tv_walk;
    if (ms) *ms = 0.0;
    return 0;
  }
  std::vector<int> cand{0};
  const int wmax = tv_walk_max(p->d);
  for (int w = 1; w < wmax; w *= 2) cand.push_back(w);
  cand.push_back(wmax);
  cudaEvent_t e0, e1;
  ASD_CUDA(cudaEventCreate(&e0));
  ASD_CUDA(cudaEventCreate(&e1));
  int best = 0;
  float best_ms = 0.f;
  cudaError_t e = cudaSuccess;
  // steps 0, 1, ..., ng - 2, 1, ... as in an iteration, each reading the
  // previous one's output; never the last step, so only the work buffers
  // and the step size (both rewritten every iteration) change
  const int ng = p->max_ng;
  auto step_of = [&](int r) { return ng > 2 ? (r == 0 ? 0 : 1 + (r - 1) % (ng - 2)) : 0; };
  for (size_t c = 0; c < cand.size() && e == cudaSuccess; c++) {
    e = launch_tv_step(p->d_inst, p->batch, p->d, 0, ng, p->st, cand[c]);  // warm-up
    if (e == cudaSuccess) e = cudaEventRecord(e0, p->st);
    for (int r = 0; r < reps && e == cudaSuccess; r++)
      e = launch_tv_step(p->d_inst, p->batch, p->d, step_of(r), ng, p->st, cand[c]);
    if (e == cudaSuccess) e = cudaEventRecord(e1, p->st);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    float t = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&t, e0, e1);
    if (e == cudaSuccess && (c == 0 || t < best_ms)) {
      best_ms = t;
      best = cand[c];
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  ASD_CUDA(e);
  if (int rc = asdpocs_plan_set_tv_walk(p, best)) return rc;
  if (walk) *walk = best;
  if (ms) *ms = (double)best_ms / reps;
  return 0;
}

int asdpocs_plan_get_shapes(asdpocs_plan p, asdpocs_shapes *out) {
  clear_error();
  if (!p || !out) return set_error(ASDPOCS_ERR_ARG, "null argument");
  out->tv_walk = p->tv_walk;
  out->ax_cols = p->ax_u;
  out->ax_quads = p->ax_q;
  out->zcol_segment = p->zseg;
  out->pdl = p->pdl;
  out->iteration_ms = 0.0;
  return 0;
}

int asdpocs_plan_set_shapes(asdpocs_plan p, const asdpocs_shapes *s) {
  clear_error();
  if (!p || !s) return set_error(ASDPOCS_ERR_ARG, "null argument");
  if (s->tv_walk < 0 || s->ax_cols < 0 || s->ax_cols > 2 || s->ax_quads < 0 ||
      s->ax_quads > 2 || s->zcol_segment < 0 || s->zcol_segment > 256 || s->pdl < -1 ||
      s->pdl > 1)
    return set_error(ASDPOCS_ERR_ARG, "launch shape out of range");
  plan_drop_graph(p);  // the captured launches change
  p->tv_walk = s->tv_walk;
  p->ax_u = s->ax_cols;
  p->ax_q = s->ax_quads;
  p->zseg = s->zcol_segment;
  p->pdl = s->pdl;
  return 0;
}

int asdpocs_plan_autotune_shapes(asdpocs_plan p, int reps, asdpocs_shapes *out) {
  clear_error();
  if (!p || reps <= 0) return set_error(ASDPOCS_ERR_ARG, "bad autotune arguments");
  // the TV walk: its own tuner (steps of the plan's data, state unchanged)
  if (int rc = asdpocs_plan_autotune(p, reps, nullptr, nullptr)) return rc;
  cudaEvent_t e0, e1;
  ASD_CUDA(cudaEventCreate(&e0));
  ASD_CUDA(cudaEventCreate(&e1));
  // device milliseconds of one iteration run as asdpocs_plan_run runs it:
  // the captured graphs, concurrent sub-batches overlapping
  // (at most maxnumIter of them after a reset: later ones find every
  // instance finished and would time empty launches)
  const int n_it = std::max(1, std::min(reps, p->max_iter));
  auto iter_ms = [&](double *t) -> int {
    plan_drop_graph(p);  // the shapes changed
    if (int r = asdpocs_plan_reset(p)) return r;
    if (int r = plan_iterations(p, 1, true)) return r;  // capture, warm-up
    if (int r = asdpocs_plan_reset(p)) return r;
    ASD_CUDA(cudaEventRecord(e0, p->st));
    if (int r = plan_iterations(p, n_it, true)) return r;
    ASD_CUDA(cudaEventRecord(e1, p->st));
    ASD_CUDA(cudaEventSynchronize(e1));
    float f = 0.f;
    ASD_CUDA(cudaEventElapsedTime(&f, e0, e1));
    *t = (double)f / n_it;
    return 0;
  };
  // the fastest candidate of one knob, by whole iterations (timer 0) or by
  // the backward step's launches (timer 1); cand[0] is the default, which
  // another candidate replaces only when faster by more than 2 %
  auto pick = [&](int timer, int *knob, const std::vector<int> &cand) -> int {
    int best = cand[0];
    double best_ms = 0.0, ms = 0.0;
    for (size_t k = 0; k < cand.size(); k++) {
      *knob = cand[k];
      if (int rc = timer == 0 ? iter_ms(&ms) : asdpocs_plan_time_phase(p, 1, reps, &ms))
        return rc;
      if (k == 0 || ms < 0.98 * best_ms) {
        best_ms = ms;
        best = cand[k];
      }
    }
    *knob = best;
    return 0;
  };
  int rc = 0;
  p->pdl = 0;
  if (p->shared) {
    // the shared forward step's shape, on whole iterations: its kernels share
    // the GPU with the other sub-batch's, which a kernel timed alone misses
    const int dflt = p->d.nz > 1 || p->d.nb > 1 ? 1 * 4 + 2 : 2 * 4 + 1;
    int uq = dflt;
    std::vector<int> cand{dflt};
    for (int c : {1 * 4 + 1, 2 * 4 + 1, 1 * 4 + 2, 2 * 4 + 2})
      if (c != dflt) cand.push_back(c);
    rc = pick(0, &uq, cand);
    p->ax_u = uq / 4;
    p->ax_q = uq % 4;
  } else if (p->d.nz > 1 && p->zcol) {
    rc = pick(1, &p->zseg, {0, 4, 8, 16, 32});  // the z-column segment length (0: by size)
  }
  double t_best = 0.0;
  // programmatic launches only where the plan runs on one stream (PdlScope)
  if (!rc && p->subs.size() == 1) rc = pick(0, &p->pdl, {0, 1});
  if (!rc) rc = iter_ms(&t_best);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc) return rc;
  plan_drop_graph(p);
  if (int r2 = asdpocs_plan_reset(p)) return r2;
  if (out) {
    asdpocs_plan_get_shapes(p, out);
    out->iteration_ms = t_best;
  }
  return 0;
}

// --------------------------------------------------- one-call drivers
int ASD_POCS_cuda(const double *P, const double *phi_vec_deg,
                  const asdpocs_geometry *geom, const asdpocs_options *opt,
                  const double *m0, const double *I0, double *m_res,
                  double *rmse, asdpocs_stats *out) {
  clear_error();
  if (!P || !phi_vec_deg || !geom || !m_res)
    return set_error(ASDPOCS_ERR_ARG, "null argument");
  asdpocs_plan p = nullptr;
  if (int e = asdpocs_plan_create(&p, 1, geom, phi_vec_deg, opt, 0, nullptr))
    return e;
  const size_t N = (size_t)geom->nx * geom->ny * geom->nz;
  const size_t PM = (size_t)geom->na * geom->nb * geom->nv;
  std::vector<float> buf(PM > N ? PM : N);
  int rc = 0;
  for (size_t i = 0; i < PM; i++) buf[i] = (float)P[i];
  rc = asdpocs_plan_set_sinogram(p, 0, buf.data(), 0);
  if (!rc && m0) {
    for (size_t i = 0; i < N; i++) buf[i] = (float)m0[i];
    rc = asdpocs_plan_set_initial(p, 0, buf.data(), 0);
  }
  if (!rc && I0) {
    for (size_t i = 0; i < N; i++) buf[i] = (float)I0[i];
    rc = asdpocs_plan_set_reference(p, 0, buf.data(), 0);
  }
  if (!rc) rc = asdpocs_plan_reset(p);
  if (!rc) rc = asdpocs_plan_run(p, 1);
  if (!rc) rc = asdpocs_plan_get_image(p, 0, buf.data(), 0);
  if (!rc) {
    for (size_t i = 0; i < N; i++) m_res[i] = buf[i];
    rc = asdpocs_plan_get_stats(p, 0, out, I0 ? rmse : nullptr);
  }
  const int saved = g_status;
  char msg[512];
  memcpy(msg, g_msg, sizeof msg);
  asdpocs_plan_destroy(p);
  if (rc) {
    g_status = saved;
    memcpy(g_msg, msg, sizeof msg);
  }
  return rc;
}

int SART_cuda_inline(const double *P, const double *phi_vec_deg,
                     const asdpocs_geometry *geom, double lambda,
                     const double *m0, double *m_out, double *dataTolerance) {
  clear_error();
  asdpocs_options o;
  asdpocs_options_default(&o);
  // one sweep, relaxation lambda, no TV (SART_cuda_inline.m:56-87)
  o.maxnumIter = 1;
  o.numOfgradients = 0;
  o.beta = lambda;
  asdpocs_stats st;
  const int rc = ASD_POCS_cuda(P, phi_vec_deg, geom, &o, m0, nullptr, m_out,
                               nullptr, &st);
  if (rc == 0 && dataTolerance) *dataTolerance = st.dataTolerance;
  return rc;
}

}  // extern "C"
