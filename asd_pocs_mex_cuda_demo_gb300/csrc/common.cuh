// Shared definitions of the asdpocs_gb300 library (internal).
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdlib.h>

#include <utility>

#include "../../include/asdpocs_gb300.h"

namespace asd {

// ---------------------------------------------------------------------------
// Bounds-checked builds (compiled with -DASDPOCS_CHECKED, the library
// libasdpocs_gb300_checked.so).  Every volume, sinogram, residual and table
// index of the projector and TV kernels goes through ASD_IN(i, n) before its
// access: an index outside [0, n) is counted in a device word of the
// translation unit (the first one kept with its extent) and the access is
// skipped -- a load gives 0, a store is dropped -- so a bad index never
// faults or traps.  asdpocs_checked_errors reads and clears the words.  In
// the normal build ASD_IN is `true` and costs nothing.
// ---------------------------------------------------------------------------
#ifdef ASDPOCS_CHECKED
static __device__ unsigned long long g_oob_count;
static __device__ long long g_oob_first[2];  // first bad index and its extent
__device__ __forceinline__ bool asd_in(long long i, long long n) {
  if (i >= 0 && i < n) return true;
  if (atomicAdd(&g_oob_count, 1ull) == 0ull) {
    g_oob_first[0] = i;
    g_oob_first[1] = n;
  }
  return false;
}
#define ASD_IN(i, n) ::asd::asd_in((long long)(i), (long long)(n))
// Reads and clears this translation unit's words: count, first index, extent.
#define ASD_CHECKED_READER(name)                                                   \
  cudaError_t name(unsigned long long *count, long long *first) {                \
    unsigned long long c = 0, z = 0;                                             \
    long long f[2] = {0, 0}, zf[2] = {0, 0};                                     \
    cudaError_t e = cudaMemcpyFromSymbol(&c, g_oob_count, sizeof c);             \
    if (e == cudaSuccess) e = cudaMemcpyFromSymbol(f, g_oob_first, sizeof f);    \
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(g_oob_count, &z, sizeof z);     \
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(g_oob_first, zf, sizeof zf);    \
    *count = c;                                                                  \
    first[0] = f[0];                                                             \
    first[1] = f[1];                                                             \
    return e;                                                                    \
  }
#else
#define ASD_IN(i, n) true
#endif

// ---------------------------------------------------------------------------
// Programmatic dependent launch.  The kernels of an ASD-POCS iteration of a
// plan that runs on one stream are launched with programmatic stream
// serialization (launch_iter inside a PdlScope), so a kernel's launch and
// block scheduling overlap the tail of the kernel before it.  Each such
// kernel calls pdl_enter() before its first global-memory access: it waits
// there until the preceding kernel has completed and its writes are visible
// (so every kernel still sees all earlier ones), then lets its own successor
// be scheduled -- once all of its blocks are resident, so the successor's
// waiting blocks never take the slots of its own.  In a kernel launched the
// ordinary way both instructions do nothing.  Plans that run sub-batches on
// concurrent streams (and the serving lanes) launch the ordinary way: there
// the successor's early, waiting blocks hold SM slots the other stream's
// kernels would use (measured 22 % slower at batch 64, against 4 % faster
// for a single instance).  ASDPOCS_NO_PDL in the environment turns it off.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void pdl_enter() {
  asm volatile("griddepcontrol.wait;\n" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory");
}

inline bool pdl_on() {
  static const bool on = getenv("ASDPOCS_NO_PDL") == nullptr;
  return on;
}

// Launches of this host thread use programmatic serialization while a
// PdlScope(true) is alive.
inline bool &pdl_now() {
  static thread_local bool now = false;
  return now;
}
struct PdlScope {
  bool prev;
  explicit PdlScope(bool on) : prev(pdl_now()) { pdl_now() = on && pdl_on(); }
  ~PdlScope() { pdl_now() = prev; }
};

// Launches kernel k (its kernel calls pdl_enter first) on st, with
// programmatic stream serialization inside a PdlScope(true).
template <typename... KArgs, typename... Args>
cudaError_t launch_iter(void (*k)(KArgs...), dim3 grid, dim3 block, cudaStream_t st,
                        Args &&...args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = 0;
  cfg.stream = st;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = pdl_now() ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, k, std::forward<Args>(args)...);
}

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
  int cor_finite;   // current view: every residual finite (set by Ax)
};

struct Inst {
  Dims d;                    // this instance's volume and detector sizes
  int nv;                    // and number of views (a plan's grids are sized
                             // for its largest instance)
  ViewGeo g;                 // geometry (cos/sin filled per view from trig)
  const float2 *trig;        // [nv] (cos_phi, sin_phi) per view
  const void *P;             // sinogram, view-major, na*nb*nv, stored as
  int p_fmt;                 //   ASDPOCS_STORE_F32 / _F16 / _BF16 (sino_at)
  float *m;                  // current image (A)
  float *m_pre;              // image at sweep start
  float *m_res;              // post-SART snapshot (returned image)
  float *m_k1;               // TV distance reference (m0)
  float *I0;                 // reference image or nullptr
  float *tv_b, *tv_c;        // TV ping-pong buffers
                             //   starts from (ping-pong), so the step's update
                             //   reads it instead of recomputing it
  float *cor;                // correction of the current view: element r at
  int cor_stride;            //   cor[r * cor_stride] (1, or kShareSlots when
                             //   a shared-geometry group interleaves them)
  float *m_il;               // shared-geometry groups: the group's images
                             //   during the SART sweep, voxel-major, slot
                             //   minor (m_il[v * kShareSlots + slot]); the
                             //   group's base, or nullptr
  float4 *tabA;              // ray slopes of every view, nv*na (ray_tab_a)
  int *vflags;               // per view: kViewAxisParallel | kViewNotX | kViewNotY
  float4 *tabC;              // 3D ray slopes of the current view, na*nb
  int tabc_mode;             // who writes tabC in the forward step (kTabc*)
  const int *chtab;          // 2-D plans of one instance or sharing geometry:
                             //   the backward step's chords of every view
                             //   (k_atx_chords), or nullptr
  int chK;                   //   chord slots per voxel and view in chtab
  double *rmse;              // [maxIter]
  double *partials;          // reduction partials [blocks * kMaxReduceK]
  unsigned *counter;         // reduction ticket
  Scalars *s;
};

// Sinogram value i of an instance, widened to FP32 from its storage.
__device__ __forceinline__ float sino_at(const Inst &I, long long i) {
  if (I.p_fmt == ASDPOCS_STORE_F16) return __half2float(((const __half *)I.P)[i]);
  if (I.p_fmt == ASDPOCS_STORE_BF16) return __bfloat162float(((const __nv_bfloat16 *)I.P)[i]);
  return ((const float *)I.P)[i];
}

// Bytes of one stored sinogram value.
__host__ __device__ inline size_t sino_elem_bytes(int fmt) {
  return fmt == ASDPOCS_STORE_F32 ? 4 : 2;
}

constexpr int kMaxPartials = 1 << 22;  // blocks per reduction (sanity bound)

// Instances per group of the shared-geometry kernels; their residuals are
// stored interleaved, cor[r * kShareSlots + slot].
constexpr int kShareSlots = 8;

// Inst::tabc_mode.  kTabcOwn: the instance writes its own table while it
// runs.  Instances sharing geometry share one table: its writer
// (kTabcShared) refreshes it every view even after it has finished, so the
// others (kTabcNone) keep reading current slopes.
constexpr int kTabcOwn = 0, kTabcShared = 1, kTabcNone = 2;

// View flags (Inst::vflags): some ray of the view has no x (or no y)
// extent; some ray is not x-dominant; some ray is not y-dominant.
constexpr int kViewAxisParallel = 1, kViewNotX = 2, kViewNotY = 4;

// Voxel tiles of the voxel-driven kernels: 32 (x) by 8 (y) voxels of one z
// slice per 256-thread block.  Grids are (x tiles, y tiles * nz, instances).
constexpr int kTileX = 32, kTileY = 8;
constexpr int kTileThreads = kTileX * kTileY;

__host__ __device__ inline dim3 tile_grid(int nx, int ny, int nz, int batch) {
  return dim3((nx + kTileX - 1) / kTileX, ((ny + kTileY - 1) / kTileY) * nz,
              batch);
}

// Launch rows of a tile grid: (ny / kTileY rounded up) * nz, at most 65535
// (the GPU's grid y limit).  The TV entry points reject images beyond it.
constexpr long long kMaxGridRows = 65535;
__host__ __device__ inline long long tile_rows(int ny, int nz) {
  return (long long)((ny + kTileY - 1) / kTileY) * nz;
}

// Voxel of this thread; true if inside the volume.
__device__ __forceinline__ bool tile_voxel(int nx, int ny, int nz, int &ix,
                                           int &iy, int &iz) {
  int by = blockIdx.y;
  iz = 0;
  if (nz > 1) {
    const int ty = (ny + kTileY - 1) / kTileY;
    iz = by / ty;
    by -= iz * ty;
  }
  ix = blockIdx.x * kTileX + (threadIdx.x % kTileX);
  iy = by * kTileY + (threadIdx.x / kTileX);
  return ix < nx && iy < ny;
}

// Batched voxel kernels give each block a group of kTilesPerBlock tile rows
// (same x tile, consecutive y tiles of one z slice) so that the block's
// fixed cost -- instance and view set-up, dependent loads -- is paid once per
// group.  Grids are (x tiles, y groups * nz, instances).
constexpr int kTilesPerBlock = 4;

__host__ __device__ inline dim3 group_grid(int nx, int ny, int nz, int batch) {
  const int ty = (ny + kTileY - 1) / kTileY;
  const int gy = (ty + kTilesPerBlock - 1) / kTilesPerBlock;
  return dim3((nx + kTileX - 1) / kTileX, gy * nz, batch);
}

// Origin of tile t (0 <= t < kTilesPerBlock) of this block's group; false
// when the group has fewer tiles (block-uniform).
__device__ __forceinline__ bool group_tile(int ny, int nz, int t, int &x0,
                                           int &y0, int &z) {
  const int ty = (ny + kTileY - 1) / kTileY;
  int g = blockIdx.y;
  z = 0;
  if (nz > 1) {
    const int gy = (ty + kTilesPerBlock - 1) / kTilesPerBlock;
    z = g / gy;
    g -= z * gy;
  }
  const int tyi = g * kTilesPerBlock + t;
  x0 = blockIdx.x * kTileX;
  y0 = tyi * kTileY;
  return tyi < ty;
}

// Index of this block among the blocks of its instance, and their number.
__device__ __forceinline__ int inst_block() {
  return blockIdx.x + gridDim.x * blockIdx.y;
}
__device__ __forceinline__ int inst_blocks() { return gridDim.x * gridDim.y; }

// Batched kernels run every instance of a plan in one grid sized for its
// largest instance.  A block keeps the (x, y) position it would have in a
// grid sized for its own instance alone -- so its tiles, its index among the
// instance's reduction partials and their number are the same as when the
// instance runs alone, and so are the results, bit for bit -- and blocks
// outside that grid have nothing to do.
struct OwnBlock {
  int bid, nblocks;  // bid < 0: outside the instance's own grid
};
__device__ __forceinline__ OwnBlock own_block(dim3 own) {
  OwnBlock b;
  b.nblocks = (int)(own.x * own.y);
  b.bid = (blockIdx.x < own.x && blockIdx.y < own.y)
              ? (int)(blockIdx.x + own.x * blockIdx.y)
              : -1;
  return b;
}
constexpr int kMaxReduceK = 4;          // values reduced together (partials sizing)

}  // namespace asd
