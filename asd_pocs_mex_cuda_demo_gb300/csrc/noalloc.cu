// Allocation-free variant of the FP32 device TV minimisation
// (asdpocs_tv_device_noalloc).
//
// Some callers cannot call cudaMalloc: code running under an allocator that
// owns all device memory (a framework's caching pool, a fixed HBM budget
// enforced by a serving layer), a real-time loop where an allocation could
// stall on a device-wide synchronisation, or a plugin host that forbids its
// extensions from allocating.  For them this entry point keeps its scratch
// (two work images, the reduction partials, the ticket counter and the step
// scalars) in one file-scope __device__ array of fixed size, which every GPU
// that loads the library holds until the process exits.  The caller still
// passes the image (in/out) and the reference image.
//
// Limits: at most kMaxVoxels voxels (nx*ny*nz <= 1,048,576, e.g. 1024^2 or
// 128^2 x 64), kMaxTiles 32x8 voxel tiles and 65535 tile rows
// (ceil(ny/8)*nz, the GPU's grid limit); other images are rejected.
// All calls share the one array: calls that overlap on the GPU (different
// streams, or several host threads) race on it and corrupt each other.
// The first call on a device looks up the array's device address (with that
// device current); that first call should come before any stream capture.
#include <mutex>

#include "kernels.h"

namespace asd {
namespace {

constexpr size_t kMaxVoxels = size_t(1) << 20;
constexpr size_t kMaxTiles = size_t(1) << 16;
constexpr size_t kImgBytes = kMaxVoxels * sizeof(float);  // 4 MiB
constexpr size_t kOffA = 0;
constexpr size_t kOffB = kImgBytes;
constexpr size_t kOffScal = 2 * kImgBytes;        // 256 B of step scalars
constexpr size_t kOffCounter = kOffScal + 256;    // ticket, must start at 0
constexpr size_t kOffPartials = kOffCounter + 256;
constexpr size_t kScratchBytes = kOffPartials + kMaxTiles * sizeof(double);

static __device__ __align__(256) unsigned char g_tv_scratch[kScratchBytes];

std::mutex g_mu;
void *g_addr[64] = {};  // device address of g_tv_scratch, per device

// Device address of the scratch array on the current device (looked up once
// per device; a host-side reference to g_tv_scratch is not a device address).
int scratch_address(char **out) {
  int dev = 0;
  ASD_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= 64) return set_error(ASDPOCS_ERR_NODEV, "device id");
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_addr[dev]) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_tv_scratch);
    if (e != cudaSuccess) return cuda_status(e, "cudaGetSymbolAddress(tv scratch)");
    g_addr[dev] = p;
  }
  *out = (char *)g_addr[dev];
  return 0;
}

}  // namespace
}  // namespace asd

using namespace asd;

extern "C" int asdpocs_tv_device_noalloc(float *img_d, const float *img_old_d,
                                         int nx, int ny, int nz, double alpha,
                                         int nTVIter, int pos, void *stream) {
  clear_error();
  if (!img_d) return set_error(ASDPOCS_ERR_ARG, "null pointer");
  if (nx <= 0 || ny <= 0 || nz <= 0)
    return set_error(ASDPOCS_ERR_ARG, "bad image dimensions");
  const size_t N = (size_t)nx * ny * nz;
  const size_t tiles = (size_t)((nx + kTileX - 1) / kTileX) *
                       ((ny + kTileY - 1) / kTileY) * nz;
  if (N > kMaxVoxels)
    return set_error(ASDPOCS_ERR_ARG,
                     "image of %zu voxels exceeds the %zu-voxel limit of the "
                     "allocation-free TV entry point",
                     N, kMaxVoxels);
  if (tiles > kMaxTiles)
    return set_error(ASDPOCS_ERR_ARG,
                     "image needs %zu tiles, over the %zu-tile limit of the "
                     "allocation-free TV entry point",
                     tiles, kMaxTiles);
  if (tile_rows(ny, nz) > kMaxGridRows)
    return set_error(ASDPOCS_ERR_ARG,
                     "image needs %lld tile rows (ceil(ny/8)*nz), over the limit of "
                     "%lld of the allocation-free TV entry point",
                     tile_rows(ny, nz), kMaxGridRows);
  char *b = nullptr;
  if (int e = scratch_address(&b)) return e;
  cudaStream_t st = (cudaStream_t)stream;
  // the ticket keeps the previous call's contents: clear it
  ASD_CUDA(cudaMemsetAsync(b + kOffCounter, 0, 256, st));
  ASD_CUDA(tv_minimize_f32(img_d, img_old_d, (float *)(b + kOffA),
                           (float *)(b + kOffB), (double *)(b + kOffScal),
                           (double *)(b + kOffPartials),
                           (unsigned *)(b + kOffCounter), nx, ny, nz, alpha,
                           nTVIter, pos, st));
  return 0;
}
