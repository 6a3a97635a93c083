// Device-side synthetic inputs: ellipsoid phantoms and Poisson noise, so
// serving and benchmark inputs need no host round trip.
//
// Phantoms follow utilities/phantom3d.m (lines 84-113): an n^3 grid on
// [-1, 1] (n = the largest dimension), voxel (r, c, k) sampled at
// (x = g[c], y = g[r], z = g[k]), every ellipsoid adding its amplitude where
// the rotated, centred point satisfies sum((q - p0)^2 / axes^2) <= 1.  The
// arithmetic is FP64, one rounding per operation (no contraction), in the
// order of the host restatement (phantoms.ellipsoids), so both give the same
// volume bit for bit.
//
// Noise: P' = -ln(max(k, 1) / I0) with k ~ Poisson(I0 exp(-P)), drawn from a
// counter-based generator (Philox-4x32-10, Salmon et al., SC'11) keyed by the
// seed and counted by the element, so the result depends on (seed, element)
// only -- not on the launch shape.  Poisson variates use the multiplication
// method for means below 10 and the transformed rejection method PTRS
// (Hormann 1993) above.
#include <math.h>

#include "kernels.h"

namespace asd {
namespace {

constexpr int kMaxEllipsoids = 32;

struct EllipsoidTable {
  int n;
  // per ellipsoid: A, a, b, c, x0, y0, z0, R (row-major 3 x 3)
  double e[kMaxEllipsoids][16];
};

__global__ void __launch_bounds__(256)
    k_phantom(float *__restrict__ vol, int nx, int ny, int nz, EllipsoidTable t,
              double scale) {
  const long long N = (long long)nx * ny * nz;
  const long long v = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= N) return;
  const int ix = (int)(v % nx), iy = (int)((v / nx) % ny), iz = (int)(v / ((long long)nx * ny));
  const int n = max(nx, max(ny, nz));
  const double h = __dmul_rn((double)(n - 1), 0.5);  // (n - 1) / 2
  auto g = [&](int i) { return n > 1 ? __ddiv_rn(__dsub_rn((double)i, h), h) : 0.0; };
  const double X = g(iy), Y = g(ix), Z = g(iz);
  double acc = 0.0;
  for (int k = 0; k < t.n; k++) {
    const double *e = t.e[k];
    const double q0 = __dadd_rn(__dadd_rn(__dmul_rn(e[7], X), __dmul_rn(e[8], Y)), __dmul_rn(e[9], Z));
    const double q1 = __dadd_rn(__dadd_rn(__dmul_rn(e[10], X), __dmul_rn(e[11], Y)), __dmul_rn(e[12], Z));
    const double q2 = __dadd_rn(__dadd_rn(__dmul_rn(e[13], X), __dmul_rn(e[14], Y)), __dmul_rn(e[15], Z));
    const double d0 = __dsub_rn(q0, e[4]), d1 = __dsub_rn(q1, e[5]), d2 = __dsub_rn(q2, e[6]);
    const double s = __dadd_rn(__dadd_rn(__ddiv_rn(__dmul_rn(d0, d0), __dmul_rn(e[1], e[1])),
                                         __ddiv_rn(__dmul_rn(d1, d1), __dmul_rn(e[2], e[2]))),
                               __ddiv_rn(__dmul_rn(d2, d2), __dmul_rn(e[3], e[3])));
    if (s <= 1.0) acc = __dadd_rn(acc, e[0]);
  }
  vol[v] = (float)__dmul_rn(acc, scale);
}

// Philox-4x32-10 (Salmon, Moraes, Dror, Shaw: "Parallel random numbers: as
// easy as 1, 2, 3", SC'11): ten rounds of the published multipliers and Weyl
// key increments.
struct Philox {
  uint32_t k0, k1;
  __device__ uint4 operator()(uint4 c) const {
    uint32_t a = k0, b = k1;
#pragma unroll
    for (int i = 0; i < 10; i++) {
      const uint32_t hi0 = __umulhi(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
      const uint32_t hi1 = __umulhi(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
      c = make_uint4(hi1 ^ c.y ^ a, lo1, hi0 ^ c.w ^ b, lo0);
      a += 0x9E3779B9u;
      b += 0xBB67AE85u;
    }
    return c;
  }
};

// Uniform in (0, 1) from 24 random bits.
__device__ __forceinline__ float unit(uint32_t x) {
  return ((float)(x >> 8) + 0.5f) * (1.0f / 16777216.0f);
}

// Poisson(lam) from the stream of element `idx`; `draws` numbers per call of
// the generator, a fresh counter per call.
__device__ long long poisson(double lam, const Philox &rng, unsigned long long idx) {
  uint32_t ctr = 0;
  uint4 buf = make_uint4(0, 0, 0, 0);
  int left = 0;
  auto next = [&]() {
    if (left == 0) {
      buf = rng(make_uint4((uint32_t)idx, (uint32_t)(idx >> 32), ctr++, 0u));
      left = 4;
    }
    const uint32_t r = left == 4 ? buf.x : left == 3 ? buf.y : left == 2 ? buf.z : buf.w;
    left--;
    return unit(r);
  };
  if (!(lam > 0.0)) return 0;
  if (lam < 10.0) {
    // multiplication method: the number of uniforms whose running product
    // stays above exp(-lam)
    const float L = expf(-(float)lam);
    float p = 1.f;
    long long k = 0;
    for (int it = 0; it < 1000; it++) {
      p *= next();
      if (p <= L) return k;
      k++;
    }
    return k;
  }
  // PTRS
  const float fl = (float)lam;
  const float slam = sqrtf(fl), loglam = logf(fl);
  const float b = 0.931f + 2.53f * slam;
  const float a = -0.059f + 0.02483f * b;
  const float inv_alpha = 1.1239f + 1.1328f / (b - 3.4f);
  const float vr = 0.9277f - 3.6224f / (b - 2.0f);
  for (int it = 0; it < 100; it++) {
    const float U = next() - 0.5f, V = next();
    const float us = 0.5f - fabsf(U);
    const float kf = floorf((2.0f * a / us + b) * U + fl + 0.43f);
    if (us >= 0.07f && V <= vr) return (long long)kf;
    if (kf < 0.0f || (us < 0.013f && V > us)) continue;
    if (logf(V) + logf(inv_alpha) - logf(a / (us * us) + b) <=
        -fl + kf * loglam - lgammaf(kf + 1.0f))
      return (long long)kf;
  }
  return (long long)rintf(fl);
}

__global__ void __launch_bounds__(256)
    k_poisson_noise(const float *__restrict__ p, float *__restrict__ out,
                    long long n, double I0, Philox rng) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const double lam = I0 * exp(-(double)p[i]);
    long long k = poisson(lam, rng, (unsigned long long)i);
    if (k < 1) k = 1;
    out[i] = (float)(-log((double)k / I0));
  }
}

}  // namespace
}  // namespace asd

using namespace asd;

extern "C" {

int asdpocs_phantom_device(float *vol_d, int nx, int ny, int nz,
                           const double *ellipsoids, int n_ellipsoids,
                           double scale, void *stream) {
  clear_error();
  if (!vol_d || (n_ellipsoids > 0 && !ellipsoids))
    return set_error(ASDPOCS_ERR_ARG, "null pointer");
  if (nx <= 0 || ny <= 0 || nz <= 0)
    return set_error(ASDPOCS_ERR_ARG, "bad phantom dimensions");
  if (n_ellipsoids < 0 || n_ellipsoids > kMaxEllipsoids)
    return set_error(ASDPOCS_ERR_ARG, "at most %d ellipsoids", kMaxEllipsoids);
  EllipsoidTable t;
  t.n = n_ellipsoids;
  for (int k = 0; k < n_ellipsoids; k++)
    for (int j = 0; j < 16; j++) t.e[k][j] = ellipsoids[k * 16 + j];
  const long long N = (long long)nx * ny * nz;
  k_phantom<<<(unsigned)((N + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
      vol_d, nx, ny, nz, t, scale);
  ASD_CUDA(cudaGetLastError());
  return 0;
}

int asdpocs_poisson_noise_device(const float *p_d, float *out_d, long long n,
                                 double I0, unsigned long long seed,
                                 void *stream) {
  clear_error();
  if (!p_d || !out_d) return set_error(ASDPOCS_ERR_ARG, "null pointer");
  if (n < 0 || !(I0 > 0.0)) return set_error(ASDPOCS_ERR_ARG, "bad noise arguments");
  if (n == 0) return 0;
  const Philox rng{(uint32_t)seed, (uint32_t)(seed >> 32)};
  const long long blocks = (n + 255) / 256;
  k_poisson_noise<<<(unsigned)(blocks < 152 * 64 ? blocks : 152 * 64), 256, 0,
                    (cudaStream_t)stream>>>(p_d, out_d, n, I0, rng);
  ASD_CUDA(cudaGetLastError());
  return 0;
}

}  // extern "C"
