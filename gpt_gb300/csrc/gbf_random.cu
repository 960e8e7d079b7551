// gbf_random.cu -- synthetic inputs generated on the device: random SU(3)
// gauge fields U = exp(i eps H) (H Hermitian traceless, complex-Gaussian
// entries) and complex-Gaussian spinors, in the natural host layout.
//
// Random numbers: Philox4x32-10, the counter-based generator of Salmon,
// Moraes, Dror and Shaw, "Parallel random numbers: as easy as 1, 2, 3"
// (SC'11); counter = (element index, draw index), key = seed.  Normals by the
// Box-Muller transform.  The exponential uses the closed Cayley-Hamilton form
// of Morningstar and Peardon, Phys. Rev. D 69 (2004) 054501, in FP64.
// These are input generators for benchmarks and the serving loop, not part
// of the operator path.
#include <cstdint>

#include "gbf_launch.cuh"
#include "../../include/gbferm.h"

namespace {

struct U4 {
  uint32_t x, y, z, w;
};

__device__ __forceinline__ U4 philox4x32_10(U4 c, uint32_t k0, uint32_t k1) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u, W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const uint32_t hi0 = __umulhi(M0, c.x), lo0 = M0 * c.x;
    const uint32_t hi1 = __umulhi(M1, c.z), lo1 = M1 * c.z;
    c = U4{hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
    k0 += W0;
    k1 += W1;
  }
  return c;
}

// uniform in (0, 1] from 64 bits (53 significant)
__device__ __forceinline__ double u01(uint32_t a, uint32_t b) {
  const uint64_t v = ((uint64_t)a << 21) ^ (uint64_t)(b >> 11);
  return ((double)(v & ((1ull << 53) - 1)) + 1.0) * (1.0 / 9007199254740992.0);
}

// two standard normals per Philox call (uses all four words)
__device__ __forceinline__ double2 normal2(uint64_t elem, uint32_t draw, uint64_t seed) {
  U4 c{(uint32_t)elem, (uint32_t)(elem >> 32), draw, 0x6a09e667u};
  U4 r = philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
  const double u1 = u01(r.x, r.y), u2 = u01(r.z, r.w);
  const double rad = sqrt(-2.0 * log(u1));
  double s, co;
  sincospi(2.0 * u2, &s, &co);
  return make_double2(rad * co, rad * s);
}

__device__ __forceinline__ double2 zm(double2 a, double2 b) { return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }

__global__ void gauge_random_kernel(double2* U, long long nlinks, double eps, uint64_t seed) {
  const long long l = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= nlinks) return;
  // A: 9 complex Gaussian entries
  double2 A[9];
  for (int k = 0; k < 9; ++k) A[k] = normal2((uint64_t)l, (uint32_t)k, seed);
  // H = (A + A^+)/2 - tr/3, Q = eps H
  double2 Q[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j)
      Q[3 * i + j] = make_double2(0.5 * (A[3 * i + j].x + A[3 * j + i].x), 0.5 * (A[3 * i + j].y - A[3 * j + i].y));
  const double tr = (Q[0].x + Q[4].x + Q[8].x) / 3.0;
  for (int i = 0; i < 3; ++i) {
    Q[4 * i].x -= tr;
    Q[4 * i].y = 0.0;
  }
  for (int k = 0; k < 9; ++k) Q[k] = make_double2(eps * Q[k].x, eps * Q[k].y);
  double2 Q2[9];
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double2 s = make_double2(0, 0);
      for (int k = 0; k < 3; ++k) {
        double2 t = zm(Q[3 * i + k], Q[3 * k + j]);
        s.x += t.x;
        s.y += t.y;
      }
      Q2[3 * i + j] = s;
    }
  // c0 = det Q = tr(Q^3)/3, c1 = tr(Q^2)/2
  double c0 = 0.0;
  for (int i = 0; i < 3; ++i)
    for (int k = 0; k < 3; ++k) c0 += zm(Q2[3 * i + k], Q[3 * k + i]).x;
  c0 /= 3.0;
  const double c1 = 0.5 * (Q2[0].x + Q2[4].x + Q2[8].x);
  const bool neg = c0 < 0.0;
  const double c0a = fabs(c0);
  const double c0max = 2.0 * pow(c1 / 3.0, 1.5);
  const double ratio = c0max > 0.0 ? fmin(1.0, c0a / c0max) : 0.0;
  const double theta = acos(ratio);
  const double u = sqrt(c1 / 3.0) * cos(theta / 3.0);
  const double w = sqrt(c1) * sin(theta / 3.0);
  const double w2 = w * w, u2 = u * u;
  const double xi0 = fabs(w) < 0.05 ? 1.0 - w2 / 6.0 * (1.0 - w2 / 20.0 * (1.0 - w2 / 42.0)) : sin(w) / w;
  double s2u, c2u, su, cu;
  sincos(2.0 * u, &s2u, &c2u);
  sincos(u, &su, &cu);
  const double2 e2iu = make_double2(c2u, s2u), emiu = make_double2(cu, -su);
  const double cw = cos(w);
  // h0 = (u^2 - w^2) e^{2iu} + e^{-iu} (8u^2 cos w + 2iu(3u^2 + w^2) xi0)
  double2 h0 = make_double2((u2 - w2) * e2iu.x, (u2 - w2) * e2iu.y);
  double2 t0 = zm(emiu, make_double2(8.0 * u2 * cw, 2.0 * u * (3.0 * u2 + w2) * xi0));
  h0.x += t0.x; h0.y += t0.y;
  // h1 = 2u e^{2iu} - e^{-iu} (2u cos w - i(3u^2 - w^2) xi0)
  double2 t1 = zm(emiu, make_double2(2.0 * u * cw, -(3.0 * u2 - w2) * xi0));
  double2 h1 = make_double2(2.0 * u * e2iu.x - t1.x, 2.0 * u * e2iu.y - t1.y);
  // h2 = e^{2iu} - e^{-iu} (cos w + 3iu xi0)
  double2 t2 = zm(emiu, make_double2(cw, 3.0 * u * xi0));
  double2 h2 = make_double2(e2iu.x - t2.x, e2iu.y - t2.y);
  double den = 9.0 * u2 - w2;
  double2 f0, f1, f2;
  if (fabs(den) < 1e-12) {  // Q ~ 0: exp(iQ) ~ 1 + iQ - Q^2/2
    f0 = make_double2(1.0, 0.0);
    f1 = make_double2(0.0, 1.0);
    f2 = make_double2(-0.5, 0.0);
  } else {
    f0 = make_double2(h0.x / den, h0.y / den);
    f1 = make_double2(h1.x / den, h1.y / den);
    f2 = make_double2(h2.x / den, h2.y / den);
    if (neg) {
      f0.y = -f0.y;
      f1.x = -f1.x;
      f2.y = -f2.y;
    }
  }
  double2* out = U + (size_t)l * 9;
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      double2 v = zm(f1, Q[3 * i + j]);
      double2 v2 = zm(f2, Q2[3 * i + j]);
      v.x += v2.x;
      v.y += v2.y;
      if (i == j) {
        v.x += f0.x;
        v.y += f0.y;
      }
      out[3 * i + j] = v;
    }
}

__global__ void spinor_random_kernel(double2* out, long long n, uint64_t seed) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  out[i] = normal2((uint64_t)i, 0x5EEDu, seed);
}

}  // namespace

extern "C" int gbf_random_gauge(const int* dims, double eps, unsigned long long seed, void* U, void* stream) {
  if (!dims || !U) return GBF_E_ARG;
  const long long V = (long long)dims[0] * dims[1] * dims[2] * dims[3];
  const long long n = 4 * V;
  gauge_random_kernel<<<(unsigned)((n + 127) / 128), 128, 0, (cudaStream_t)stream>>>((double2*)U, n, eps, seed);
  return cudaGetLastError() == cudaSuccess ? GBF_OK : GBF_E_CUDA;
}

extern "C" int gbf_random_spinor(long long n_complex, unsigned long long seed, void* out, void* stream) {
  if (!out || n_complex < 0) return GBF_E_ARG;
  if (n_complex == 0) return GBF_OK;
  spinor_random_kernel<<<(unsigned)((n_complex + 255) / 256), 256, 0, (cudaStream_t)stream>>>((double2*)out, n_complex, seed);
  return cudaGetLastError() == cudaSuccess ? GBF_OK : GBF_E_CUDA;
}
