// gbf_common.cuh -- shared device types for the GB300 fermion-matrix kernels.
//
// Internal field layout (one checkerboard half):
//   a "5D site" n = cb4 * N5 + i5, with cb4 the checkerboard index of the 4D
//   site and i5 = rhs * Ls + s the inner index (Ls = 1 for Wilson-clover).
//   Consecutive threads take consecutive n, so every component load is a
//   fully coalesced 16-byte vector load:
//     FP64: double2 [12][N]             (192 B per 5D site)
//     FP32: float4  [6][N]              ( 96 B per 5D site)
//     FP16: uint4   [3][N] + float [N]  ( 52 B per 5D site; __half2 values
//           normalised by a per-site FP32 scale = max |component|)
//     double-float: float4 [12][N]      (192 B per 5D site; (re.h, im.h, re.l, im.l))
//   A full field is [even half][odd half].
//   cb4 = (x0/2) + (L0/2)*(x1 + L1*(x2 + L2*x3)); parity = (x0+x1+x2+x3) & 1.
//
// Gauge links, [parity][mu][chunk][Vh] for the sites of that parity:
//     L64  : double2 [9]  (full 3x3, boundary phase and -cc_mu/2 folded in)
//     L32  : float2  [9]  (same, FP32)
//     L32R : float4  [3]  (rows 0,1 of an SU(3) matrix; row 2 rebuilt as
//                          conj(row0 x row1); phase and -cc_mu/2 at run time)
//     LDD  : float4  [9]  (as L64, each complex as (re.h, im.h, re.l, im.l))
#pragma once
#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include <cstdint>

namespace gbf {

// PDD: double-float storage and arithmetic (value = h + l, two FP32 words;
// see struct dd below), the FP64-accurate path that runs on the FP32 pipe.
enum Prec { P64 = 0, P32 = 1, P16 = 2, PDD = 3 };
enum LinkStore { L64 = 0, L32 = 1, L32R = 2, LDD = 3 };
enum LocalKind { LOC_NONE = 0, LOC_CLOVER = 1, LOC_SMAT = 2, LOC_SCALAR = 3, LOC_TWIST = 4 };

constexpr int kMaxLs = 32;
constexpr int kMaxRhs = 16;

// Division of a 32-bit unsigned n < 2^31 by a run-time constant d >= 1 as a
// multiply-high and a shift (Granlund & Montgomery, "Division by invariant
// integers using multiplication", PLDI 1994): with l = ceil(log2 d),
// m = floor(2^32 (2^l - d) / d) + 1,  n / d = (umulhi(n, m) + n) >> l.
struct FastDiv {
  unsigned d, m, l;
  __host__ __device__ FastDiv() : d(1), m(1), l(0) {}
  __host__ explicit FastDiv(unsigned dd) : d(dd) {
    l = 0;
    while ((1ull << l) < dd) ++l;
    m = (unsigned)(((1ull << 32) * ((1ull << l) - dd)) / dd + 1);
  }
  __device__ __forceinline__ unsigned div(unsigned n) const { return (__umulhi(n, m) + n) >> l; }
};

// Geometry and run-time constants of one operator.
struct Geo {
  int L[4];
  int Lh0;      // L0 / 2
  int Vh;       // 4D sites per parity
  int N5;       // inner extent = Ls * nrhs
  int Ls;       // 5th dimension (1 for Wilson-clover)
  int nrhs;
  long long N;  // 5D sites per parity = Vh * N5 (12 N < 2^31 is checked at creation)
  // run-time link factors for reconstructed links: lambda_mu = -cc_mu/2 and phase_mu
  float lam[4];
  float ph_re[4], ph_im[4];
  FastDiv fLh0, fL1, fL2, fN5, fLs;
};

template <typename R> struct C2;
template <> struct C2<double> { using T = double2; };
template <> struct C2<float> { using T = float2; };
template <typename R> using cplx = typename C2<R>::T;

template <typename R> __device__ __forceinline__ cplx<R> mk(R a, R b) { cplx<R> r; r.x = a; r.y = b; return r; }
template <typename R> __device__ __forceinline__ cplx<R> cz() { return mk<R>(0, 0); }
template <typename R> __device__ __forceinline__ cplx<R> add(cplx<R> a, cplx<R> b) { return mk<R>(a.x + b.x, a.y + b.y); }
template <typename R> __device__ __forceinline__ cplx<R> sub(cplx<R> a, cplx<R> b) { return mk<R>(a.x - b.x, a.y - b.y); }
template <typename R> __device__ __forceinline__ cplx<R> scl(R s, cplx<R> a) { return mk<R>(s * a.x, s * a.y); }
// acc + a*b
template <typename R> __device__ __forceinline__ cplx<R> cmadd(cplx<R> acc, cplx<R> a, cplx<R> b) {
  acc.x = fma(a.x, b.x, acc.x); acc.x = fma(-a.y, b.y, acc.x);
  acc.y = fma(a.x, b.y, acc.y); acc.y = fma(a.y, b.x, acc.y);
  return acc;
}
// acc + conj(a)*b
template <typename R> __device__ __forceinline__ cplx<R> cmaddc(cplx<R> acc, cplx<R> a, cplx<R> b) {
  acc.x = fma(a.x, b.x, acc.x); acc.x = fma(a.y, b.y, acc.x);
  acc.y = fma(a.x, b.y, acc.y); acc.y = fma(-a.y, b.x, acc.y);
  return acc;
}
template <typename R> __device__ __forceinline__ cplx<R> cmul(cplx<R> a, cplx<R> b) { return cmadd<R>(cz<R>(), a, b); }
template <typename R> __device__ __forceinline__ R rzero() { return R(0); }

// ---------------------------------------------------------------------------
// Double-float numbers.  A value is the unevaluated sum h + l of two FP32
// words with |l| <= ulp(h)/2 after an addition or a product (a 48-bit
// significand, unit roundoff 2^-48 ~ 3.6e-15), so FP64-class accuracy runs
// on the FP32 pipe, which on GB300 issues about 70 times the FP64 pipe's
// operations.  fma leaves the pair un-normalised (|l| a few ulp(h)): the
// next operation absorbs it, and the saved fast-two-sum is a fifth of the
// cost of an fma (build with GBF_DD_RENORM to normalise there too).
// The operations are built from two error-free transformations:
//   TwoSum(a, b) = (s, e), s = fl(a + b), s + e = a + b exactly
//     (Knuth, TAOCP vol. 2, sec. 4.2.2, Theorem B);
//   TwoProd(a, b) = (p, e), p = fl(a b), e = fma(a, b, -p), p + e = a b exactly.
// Addition is the "sloppy" double-word sum and the product keeps the cross
// terms a.h b.l + a.l b.h and drops a.l b.l (Joldes, Muller, Popescu, ACM
// TOMS 44 (2017) 15, algorithms 4 and 10): the error of each operation is a
// few 2^-48 relative to its operands.  Every intrinsic is round-to-nearest
// and un-contracted, so the compiler cannot fuse or reorder the steps.
// ---------------------------------------------------------------------------
struct dd {
  float h, l;
  dd() = default;
  __host__ __device__ constexpr dd(float hi, float lo) : h(hi), l(lo) {}
  __host__ __device__ explicit dd(int a) : h((float)a), l(0.f) {}
  __host__ __device__ explicit dd(float a) : h(a), l(0.f) {}
  // round-to-nearest split of a double: h = fl32(a), l = fl32(a - h); a - h is exact
  __host__ __device__ explicit dd(double a) : h((float)a), l((float)(a - (double)(float)a)) {}
  __host__ __device__ explicit operator double() const { return (double)h + (double)l; }
};

__device__ __forceinline__ dd dd_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return dd(s, e);
}
// exact when |a| >= |b| (or a == 0)
__device__ __forceinline__ dd dd_fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return dd(s, __fsub_rn(b, __fsub_rn(s, a)));
}
__device__ __forceinline__ dd operator-(dd a) { return dd(-a.h, -a.l); }
__device__ __forceinline__ dd operator+(dd a, dd b) {
  const dd s = dd_two_sum(a.h, b.h);
  return dd_fast_two_sum(s.h, __fadd_rn(s.l, __fadd_rn(a.l, b.l)));
}
__device__ __forceinline__ dd operator-(dd a, dd b) { return a + (-b); }
__device__ __forceinline__ dd operator*(dd a, dd b) {
  const float p = __fmul_rn(a.h, b.h);
  float e = __fmaf_rn(a.h, b.h, -p);
  e = __fmaf_rn(a.h, b.l, e);
  e = __fmaf_rn(a.l, b.h, e);
  return dd_fast_two_sum(p, e);
}
// a * b + c
using ::fma;
__device__ __forceinline__ dd fma(dd a, dd b, dd c) {
  const float p = __fmul_rn(a.h, b.h);
  float e = __fmaf_rn(a.h, b.h, -p);
  e = __fmaf_rn(a.h, b.l, e);
  e = __fmaf_rn(a.l, b.h, e);
  const dd s = dd_two_sum(p, c.h);
#ifdef GBF_DD_RENORM
  return dd_fast_two_sum(s.h, __fadd_rn(s.l, __fadd_rn(e, c.l)));
#else
  return dd(s.h, __fadd_rn(s.l, __fadd_rn(e, c.l)));
#endif
}
// exact scaling by +-1 (or any power of two)
__device__ __forceinline__ dd dd_scale2(float f, dd a) { return dd(__fmul_rn(f, a.h), __fmul_rn(f, a.l)); }

struct ddc {
  dd x, y;
};
template <> struct C2<dd> { using T = ddc; };
template <> __device__ __forceinline__ dd rzero<dd>() { return dd(0.f, 0.f); }
template <> __device__ __forceinline__ cplx<dd> cz<dd>() { return mk<dd>(dd(0.f, 0.f), dd(0.f, 0.f)); }

// Two double-float numbers as lanes of FP32 pairs (fma.rn.f32x2 and
// add.rn.f32x2 on sm_100 and later): value_k = h.k + l.k for k = x, y.  As a
// complex double-float, x is the real and y the imaginary part, which is the
// float4 storage (x.h, y.h, x.l, y.l) of double-float fields and links, so a
// 16-byte load is a pdd.  Every operation is the lane-wise form of the
// scalar one above (the same steps in the same order), so the results equal
// the scalar code's while the FP32 pipe is issued half the instructions.
struct pdd {
  float2 h, l;
};
__device__ __forceinline__ pdd pdd_ld(const float4 q) { return pdd{make_float2(q.x, q.y), make_float2(q.z, q.w)}; }
__device__ __forceinline__ float4 pdd_st(const pdd a) { return make_float4(a.h.x, a.h.y, a.l.x, a.l.y); }
__device__ __forceinline__ float2 neg2(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ void two_sum2(float2 a, float2 b, float2& s, float2& e) {
  s = __fadd2_rn(a, b);
  const float2 bb = __fadd2_rn(s, neg2(a));
  e = __fadd2_rn(__fadd2_rn(a, neg2(__fadd2_rn(s, neg2(bb)))), __fadd2_rn(b, neg2(bb)));
}
__device__ __forceinline__ pdd fast_two_sum2(float2 a, float2 b) {
  const float2 s = __fadd2_rn(a, b);
  return pdd{s, __fadd2_rn(b, neg2(__fadd2_rn(s, neg2(a))))};
}
// a + b
__device__ __forceinline__ pdd pdd_add(pdd a, pdd b) {
  float2 s, e;
  two_sum2(a.h, b.h, s, e);
  return fast_two_sum2(s, __fadd2_rn(e, __fadd2_rn(a.l, b.l)));
}
// f a + c for a double-float scalar f (as fma(dd, dd, dd); c = 0 gives the
// un-normalised product, as cmul)
__device__ __forceinline__ pdd pdd_fma_s(dd f, pdd a, pdd c) {
  const float2 fh = make_float2(f.h, f.h), fl = make_float2(f.l, f.l);
  const float2 p = __fmul2_rn(fh, a.h);
  float2 e = __ffma2_rn(fh, a.h, neg2(p));
  e = __ffma2_rn(fh, a.l, e);
  e = __ffma2_rn(fl, a.h, e);
  float2 s, t;
  two_sum2(p, c.h, s, t);
#ifdef GBF_DD_RENORM
  return fast_two_sum2(s, __fadd2_rn(t, __fadd2_rn(e, c.l)));
#else
  return pdd{s, __fadd2_rn(t, __fadd2_rn(e, c.l))};
#endif
}
// f a: fma with c = 0 without the two-sum with zero (equal up to the sign
// of a zero low word)
__device__ __forceinline__ pdd pdd_mul_s(dd f, pdd a) {
  const float2 fh = make_float2(f.h, f.h), fl = make_float2(f.l, f.l);
  const float2 p = __fmul2_rn(fh, a.h);
  float2 e = __ffma2_rn(fh, a.h, neg2(p));
  e = __ffma2_rn(fh, a.l, e);
  e = __ffma2_rn(fl, a.h, e);
  return pdd{p, e};
}
// i a
__device__ __forceinline__ pdd pdd_i(pdd a) { return pdd{make_float2(-a.h.y, a.h.x), make_float2(-a.l.y, a.l.x)}; }
__device__ __forceinline__ pdd pdd_nrm(pdd a) { return fast_two_sum2(a.h, a.l); }
// a + s coef v with run-time coefficient code and sign (as coefmadd_rt)
__device__ __forceinline__ pdd pdd_coefmadd_rt(int code, float s, pdd v, pdd a) {
  const bool im = code >= 2;
  const float sg = (code == 1 || code == 3) ? -s : s;
  const pdd w = im ? pdd_i(v) : v;
  const float2 f = make_float2(sg, sg);
  return pdd_add(a, pdd{__fmul2_rn(f, w.h), __fmul2_rn(f, w.l)});
}

// Normalise an fma result before it is stored or used as a factor: with
// cancellation in the un-normalised pair |l| can exceed |h|, and a product
// (which drops l_a l_b) would then be wrong.  No-op for FP32 / FP64.
template <typename R> __device__ __forceinline__ void nrm(cplx<R>&) {}
template <> __device__ __forceinline__ void nrm<dd>(cplx<dd>& v) {
  v.x = dd_fast_two_sum(v.x.h, v.x.l);
  v.y = dd_fast_two_sum(v.y.h, v.y.l);
}

// ---------------------------------------------------------------------------
// spinor storage
// ---------------------------------------------------------------------------
template <int P> struct SpinorT;
template <> struct SpinorT<P64> { using R = double; static constexpr int bytes = 192; };
template <> struct SpinorT<P32> { using R = float; static constexpr int bytes = 96; };
template <> struct SpinorT<P16> { using R = float; static constexpr int bytes = 52; };
template <> struct SpinorT<PDD> { using R = dd; static constexpr int bytes = 192; };

__host__ __device__ inline long long half_bytes(int P, long long N) {
  return (P == P64 || P == PDD) ? 192 * N : (P == P32 ? 96 * N : 52 * N);
}

// Element indices are 32-bit: gbf_create checks 12 N < 2^31 (and the link and
// clover extents), so `n + k N` never overflows and each address is a single
// 32-bit multiply-add into a 64-bit pointer.
template <int P> __device__ __forceinline__ void load_spinor(const void* base, long long N, long long n, cplx<typename SpinorT<P>::R> (&v)[12]);
template <int P> __device__ __forceinline__ void store_spinor(void* base, long long N, long long n, const cplx<typename SpinorT<P>::R> (&v)[12]);

template <> __device__ __forceinline__ void load_spinor<P64>(const void* base, long long N_, long long n_, double2 (&v)[12]) {
  const double2* p = reinterpret_cast<const double2*>(base);
  const unsigned N = (unsigned)N_, n = (unsigned)n_;
#pragma unroll
  for (int k = 0; k < 12; ++k) v[k] = __ldg(p + (n + k * N));
}
template <> __device__ __forceinline__ void store_spinor<P64>(void* base, long long N_, long long n_, const double2 (&v)[12]) {
  double2* p = reinterpret_cast<double2*>(base);
  const unsigned N = (unsigned)N_, n = (unsigned)n_;
#pragma unroll
  for (int k = 0; k < 12; ++k) p[n + k * N] = v[k];
}
// double-float: float4 (re.h, im.h, re.l, im.l) [12][N]: one 16-byte load
// gives the packed high pair and the packed low pair of a complex number
template <> __device__ __forceinline__ void load_spinor<PDD>(const void* base, long long N_, long long n_, ddc (&v)[12]) {
  const float4* p = reinterpret_cast<const float4*>(base);
  const unsigned N = (unsigned)N_, n = (unsigned)n_;
#pragma unroll
  for (int k = 0; k < 12; ++k) {
    const float4 q = __ldg(p + (n + k * N));
    v[k].x = dd(q.x, q.z);
    v[k].y = dd(q.y, q.w);
  }
}
template <> __device__ __forceinline__ void store_spinor<PDD>(void* base, long long N_, long long n_, const ddc (&v)[12]) {
  float4* p = reinterpret_cast<float4*>(base);
  const unsigned N = (unsigned)N_, n = (unsigned)n_;
#pragma unroll
  for (int k = 0; k < 12; ++k) {
    ddc w = v[k];
    nrm<dd>(w);  // memory holds normalised pairs
    p[n + k * N] = make_float4(w.x.h, w.y.h, w.x.l, w.y.l);
  }
}
template <> __device__ __forceinline__ void load_spinor<P32>(const void* base, long long N_, long long n_, float2 (&v)[12]) {
  const float4* p = reinterpret_cast<const float4*>(base);
  const unsigned N = (unsigned)N_, n = (unsigned)n_;
#pragma unroll
  for (int k = 0; k < 6; ++k) {
    float4 q = __ldg(p + (n + k * N));
    v[2 * k] = make_float2(q.x, q.y);
    v[2 * k + 1] = make_float2(q.z, q.w);
  }
}
template <> __device__ __forceinline__ void store_spinor<P32>(void* base, long long N_, long long n_, const float2 (&v)[12]) {
  float4* p = reinterpret_cast<float4*>(base);
  const unsigned N = (unsigned)N_, n = (unsigned)n_;
#pragma unroll
  for (int k = 0; k < 6; ++k) p[n + k * N] = make_float4(v[2 * k].x, v[2 * k].y, v[2 * k + 1].x, v[2 * k + 1].y);
}
template <> __device__ __forceinline__ void load_spinor<P16>(const void* base, long long N_, long long n_, float2 (&v)[12]) {
  const uint4* p = reinterpret_cast<const uint4*>(base);
  const unsigned N = (unsigned)N_, n = (unsigned)n_;
  const float s = __ldg(reinterpret_cast<const float*>(p + 3 * N) + n);
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    uint4 q = __ldg(p + (n + k * N));
    const unsigned w[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      __half2 h = *reinterpret_cast<const __half2*>(&w[j]);
      float2 f = __half22float2(h);
      v[4 * k + j] = make_float2(f.x * s, f.y * s);
    }
  }
}
template <> __device__ __forceinline__ void store_spinor<P16>(void* base, long long N_, long long n_, const float2 (&v)[12]) {
  float m = 0.f;
#pragma unroll
  for (int k = 0; k < 12; ++k) m = fmaxf(m, fmaxf(fabsf(v[k].x), fabsf(v[k].y)));
  const float inv = m > 0.f ? 1.f / m : 0.f;
  uint4* p = reinterpret_cast<uint4*>(base);
  const unsigned N = (unsigned)N_, n = (unsigned)n_;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    unsigned w[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      __half2 h = __floats2half2_rn(v[4 * k + j].x * inv, v[4 * k + j].y * inv);
      w[j] = *reinterpret_cast<unsigned*>(&h);
    }
    p[n + k * N] = make_uint4(w[0], w[1], w[2], w[3]);
  }
  reinterpret_cast<float*>(p + 3 * N)[n] = m;
}

// ---------------------------------------------------------------------------
// links
// ---------------------------------------------------------------------------
template <int LS> struct LinkT;
template <> struct LinkT<L64> { using R = double; static constexpr int chunks = 9; static constexpr int chunk_bytes = 16; };
template <> struct LinkT<L32> { using R = float; static constexpr int chunks = 9; static constexpr int chunk_bytes = 8; };
template <> struct LinkT<L32R> { using R = float; static constexpr int chunks = 3; static constexpr int chunk_bytes = 16; };
template <> struct LinkT<LDD> { using R = dd; static constexpr int chunks = 9; static constexpr int chunk_bytes = 16; };

__host__ __device__ inline long long link_bytes_per_parity_mu(int LS, int Vh) {
  return (long long)Vh * ((LS == L64 || LS == LDD) ? 144 : (LS == L32 ? 72 : 48));
}

// Load U_mu at checkerboard index cb of parity p into u[9] (row major).
template <int LS, typename R>
__device__ __forceinline__ void load_link(const void* links, int Vh, int p, int mu, int cb, cplx<R> (&u)[9]);

template <> __device__ __forceinline__ void load_link<L64, double>(const void* links, int Vh, int p, int mu, int cb, double2 (&u)[9]) {
  const double2* b = reinterpret_cast<const double2*>(links);
  const unsigned o = (unsigned)((p * 4 + mu) * 9) * (unsigned)Vh + (unsigned)cb;
#pragma unroll
  for (int k = 0; k < 9; ++k) u[k] = __ldg(b + (o + (unsigned)k * (unsigned)Vh));
}
template <> __device__ __forceinline__ void load_link<LDD, dd>(const void* links, int Vh, int p, int mu, int cb, ddc (&u)[9]) {
  const float4* b = reinterpret_cast<const float4*>(links);
  const unsigned o = (unsigned)((p * 4 + mu) * 9) * (unsigned)Vh + (unsigned)cb;
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    const float4 q = __ldg(b + (o + (unsigned)k * (unsigned)Vh));
    u[k].x = dd(q.x, q.z);
    u[k].y = dd(q.y, q.w);
  }
}
template <> __device__ __forceinline__ void load_link<L32, float>(const void* links, int Vh, int p, int mu, int cb, float2 (&u)[9]) {
  const float2* b = reinterpret_cast<const float2*>(links);
  const unsigned o = (unsigned)((p * 4 + mu) * 9) * (unsigned)Vh + (unsigned)cb;
#pragma unroll
  for (int k = 0; k < 9; ++k) u[k] = __ldg(b + (o + (unsigned)k * (unsigned)Vh));
}
// SU(3) link from its first two rows (three float4): row 2 = conj(row0 x row1)
__device__ __forceinline__ void link12_rebuild(const float4 a0, const float4 a1, const float4 a2, float2 (&u)[9]) {
  u[0] = make_float2(a0.x, a0.y); u[1] = make_float2(a0.z, a0.w); u[2] = make_float2(a1.x, a1.y);
  u[3] = make_float2(a1.z, a1.w); u[4] = make_float2(a2.x, a2.y); u[5] = make_float2(a2.z, a2.w);
  // row2 = conj(row0 x row1)
  u[6] = make_float2(u[1].x * u[5].x - u[1].y * u[5].y - (u[2].x * u[4].x - u[2].y * u[4].y),
                     -(u[1].x * u[5].y + u[1].y * u[5].x - (u[2].x * u[4].y + u[2].y * u[4].x)));
  u[7] = make_float2(u[2].x * u[3].x - u[2].y * u[3].y - (u[0].x * u[5].x - u[0].y * u[5].y),
                     -(u[2].x * u[3].y + u[2].y * u[3].x - (u[0].x * u[5].y + u[0].y * u[5].x)));
  u[8] = make_float2(u[0].x * u[4].x - u[0].y * u[4].y - (u[1].x * u[3].x - u[1].y * u[3].y),
                     -(u[0].x * u[4].y + u[0].y * u[4].x - (u[1].x * u[3].y + u[1].y * u[3].x)));
}
template <> __device__ __forceinline__ void load_link<L32R, float>(const void* links, int Vh, int p, int mu, int cb, float2 (&u)[9]) {
  const float4* b = reinterpret_cast<const float4*>(links);
  const unsigned o = (unsigned)((p * 4 + mu) * 3) * (unsigned)Vh + (unsigned)cb;
  link12_rebuild(__ldg(b + o), __ldg(b + (o + (unsigned)Vh)), __ldg(b + (o + 2u * (unsigned)Vh)), u);
}

// ---------------------------------------------------------------------------
// gamma matrices of the gpt/Grid basis (lib/gpt/core/gamma.py:28-41):
// gamma_mu[r][perm(mu,r)] = coef(mu,r), coef in {+1,-1,+i,-i}
// coef codes: 0:+1 1:-1 2:+i 3:-i
// ---------------------------------------------------------------------------
__host__ __device__ constexpr int gperm(int mu, int r) { return (mu < 2) ? (3 - r) : ((r + 2) & 3); }
__host__ __device__ constexpr int gcoef(int mu, int r) {
  return mu == 0 ? (r < 2 ? 2 : 3) : mu == 1 ? (r == 0 || r == 3 ? 1 : 0) : mu == 2 ? (r == 0 || r == 3 ? 2 : 3) : 0;
}
// s * coef * v  (s = +-1 as a real factor)
template <typename R> __device__ __forceinline__ cplx<R> coefmul(int code, R s, cplx<R> v) {
  switch (code) {
    case 0: return mk<R>(s * v.x, s * v.y);
    case 1: return mk<R>(-s * v.x, -s * v.y);
    case 2: return mk<R>(-s * v.y, s * v.x);
    default: return mk<R>(s * v.y, -s * v.x);
  }
}
// a + s * coef * v as fused multiply-adds
template <typename R> __device__ __forceinline__ cplx<R> coefmadd(int code, R s, cplx<R> v, cplx<R> a) {
  switch (code) {
    case 0: return mk<R>(fma(s, v.x, a.x), fma(s, v.y, a.y));
    case 1: return mk<R>(fma(-s, v.x, a.x), fma(-s, v.y, a.y));
    case 2: return mk<R>(fma(-s, v.y, a.x), fma(s, v.x, a.y));
    default: return mk<R>(fma(s, v.y, a.x), fma(-s, v.x, a.y));
  }
}
// double-float: the callers' s is the projector sign +-1, so s*v is an exact
// rescaling and the term is a double-float addition
template <> __device__ __forceinline__ cplx<dd> coefmadd<dd>(int code, dd s, cplx<dd> v, cplx<dd> a) {
  const dd vx = dd_scale2(s.h, v.x), vy = dd_scale2(s.h, v.y);
  switch (code) {
    case 0: return mk<dd>(a.x + vx, a.y + vy);
    case 1: return mk<dd>(a.x - vx, a.y - vy);
    case 2: return mk<dd>(a.x - vy, a.y + vx);
    default: return mk<dd>(a.x + vy, a.y - vx);
  }
}

// a + s * coef * v with the coefficient code and the sign known only at run
// time (rolled direction loops): branch-free, s = +-1
__device__ __forceinline__ cplx<dd> coefmadd_rt(int code, float s, cplx<dd> v, cplx<dd> a) {
  const bool im = code >= 2;
  const float sg = (code == 1 || code == 3) ? -s : s;
  const dd tx = im ? -v.y : v.x;  // coef = +-i multiplies by i: (x, y) -> (-y, x)
  const dd ty = im ? v.x : v.y;
  return mk<dd>(a.x + dd_scale2(sg, tx), a.y + dd_scale2(sg, ty));
}

// the three colour components of spin k of a double-float spinor
__device__ __forceinline__ void load_spin_dd(const void* base, long long N_, unsigned n, int k, ddc (&v)[3]) {
  const float4* p = reinterpret_cast<const float4*>(base);
  const unsigned N = (unsigned)N_;
#pragma unroll
  for (int col = 0; col < 3; ++col) {
    const float4 q = __ldg(p + (n + (unsigned)(3 * k + col) * N));
    v[col].x = dd(q.x, q.z);
    v[col].y = dd(q.y, q.w);
  }
}

// 4D coordinates of checkerboard index cb at parity p
struct Coord { int x[4]; };
__device__ __forceinline__ Coord cb_coords(const Geo& g, int cb, int p) {
  Coord c;
  const unsigned r0 = g.fLh0.div((unsigned)cb);
  const int xh = cb - (int)r0 * g.Lh0;
  const unsigned r1 = g.fL1.div(r0);
  c.x[1] = (int)r0 - (int)r1 * g.L[1];
  const unsigned r2 = g.fL2.div(r1);
  c.x[2] = (int)r1 - (int)r2 * g.L[2];
  c.x[3] = (int)r2;
  c.x[0] = 2 * xh + ((c.x[1] + c.x[2] + c.x[3] + p) & 1);
  return c;
}
__device__ __forceinline__ int cb_index(const Geo& g, const int (&x)[4]) {
  return (x[0] >> 1) + g.Lh0 * (x[1] + g.L[1] * (x[2] + g.L[2] * x[3]));
}

// ---------------------------------------------------------------------------
// reductions: deterministic two-level sum (fixed block order)
// ---------------------------------------------------------------------------
struct CGState {
  double cp[kMaxRhs];    // |r|^2
  double rsq[kMaxRhs];   // eps^2 |b|^2
  double alpha[kMaxRhs];
  double beta[kMaxRhs];
  double d[kMaxRhs];
  double last[kMaxRhs];  // last reduction result (generic)
  double last_im[kMaxRhs];
  int done[kMaxRhs];
  int all_done;
  int iter;
  int nrhs;
  int breakdown;
  int maxiter;
  // set by a kernel whose bounded wait for an asynchronous copy ran out
  // (never expected; the host turns it into an error)
  int kernel_error;
};

}  // namespace gbf
