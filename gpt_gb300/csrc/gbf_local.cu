// gbf_local.cu -- site-local kernels: clover / s-matrix application, the CG
// vector updates, BLAS with deterministic reductions, precision conversion,
// natural <-> internal layout transfer, gauge packing and the clover build.
//
// All of these are HBM-bound streaming kernels (bytes per 5D site listed at
// each kernel); the clover build is a one-time set-up kernel.
#include "gbf_launch.cuh"

namespace gbf {

// ---------------------------------------------------------------------------
// site-local op with optional CG pre-step (p = r + beta p):
// bytes/site: A + (W read+write if pre) + out + (X) + clover (288 B FP32, 576 B FP64)
// ---------------------------------------------------------------------------
template <int P, int LK, bool LOOP>
__global__ void __launch_bounds__(256) local_kernel(const LocalArgs a) {
  using R = typename SpinorT<P>::R;
  using V = cplx<R>;
  extern __shared__ __align__(16) double smem_d[];
  const Geo& g = a.g;
  if (a.check_done && a.ra.st->all_done) return;
  double red_re = 0, red_im = 0;
  const long long ntiles = (g.N + blockDim.x - 1) / blockDim.x;
  long long tile = blockIdx.x;
  do {
  const long long n = tile * blockDim.x + threadIdx.x;
  const bool active = n < g.N;
  V v[12];
#pragma unroll
  for (int k = 0; k < 12; ++k) v[k] = cz<R>();
  int cb = 0;
  if (active) {
    cb = (int)g.fN5.div((unsigned)n);
    load_spinor<P>(a.A, g.N, n, v);
    if (a.pre) {
      const int rhs = (int)g.fLs.div((unsigned)n - (unsigned)cb * (unsigned)g.N5);
      const R beta = (R)a.ra.st->beta[rhs];
      V w[12];
      load_spinor<P>(a.W, g.N, n, w);
#pragma unroll
      for (int k = 0; k < 12; ++k) {
        v[k] = mk<R>(fma(beta, w[k].x, v[k].x), fma(beta, w[k].y, v[k].y));
        nrm<R>(v[k]);  // a factor of the local op below
      }
      store_spinor<P>(a.W, g.N, n, v);
    }
  }
  if (LK == LOC_SMAT) {
    if (a.l.kind == LOC_SMAT) {
      R* tile = reinterpret_cast<R*>(smem_d);
      R* mat = tile + 24 * blockDim.x;
      if (a.l.cplx) smat_apply_block_c<R>(reinterpret_cast<const R*>(a.l.smat), g.Ls, tile, mat, v);
      else smat_apply_block<R>(reinterpret_cast<const R*>(a.l.smat), g.Ls, tile, mat, v, true);
    }
  } else if (active && a.l.kind != LOC_NONE) {
    local_apply_thread<R>(a.l, g.Vh, a.parity, cb, v);
  }
  if (active) {
    if (a.c1 != 1.0) {
      const R c1 = (R)a.c1;
#pragma unroll
      for (int k = 0; k < 12; ++k) {
        nrm<R>(v[k]);
        v[k] = scl<R>(c1, v[k]);
      }
    }
    if (a.X) {
      V xv[12];
      load_spinor<P>(a.X, g.N, n, xv);
      const R c2 = (R)a.c2;
#pragma unroll
      for (int k = 0; k < 12; ++k) v[k] = mk<R>(fma(c2, xv[k].x, v[k].x), fma(c2, xv[k].y, v[k].y));
    }
    if (a.out) store_spinor<P>(a.out, g.N, n, v);
  }
  if (a.red && active) {
    double vr = 0, vi = 0;
    if (a.red == 1) {
      V yv[12];
      load_spinor<P>(a.Y, g.N, n, yv);
      site_dot<R>(yv, v, vr, vi);
    } else {
      vr = site_norm2<R>(v);
    }
    red_re += vr;
    red_im += vi;
  }
  tile += gridDim.x;
  } while (LOOP && tile < ntiles);
  if (a.red) {
    double* sm = smem_d + (LK == LOC_SMAT ? (24 * blockDim.x + kSmatWords) * sizeof(R) / sizeof(double) + 1 : 0);
    block_reduce_finalize(a.ra, red_re, red_im, g.N5, g.Ls, g.nrhs, sm);
  }
}

static size_t local_smem(int P, int LK, int bd) {
  size_t rb = (P == P64 || P == PDD) ? 8 : 4;
  size_t s = 0;
  if (LK == LOC_SMAT) s += (24 * (size_t)bd + kSmatWords) * rb + 8;
  return s + 2 * (size_t)bd * 8;
}

template <int P, int LK, bool LOOP>
static cudaError_t launch_local_tl(const LocalArgs& a, cudaStream_t st) {
  const int bd = pick_bd(a.bd, a.g.N5);
  if (bd <= 0) return cudaErrorInvalidValue;
  const long long ntiles = (a.g.N + bd - 1) / bd;
  const size_t sm = local_smem(P, LK, bd);
  auto k = local_kernel<P, LK, LOOP>;
  const int res = resident_blocks((const void*)k, bd, sm);
  const long long nb = a.red ? reduce_grid(ntiles, a.g.nrhs, res) : ntiles;
  k<<<(unsigned)nb, bd, sm, st>>>(a);
  return cudaGetLastError();
}

template <int P, int LK>
static cudaError_t launch_local_t(const LocalArgs& a, cudaStream_t st) {
  const int bd = pick_bd(a.bd, a.g.N5);
  if (bd <= 0) return cudaErrorInvalidValue;
  const long long ntiles = (a.g.N + bd - 1) / bd;
  const int res = resident_blocks((const void*)local_kernel<P, LK, true>, bd, local_smem(P, LK, bd));
  const bool loop = a.red && reduce_grid(ntiles, a.g.nrhs, res) < ntiles;
  return loop ? launch_local_tl<P, LK, true>(a, st) : launch_local_tl<P, LK, false>(a, st);
}

cudaError_t launch_local(int P, const LocalArgs& a, cudaStream_t st) {
  const bool sm = a.l.kind == LOC_SMAT;
  if (P == P64) return sm ? launch_local_t<P64, LOC_SMAT>(a, st) : launch_local_t<P64, LOC_CLOVER>(a, st);
  if (P == P32) return sm ? launch_local_t<P32, LOC_SMAT>(a, st) : launch_local_t<P32, LOC_CLOVER>(a, st);
  if (P == P16) return sm ? launch_local_t<P16, LOC_SMAT>(a, st) : launch_local_t<P16, LOC_CLOVER>(a, st);
  if (P == PDD) return sm ? launch_local_t<PDD, LOC_SMAT>(a, st) : launch_local_t<PDD, LOC_CLOVER>(a, st);
  return cudaErrorInvalidValue;
}

// ---------------------------------------------------------------------------
// CG update: r -= alpha mmp; x += alpha p; |r|^2 -> beta, convergence.
// bytes/site: r, mmp, x, p read + r, x written = 6 spinors
// ---------------------------------------------------------------------------
template <int P>
__global__ void __launch_bounds__(256) cg_update_kernel(const CGUpdateArgs a) {
  using R = typename SpinorT<P>::R;
  using V = cplx<R>;
  extern __shared__ __align__(16) double smem_d[];
  const Geo& g = a.g;
  if (a.ra.st->all_done) {
    // every execution of the CG loop's last kernel sets the loop condition
    if (a.ra.use_cond && blockIdx.x == 0 && threadIdx.x == 0) cudaGraphSetConditional(a.ra.cond, 0u);
    return;
  }
  double vr = 0;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x; n < g.N; n += stride) {
    const unsigned i5 = (unsigned)n - g.fN5.div((unsigned)n) * (unsigned)g.N5;
    const int rhs = (int)g.fLs.div(i5);
    const R al = (R)a.ra.st->alpha[rhs];
    V r[12], m[12], x[12], p[12];
    load_spinor<P>(a.r, g.N, n, r);
    load_spinor<P>(a.mmp, g.N, n, m);
    load_spinor<P>(a.x, g.N, n, x);
    load_spinor<P>(a.p, g.N, n, p);
#pragma unroll
    for (int k = 0; k < 12; ++k) {
      r[k] = mk<R>(fma(-al, m[k].x, r[k].x), fma(-al, m[k].y, r[k].y));
      x[k] = mk<R>(fma(al, p[k].x, x[k].x), fma(al, p[k].y, x[k].y));
    }
    vr += site_norm2<R>(r);
    store_spinor<P>(a.r, g.N, n, r);
    store_spinor<P>(a.x, g.N, n, x);
  }
  block_reduce_finalize(a.ra, vr, 0.0, g.N5, g.Ls, g.nrhs, smem_d);
}

cudaError_t launch_cg_update(int P, const CGUpdateArgs& a, cudaStream_t st) {
  const int bd = pick_bd(a.bd, a.g.N5);
  if (bd <= 0) return cudaErrorInvalidValue;
  const size_t sm = 2 * (size_t)bd * 8;
  const void* k = P == P64 ? (const void*)cg_update_kernel<P64>
                : P == P32 ? (const void*)cg_update_kernel<P32>
                : P == P16 ? (const void*)cg_update_kernel<P16>
                : P == PDD ? (const void*)cg_update_kernel<PDD> : nullptr;
  if (!k) return cudaErrorInvalidValue;
  const long long nb = reduce_grid((a.g.N + bd - 1) / bd, a.g.nrhs, resident_blocks(k, bd, sm));
  if (P == P64) cg_update_kernel<P64><<<(unsigned)nb, bd, sm, st>>>(a);
  else if (P == P32) cg_update_kernel<P32><<<(unsigned)nb, bd, sm, st>>>(a);
  else if (P == P16) cg_update_kernel<P16><<<(unsigned)nb, bd, sm, st>>>(a);
  else cg_update_kernel<PDD><<<(unsigned)nb, bd, sm, st>>>(a);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// BLAS: out = a x + b y (complex a, real b, per rhs), reductions
// ---------------------------------------------------------------------------
template <int P>
__global__ void __launch_bounds__(256) blas_kernel(const BlasArgs a) {
  using R = typename SpinorT<P>::R;
  using V = cplx<R>;
  extern __shared__ __align__(16) double smem_d[];
  const Geo& g = a.g;
  double vr = 0, vi = 0;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x; n < g.N; n += stride) {
    const unsigned i5 = (unsigned)n - g.fN5.div((unsigned)n) * (unsigned)g.N5;
    const int rhs = (int)g.fLs.div(i5);
    V x[12], y[12], o[12];
    load_spinor<P>(a.x, g.N, n, x);
    if (a.y) load_spinor<P>(a.y, g.N, n, y);
    else
#pragma unroll
      for (int k = 0; k < 12; ++k) y[k] = cz<R>();
    if (a.red == 3) {
      double dr, di;
      site_dot<R>(x, y, dr, di);
      vr += dr;
      vi += di;
    } else {
      const V ac = mk<R>((R)a.a_re[rhs], (R)a.a_im[rhs]);
      const R bc = (R)a.b_re[rhs];
#pragma unroll
      for (int k = 0; k < 12; ++k) {
        V t = cmul<R>(ac, x[k]);
        o[k] = mk<R>(fma(bc, y[k].x, t.x), fma(bc, y[k].y, t.y));
      }
      if (a.write) store_spinor<P>(a.out, g.N, n, o);
      if (a.red == 2) vr += site_norm2<R>(o);
    }
  }
  if (a.red) block_reduce_finalize(a.ra, vr, vi, g.N5, g.Ls, g.nrhs, smem_d);
}

cudaError_t launch_blas(int P, const BlasArgs& a, cudaStream_t st) {
  const int bd = block_size_for(a.g.N5, LOC_NONE);
  if (bd <= 0) return cudaErrorInvalidValue;
  const long long ntiles = (a.g.N + bd - 1) / bd;
  const size_t sm = 2 * (size_t)bd * 8;
  const void* k = P == P64 ? (const void*)blas_kernel<P64>
                : P == P32 ? (const void*)blas_kernel<P32>
                : P == P16 ? (const void*)blas_kernel<P16>
                : P == PDD ? (const void*)blas_kernel<PDD> : nullptr;
  if (!k) return cudaErrorInvalidValue;
  const long long nb = a.red ? reduce_grid(ntiles, a.g.nrhs, resident_blocks(k, bd, sm)) : ntiles;
  if (P == P64) blas_kernel<P64><<<(unsigned)nb, bd, sm, st>>>(a);
  else if (P == P32) blas_kernel<P32><<<(unsigned)nb, bd, sm, st>>>(a);
  else if (P == P16) blas_kernel<P16><<<(unsigned)nb, bd, sm, st>>>(a);
  else if (P == PDD) blas_kernel<PDD><<<(unsigned)nb, bd, sm, st>>>(a);
  else return cudaErrorInvalidValue;
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// precision conversion
// ---------------------------------------------------------------------------
template <int PO, int PI>
__global__ void convert_kernel(void* out, const void* in, long long N, double scale) {
  const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  using RI = typename SpinorT<PI>::R;
  using RO = typename SpinorT<PO>::R;
  cplx<RI> v[12];
  load_spinor<PI>(in, N, n, v);
  cplx<RO> o[12];
#pragma unroll
  for (int k = 0; k < 12; ++k) o[k] = mk<RO>((RO)(scale * (double)v[k].x), (RO)(scale * (double)v[k].y));
  store_spinor<PO>(out, N, n, o);
}

cudaError_t launch_convert(int Pout, void* out, int Pin, const void* in, long long N, double scale, cudaStream_t st) {
  const int bd = 256;
  const unsigned nb = (unsigned)((N + bd - 1) / bd);
#define GBF_CV(A, B) \
  if (Pout == A && Pin == B) { convert_kernel<A, B><<<nb, bd, 0, st>>>(out, in, N, scale); return cudaGetLastError(); }
  GBF_CV(P64, P64) GBF_CV(P64, P32) GBF_CV(P64, P16)
  GBF_CV(P32, P64) GBF_CV(P32, P32) GBF_CV(P32, P16)
  GBF_CV(P16, P64) GBF_CV(P16, P32) GBF_CV(P16, P16)
  GBF_CV(PDD, P64) GBF_CV(PDD, P32) GBF_CV(PDD, P16) GBF_CV(PDD, PDD)
  GBF_CV(P64, PDD) GBF_CV(P32, PDD) GBF_CV(P16, PDD)
#undef GBF_CV
  return cudaErrorInvalidValue;
}

__global__ void cg_init_kernel(CGState* st, int nrhs, double eps, int maxiter) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  int all = 1;
  st->nrhs = nrhs;
  st->iter = 0;
  st->breakdown = 0;
  st->maxiter = maxiter;
  for (int r = 0; r < nrhs; ++r) {
    const double ssq = st->last[r];
    st->cp[r] = ssq;
    st->rsq[r] = eps * eps * ssq;
    st->alpha[r] = 0.0;
    st->beta[r] = 0.0;
    st->done[r] = (ssq == 0.0) ? 1 : 0;
    all &= st->done[r];
  }
  st->all_done = all;
}

cudaError_t launch_cg_init(CGState* st, int nrhs, double eps, int maxiter, cudaStream_t s) {
  cg_init_kernel<<<1, 32, 0, s>>>(st, nrhs, eps, maxiter);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// natural <-> internal: natural = complex128 [V][Ls][12] (site lexicographic,
// x0 fastest; s fastest within a site); internal full field [even][odd].
// ---------------------------------------------------------------------------
template <int P>
__global__ void import_kernel(Geo g, const double2* nat, void* full, int rhs, int to_natural) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long V = 2LL * g.Vh;
  if (t >= V * g.Ls) return;
  const long long xs = t / g.Ls;
  const int s = (int)(t - xs * g.Ls);
  int x[4];
  long long r = xs;
  for (int m = 0; m < 4; ++m) { x[m] = (int)(r % g.L[m]); r /= g.L[m]; }
  const int par = (x[0] + x[1] + x[2] + x[3]) & 1;
  const int cb = cb_index(g, x);
  const long long n = (long long)cb * g.N5 + (long long)rhs * g.Ls + s;
  using R = typename SpinorT<P>::R;
  char* half = reinterpret_cast<char*>(full) + (par ? half_bytes(P, g.N) : 0);
  const double2* src = nat + (size_t)t * 12;
  cplx<R> v[12];
  if (!to_natural) {
#pragma unroll
    for (int k = 0; k < 12; ++k) v[k] = mk<R>((R)src[k].x, (R)src[k].y);
    store_spinor<P>(half, g.N, n, v);
  } else {
    load_spinor<P>(half, g.N, n, v);
    double2* dst = const_cast<double2*>(src);
#pragma unroll
    for (int k = 0; k < 12; ++k) dst[k] = make_double2((double)v[k].x, (double)v[k].y);
  }
}

cudaError_t launch_import(int P, const Geo& g, const double2* nat, void* full, int rhs, int to_natural, cudaStream_t st) {
  const long long tot = 2LL * g.Vh * g.Ls;
  const unsigned nb = (unsigned)((tot + 255) / 256);
  if (P == P64) import_kernel<P64><<<nb, 256, 0, st>>>(g, nat, full, rhs, to_natural);
  else if (P == P32) import_kernel<P32><<<nb, 256, 0, st>>>(g, nat, full, rhs, to_natural);
  else if (P == P16) import_kernel<P16><<<nb, 256, 0, st>>>(g, nat, full, rhs, to_natural);
  else if (P == PDD) import_kernel<PDD><<<nb, 256, 0, st>>>(g, nat, full, rhs, to_natural);
  else return cudaErrorInvalidValue;
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// gauge packing
// ---------------------------------------------------------------------------
__device__ __forceinline__ double2 zmul(double2 a, double2 b) { return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
__device__ __forceinline__ double2 zconj(double2 a) { return make_double2(a.x, -a.y); }

__device__ void atomic_max_err(unsigned* e, double v) {
  float f = (float)fmin(v, 3.0e38);
  if (!(f >= 0.f)) f = 3.0e38f;  // NaN
  atomicMax(e, __float_as_uint(f));
}

// per-direction link factor: lam = -cc_mu/2 and the boundary phase (re, im)
struct LamPh {
  double lam, re, im;
};

template <int LS>
__global__ void pack_links_kernel(Geo g, const double2* U, void* links, LamPh lam_ph0, LamPh lam_ph1, LamPh lam_ph2,
                                  LamPh lam_ph3, unsigned* err) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long V = 2LL * g.Vh;
  if (t >= 4 * V) return;
  const int mu = (int)(t / V);
  const long long xs = t - (long long)mu * V;
  int x[4];
  long long r = xs;
  for (int m = 0; m < 4; ++m) { x[m] = (int)(r % g.L[m]); r /= g.L[m]; }
  const int par = (x[0] + x[1] + x[2] + x[3]) & 1;
  const int cb = cb_index(g, x);
  double2 u[9];
  for (int k = 0; k < 9; ++k) u[k] = U[(size_t)t * 9 + k];
  const LamPh lp = mu == 0 ? lam_ph0 : mu == 1 ? lam_ph1 : mu == 2 ? lam_ph2 : lam_ph3;
  if (LS == L32R) {
    // unitarity and det = 1 check for the 12-real storage
    double e = 0;
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j) {
        double2 s = make_double2(0, 0);
        for (int k = 0; k < 3; ++k) {
          double2 q = zmul(zconj(u[3 * k + i]), u[3 * k + j]);
          s.x += q.x; s.y += q.y;
        }
        if (i == j) s.x -= 1.0;
        e = fmax(e, fabs(s.x) + fabs(s.y));
      }
    double2 c0 = zmul(u[4], u[8]), c1 = zmul(u[5], u[7]);
    double2 m0 = make_double2(c0.x - c1.x, c0.y - c1.y);
    double2 c2 = zmul(u[3], u[8]), c3 = zmul(u[5], u[6]);
    double2 m1 = make_double2(c2.x - c3.x, c2.y - c3.y);
    double2 c4 = zmul(u[3], u[7]), c5 = zmul(u[4], u[6]);
    double2 m2 = make_double2(c4.x - c5.x, c4.y - c5.y);
    double2 a0 = zmul(u[0], m0), a1 = zmul(u[1], m1), a2 = zmul(u[2], m2);
    double2 det = make_double2(a0.x - a1.x + a2.x, a0.y - a1.y + a2.y);
    e = fmax(e, fabs(det.x - 1.0) + fabs(det.y));
    atomic_max_err(err, e);
    float4* b = reinterpret_cast<float4*>(links) + (size_t)(par * 4 + mu) * 3 * g.Vh + cb;
    b[0] = make_float4((float)u[0].x, (float)u[0].y, (float)u[1].x, (float)u[1].y);
    b[g.Vh] = make_float4((float)u[2].x, (float)u[2].y, (float)u[3].x, (float)u[3].y);
    b[2 * (size_t)g.Vh] = make_float4((float)u[4].x, (float)u[4].y, (float)u[5].x, (float)u[5].y);
    return;
  }
  double2 lam = make_double2(lp.lam, 0.0);
  if (x[mu] == g.L[mu] - 1) lam = make_double2(lp.lam * lp.re, lp.lam * lp.im);
  for (int k = 0; k < 9; ++k) u[k] = zmul(lam, u[k]);
  if (LS == L64) {
    double2* b = reinterpret_cast<double2*>(links) + (size_t)(par * 4 + mu) * 9 * g.Vh + cb;
    for (int k = 0; k < 9; ++k) b[(size_t)k * g.Vh] = u[k];
  } else if (LS == LDD) {
    float4* b = reinterpret_cast<float4*>(links) + (size_t)(par * 4 + mu) * 9 * g.Vh + cb;
    for (int k = 0; k < 9; ++k) {
      const dd re(u[k].x), im(u[k].y);
      b[(size_t)k * g.Vh] = make_float4(re.h, im.h, re.l, im.l);
    }
  } else {
    float2* b = reinterpret_cast<float2*>(links) + (size_t)(par * 4 + mu) * 9 * g.Vh + cb;
    for (int k = 0; k < 9; ++k) b[(size_t)k * g.Vh] = make_float2((float)u[k].x, (float)u[k].y);
  }
}

cudaError_t launch_pack_links(int LS, const Geo& g, const double2* U, void* links, const double* lam_mu, const double* ph,
                              unsigned* err, cudaStream_t st) {
  const long long tot = 8LL * g.Vh;
  const unsigned nb = (unsigned)((tot + 255) / 256);
  LamPh lp[4];
  for (int m = 0; m < 4; ++m) lp[m] = LamPh{lam_mu[m], ph[2 * m], ph[2 * m + 1]};
  if (LS == L64) pack_links_kernel<L64><<<nb, 256, 0, st>>>(g, U, links, lp[0], lp[1], lp[2], lp[3], err);
  else if (LS == L32) pack_links_kernel<L32><<<nb, 256, 0, st>>>(g, U, links, lp[0], lp[1], lp[2], lp[3], err);
  else if (LS == L32R) pack_links_kernel<L32R><<<nb, 256, 0, st>>>(g, U, links, lp[0], lp[1], lp[2], lp[3], err);
  else if (LS == LDD) pack_links_kernel<LDD><<<nb, 256, 0, st>>>(g, U, links, lp[0], lp[1], lp[2], lp[3], err);
  else return cudaErrorInvalidValue;
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// clover build (one thread per 4D site, FP64):
//   F_munu = 1/8 (Q - Q^+), Q the four-leaf clover (lib/gpt/qcd/gauge/loops.py:162-174)
//   C = sum_{mu<nu} -1/2 c_p sigma_munu (x) F_munu + diag   (reference/wilson_clover.py:91-127)
// sigma_munu restricted to the chiral blocks comes from the host.
// ---------------------------------------------------------------------------
struct SigmaBlocks {
  double2 s[6][2][4];  // [plane][block][2x2]
};

struct NatGeo {
  int L[4];
  __device__ long long idx(const int (&x)[4]) const { return x[0] + (long long)L[0] * (x[1] + (long long)L[1] * (x[2] + (long long)L[2] * x[3])); }
  __device__ long long shift(long long s, int mu, int d) const {
    int x[4];
    long long r = s;
    for (int m = 0; m < 4; ++m) { x[m] = (int)(r % L[m]); r /= L[m]; }
    x[mu] = (x[mu] + d + L[mu]) % L[mu];
    return idx(x);
  }
};

// 3x3 products with operands either in registers or straight from the
// natural gauge field in memory (no local copies; every index is static so
// the matrices stay in registers).  op(X) = X or X^dagger.
template <bool ADJ>
__device__ __forceinline__ double2 mel(const double2* X, int i, int j) {
  return ADJ ? zconj(__ldg(X + 3 * j + i)) : __ldg(X + 3 * i + j);
}
// out = op(A) op(B), both in memory
template <bool AA, bool AB>
__device__ __forceinline__ void mul_mm(const double2* A, const double2* B, double2 (&out)[9]) {
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      double2 s = make_double2(0.0, 0.0);
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const double2 q = zmul(mel<AA>(A, i, k), mel<AB>(B, k, j));
        s.x += q.x;
        s.y += q.y;
      }
      out[3 * i + j] = s;
    }
}
// acc += sgn R op(B), R in registers, B in memory
template <bool AB>
__device__ __forceinline__ void mul_rm_acc(const double2 (&R)[9], const double2* B, double sgn, double2 (&acc)[9]) {
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      double2 s = make_double2(0.0, 0.0);
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const double2 q = zmul(R[3 * i + k], mel<AB>(B, k, j));
        s.x += q.x;
        s.y += q.y;
      }
      acc[3 * i + j].x += sgn * s.x;
      acc[3 * i + j].y += sgn * s.y;
    }
}
// acc += A R, A in memory, R in registers
__device__ __forceinline__ void mul_mr_acc(const double2* A, const double2 (&R)[9], double2 (&acc)[9]) {
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      double2 s = make_double2(0.0, 0.0);
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const double2 q = zmul(mel<false>(A, i, k), R[3 * k + j]);
        s.x += q.x;
        s.y += q.y;
      }
      acc[3 * i + j].x += s.x;
      acc[3 * i + j].y += s.y;
    }
}

// v(y) = staple_up(y) - staple_down(y) of the (mu, nu) plane:
//   staple_up(y)   = U_nu(y+mu) U_mu(y+nu)^+ U_nu(y)^+
//   staple_down(y) = U_nu(z+mu)^+ U_mu(z)^+ U_nu(z),  z = y - nu
__device__ __forceinline__ void vfield(const NatGeo& G, const double2* U, long long V, int mu, int nu, long long y,
                                       double2 (&v)[9]) {
  auto L = [&](int m, long long s) { return U + ((size_t)m * V + s) * 9; };
  double2 t[9];
#pragma unroll
  for (int e = 0; e < 9; ++e) v[e] = make_double2(0.0, 0.0);
  mul_mm<false, true>(L(nu, G.shift(y, mu, 1)), L(mu, G.shift(y, nu, 1)), t);
  mul_rm_acc<true>(t, L(nu, y), 1.0, v);
  const long long z = G.shift(y, nu, -1);
  mul_mm<true, true>(L(nu, G.shift(z, mu, 1)), L(mu, z), t);
  mul_rm_acc<false>(t, L(nu, z), -1.0, v);
}

__device__ bool invert6(double2 (&A)[36], double2 (&I)[36]) {
  for (int i = 0; i < 36; ++i) I[i] = make_double2((i % 7 == 0) ? 1.0 : 0.0, 0.0);
  for (int col = 0; col < 6; ++col) {
    int piv = col;
    double best = -1;
    for (int r = col; r < 6; ++r) {
      double m = A[6 * r + col].x * A[6 * r + col].x + A[6 * r + col].y * A[6 * r + col].y;
      if (m > best) { best = m; piv = r; }
    }
    if (!(best > 0)) return false;
    if (piv != col)
      for (int k = 0; k < 6; ++k) {
        double2 t = A[6 * col + k]; A[6 * col + k] = A[6 * piv + k]; A[6 * piv + k] = t;
        t = I[6 * col + k]; I[6 * col + k] = I[6 * piv + k]; I[6 * piv + k] = t;
      }
    double2 pv = A[6 * col + col];
    double pn = pv.x * pv.x + pv.y * pv.y;
    double2 pinv = make_double2(pv.x / pn, -pv.y / pn);
    for (int k = 0; k < 6; ++k) { A[6 * col + k] = zmul(A[6 * col + k], pinv); I[6 * col + k] = zmul(I[6 * col + k], pinv); }
    for (int r = 0; r < 6; ++r) {
      if (r == col) continue;
      double2 f = A[6 * r + col];
      for (int k = 0; k < 6; ++k) {
        double2 a = zmul(f, A[6 * col + k]), b = zmul(f, I[6 * col + k]);
        A[6 * r + k] = make_double2(A[6 * r + k].x - a.x, A[6 * r + k].y - a.y);
        I[6 * r + k] = make_double2(I[6 * r + k].x - b.x, I[6 * r + k].y - b.y);
      }
    }
  }
  return true;
}

// Clover term of every site, one thread per site: for each plane
// F_munu = 1/8 (Q - Q^+), Q = U_mu(x) v(x) + v(x-mu) U_mu(x-mu), in registers;
// -1/2 c_p sigma_munu (x) F_munu is added to the two Hermitian chiral blocks,
// whose 2 x 36 reals (6 diagonal, 15 complex lower entries each) live in
// shared memory ([72][blockDim], one column per thread).  Writes the clover
// blocks in FP64 and FP32 storage; clover_invert_kernel inverts them.
constexpr int kCloverBlock = 64;
__global__ void __launch_bounds__(kCloverBlock) clover_kernel(Geo g, const double2* U, SigmaBlocks sig, double diag,
                                                               double csw_r, double csw_t, double2* c64, float4* c32) {
  __shared__ double acc[72][kCloverBlock];
  const int t = threadIdx.x;
  const long long xs = (long long)blockIdx.x * blockDim.x + t;
  const long long V = 2LL * g.Vh;
  if (xs >= V) return;  // no block-wide synchronisation below: each thread owns its column
  NatGeo G;
  for (int m = 0; m < 4; ++m) G.L[m] = g.L[m];
  int x[4];
  long long r = xs;
  for (int m = 0; m < 4; ++m) { x[m] = (int)(r % g.L[m]); r /= g.L[m]; }
  const int par = (x[0] + x[1] + x[2] + x[3]) & 1;
  const int cb = cb_index(g, x);
#pragma unroll
  for (int e = 0; e < 72; ++e) acc[e][t] = ((e % 36) < 6) ? diag : 0.0;
  int plane = 0;
#pragma unroll 1
  for (int mu = 0; mu < 4; ++mu)
#pragma unroll 1
    for (int nu = mu + 1; nu < 4; ++nu, ++plane) {
      const double cp = (nu == 3) ? csw_t : csw_r;
      if (cp == 0.0) continue;
      double2 v[9], Q[9];
#pragma unroll
      for (int e = 0; e < 9; ++e) Q[e] = make_double2(0.0, 0.0);
      vfield(G, U, V, mu, nu, xs, v);
      mul_mr_acc(U + ((size_t)mu * V + xs) * 9, v, Q);
      const long long xm = G.shift(xs, mu, -1);
      vfield(G, U, V, mu, nu, xm, v);
      mul_rm_acc<false>(v, U + ((size_t)mu * V + xm) * 9, 1.0, Q);
      double2 F[9];
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          const double2 dq = zconj(Q[3 * j + i]);
          F[3 * i + j] = make_double2(0.125 * (Q[3 * i + j].x - dq.x), 0.125 * (Q[3 * i + j].y - dq.y));
        }
#pragma unroll
      for (int b = 0; b < 2; ++b)
#pragma unroll
        for (int s1 = 0; s1 < 2; ++s1)
#pragma unroll
          for (int s2 = 0; s2 < 2; ++s2) {
            const double2 sg = sig.s[plane][b][2 * s1 + s2];
            const double2 f = make_double2(-0.5 * cp * sg.x, -0.5 * cp * sg.y);
#pragma unroll
            for (int a = 0; a < 3; ++a)
#pragma unroll
              for (int c = 0; c < 3; ++c) {
                const int i = 3 * s1 + a, j = 3 * s2 + c;
                if (i < j) continue;  // Hermitian: the lower triangle and the diagonal
                const double2 q = zmul(f, F[3 * a + c]);
                if (i == j) {
                  acc[36 * b + i][t] += q.x;
                } else {
                  const int tt = tri(i, j);
                  acc[36 * b + 6 + 2 * tt][t] += q.x;
                  acc[36 * b + 7 + 2 * tt][t] += q.y;
                }
              }
          }
    }
  const size_t poff36 = (size_t)par * 36 * g.Vh, poff18 = (size_t)par * 18 * g.Vh;
#pragma unroll
  for (int b = 0; b < 2; ++b) {
#pragma unroll
    for (int k = 0; k < 18; ++k)
      c64[poff36 + (size_t)(18 * b + k) * g.Vh + cb] = make_double2(acc[36 * b + 2 * k][t], acc[36 * b + 2 * k + 1][t]);
#pragma unroll
    for (int k = 0; k < 9; ++k)
      c32[poff18 + (size_t)(9 * b + k) * g.Vh + cb] =
          make_float4((float)acc[36 * b + 4 * k][t], (float)acc[36 * b + 4 * k + 1][t], (float)acc[36 * b + 4 * k + 2][t],
                      (float)acc[36 * b + 4 * k + 3][t]);
  }
}

// Inverse of every Hermitian 6x6 clover block, one thread per (site, parity,
// block), Gauss-Jordan with partial pivoting in FP64 on matrices in shared
// memory; reads the FP64 clover, writes the FP64 and FP32 inverse.
constexpr int kInvBlock = 32;
__global__ void __launch_bounds__(kInvBlock) clover_invert_kernel(int Vh, const double2* c64, double2* ci64, float4* ci32,
                                                                  unsigned* err) {
  __shared__ double2 sA[kInvBlock][36], sI[kInvBlock][36];
  const long long tt = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (tt >= 4LL * Vh) return;
  const int cb = (int)(tt % Vh);
  const int pb = (int)(tt / Vh);
  const int par = pb >> 1, b = pb & 1;
  const double2* src = c64 + (size_t)par * 36 * Vh;
  double re[36];
#pragma unroll
  for (int k = 0; k < 18; ++k) {
    const double2 q = src[(size_t)(18 * b + k) * Vh + cb];
    re[2 * k] = q.x;
    re[2 * k + 1] = q.y;
  }
  double2(&A)[36] = sA[threadIdx.x];
  double2(&I)[36] = sI[threadIdx.x];
  for (int i = 0; i < 6; ++i) A[7 * i] = make_double2(re[i], 0.0);
  for (int i = 1; i < 6; ++i)
    for (int j = 0; j < i; ++j) {
      const double2 v = make_double2(re[6 + 2 * tri(i, j)], re[6 + 2 * tri(i, j) + 1]);
      A[6 * i + j] = v;
      A[6 * j + i] = zconj(v);
    }
  if (!invert6(A, I)) atomic_max_err(err, 1e30);
  for (int i = 0; i < 6; ++i) re[i] = I[7 * i].x;
  for (int i = 1; i < 6; ++i)
    for (int j = 0; j < i; ++j) {
      re[6 + 2 * tri(i, j)] = I[6 * i + j].x;
      re[6 + 2 * tri(i, j) + 1] = I[6 * i + j].y;
    }
  double2* d64 = ci64 + (size_t)par * 36 * Vh;
  float4* d32 = ci32 + (size_t)par * 18 * Vh;
#pragma unroll
  for (int k = 0; k < 18; ++k) d64[(size_t)(18 * b + k) * Vh + cb] = make_double2(re[2 * k], re[2 * k + 1]);
#pragma unroll
  for (int k = 0; k < 9; ++k)
    d32[(size_t)(9 * b + k) * Vh + cb] = make_float4((float)re[4 * k], (float)re[4 * k + 1], (float)re[4 * k + 2], (float)re[4 * k + 3]);
}

cudaError_t launch_clover(const Geo& g, const double2* U, double diag, double csw_r, double csw_t, void* c64, void* ci64,
                          void* c32, void* ci32, unsigned* err, cudaStream_t st) {
  // sigma_munu = 1/2 [g_mu, g_nu] in the chiral blocks, from the sparse gamma tables
  SigmaBlocks sig;
  auto gm = [](int mu, int r, int c) -> double2 {
    if (gperm(mu, r) != c) return make_double2(0, 0);
    switch (gcoef(mu, r)) {
      case 0: return make_double2(1, 0);
      case 1: return make_double2(-1, 0);
      case 2: return make_double2(0, 1);
      default: return make_double2(0, -1);
    }
  };
  int plane = 0;
  for (int mu = 0; mu < 4; ++mu)
    for (int nu = mu + 1; nu < 4; ++nu, ++plane) {
      double2 S[16];
      for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) {
          double re = 0, im = 0;
          for (int k = 0; k < 4; ++k) {
            double2 a = gm(mu, i, k), b = gm(nu, k, j), c = gm(nu, i, k), d = gm(mu, k, j);
            re += (a.x * b.x - a.y * b.y) - (c.x * d.x - c.y * d.y);
            im += (a.x * b.y + a.y * b.x) - (c.x * d.y + c.y * d.x);
          }
          S[4 * i + j] = make_double2(0.5 * re, 0.5 * im);
        }
      for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j)
          if ((i < 2) != (j < 2) && (S[4 * i + j].x != 0 || S[4 * i + j].y != 0)) return cudaErrorInvalidValue;
      for (int b = 0; b < 2; ++b)
        for (int s1 = 0; s1 < 2; ++s1)
          for (int s2 = 0; s2 < 2; ++s2) sig.s[plane][b][2 * s1 + s2] = S[4 * (2 * b + s1) + (2 * b + s2)];
    }
  const long long V = 2LL * g.Vh;
  clover_kernel<<<(unsigned)((V + kCloverBlock - 1) / kCloverBlock), kCloverBlock, 0, st>>>(
      g, U, sig, diag, csw_r, csw_t, (double2*)c64, (float4*)c32);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  clover_invert_kernel<<<(unsigned)((2 * V + kInvBlock - 1) / kInvBlock), kInvBlock, 0, st>>>(
      g.Vh, (const double2*)c64, (double2*)ci64, (float4*)ci32, err);
  return cudaGetLastError();
}

// Mass change of a clover operator (set_mass): add `shift` to the diagonal
// of both chiral blocks of every site's clover term, in place, and rebuild
// the inverse blocks (Gauss-Jordan with partial pivoting in FP64; the
// matrices of one thread live in shared memory).  One thread per (site,
// parity, block); `prec` is the storage of the operator (P64 double2
// [36][Vh], P32 / P16 float4 [18][Vh], PDD float4 [36][Vh] per parity).
constexpr int kShiftBlock = 32;
__device__ __forceinline__ void clover_row_load(int prec, const void* base, int Vh, size_t off_rows, int b, int cb,
                                                double (&re)[36]) {
  if (prec == P64) {
    const double2* p = reinterpret_cast<const double2*>(base) + off_rows * 2 * Vh;
    for (int k = 0; k < 18; ++k) {
      const double2 q = p[(size_t)(18 * b + k) * Vh + cb];
      re[2 * k] = q.x;
      re[2 * k + 1] = q.y;
    }
  } else if (prec == PDD) {
    const float4* p = reinterpret_cast<const float4*>(base) + off_rows * 2 * Vh;
    for (int k = 0; k < 18; ++k) {
      const float4 q = p[(size_t)(18 * b + k) * Vh + cb];
      re[2 * k] = (double)q.x + (double)q.z;
      re[2 * k + 1] = (double)q.y + (double)q.w;
    }
  } else {
    const float4* p = reinterpret_cast<const float4*>(base) + off_rows * Vh;
    for (int k = 0; k < 9; ++k) {
      const float4 q = p[(size_t)(9 * b + k) * Vh + cb];
      re[4 * k] = q.x; re[4 * k + 1] = q.y; re[4 * k + 2] = q.z; re[4 * k + 3] = q.w;
    }
  }
}
__device__ __forceinline__ void clover_row_store(int prec, void* base, int Vh, size_t off_rows, int b, int cb,
                                                 const double (&re)[36]) {
  if (prec == P64) {
    double2* p = reinterpret_cast<double2*>(base) + off_rows * 2 * Vh;
    for (int k = 0; k < 18; ++k) p[(size_t)(18 * b + k) * Vh + cb] = make_double2(re[2 * k], re[2 * k + 1]);
  } else if (prec == PDD) {
    float4* p = reinterpret_cast<float4*>(base) + off_rows * 2 * Vh;
    for (int k = 0; k < 18; ++k) {
      const dd x(re[2 * k]), y(re[2 * k + 1]);
      p[(size_t)(18 * b + k) * Vh + cb] = make_float4(x.h, y.h, x.l, y.l);
    }
  } else {
    float4* p = reinterpret_cast<float4*>(base) + off_rows * Vh;
    for (int k = 0; k < 9; ++k)
      p[(size_t)(9 * b + k) * Vh + cb] =
          make_float4((float)re[4 * k], (float)re[4 * k + 1], (float)re[4 * k + 2], (float)re[4 * k + 3]);
  }
}

__global__ void __launch_bounds__(kShiftBlock) clover_shift_kernel(int prec, void* clov, void* clov_inv, int Vh,
                                                                     double shift, unsigned* err) {
  __shared__ double2 sA[kShiftBlock][36], sI[kShiftBlock][36];
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 4LL * Vh) return;
  const int cb = (int)(t % Vh);
  const int pb = (int)(t / Vh);  // parity * 2 + block
  const int par = pb >> 1, b = pb & 1;
  // rows of one parity: 36 (FP64 and double-float, in 16-byte units of the
  // storage) or 18 (FP32 float4); offsets in units of the storage row / 2
  const size_t off = (size_t)par * 18;
  double re[36];
  clover_row_load(prec, clov, Vh, off, b, cb, re);
  for (int i = 0; i < 6; ++i) re[i] += shift;
  clover_row_store(prec, clov, Vh, off, b, cb, re);
  double2(&A)[36] = sA[threadIdx.x];
  double2(&I)[36] = sI[threadIdx.x];
  for (int i = 0; i < 6; ++i) A[7 * i] = make_double2(re[i], 0.0);
  for (int i = 1; i < 6; ++i)
    for (int j = 0; j < i; ++j) {
      const double2 v = make_double2(re[6 + 2 * tri(i, j)], re[6 + 2 * tri(i, j) + 1]);
      A[6 * i + j] = v;
      A[6 * j + i] = zconj(v);
    }
  if (!invert6(A, I)) atomic_max_err(err, 1e30);
  for (int i = 0; i < 6; ++i) re[i] = I[7 * i].x;
  for (int i = 1; i < 6; ++i)
    for (int j = 0; j < i; ++j) {
      re[6 + 2 * tri(i, j)] = I[6 * i + j].x;
      re[6 + 2 * tri(i, j) + 1] = I[6 * i + j].y;
    }
  clover_row_store(prec, clov_inv, Vh, off, b, cb, re);
}

cudaError_t launch_clover_shift(int prec, void* clov, void* clov_inv, int Vh, double shift, unsigned* err, cudaStream_t st) {
  const long long n = 4LL * Vh;
  clover_shift_kernel<<<(unsigned)((n + kShiftBlock - 1) / kShiftBlock), kShiftBlock, 0, st>>>(prec, clov, clov_inv, Vh,
                                                                                               shift, err);
  return cudaGetLastError();
}

__global__ void clover_narrow_kernel(const double2* src, float4* dst, long long nrows32, int Vh) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nrows32 * Vh) return;
  const long long row = t / Vh, cb = t - row * Vh;
  const double2 a = src[(2 * row) * Vh + cb], b = src[(2 * row + 1) * Vh + cb];
  dst[row * Vh + cb] = make_float4((float)a.x, (float)a.y, (float)b.x, (float)b.y);
}

cudaError_t launch_clover_narrow(const void* src64, void* dst32, long long nrows32, int Vh, cudaStream_t st) {
  const long long n = nrows32 * Vh;
  clover_narrow_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>((const double2*)src64, (float4*)dst32, nrows32, Vh);
  return cudaGetLastError();
}

// double-float source: each double2 of the FP64 layout is a float4 (x.h, y.h, x.l, y.l)
__global__ void clover_narrow_dd_kernel(const float4* src, float4* dst, long long nrows32, int Vh) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nrows32 * Vh) return;
  const long long row = t / Vh, cb = t - row * Vh;
  const float4 a = src[(2 * row) * Vh + cb], b = src[(2 * row + 1) * Vh + cb];
  dst[row * Vh + cb] = make_float4(__fadd_rn(a.x, a.z), __fadd_rn(a.y, a.w), __fadd_rn(b.x, b.z), __fadd_rn(b.y, b.w));
}

cudaError_t launch_clover_narrow_dd(const void* srcdd, void* dst32, long long nrows32, int Vh, cudaStream_t st) {
  const long long n = nrows32 * Vh;
  clover_narrow_dd_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>((const float4*)srcdd, (float4*)dst32, nrows32, Vh);
  return cudaGetLastError();
}

__global__ void split_dd_kernel(const double2* src, float4* dst, long long n) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const double2 a = src[t];
  const dd x(a.x), y(a.y);
  dst[t] = make_float4(x.h, y.h, x.l, y.l);
}

cudaError_t launch_split_dd(const void* src64, void* dst, long long n_complex, cudaStream_t st) {
  split_dd_kernel<<<(unsigned)((n_complex + 255) / 256), 256, 0, st>>>((const double2*)src64, (float4*)dst, n_complex);
  return cudaGetLastError();
}

}  // namespace gbf

namespace gbf {

// ---------------------------------------------------------------------------
// Fifth-dimension data movement of the MADWF preconditioner
// (lib/gpt/qcd/fermion/preconditioner/mixed_dwf.py:43-98).  Thread per 5D
// site; bytes/site: two reads and one write (chiral shift), one read and one
// write (slice copy).
// ---------------------------------------------------------------------------

// dst_s = P- src_s + P+ src_{(s + offset) mod Ls}, P+- = (1 +- gamma5) / 2 with
// gamma5 = diag(1, 1, -1, -1): spins 0, 1 from slice s + offset, spins 2, 3
// from slice s (the operator P of mixed_dwf.py:46-54; offset -1 is P^+ = P^-1)
template <int P>
__global__ void __launch_bounds__(256) chiral_shift_kernel(const Geo g, const void* src, void* dst, int offset) {
  using R = typename SpinorT<P>::R;
  using V = cplx<R>;
  const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= g.N) return;
  const unsigned cb = g.fN5.div((unsigned)n);
  const unsigned i5 = (unsigned)n - cb * (unsigned)g.N5;
  const unsigned rhs = g.fLs.div(i5);
  const int s = (int)(i5 - rhs * (unsigned)g.Ls);
  int s2 = (s + offset) % g.Ls;
  if (s2 < 0) s2 += g.Ls;
  const long long n2 = (long long)cb * g.N5 + (long long)rhs * g.Ls + s2;
  V a[12], b[12];
  load_spinor<P>(src, g.N, n, a);
  load_spinor<P>(src, g.N, n2, b);
#pragma unroll
  for (int k = 0; k < 6; ++k) a[k] = b[k];
  store_spinor<P>(dst, g.N, n, a);
}

// dst slices [d0, d0 + count) = scale * src slices [s0, s0 + count), every
// 4D site and right-hand side; the two fields may have different Ls
// (g.separate / g.merge along the fifth dimension, mixed_dwf.py:43-48)
template <int P>
__global__ void __launch_bounds__(256) copy_slices_kernel(const Geo gd, void* dst, int d0, const Geo gs, const void* src,
                                                          int s0, int count, double scale) {
  using R = typename SpinorT<P>::R;
  using V = cplx<R>;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long total = (long long)gs.Vh * gs.nrhs * count;
  if (t >= total) return;
  const long long q = t / count;
  const int j = (int)(t - q * count);
  const long long cb = q / gs.nrhs;
  const int rhs = (int)(q - cb * gs.nrhs);
  const long long ns = cb * gs.N5 + (long long)rhs * gs.Ls + s0 + j;
  const long long nd = cb * gd.N5 + (long long)rhs * gd.Ls + d0 + j;
  V v[12];
  load_spinor<P>(src, gs.N, ns, v);
  if (scale != 1.0) {
    const R sc = (R)scale;
#pragma unroll
    for (int k = 0; k < 12; ++k) {
      nrm<R>(v[k]);
      v[k] = scl<R>(sc, v[k]);
      nrm<R>(v[k]);
    }
  }
  store_spinor<P>(dst, gd.N, nd, v);
}

cudaError_t launch_chiral_shift(int P, const Geo& g, const void* src, void* dst, int offset, cudaStream_t st) {
  const int bd = 256;
  const unsigned nb = (unsigned)((g.N + bd - 1) / bd);
  if (P == P64) chiral_shift_kernel<P64><<<nb, bd, 0, st>>>(g, src, dst, offset);
  else if (P == P32) chiral_shift_kernel<P32><<<nb, bd, 0, st>>>(g, src, dst, offset);
  else if (P == P16) chiral_shift_kernel<P16><<<nb, bd, 0, st>>>(g, src, dst, offset);
  else if (P == PDD) chiral_shift_kernel<PDD><<<nb, bd, 0, st>>>(g, src, dst, offset);
  else return cudaErrorInvalidValue;
  return cudaGetLastError();
}

cudaError_t launch_copy_slices(int P, const Geo& gd, void* dst, int d0, const Geo& gs, const void* src, int s0, int count,
                               double scale, cudaStream_t st) {
  const int bd = 256;
  const long long total = (long long)gs.Vh * gs.nrhs * count;
  if (total == 0) return cudaSuccess;
  const unsigned nb = (unsigned)((total + bd - 1) / bd);
  if (P == P64) copy_slices_kernel<P64><<<nb, bd, 0, st>>>(gd, dst, d0, gs, src, s0, count, scale);
  else if (P == P32) copy_slices_kernel<P32><<<nb, bd, 0, st>>>(gd, dst, d0, gs, src, s0, count, scale);
  else if (P == P16) copy_slices_kernel<P16><<<nb, bd, 0, st>>>(gd, dst, d0, gs, src, s0, count, scale);
  else if (P == PDD) copy_slices_kernel<PDD><<<nb, bd, 0, st>>>(gd, dst, d0, gs, src, s0, count, scale);
  else return cudaErrorInvalidValue;
  return cudaGetLastError();
}

}  // namespace gbf
