// gbf_block.cu -- kernels of the block CG over the packed right-hand sides
// of one field (lib/gpt/algorithms/inverter/block_cg.py:36-149): the Gram
// matrix of two block vectors and the block linear combination.
//
// A packed field holds k = n_rhs block vectors; the 5D site n = cb N5 + i5,
// i5 = i Ls + s, belongs to vector i.  Both kernels run one thread per 5D
// site; the k sites (cb, j, s), j = 0..k-1, that a thread needs lie in the
// same block (blockDim is a multiple of N5), which stages them in shared
// memory once.
//
// Bytes per 5D site: Gram reads A and B once; the linear combination reads X
// and Y once and writes out (HBM-bound streaming kernels).
#include "gbf_launch.cuh"

namespace gbf {

// Stage the block's tile of a packed field in shared memory, component-major
// ([24 reals][bd sites]: conflict-free writes, and broadcast reads for the
// threads of one (cb, s) that need the same site).
template <typename R>
__device__ __forceinline__ void tile_store(R* tile, int bd, int t, const cplx<R> (&v)[12]) {
#pragma unroll
  for (int c = 0; c < 12; ++c) {
    tile[(2 * c) * bd + t] = v[c].x;
    tile[(2 * c + 1) * bd + t] = v[c].y;
  }
}
template <typename R>
__device__ __forceinline__ void tile_load(const R* tile, int bd, int t, cplx<R> (&v)[12]) {
#pragma unroll
  for (int c = 0; c < 12; ++c) v[c] = mk<R>(tile[(2 * c) * bd + t], tile[(2 * c + 1) * bd + t]);
}

// conj(a) . b of one site in the arithmetic precision R
template <typename R>
__device__ __forceinline__ void site_dot_r(const cplx<R> (&a)[12], const cplx<R> (&b)[12], R& re, R& im) {
  R r = rzero<R>(), i = rzero<R>();
#pragma unroll
  for (int k = 0; k < 12; ++k) {
    r = fma(a[k].x, b[k].x, r);
    r = fma(a[k].y, b[k].y, r);
    i = fma(a[k].x, b[k].y, i);
    i = fma(-a[k].y, b[k].x, i);
  }
  re = r;
  im = i;
}

// G[i][j] = sum_sites conj(A_i) . B_j, reduced deterministically: per-thread
// partials (over the thread's tiles, in the arithmetic precision, as the
// per-site sums of the other reductions) in shared memory [2k][bd], per-block
// sums in FP64 over the threads of each vector i in a fixed order, then the
// last block sums the [block][k*k] partials in block order.  The B tile of
// the block is staged in shared memory, so each B site is read from memory
// once.
template <int P>
__global__ void __launch_bounds__(256) gram_kernel(const Geo g, const void* A, const void* B, double2* partial,
                                                   unsigned* counter, double2* out) {
  using R = typename SpinorT<P>::R;
  using V = cplx<R>;
  extern __shared__ __align__(16) double sm_d[];  // [2k][bd] partials, then the [24][bd] tile, both R
  const int k = g.nrhs, t = threadIdx.x, bd = blockDim.x;
  R* sm = reinterpret_cast<R*>(sm_d);
  R* tile = sm + 2 * k * bd;
  for (int j = 0; j < 2 * k; ++j) sm[j * bd + t] = rzero<R>();
  const int i = (int)g.fLs.div((unsigned)(t % g.N5));  // vector of this thread (bd is a multiple of N5)
  const long long ntiles = (g.N + bd - 1) / bd;
  for (long long tl = blockIdx.x; tl < ntiles; tl += gridDim.x) {
    const long long n = tl * bd + t;
    const bool active = n < g.N;
    V a[12];
    if (active) {
      V b[12];
      load_spinor<P>(B, g.N, n, b);
#pragma unroll
      for (int c = 0; c < 12; ++c) nrm<R>(b[c]);
      tile_store<R>(tile, bd, t, b);
      load_spinor<P>(A, g.N, n, a);
#pragma unroll
      for (int c = 0; c < 12; ++c) nrm<R>(a[c]);
    }
    __syncthreads();
    if (active) {
      for (int j = 0; j < k; ++j) {
        V b[12];
        tile_load<R>(tile, bd, t + (j - i) * g.Ls, b);
        R re, im;
        site_dot_r<R>(a, b, re, im);
        sm[(2 * j) * bd + t] = sm[(2 * j) * bd + t] + re;
        sm[(2 * j + 1) * bd + t] = sm[(2 * j + 1) * bd + t] + im;
      }
    }
    __syncthreads();
  }
  // entry q = i k + j: threads of vector i are t = S N5 + i Ls + s
  const int S = bd / g.N5;
  for (int q = t; q < k * k; q += bd) {
    const int qi = q / k, qj = q - qi * k;
    double re = 0.0, im = 0.0;
    for (int a = 0; a < S; ++a)
      for (int s = 0; s < g.Ls; ++s) {
        const int tt = a * g.N5 + qi * g.Ls + s;
        re += (double)sm[(2 * qj) * bd + tt];
        im += (double)sm[(2 * qj + 1) * bd + tt];
      }
    partial[(size_t)blockIdx.x * k * k + q] = make_double2(re, im);
  }
  __threadfence();
  __syncthreads();
  __shared__ int s_last;
  if (t == 0) s_last = (atomicAdd(counter, 1u) == gridDim.x - 1);
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  // full warp w sums entries q = w, w + nw, ...: lane l adds blocks l,
  // l + 32, ... in order, then a fixed shuffle tree (deterministic).  bd >= 129
  // (block_size_for), so nw >= 4; a partial last warp takes no part.
  const int lane = t & 31, nw = bd >> 5;
  for (int q = t >> 5; q < k * k && (t >> 5) < nw; q += nw) {
    double re = 0.0, im = 0.0;
    for (unsigned b = lane; b < gridDim.x; b += 32) {
      const double2 v = __ldcg(partial + (size_t)b * k * k + q);
      re += v.x;
      im += v.y;
    }
    re = warp_sum(re);
    im = warp_sum(im);
    if (lane == 0) out[q] = make_double2(re, im);
  }
  if (t == 0) *counter = 0u;
}

// out_i = beta Y_i + sum_j X_j W[j][i]  (W: k x k complex, row j = coefficients
// of X_j).  out may be Y (each thread reads and writes its own site); out must
// not be X.  The X tile of the block is staged in shared memory.
template <int P>
__global__ void __launch_bounds__(256) lincomb_kernel(const Geo g, void* out, const void* Y, double beta, const void* X,
                                                      const double2* W) {
  using R = typename SpinorT<P>::R;
  using V = cplx<R>;
  extern __shared__ __align__(16) double sm[];
  R* tile = reinterpret_cast<R*>(sm);  // [24][bd]
  const int k = g.nrhs, t = threadIdx.x, bd = blockDim.x;
  const int i = (int)g.fLs.div((unsigned)(t % g.N5));
  const long long ntiles = (g.N + bd - 1) / bd;
  for (long long tl = blockIdx.x; tl < ntiles; tl += gridDim.x) {
    const long long n = tl * bd + t;
    const bool active = n < g.N;
    if (active) {
      V x[12];
      load_spinor<P>(X, g.N, n, x);
      tile_store<R>(tile, bd, t, x);
    }
    __syncthreads();
    if (active) {
      V acc[12];
      if (Y) {
        load_spinor<P>(Y, g.N, n, acc);
        const R b = (R)beta;
#pragma unroll
        for (int c = 0; c < 12; ++c) {
          nrm<R>(acc[c]);
          acc[c] = scl<R>(b, acc[c]);
        }
      } else {
#pragma unroll
        for (int c = 0; c < 12; ++c) acc[c] = cz<R>();
      }
      for (int j = 0; j < k; ++j) {
        V x[12];
        tile_load<R>(tile, bd, t + (j - i) * g.Ls, x);
        const double2 w = __ldg(W + j * k + i);
        const V wc = mk<R>((R)w.x, (R)w.y);
#pragma unroll
        for (int c = 0; c < 12; ++c) acc[c] = cmadd<R>(acc[c], wc, x[c]);
      }
      store_spinor<P>(out, g.N, n, acc);
    }
    __syncthreads();
  }
}

// Two block linear combinations in one pass (the pairs of one block-CG half
// iteration):  out1_i = b1 Y1_i + sum_j X1_j W1[j][i]
//              out2_i = b2 Y2_i + c out1_i + sum_j X2_j W2[j][i]
// out1 and out2 may equal Y1 and Y2 (own site only); neither may be X1 or X2.
template <int P>
__global__ void __launch_bounds__(256) lincomb2_kernel(const Geo g, void* out1, const void* Y1, double b1, const void* X1,
                                                       const double2* W1, void* out2, const void* Y2, double b2,
                                                       double c, const void* X2, const double2* W2) {
  using R = typename SpinorT<P>::R;
  using V = cplx<R>;
  extern __shared__ __align__(16) double sm[];
  R* tile1 = reinterpret_cast<R*>(sm);  // [24][bd] each
  const int k = g.nrhs, t = threadIdx.x, bd = blockDim.x;
  R* tile2 = tile1 + 24 * bd;
  const int i = (int)g.fLs.div((unsigned)(t % g.N5));
  const long long ntiles = (g.N + bd - 1) / bd;
  for (long long tl = blockIdx.x; tl < ntiles; tl += gridDim.x) {
    const long long n = tl * bd + t;
    const bool active = n < g.N;
    if (active) {
      V x[12];
      load_spinor<P>(X1, g.N, n, x);
      tile_store<R>(tile1, bd, t, x);
      load_spinor<P>(X2, g.N, n, x);
      tile_store<R>(tile2, bd, t, x);
    }
    __syncthreads();
    if (active) {
      V acc[12];
      if (Y1) {
        load_spinor<P>(Y1, g.N, n, acc);
        const R b = (R)b1;
#pragma unroll
        for (int q = 0; q < 12; ++q) {
          nrm<R>(acc[q]);
          acc[q] = scl<R>(b, acc[q]);
        }
      } else {
#pragma unroll
        for (int q = 0; q < 12; ++q) acc[q] = cz<R>();
      }
      for (int j = 0; j < k; ++j) {
        V x[12];
        tile_load<R>(tile1, bd, t + (j - i) * g.Ls, x);
        const double2 w = __ldg(W1 + j * k + i);
        const V wc = mk<R>((R)w.x, (R)w.y);
#pragma unroll
        for (int q = 0; q < 12; ++q) acc[q] = cmadd<R>(acc[q], wc, x[q]);
      }
#pragma unroll
      for (int q = 0; q < 12; ++q) nrm<R>(acc[q]);
      store_spinor<P>(out1, g.N, n, acc);
      V acc2[12];
      const R cc = (R)c;
      if (Y2) {
        load_spinor<P>(Y2, g.N, n, acc2);
        const R b = (R)b2;
#pragma unroll
        for (int q = 0; q < 12; ++q) {
          nrm<R>(acc2[q]);
          acc2[q] = mk<R>(fma(cc, acc[q].x, b * acc2[q].x), fma(cc, acc[q].y, b * acc2[q].y));
        }
      } else {
#pragma unroll
        for (int q = 0; q < 12; ++q) acc2[q] = scl<R>(cc, acc[q]);
      }
      for (int j = 0; j < k; ++j) {
        V x[12];
        tile_load<R>(tile2, bd, t + (j - i) * g.Ls, x);
        const double2 w = __ldg(W2 + j * k + i);
        const V wc = mk<R>((R)w.x, (R)w.y);
#pragma unroll
        for (int q = 0; q < 12; ++q) acc2[q] = cmadd<R>(acc2[q], wc, x[q]);
      }
      store_spinor<P>(out2, g.N, n, acc2);
    }
    __syncthreads();
  }
}

static size_t tile_bytes(int P, int bd) { return (size_t)24 * bd * ((P == P64 || P == PDD) ? 8 : 4); }

cudaError_t launch_lincomb2(int P, const Geo& g, void* out1, const void* Y1, double b1, const void* X1, const double2* W1,
                            void* out2, const void* Y2, double b2, double c, const void* X2, const double2* W2,
                            cudaStream_t st) {
  const int bd = block_size_for(g.N5, LOC_NONE);
  if (bd <= 0 || out1 == X1 || out1 == X2 || out2 == X1 || out2 == X2 || out1 == out2) return cudaErrorInvalidValue;
  const void* k = P == P64 ? (const void*)lincomb2_kernel<P64>
                : P == P32 ? (const void*)lincomb2_kernel<P32>
                : P == P16 ? (const void*)lincomb2_kernel<P16>
                : P == PDD ? (const void*)lincomb2_kernel<PDD> : nullptr;
  if (!k) return cudaErrorInvalidValue;
  const size_t sm = 2 * tile_bytes(P, bd);
  const long long nb = reduce_grid((g.N + bd - 1) / bd, g.nrhs, resident_blocks(k, bd, sm));
#define GBF_L2(PP) lincomb2_kernel<PP><<<(unsigned)nb, bd, sm, st>>>(g, out1, Y1, b1, X1, W1, out2, Y2, b2, c, X2, W2)
  if (P == P64) GBF_L2(P64);
  else if (P == P32) GBF_L2(P32);
  else if (P == P16) GBF_L2(P16);
  else GBF_L2(PDD);
#undef GBF_L2
  return cudaGetLastError();
}

template <int P>
static cudaError_t launch_gram_t(const Geo& g, const void* A, const void* B, double2* partial, long long max_blocks,
                                 unsigned* counter, double2* out, int bd, cudaStream_t st) {
  const size_t sm = (size_t)2 * g.nrhs * bd * ((P == P64 || P == PDD) ? 8 : 4) + tile_bytes(P, bd);
  auto k = gram_kernel<P>;
  const int res = resident_blocks((const void*)k, bd, sm);
  long long nb = reduce_grid((g.N + bd - 1) / bd, g.nrhs, res);
  if (nb > max_blocks) nb = max_blocks;
  k<<<(unsigned)nb, bd, sm, st>>>(g, A, B, partial, counter, out);
  return cudaGetLastError();
}

cudaError_t launch_gram(int P, const Geo& g, const void* A, const void* B, double2* partial, long long max_blocks,
                        unsigned* counter, double2* out, cudaStream_t st) {
  const int bd = block_size_for(g.N5, LOC_NONE);
  if (bd <= 0 || g.nrhs > kMaxRhs) return cudaErrorInvalidValue;
  if (P == P64) return launch_gram_t<P64>(g, A, B, partial, max_blocks, counter, out, bd, st);
  if (P == P32) return launch_gram_t<P32>(g, A, B, partial, max_blocks, counter, out, bd, st);
  if (P == P16) return launch_gram_t<P16>(g, A, B, partial, max_blocks, counter, out, bd, st);
  if (P == PDD) return launch_gram_t<PDD>(g, A, B, partial, max_blocks, counter, out, bd, st);
  return cudaErrorInvalidValue;
}

cudaError_t launch_lincomb(int P, const Geo& g, void* out, const void* Y, double beta, const void* X, const double2* W,
                           cudaStream_t st) {
  const int bd = block_size_for(g.N5, LOC_NONE);
  if (bd <= 0 || out == X) return cudaErrorInvalidValue;
  const void* k = P == P64 ? (const void*)lincomb_kernel<P64>
                : P == P32 ? (const void*)lincomb_kernel<P32>
                : P == P16 ? (const void*)lincomb_kernel<P16>
                : P == PDD ? (const void*)lincomb_kernel<PDD> : nullptr;
  if (!k) return cudaErrorInvalidValue;
  const size_t sm = tile_bytes(P, bd);
  const long long nb = reduce_grid((g.N + bd - 1) / bd, g.nrhs, resident_blocks(k, bd, sm));
  if (P == P64) lincomb_kernel<P64><<<(unsigned)nb, bd, sm, st>>>(g, out, Y, beta, X, W);
  else if (P == P32) lincomb_kernel<P32><<<(unsigned)nb, bd, sm, st>>>(g, out, Y, beta, X, W);
  else if (P == P16) lincomb_kernel<P16><<<(unsigned)nb, bd, sm, st>>>(g, out, Y, beta, X, W);
  else lincomb_kernel<PDD><<<(unsigned)nb, bd, sm, st>>>(g, out, Y, beta, X, W);
  return cudaGetLastError();
}

}  // namespace gbf

namespace gbf {

// Multi-shift CG vector update for the active shifts j (one pass over r):
//   x_j += a_j p_j ;  p_j = b_j p_j + g_j r
// (lib/gpt/algorithms/inverter/multi_shift_cg.py:45-47).  bytes/site: r once,
// x_j and p_j read and written per active shift.
template <int P>
__global__ void __launch_bounds__(256) multishift_kernel(const Geo g, const MultiShiftArgs a) {
  using R = typename SpinorT<P>::R;
  using V = cplx<R>;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x; n < g.N; n += stride) {
    V r[12];
    load_spinor<P>(a.r, g.N, n, r);
    for (int j = 0; j < a.n; ++j) {
      V x[12], p[12];
      load_spinor<P>(a.x[j], g.N, n, x);
      load_spinor<P>(a.p[j], g.N, n, p);
      const R aj = (R)a.a[j], bj = (R)a.b[j], gj = (R)a.g[j];
#pragma unroll
      for (int k = 0; k < 12; ++k) {
        x[k] = mk<R>(fma(aj, p[k].x, x[k].x), fma(aj, p[k].y, x[k].y));
        p[k] = mk<R>(fma(bj, p[k].x, gj * r[k].x), fma(bj, p[k].y, gj * r[k].y));
      }
      store_spinor<P>(a.x[j], g.N, n, x);
      store_spinor<P>(a.p[j], g.N, n, p);
    }
  }
}

cudaError_t launch_multishift(int P, const Geo& g, const MultiShiftArgs& a, cudaStream_t st) {
  if (a.n < 0 || a.n > kMaxShifts) return cudaErrorInvalidValue;
  if (a.n == 0) return cudaSuccess;
  const int bd = 256;
  const void* k = P == P64 ? (const void*)multishift_kernel<P64>
                : P == P32 ? (const void*)multishift_kernel<P32>
                : P == P16 ? (const void*)multishift_kernel<P16>
                : P == PDD ? (const void*)multishift_kernel<PDD> : nullptr;
  if (!k) return cudaErrorInvalidValue;
  const long long nb = reduce_grid((g.N + bd - 1) / bd, 1, resident_blocks(k, bd, 0));
  if (P == P64) multishift_kernel<P64><<<(unsigned)nb, bd, 0, st>>>(g, a);
  else if (P == P32) multishift_kernel<P32><<<(unsigned)nb, bd, 0, st>>>(g, a);
  else if (P == P16) multishift_kernel<P16><<<(unsigned)nb, bd, 0, st>>>(g, a);
  else multishift_kernel<PDD><<<(unsigned)nb, bd, 0, st>>>(g, a);
  return cudaGetLastError();
}

}  // namespace gbf

namespace gbf {

// ---------------------------------------------------------------------------
// Mode representation A = sum_n left_n right_n^+ f(eval_n)
// (lib/gpt/algorithms/modes/matrix.py:31-56: rank_inner_product of a block of
// the right modes with the source, then the linear combination of the left
// modes), used by the deflation inverter (lib/gpt/algorithms/inverter/
// deflate.py).  Every mode is a separate field; both kernels stream a block
// of up to kModeBlock of them through one pass over the sites.
// ---------------------------------------------------------------------------

// out[j] = sum_sites conj(v_j) . src: products and the per-thread sums over
// the thread's sites in the arithmetic precision (a thread handles a few
// sites: the grid is one wave of resident blocks), FP64 block sums in a fixed
// order, the last block sums the [block][j] partials in block order
// (deterministic).  NM = kModeBlock for full blocks (no predication), 0 for
// a run-time count a.n < kModeBlock.  bytes/site: src once + every v_j once.
template <int P, int NM>
__global__ void __launch_bounds__(256) mode_dot_kernel(const Geo g, const ModeDotArgs a) {
  using R = typename SpinorT<P>::R;
  using V = cplx<R>;
  __shared__ double sm[64];
  const int t = threadIdx.x;
  const int nm = NM ? NM : a.n;
  R re[kModeBlock], im[kModeBlock];
#pragma unroll
  for (int j = 0; j < kModeBlock; ++j) re[j] = im[j] = rzero<R>();
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long n = (long long)blockIdx.x * blockDim.x + t; n < g.N; n += stride) {
    V s[12];
    load_spinor<P>(a.src, g.N, n, s);
#pragma unroll
    for (int k = 0; k < 12; ++k) nrm<R>(s[k]);
#pragma unroll
    for (int j = 0; j < kModeBlock; ++j) {
      if (NM || j < nm) {
        V v[12];
        load_spinor<P>(a.v[j], g.N, n, v);
#pragma unroll
        for (int k = 0; k < 12; ++k) nrm<R>(v[k]);
        R dr, di;
        site_dot_r<R>(v, s, dr, di);
        re[j] = re[j] + dr;
        im[j] = im[j] + di;
      }
    }
  }
#pragma unroll
  for (int j = 0; j < kModeBlock; ++j) {
    if (NM || j < nm) {
      const double2 b = block_sum_shfl((double)re[j], (double)im[j], sm);
      if (t == 0) a.partial[(size_t)blockIdx.x * nm + j] = b;
    }
  }
  __threadfence();
  __syncthreads();
  __shared__ int s_last;
  if (t == 0) s_last = (atomicAdd(a.counter, 1u) == gridDim.x - 1);
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  // warp j sums mode j: lane l adds blocks l, l + 32, ... in order, then a
  // fixed shuffle tree (deterministic); blockDim = 256 gives 8 warps
  const int lane = t & 31, w = t >> 5;
  if (w < nm) {
    double sr = 0.0, si = 0.0;
    for (unsigned b = lane; b < gridDim.x; b += 32) {
      const double2 v = __ldcg(a.partial + (size_t)b * nm + w);
      sr += v.x;
      si += v.y;
    }
    sr = warp_sum(sr);
    si = warp_sum(si);
    if (lane == 0) a.out[w] = make_double2(sr, si);
  }
  if (t == 0) *a.counter = 0u;
}

// out = (accumulate ? out : 0) + sum_j w_j v_j, complex weights rounded to
// the arithmetic precision once per thread.  bytes/site: every v_j once, out
// written (+ read).
template <int P, int NM>
__global__ void __launch_bounds__(256) mode_axpy_kernel(const Geo g, const ModeAxpyArgs a) {
  using R = typename SpinorT<P>::R;
  using V = cplx<R>;
  const int nm = NM ? NM : a.n;
  V w[kModeBlock];
#pragma unroll
  for (int j = 0; j < kModeBlock; ++j) w[j] = mk<R>((R)a.w[j].x, (R)a.w[j].y);
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x; n < g.N; n += stride) {
    V o[12];
    if (a.accumulate) {
      load_spinor<P>(a.out, g.N, n, o);
    } else {
#pragma unroll
      for (int k = 0; k < 12; ++k) o[k] = cz<R>();
    }
#pragma unroll
    for (int j = 0; j < kModeBlock; ++j) {
      if (NM || j < nm) {
        V v[12];
        load_spinor<P>(a.v[j], g.N, n, v);
#pragma unroll
        for (int k = 0; k < 12; ++k) {
          nrm<R>(v[k]);
          o[k] = cmadd<R>(o[k], w[j], v[k]);
          nrm<R>(o[k]);
        }
      }
    }
    store_spinor<P>(a.out, g.N, n, o);
  }
}

template <int P, int NM>
static cudaError_t launch_mode_dot_t(const Geo& g, const ModeDotArgs& a, long long max_partials, cudaStream_t st) {
  auto k = mode_dot_kernel<P, NM>;
  const int bd = 256;
  long long nb = reduce_grid((g.N + bd - 1) / bd, 1, resident_blocks((const void*)k, bd, 0));
  if (nb * a.n > max_partials) nb = max_partials / a.n;
  if (nb < 1) return cudaErrorInvalidValue;
  k<<<(unsigned)nb, bd, 0, st>>>(g, a);
  return cudaGetLastError();
}

template <int P>
static cudaError_t launch_mode_dot_p(const Geo& g, const ModeDotArgs& a, long long max_partials, cudaStream_t st) {
  return a.n == kModeBlock ? launch_mode_dot_t<P, kModeBlock>(g, a, max_partials, st)
                           : launch_mode_dot_t<P, 0>(g, a, max_partials, st);
}

cudaError_t launch_mode_dot(int P, const Geo& g, const ModeDotArgs& a, long long max_partials, cudaStream_t st) {
  if (a.n < 1 || a.n > kModeBlock) return cudaErrorInvalidValue;
  if (P == P64) return launch_mode_dot_p<P64>(g, a, max_partials, st);
  if (P == P32) return launch_mode_dot_p<P32>(g, a, max_partials, st);
  if (P == P16) return launch_mode_dot_p<P16>(g, a, max_partials, st);
  if (P == PDD) return launch_mode_dot_p<PDD>(g, a, max_partials, st);
  return cudaErrorInvalidValue;
}

template <int P, int NM>
static cudaError_t launch_mode_axpy_t(const Geo& g, const ModeAxpyArgs& a, cudaStream_t st) {
  auto k = mode_axpy_kernel<P, NM>;
  const int bd = 256;
  const long long nb = reduce_grid((g.N + bd - 1) / bd, 1, resident_blocks((const void*)k, bd, 0));
  k<<<(unsigned)nb, bd, 0, st>>>(g, a);
  return cudaGetLastError();
}

template <int P>
static cudaError_t launch_mode_axpy_p(const Geo& g, const ModeAxpyArgs& a, cudaStream_t st) {
  return a.n == kModeBlock ? launch_mode_axpy_t<P, kModeBlock>(g, a, st) : launch_mode_axpy_t<P, 0>(g, a, st);
}

cudaError_t launch_mode_axpy(int P, const Geo& g, const ModeAxpyArgs& a, cudaStream_t st) {
  if (a.n < 0 || a.n > kModeBlock) return cudaErrorInvalidValue;
  if (P == P64) return launch_mode_axpy_p<P64>(g, a, st);
  if (P == P32) return launch_mode_axpy_p<P32>(g, a, st);
  if (P == P16) return launch_mode_axpy_p<P16>(g, a, st);
  if (P == PDD) return launch_mode_axpy_p<PDD>(g, a, st);
  return cudaErrorInvalidValue;
}

}  // namespace gbf
