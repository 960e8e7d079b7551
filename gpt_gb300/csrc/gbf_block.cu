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
// FP32: two complex components per 16-byte word ([6][bd] float4), read back
// with 6 vector loads instead of 24 scalar ones
template <>
__device__ __forceinline__ void tile_store<float>(float* tile, int bd, int t, const float2 (&v)[12]) {
  float4* q = reinterpret_cast<float4*>(tile);
#pragma unroll
  for (int c = 0; c < 6; ++c) q[c * bd + t] = make_float4(v[2 * c].x, v[2 * c].y, v[2 * c + 1].x, v[2 * c + 1].y);
}
template <>
__device__ __forceinline__ void tile_load<float>(const float* tile, int bd, int t, float2 (&v)[12]) {
  const float4* q = reinterpret_cast<const float4*>(tile);
#pragma unroll
  for (int c = 0; c < 6; ++c) {
    const float4 w = q[c * bd + t];
    v[2 * c] = make_float2(w.x, w.y);
    v[2 * c + 1] = make_float2(w.z, w.w);
  }
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
__global__ void __launch_bounds__(256) gram_kernel(const Geo g, const void* A, const void* B, double2* partial) {
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
}

// The same Gram matrix for FP32 / FP16 fields, register-tiled.  A tile of
// bd 5D sites (S 4D sites x Ls x k vectors) is staged in shared memory as
// [component c][row r = (site, s)][vector i] for A and B.  Threads form
// groups of 16, a 4 x 4 grid: thread (ti, tj) owns the T x T block of
// entries i in [T ti, T ti + T), j in [T tj, T tj + T) (T = ceil(k / 4)) and,
// for the (c, r) pairs of its group, reads T values of A and T of B and does
// 4 T^2 fused multiply-adds -- each shared-memory value feeds 2 T complex
// products instead of one.  Per tile the products are summed in FP32, then
// added to FP64 accumulators; the block sums its groups in a fixed order and
// the last block the [block][k*k] partials in block order (deterministic).
template <int P, int T>
__global__ void __launch_bounds__(256) gram_tiled_kernel(const Geo g, const void* A, const void* B, double2* partial) {
  using V = float2;
  extern __shared__ __align__(16) double sm_d[];
  const int k = g.nrhs, t = threadIdx.x, bd = blockDim.x;
  const int Ls = g.Ls, N5 = g.N5, R = (bd / N5) * Ls;  // rows per tile
  V* sA = reinterpret_cast<V*>(sm_d);                  // [12][R][k]
  V* sB = sA + 12 * R * k;
  const int grp = t >> 4, l16 = t & 15, ti = l16 >> 2, tj = l16 & 3, G = bd >> 4;
  // staging position of this thread's site: n_local = jsite N5 + iv Ls + s
  const int jsite = t / N5, i5 = t - jsite * N5, iv = i5 / Ls, s = i5 - iv * Ls;
  const int row = jsite * Ls + s;
  double dre[T][T], dim[T][T];
#pragma unroll
  for (int x = 0; x < T; ++x)
#pragma unroll
    for (int y = 0; y < T; ++y) dre[x][y] = dim[x][y] = 0.0;
  const long long ntiles = (g.N + bd - 1) / bd;
  for (long long tl = blockIdx.x; tl < ntiles; tl += gridDim.x) {
    const long long n = tl * bd + t;
    V a[12], b[12];
    if (n < g.N) {
      load_spinor<P>(A, g.N, n, a);
      load_spinor<P>(B, g.N, n, b);
    } else {
#pragma unroll
      for (int c = 0; c < 12; ++c) a[c] = b[c] = make_float2(0.f, 0.f);
    }
#pragma unroll
    for (int c = 0; c < 12; ++c) {
      sA[(c * R + row) * k + iv] = a[c];
      sB[(c * R + row) * k + iv] = b[c];
    }
    __syncthreads();
    float fre[T][T], fim[T][T];
#pragma unroll
    for (int x = 0; x < T; ++x)
#pragma unroll
      for (int y = 0; y < T; ++y) fre[x][y] = fim[x][y] = 0.f;
    for (int pq = grp; pq < 12 * R; pq += G) {
      const V* pa = sA + pq * k + T * ti;  // pq = c R + r
      const V* pb = sB + pq * k + T * tj;
      V av[T], bv[T];
#pragma unroll
      for (int x = 0; x < T; ++x) {
        av[x] = (T * ti + x < k) ? pa[x] : make_float2(0.f, 0.f);
        bv[x] = (T * tj + x < k) ? pb[x] : make_float2(0.f, 0.f);
      }
#pragma unroll
      for (int x = 0; x < T; ++x)
#pragma unroll
        for (int y = 0; y < T; ++y) {  // conj(a) b
          fre[x][y] = fmaf(av[x].x, bv[y].x, fre[x][y]);
          fre[x][y] = fmaf(av[x].y, bv[y].y, fre[x][y]);
          fim[x][y] = fmaf(av[x].x, bv[y].y, fim[x][y]);
          fim[x][y] = fmaf(-av[x].y, bv[y].x, fim[x][y]);
        }
    }
#pragma unroll
    for (int x = 0; x < T; ++x)
#pragma unroll
      for (int y = 0; y < T; ++y) {
        dre[x][y] += (double)fre[x][y];
        dim[x][y] += (double)fim[x][y];
      }
    __syncthreads();
  }
  // block sum over the groups, fixed order ([group][k*k] doubles in the tile region)
  double2* red = reinterpret_cast<double2*>(sm_d);
#pragma unroll
  for (int x = 0; x < T; ++x)
#pragma unroll
    for (int y = 0; y < T; ++y) {
      const int i = T * ti + x, j = T * tj + y;
      if (i < k && j < k) red[grp * k * k + i * k + j] = make_double2(dre[x][y], dim[x][y]);
    }
  __syncthreads();
  for (int q = t; q < k * k; q += bd) {
    double re = 0.0, im = 0.0;
    for (int gg = 0; gg < G; ++gg) {
      const double2 v = red[gg * k * k + q];
      re += v.x;
      im += v.y;
    }
    partial[(size_t)blockIdx.x * k * k + q] = make_double2(re, im);
  }
}

// The FP32 Gram with the tiles double-buffered: while a tile is reduced the
// next one streams into the other buffer with cp.async 16-byte copies (no
// registers held for staging, the loads of one tile overlap the arithmetic of
// the previous one).  Layout per buffer and field: [component pair cp][row r]
// [vector i] of float4 (components 2 cp and 2 cp + 1 of one site, exactly
// one 16-byte word of the field's FP32 layout); each (cp, r) pair gives
// 8 T^2 fused multiply-adds for 2 T vector loads.  Summation as in
// gram_tiled_kernel (FP32 within a tile, FP64 across tiles, fixed orders).
__device__ __forceinline__ void cpa16(void* dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((unsigned)__cvta_generic_to_shared(dst)), "l"(src)
               : "memory");
}
__device__ __forceinline__ void cpa_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cpa_wait1() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }
__device__ __forceinline__ void cpa_wait0() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

template <int T>
__global__ void __launch_bounds__(256) gram_async_kernel(const Geo g, const void* A, const void* B, double2* partial) {
  extern __shared__ __align__(16) double sm_d[];
  const int k = g.nrhs, t = threadIdx.x, bd = blockDim.x;
  const int Ls = g.Ls, N5 = g.N5, R = (bd / N5) * Ls;
  float4* buf = reinterpret_cast<float4*>(sm_d);  // [2 buffers][A, B][6][R][k]
  const int fld = 6 * R * k;                      // float4 per field and buffer (= 6 bd)
  const int grp = t >> 4, l16 = t & 15, ti = l16 >> 2, tj = l16 & 3, G = bd >> 4;
  const int jsite = t / N5, i5 = t - jsite * N5, iv = i5 / Ls, s = i5 - iv * Ls;
  const int row = jsite * Ls + s;
  const float4* gA = reinterpret_cast<const float4*>(A);
  const float4* gB = reinterpret_cast<const float4*>(B);
  const unsigned N = (unsigned)g.N;
  double dre[T][T], dim[T][T];
#pragma unroll
  for (int x = 0; x < T; ++x)
#pragma unroll
    for (int y = 0; y < T; ++y) dre[x][y] = dim[x][y] = 0.0;
  const long long ntiles = (g.N + bd - 1) / bd;
  // stage tile tl into buffer b (absent sites: zeros written by the thread)
  auto stage = [&](long long tl, int b) {
    const long long n = tl * bd + t;
    float4* dA = buf + (size_t)b * 2 * fld;
    float4* dB = dA + fld;
#pragma unroll
    for (int cp = 0; cp < 6; ++cp) {
      const int o = (cp * R + row) * k + iv;
      if (n < g.N) {
        cpa16(dA + o, gA + ((unsigned)n + (unsigned)cp * N));
        cpa16(dB + o, gB + ((unsigned)n + (unsigned)cp * N));
      } else {
        dA[o] = make_float4(0.f, 0.f, 0.f, 0.f);
        dB[o] = make_float4(0.f, 0.f, 0.f, 0.f);
      }
    }
    cpa_commit();
  };
  long long tl = blockIdx.x;
  int b = 0;
  if (tl < ntiles) stage(tl, 0);
  for (; tl < ntiles; tl += gridDim.x, b ^= 1) {
    const long long nxt = tl + gridDim.x;
    if (nxt < ntiles) {
      stage(nxt, b ^ 1);
      cpa_wait1();  // this thread's copies of the current tile have landed
    } else {
      cpa_wait0();
    }
    __syncthreads();  // every thread's copies of the current tile
    const float4* sA = buf + (size_t)b * 2 * fld;
    const float4* sB = sA + fld;
    float fre[T][T], fim[T][T];
#pragma unroll
    for (int x = 0; x < T; ++x)
#pragma unroll
      for (int y = 0; y < T; ++y) fre[x][y] = fim[x][y] = 0.f;
    for (int pq = grp; pq < 6 * R; pq += G) {  // pq = cp R + r
      const float4* pa = sA + pq * k + T * ti;
      const float4* pb = sB + pq * k + T * tj;
      float4 av[T], bv[T];
#pragma unroll
      for (int x = 0; x < T; ++x) {
        av[x] = (T * ti + x < k) ? pa[x] : make_float4(0.f, 0.f, 0.f, 0.f);
        bv[x] = (T * tj + x < k) ? pb[x] : make_float4(0.f, 0.f, 0.f, 0.f);
      }
#pragma unroll
      for (int x = 0; x < T; ++x)
#pragma unroll
        for (int y = 0; y < T; ++y) {  // conj(a) b over the two components
          fre[x][y] = fmaf(av[x].x, bv[y].x, fre[x][y]);
          fre[x][y] = fmaf(av[x].y, bv[y].y, fre[x][y]);
          fre[x][y] = fmaf(av[x].z, bv[y].z, fre[x][y]);
          fre[x][y] = fmaf(av[x].w, bv[y].w, fre[x][y]);
          fim[x][y] = fmaf(av[x].x, bv[y].y, fim[x][y]);
          fim[x][y] = fmaf(-av[x].y, bv[y].x, fim[x][y]);
          fim[x][y] = fmaf(av[x].z, bv[y].w, fim[x][y]);
          fim[x][y] = fmaf(-av[x].w, bv[y].z, fim[x][y]);
        }
    }
#pragma unroll
    for (int x = 0; x < T; ++x)
#pragma unroll
      for (int y = 0; y < T; ++y) {
        dre[x][y] += (double)fre[x][y];
        dim[x][y] += (double)fim[x][y];
      }
    __syncthreads();  // the buffer is refilled two tiles on
  }
  double2* red = reinterpret_cast<double2*>(sm_d);
#pragma unroll
  for (int x = 0; x < T; ++x)
#pragma unroll
    for (int y = 0; y < T; ++y) {
      const int i = T * ti + x, j = T * tj + y;
      if (i < k && j < k) red[grp * k * k + i * k + j] = make_double2(dre[x][y], dim[x][y]);
    }
  __syncthreads();
  for (int q = t; q < k * k; q += bd) {
    double re = 0.0, im = 0.0;
    for (int gg = 0; gg < G; ++gg) {
      const double2 v = red[gg * k * k + q];
      re += v.x;
      im += v.y;
    }
    partial[(size_t)blockIdx.x * k * k + q] = make_double2(re, im);
  }
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

// lincomb2_kernel for FP32 with the X1 and X2 tiles double-buffered by
// cp.async (layout [component pair][thread] float4, one 16-byte word per
// copy): the next tile's copies overlap this tile's combinations.
__global__ void __launch_bounds__(256) lincomb2_async_kernel(const Geo g, void* out1, const void* Y1, double b1,
                                                             const void* X1, const double2* W1, void* out2,
                                                             const void* Y2, double b2, double c, const void* X2,
                                                             const double2* W2) {
  using V = float2;
  extern __shared__ __align__(16) double sm[];
  float4* buf = reinterpret_cast<float4*>(sm);  // [2 buffers][X1, X2][6][bd]
  const int k = g.nrhs, t = threadIdx.x, bd = blockDim.x;
  const int i = (int)g.fLs.div((unsigned)(t % g.N5));
  const unsigned N = (unsigned)g.N;
  const float4* gx1 = reinterpret_cast<const float4*>(X1);
  const float4* gx2 = reinterpret_cast<const float4*>(X2);
  const long long ntiles = (g.N + bd - 1) / bd;
  auto stage = [&](long long tl, int b) {
    const long long n = tl * bd + t;
    float4* d1 = buf + (size_t)b * 12 * bd;
    float4* d2 = d1 + 6 * bd;
    if (n < g.N) {
#pragma unroll
      for (int cp = 0; cp < 6; ++cp) {
        cpa16(d1 + cp * bd + t, gx1 + ((unsigned)n + (unsigned)cp * N));
        cpa16(d2 + cp * bd + t, gx2 + ((unsigned)n + (unsigned)cp * N));
      }
    }
    cpa_commit();
  };
  long long tl = blockIdx.x;
  int b = 0;
  if (tl < ntiles) stage(tl, 0);
  for (; tl < ntiles; tl += gridDim.x, b ^= 1) {
    const long long nxt = tl + gridDim.x;
    if (nxt < ntiles) stage(nxt, b ^ 1);
    const long long n = tl * bd + t;
    // this site's own Y1 and Y2, loaded before the wait so that their latency
    // overlaps it
    V acc[12], y2v[12];
    if (n < g.N) {
      if (Y1) load_spinor<P32>(Y1, g.N, n, acc);
      if (Y2) load_spinor<P32>(Y2, g.N, n, y2v);
    }
    if (nxt < ntiles) cpa_wait1();
    else cpa_wait0();
    __syncthreads();
    if (n < g.N) {
      const float* tile1 = reinterpret_cast<const float*>(buf + (size_t)b * 12 * bd);
      const float* tile2 = tile1 + 24 * bd;
      if (Y1) {
        const float bb = (float)b1;
#pragma unroll
        for (int q = 0; q < 12; ++q) acc[q] = scl<float>(bb, acc[q]);
      } else {
#pragma unroll
        for (int q = 0; q < 12; ++q) acc[q] = cz<float>();
      }
      for (int j = 0; j < k; ++j) {
        V x[12];
        tile_load<float>(tile1, bd, t + (j - i) * g.Ls, x);
        const double2 w = __ldg(W1 + j * k + i);
        const V wc = make_float2((float)w.x, (float)w.y);
#pragma unroll
        for (int q = 0; q < 12; ++q) acc[q] = cmadd<float>(acc[q], wc, x[q]);
      }
      store_spinor<P32>(out1, g.N, n, acc);
      V acc2[12];
      const float cc = (float)c;
      if (Y2) {
        const float bb = (float)b2;
#pragma unroll
        for (int q = 0; q < 12; ++q) acc2[q] = make_float2(fmaf(cc, acc[q].x, bb * y2v[q].x), fmaf(cc, acc[q].y, bb * y2v[q].y));
      } else {
#pragma unroll
        for (int q = 0; q < 12; ++q) acc2[q] = scl<float>(cc, acc[q]);
      }
      for (int j = 0; j < k; ++j) {
        V x[12];
        tile_load<float>(tile2, bd, t + (j - i) * g.Ls, x);
        const double2 w = __ldg(W2 + j * k + i);
        const V wc = make_float2((float)w.x, (float)w.y);
#pragma unroll
        for (int q = 0; q < 12; ++q) acc2[q] = cmadd<float>(acc2[q], wc, x[q]);
      }
      store_spinor<P32>(out2, g.N, n, acc2);
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
  if (P == P32) {
    const size_t sma = (size_t)2 * 12 * bd * sizeof(float4);
    const long long nba =
        reduce_grid((g.N + bd - 1) / bd, g.nrhs, resident_blocks((const void*)lincomb2_async_kernel, bd, sma));
    lincomb2_async_kernel<<<(unsigned)nba, bd, sma, st>>>(g, out1, Y1, b1, X1, W1, out2, Y2, b2, c, X2, W2);
    return cudaGetLastError();
  }
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

// Sum of the [block][k*k] Gram partials: one block of 256 threads per entry
// q, its threads take blocks b = t, t + 256, ... in order and a fixed
// shuffle tree adds them (deterministic; many blocks share the work instead
// of one last block walking every entry).
__global__ void __launch_bounds__(256) gram_finalize_kernel(const double2* partial, int nblocks, int kk, double2* out) {
  __shared__ double sm[64];
  const int q = blockIdx.x, t = threadIdx.x;
  double re = 0.0, im = 0.0;
  for (int b = t; b < nblocks; b += blockDim.x) {
    const double2 v = partial[(size_t)b * kk + q];
    re += v.x;
    im += v.y;
  }
  const double2 r = block_sum_shfl(re, im, sm);
  if (t == 0) out[q] = r;
}

template <int P>
static cudaError_t launch_gram_t(const Geo& g, const void* A, const void* B, double2* partial, long long max_blocks,
                                 unsigned* counter, double2* out, int bd, cudaStream_t st) {
  const size_t sm = (size_t)2 * g.nrhs * bd * ((P == P64 || P == PDD) ? 8 : 4) + tile_bytes(P, bd);
  auto k = gram_kernel<P>;
  const int res = resident_blocks((const void*)k, bd, sm);
  long long nb = reduce_grid((g.N + bd - 1) / bd, g.nrhs, res);
  if (nb > max_blocks) nb = max_blocks;
  (void)counter;
  k<<<(unsigned)nb, bd, sm, st>>>(g, A, B, partial);
  gram_finalize_kernel<<<(unsigned)(g.nrhs * g.nrhs), 256, 0, st>>>(partial, (int)nb, g.nrhs * g.nrhs, out);
  return cudaGetLastError();
}


template <int P, int T>
static cudaError_t launch_gram_tiled(const Geo& g, const void* A, const void* B, double2* partial, long long max_blocks,
                                     unsigned* counter, double2* out, int bd, cudaStream_t st) {
  // staged tiles: 2 x 12 x bd complex floats; the group sums reuse them
  size_t sm = (size_t)2 * 12 * bd * sizeof(float2);
  const size_t red = (size_t)(bd / 16) * g.nrhs * g.nrhs * sizeof(double2);
  if (red > sm) sm = red;
  auto k = gram_tiled_kernel<P, T>;
  const int res = resident_blocks((const void*)k, bd, sm);
  long long nb = reduce_grid((g.N + bd - 1) / bd, 1, res);
  if (nb > max_blocks) nb = max_blocks;
  (void)counter;
  k<<<(unsigned)nb, bd, sm, st>>>(g, A, B, partial);
  gram_finalize_kernel<<<(unsigned)(g.nrhs * g.nrhs), 256, 0, st>>>(partial, (int)nb, g.nrhs * g.nrhs, out);
  return cudaGetLastError();
}

template <int T>
static cudaError_t launch_gram_async(const Geo& g, const void* A, const void* B, double2* partial, long long max_blocks,
                                     unsigned* counter, double2* out, int bd, cudaStream_t st) {
  // two buffers of the A and B tiles (2 x 2 x 6 bd float4); the group sums reuse them
  size_t sm = (size_t)2 * 2 * 6 * bd * sizeof(float4);
  const size_t red = (size_t)(bd / 16) * g.nrhs * g.nrhs * sizeof(double2);
  if (red > sm) sm = red;
  auto k = gram_async_kernel<T>;
  const int res = resident_blocks((const void*)k, bd, sm);
  long long nb = reduce_grid((g.N + bd - 1) / bd, 1, res);
  if (nb > max_blocks) nb = max_blocks;
  (void)counter;
  k<<<(unsigned)nb, bd, sm, st>>>(g, A, B, partial);
  gram_finalize_kernel<<<(unsigned)(g.nrhs * g.nrhs), 256, 0, st>>>(partial, (int)nb, g.nrhs * g.nrhs, out);
  return cudaGetLastError();
}

template <int P>
static cudaError_t launch_gram_tiled_k(const Geo& g, const void* A, const void* B, double2* partial, long long max_blocks,
                                       unsigned* counter, double2* out, int bd, cudaStream_t st) {
  const int T = (g.nrhs + 3) / 4;
  if (T == 1) return launch_gram_tiled<P, 1>(g, A, B, partial, max_blocks, counter, out, bd, st);
  if (T == 2) return launch_gram_tiled<P, 2>(g, A, B, partial, max_blocks, counter, out, bd, st);
  if (T == 3) return launch_gram_tiled<P, 3>(g, A, B, partial, max_blocks, counter, out, bd, st);
  return launch_gram_tiled<P, 4>(g, A, B, partial, max_blocks, counter, out, bd, st);
}

// kernels one launch_gram issues: the partial sums and their finalisation
int gram_launches(int, const Geo&) { return 2; }

cudaError_t launch_gram(int P, const Geo& g, const void* A, const void* B, double2* partial, long long max_blocks,
                        unsigned* counter, double2* out, cudaStream_t st) {
  const int bd = block_size_for(g.N5, LOC_NONE);
  if (bd <= 0 || g.nrhs > kMaxRhs) return cudaErrorInvalidValue;
  // FP32 / FP16: the register-tiled kernel (groups of 16 threads)
  if ((P == P32 || P == P16) && bd % 16 == 0) {
    if (P == P32) {
      const int T = (g.nrhs + 3) / 4;
      if (T == 1) return launch_gram_async<1>(g, A, B, partial, max_blocks, counter, out, bd, st);
      if (T == 2) return launch_gram_async<2>(g, A, B, partial, max_blocks, counter, out, bd, st);
      if (T == 3) return launch_gram_async<3>(g, A, B, partial, max_blocks, counter, out, bd, st);
      return launch_gram_async<4>(g, A, B, partial, max_blocks, counter, out, bd, st);
    }
    return launch_gram_tiled_k<P16>(g, A, B, partial, max_blocks, counter, out, bd, st);
  }
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
