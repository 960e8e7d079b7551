// gbf_kernels.cuh -- device building blocks shared by the kernel files:
// site-local operators (clover, s-matrix), the deterministic block reduction
// and its last-block finalisation, and the CG scalar updates.
#pragma once
#include "gbf_common.cuh"

namespace gbf {

// A site-local operator applied in a kernel epilogue.
//   LOC_CLOVER: per 4D site two Hermitian 6x6 blocks (spins {0,1}, {2,3});
//               72 reals per site: block b = 6 diagonal reals followed by the
//               15 strictly-lower complex entries (row-major i > j).
//               Storage per parity: FP64 double2 [36][Vh], FP32 float4 [18][Vh].
//   LOC_SMAT:   one real Ls x Ls matrix per chirality acting on the s index,
//               the same at every 4D site; [2][Ls][Ls] in the arithmetic type.
//   LOC_SCALAR: multiplication by a real constant.
//   LOC_TWIST:  multiplication by a complex constant per chirality, z[0] + i z[1]
//               on spins 0, 1 and z[2] + i z[3] on spins 2, 3 (twisted mass
//               a + i mu g5, its inverse and adjoints).
struct LocalOp {
  int kind;
  const void* clov[2];  // per parity
  const void* smat;
  int cplx;             // LOC_SMAT: complex matrices ([2][Ls][Ls] (re, im) pairs; zmobius)
  double scalar;
  double z[4];
};

template <typename R> struct CloverLoad;
template <> struct CloverLoad<double> {
  static __device__ __forceinline__ void block(const void* base, int Vh, int cb, int b, double (&c)[36]) {
    const double2* p = reinterpret_cast<const double2*>(base) + ((unsigned)cb + 18u * (unsigned)b * (unsigned)Vh);
#pragma unroll
    for (int k = 0; k < 18; ++k) {
      double2 q = __ldg(p + (unsigned)k * (unsigned)Vh);
      c[2 * k] = q.x;
      c[2 * k + 1] = q.y;
    }
  }
};
template <> struct CloverLoad<float> {
  static __device__ __forceinline__ void block(const void* base, int Vh, int cb, int b, float (&c)[36]) {
    const float4* p = reinterpret_cast<const float4*>(base) + ((unsigned)cb + 9u * (unsigned)b * (unsigned)Vh);
#pragma unroll
    for (int k = 0; k < 9; ++k) {
      float4 q = __ldg(p + (unsigned)k * (unsigned)Vh);
      c[4 * k] = q.x; c[4 * k + 1] = q.y; c[4 * k + 2] = q.z; c[4 * k + 3] = q.w;
    }
  }
};
// off-diagonal index of (i, j), i > j
__host__ __device__ constexpr int tri(int i, int j) { return i * (i - 1) / 2 + j; }

template <typename R>
__device__ __forceinline__ void clover_apply(const void* base, int Vh, int cb, cplx<R> (&v)[12]) {
#pragma unroll
  for (int b = 0; b < 2; ++b) {
    R c[36];
    CloverLoad<R>::block(base, Vh, cb, b, c);
    cplx<R> o[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) {
      cplx<R> acc = scl<R>(c[i], v[6 * b + i]);
#pragma unroll
      for (int j = 0; j < 6; ++j) {
        if (j < i) {
          const int t = tri(i, j);
          acc = cmadd<R>(acc, mk<R>(c[6 + 2 * t], c[6 + 2 * t + 1]), v[6 * b + j]);
        } else if (j > i) {
          const int t = tri(j, i);
          acc = cmaddc<R>(acc, mk<R>(c[6 + 2 * t], c[6 + 2 * t + 1]), v[6 * b + j]);
        }
      }
      o[i] = acc;
    }
#pragma unroll
    for (int i = 0; i < 6; ++i) v[6 * b + i] = o[i];
  }
}

// Double-float clover for site-local kernels: all loads of a block issued
// together, the two blocks in a rolled loop (the block is selected into w and
// written back by predicated moves) to keep the code in the instruction cache.
template <>
__device__ __forceinline__ void clover_apply<dd>(const void* base, int Vh, int cb, ddc (&v)[12]) {
  const float4* p0 = reinterpret_cast<const float4*>(base) + cb;
#pragma unroll 1
  for (int b = 0; b < 2; ++b) {
    const float4* p = p0 + 18u * (unsigned)b * (unsigned)Vh;
    float4 q[18];
#pragma unroll
    for (int k = 0; k < 18; ++k) q[k] = __ldg(p + (unsigned)k * (unsigned)Vh);
    ddc w[6], o[6];
#pragma unroll
    for (int i = 0; i < 6; ++i) w[i] = b ? v[6 + i] : v[i];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      o[2 * k] = scl<dd>(dd(q[k].x, q[k].z), w[2 * k]);
      o[2 * k + 1] = scl<dd>(dd(q[k].y, q[k].w), w[2 * k + 1]);
    }
#pragma unroll
    for (int i = 1; i < 6; ++i)
#pragma unroll
      for (int j = 0; j < i; ++j) {
        const float4 e = q[3 + tri(i, j)];
        const ddc cij = mk<dd>(dd(e.x, e.z), dd(e.y, e.w));
        o[i] = cmadd<dd>(o[i], cij, w[j]);
        o[j] = cmaddc<dd>(o[j], cij, w[i]);
      }
#pragma unroll
    for (int i = 0; i < 6; ++i) {
      if (b) v[6 + i] = o[i];
      else v[i] = o[i];
    }
  }
}

// Double-float clover for the register-capped hopping kernel: entry by entry
// (each off-diagonal entry is loaded right before its two uses, row i and,
// conjugated, row j), so that no more than one entry is live.
__device__ __forceinline__ void clover_apply_dd_lowreg(const void* base, int Vh, int cb, ddc (&v)[12]) {
  const float4* p0 = reinterpret_cast<const float4*>(base) + cb;
#pragma unroll
  for (int b = 0; b < 2; ++b) {
    const float4* p = p0 + 18u * (unsigned)b * (unsigned)Vh;
    ddc* w = v + 6 * b;
    ddc o[6];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const float4 q = __ldg(p + (unsigned)k * (unsigned)Vh);
      o[2 * k] = scl<dd>(dd(q.x, q.z), w[2 * k]);
      o[2 * k + 1] = scl<dd>(dd(q.y, q.w), w[2 * k + 1]);
    }
#pragma unroll
    for (int i = 1; i < 6; ++i)
#pragma unroll
      for (int j = 0; j < i; ++j) {
        const float4 q = __ldg(p + (unsigned)(3 + tri(i, j)) * (unsigned)Vh);
        const ddc cij = mk<dd>(dd(q.x, q.z), dd(q.y, q.w));
        o[i] = cmadd<dd>(o[i], cij, w[j]);
        o[j] = cmaddc<dd>(o[j], cij, w[i]);
      }
#pragma unroll
    for (int i = 0; i < 6; ++i) w[i] = o[i];
  }
}

// Per-thread local op (everything except LOC_SMAT, which needs the block).
template <typename R>
__device__ __forceinline__ void local_apply_thread(const LocalOp& l, int Vh, int parity, int cb, cplx<R> (&v)[12]) {
  if (l.kind == LOC_CLOVER) {
    clover_apply<R>(l.clov[parity], Vh, cb, v);
  } else if (l.kind == LOC_TWIST) {
    const cplx<R> z0 = mk<R>((R)l.z[0], (R)l.z[1]), z1 = mk<R>((R)l.z[2], (R)l.z[3]);
#pragma unroll
    for (int k = 0; k < 12; ++k) {
      nrm<R>(v[k]);
      v[k] = cmul<R>(k < 6 ? z0 : z1, v[k]);
    }
  } else if (l.kind == LOC_SCALAR) {
    const R s = (R)l.scalar;
#pragma unroll
    for (int k = 0; k < 12; ++k) {
      nrm<R>(v[k]);
      v[k] = scl<R>(s, v[k]);
    }
  }
}

// Shared-memory words reserved for the s-matrices of one block: two
// chiralities of Ls x Ls complex entries at the largest Ls.
constexpr int kSmatWords = 4 * kMaxLs * kMaxLs;

// s-matrix op through shared memory.  Threads of one block hold complete
// s-columns (blockDim is a multiple of N5, i5 = rhs*Ls + s fastest).
// tile: 24*blockDim reals, one contiguous spinor per thread so the s-column
// is read back with 16-byte loads (the threads of one column read the same
// address: shared-memory broadcast); mat: 2*Ls*Ls reals.  All threads call.
template <typename R> struct Vec4;
template <> struct Vec4<float> { using T = float4; };
template <> struct Vec4<double> { using T = double2; };
template <> struct Vec4<dd> { using T = float4; };

template <typename R>
__device__ __forceinline__ void smat_apply_block(const R* mat_g, int Ls, R* tile, R* mat, cplx<R> (&v)[12], bool load_mat) {
  using W = typename Vec4<R>::T;
  constexpr int per = (int)(sizeof(W) / sizeof(R));  // reals per vector load
  const int t = threadIdx.x, bd = blockDim.x;
  if (load_mat)
    for (int k = t; k < 2 * Ls * Ls; k += bd) mat[k] = mat_g[k];
  R* mine = tile + 24 * t;
#pragma unroll
  for (int k = 0; k < 12; ++k) {
    mine[2 * k] = v[k].x;
    mine[2 * k + 1] = v[k].y;
  }
  __syncthreads();
  const int s = t % Ls;
  const R* col = tile + 24 * (t - s);
  const R* m0 = mat + s * Ls;
  const R* m1 = mat + Ls * Ls + s * Ls;
  R acc[24];
#pragma unroll
  for (int k = 0; k < 24; ++k) acc[k] = rzero<R>();
  for (int sp = 0; sp < Ls; ++sp) {
    const R a0 = m0[sp], a1 = m1[sp];
    const W* src = reinterpret_cast<const W*>(col + 24 * sp);
#pragma unroll
    for (int q = 0; q < 24 / per; ++q) {
      const W w = src[q];
      const R* e = reinterpret_cast<const R*>(&w);
#pragma unroll
      for (int j = 0; j < per; ++j) {
        const int k = q * per + j;
        acc[k] = fma(k < 12 ? a0 : a1, e[j], acc[k]);
      }
    }
  }
#pragma unroll
  for (int k = 0; k < 12; ++k) v[k] = mk<R>(acc[2 * k], acc[2 * k + 1]);
  __syncthreads();
}

// The same with complex matrices ([2][Ls][Ls] entries of (re, im)), the
// per-slice complex Cayley coefficients of zmobius.
template <typename R>
__device__ __forceinline__ void smat_apply_block_c(const R* mat_g, int Ls, R* tile, R* mat, cplx<R> (&v)[12]) {
  using W = typename Vec4<R>::T;
  constexpr int per = (int)(sizeof(W) / sizeof(R));  // reals per vector load (even)
  const int t = threadIdx.x, bd = blockDim.x;
  for (int k = t; k < 4 * Ls * Ls; k += bd) mat[k] = mat_g[k];
  R* mine = tile + 24 * t;
#pragma unroll
  for (int k = 0; k < 12; ++k) {
    mine[2 * k] = v[k].x;
    mine[2 * k + 1] = v[k].y;
  }
  __syncthreads();
  const int s = t % Ls;
  const R* col = tile + 24 * (t - s);
  const R* m0 = mat + 2 * (s * Ls);
  const R* m1 = mat + 2 * (Ls * Ls + s * Ls);
  R acc[24];
#pragma unroll
  for (int k = 0; k < 24; ++k) acc[k] = rzero<R>();
  for (int sp = 0; sp < Ls; ++sp) {
    const R a0r = m0[2 * sp], a0i = m0[2 * sp + 1], a1r = m1[2 * sp], a1i = m1[2 * sp + 1];
    const W* src = reinterpret_cast<const W*>(col + 24 * sp);
#pragma unroll
    for (int q = 0; q < 24 / per; ++q) {
      const W w = src[q];
      const R* e = reinterpret_cast<const R*>(&w);
#pragma unroll
      for (int j = 0; j < per; j += 2) {
        const int k = q * per + j;
        const R ar = k < 12 ? a0r : a1r, ai = k < 12 ? a0i : a1i;
        acc[k] = fma(ar, e[j], acc[k]);
        acc[k] = fma(-ai, e[j + 1], acc[k]);
        acc[k + 1] = fma(ar, e[j + 1], acc[k + 1]);
        acc[k + 1] = fma(ai, e[j], acc[k + 1]);
      }
    }
  }
#pragma unroll
  for (int k = 0; k < 12; ++k) v[k] = mk<R>(acc[2 * k], acc[2 * k + 1]);
  __syncthreads();
}

// Per-site <a, b> and |a|^2: the 12 products of one site are summed in the
// arithmetic precision R (FP32 kernels stay on the FP32 pipe; FP64 throughput
// is 1/58 of FP32 on GB300), the cross-site sums below are FP64.
template <typename R>
__device__ __forceinline__ void site_dot(const cplx<R> (&a)[12], const cplx<R> (&b)[12], double& re, double& im) {
  R r = 0, i = 0;
#pragma unroll
  for (int k = 0; k < 12; ++k) {
    r = fma(a[k].x, b[k].x, r);
    r = fma(a[k].y, b[k].y, r);
    i = fma(a[k].x, b[k].y, i);
    i = fma(-a[k].y, b[k].x, i);
  }
  re = (double)r;
  im = (double)i;
}
template <typename R>
__device__ __forceinline__ double site_norm2(const cplx<R> (&a)[12]) {
  R r = 0;
#pragma unroll
  for (int k = 0; k < 12; ++k) {
    r = fma(a[k].x, a[k].x, r);
    r = fma(a[k].y, a[k].y, r);
  }
  return (double)r;
}
template <>
__device__ __forceinline__ void site_dot<dd>(const ddc (&a_)[12], const ddc (&b_)[12], double& re, double& im) {
  ddc a[12], b[12];
#pragma unroll
  for (int k = 0; k < 12; ++k) {
    a[k] = a_[k];
    b[k] = b_[k];
    nrm<dd>(a[k]);
    nrm<dd>(b[k]);
  }
  dd r = rzero<dd>(), i = rzero<dd>();
#pragma unroll
  for (int k = 0; k < 12; ++k) {
    r = fma(a[k].x, b[k].x, r);
    r = fma(a[k].y, b[k].y, r);
    i = fma(a[k].x, b[k].y, i);
    i = fma(-a[k].y, b[k].x, i);
  }
  re = (double)r;
  im = (double)i;
}
template <>
__device__ __forceinline__ double site_norm2<dd>(const ddc (&a_)[12]) {
  ddc a[12];
#pragma unroll
  for (int k = 0; k < 12; ++k) {
    a[k] = a_[k];
    nrm<dd>(a[k]);
  }
  dd r = rzero<dd>();
#pragma unroll
  for (int k = 0; k < 12; ++k) {
    r = fma(a[k].x, a[k].x, r);
    r = fma(a[k].y, a[k].y, r);
  }
  return (double)r;
}

// ---------------------------------------------------------------------------
// deterministic reduction: block tree over sites (stride N5), per-rhs sum of
// the s entries, per-block partials, last block sums the partials in block
// order and applies a finaliser to the CG state.
// ---------------------------------------------------------------------------
enum Fin { FIN_STORE = 0, FIN_ALPHA = 1, FIN_BETA = 2, FIN_INIT = 3 };

struct RedArgs {
  int fin;
  double2* partial;   // [gridDim][nrhs]
  unsigned* counter;  // zero on entry, restored to zero by the last block
  CGState* st;
  // FIN_BETA inside a conditional while graph: the last block sets the loop
  // condition to !all_done (all_done also covers maxiter and breakdown)
  unsigned long long cond;
  int use_cond;
};

__device__ __forceinline__ void finalize(const RedArgs& r, int rhs, double re, double im) {
  CGState* st = r.st;
  switch (r.fin) {
    case FIN_STORE:
      st->last[rhs] = re;
      st->last_im[rhs] = im;
      break;
    case FIN_ALPHA: {
      st->d[rhs] = re;
      double a = 0.0;
      if (!st->done[rhs]) {
        if (!(re > 0.0) || !isfinite(re)) {
          st->done[rhs] = 1;
          st->breakdown = 1;
        } else {
          a = st->cp[rhs] / re;
        }
      }
      st->alpha[rhs] = a;
      break;
    }
    case FIN_BETA: {
      if (!st->done[rhs]) {
        double b = re / st->cp[rhs];
        st->beta[rhs] = b;
        st->cp[rhs] = re;
        if (re <= st->rsq[rhs]) st->done[rhs] = 1;
        if (!isfinite(re)) { st->done[rhs] = 1; st->breakdown = 1; }
      } else {
        st->beta[rhs] = 0.0;
      }
      break;
    }
    case FIN_INIT:
      st->cp[rhs] = re;
      st->alpha[rhs] = 0.0;
      st->beta[rhs] = 0.0;
      st->done[rhs] = (re <= st->rsq[rhs]) ? 1 : 0;
      break;
  }
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// Sum (a, b) over the block in a fixed order: shuffle within warps, then the
// warp sums in warp 0.  Needs blockDim % 32 == 0; result valid in thread 0.
__device__ __forceinline__ double2 block_sum_shfl(double a, double b, double* sm) {
  const int t = threadIdx.x, lane = t & 31, w = t >> 5, nw = blockDim.x >> 5;
  a = warp_sum(a);
  b = warp_sum(b);
  if (lane == 0) {
    sm[w] = a;
    sm[32 + w] = b;
  }
  __syncthreads();
  if (w == 0) {
    a = lane < nw ? sm[lane] : 0.0;
    b = lane < nw ? sm[32 + lane] : 0.0;
    a = warp_sum(a);
    b = warp_sum(b);
  }
  __syncthreads();
  return make_double2(a, b);
}

// sm: 2*blockDim doubles of shared memory.  Every thread of the block calls.
__device__ __forceinline__ void block_reduce_finalize(const RedArgs& r, double vre, double vim, int N5, int Ls, int nrhs, double* sm) {
  const int t = threadIdx.x, bd = blockDim.x;
  const bool shfl = (bd & 31) == 0;
  if (nrhs == 1 && shfl) {
    // one right-hand side: every thread's value belongs to it
    const double2 s = block_sum_shfl(vre, vim, sm);
    if (t == 0) r.partial[blockIdx.x] = s;
  } else {
    const int S = bd / N5;  // power of two by construction
    sm[t] = vre;
    sm[bd + t] = vim;
    __syncthreads();
    for (int k = S >> 1; k >= 1; k >>= 1) {
      if (t < k * N5) {
        sm[t] += sm[t + k * N5];
        sm[bd + t] += sm[bd + t + k * N5];
      }
      __syncthreads();
    }
    if (t < nrhs) {
      double ar = 0, ai = 0;
      for (int s = 0; s < Ls; ++s) {
        ar += sm[t * Ls + s];
        ai += sm[bd + t * Ls + s];
      }
      r.partial[(size_t)blockIdx.x * nrhs + t] = make_double2(ar, ai);
    }
  }
  __threadfence();
  __syncthreads();
  __shared__ int s_last;
  if (t == 0) s_last = (atomicAdd(r.counter, 1u) == gridDim.x - 1);
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  // The partials form a flat [block][rhs] array.  Thread t sums entries
  // t, t + bd, t + 2bd, ... (coalesced); since bd is a multiple of nrhs all of
  // them belong to rhs t % nrhs.  Then thread r < nrhs adds the bd/nrhs
  // thread sums of its rhs in order.  Fixed order: bitwise reproducible.
  {
    const long long total = (long long)gridDim.x * nrhs;
    double ar = 0, ai = 0;
#pragma unroll 4
    for (long long e = t; e < total; e += bd) {
      const double2 q = __ldcg(r.partial + e);
      ar += q.x;
      ai += q.y;
    }
    if (nrhs == 1 && shfl) {
      const double2 s = block_sum_shfl(ar, ai, sm);
      if (t == 0) finalize(r, 0, s.x, s.y);
    } else {
      sm[t] = ar;
      sm[bd + t] = ai;
      __syncthreads();
      if (t < nrhs) {
        double sr = 0, si = 0;
        for (int j = t; j < bd; j += nrhs) {
          sr += sm[j];
          si += sm[bd + j];
        }
        finalize(r, t, sr, si);
      }
    }
    __syncthreads();
  }
  if (t == 0) {
    if (r.fin == FIN_BETA || r.fin == FIN_INIT) {
      int all = 1;
      for (int rhs = 0; rhs < nrhs; ++rhs) all &= r.st->done[rhs];
      if (r.fin == FIN_BETA) {
        r.st->iter += 1;
        if (r.st->iter >= r.st->maxiter) all = 1;
      }
      r.st->all_done = all;
      if (r.fin == FIN_BETA && r.use_cond) cudaGraphSetConditional(r.cond, all ? 0u : 1u);
    }
    *r.counter = 0;
    __threadfence();
  }
}

}  // namespace gbf
