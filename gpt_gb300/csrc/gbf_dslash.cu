// gbf_dslash.cu -- the even-odd Wilson hopping kernel with fused epilogues.
//
// Computes, for every 5D site n of the output parity p (thread per site):
//   hop(x) = -1/2 sum_mu cc_mu [ (1 + s g_mu) U_mu(x) in(x+mu)
//                               + (1 - s g_mu) U_mu(x-mu)^+ in(x-mu) ]
// with s = -1 for Dhop and s = +1 for Dhop^dag (the statement of
// lib/gpt/qcd/fermion/reference/wilson_clover.py:182-200, which Grid's
// WilsonKernels implement for opcodes 3001/3002/4001/4002, and the 4D part of
// Grid's Cayley Meooe for Mobius), followed by the epilogue
//   out = c1 * L1(hop) + c2 * L2(X)       (L1, L2 site-local operators)
// and optionally the deterministic reduction of <Y, out> or |out|^2 with a
// CG finaliser.  The input spinor is projected to two spin components before
// the colour multiply (8 x 2 SU(3) matvecs per site) and the lower two spin
// components of each term are rebuilt from the upper two.
//
// Roofline: HBM-bound in FP32/FP16 (per output site: 8 neighbour spinors that
// the L2 mostly serves once, 8 links, 1 output); FP64 is bound by the FP64
// pipe on GB300 (about 1.2 TFLOP/s measured).
#include <array>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <mutex>
#include <tuple>
#include "gbf_launch.cuh"

// resident blocks of 256 threads per SM requested for the FP32/FP16 variants
// (register cap 65536 / (256 * minblocks))
#ifndef GBF_DSLASH_MINB
#define GBF_DSLASH_MINB 2
#endif
// the same for the double-float variant (2: 128 registers, a few spills in
// the clover epilogue, measured faster than 1 block of 255 registers)
#ifndef GBF_DSLASH_MINB_DD
#define GBF_DSLASH_MINB_DD 2
#endif

namespace gbf {

// Offset (in 16-byte units) of the double-float accumulators in dynamic
// shared memory: after the s-matrix tile and the reduction scratch.
__host__ __device__ inline unsigned dd_acc_offset16(int LK, unsigned bd) {
  size_t s = 0;
  if (LK == LOC_SMAT) s += (24 * (size_t)bd + kSmatWords) * 8 + 8;
  s += 2 * (size_t)bd * 8;
  return (unsigned)((s + 15) / 16);
}

// Epilogue of the hopping kernels for the 5D site n (4D site cb of the
// output parity): out = c1 L1(hop) + c2 L2(X), store, and the per-thread
// part of the optional reduction.  Every thread of the block calls (the
// s-matrix op synchronises the block).
template <int P, int LK>
__device__ __forceinline__ void hop_epilogue(const DslashArgs& a, bool active, long long n, int cb,
                                             cplx<typename SpinorT<P>::R> (&res)[12], double& red_re, double& red_im,
                                             double* smem_d) {
  using R = typename SpinorT<P>::R;
  using V = cplx<R>;
  const Geo& g = a.g;
  const int p = a.out_parity;
  if (LK == LOC_SMAT) {
    if (a.l1.kind == LOC_SMAT) {
      R* tile = reinterpret_cast<R*>(smem_d);
      R* mat = tile + 24 * blockDim.x;
      if (a.l1.cplx) smat_apply_block_c<R>(reinterpret_cast<const R*>(a.l1.smat), g.Ls, tile, mat, res);
      else smat_apply_block<R>(reinterpret_cast<const R*>(a.l1.smat), g.Ls, tile, mat, res, true);
    }
  } else if (active && a.l1.kind != LOC_NONE) {
    if constexpr (P == PDD) {
      if (a.l1.kind == LOC_CLOVER) clover_apply_dd_lowreg(a.l1.clov[p], g.Vh, cb, res);
      else local_apply_thread<R>(a.l1, g.Vh, p, cb, res);
    } else {
      local_apply_thread<R>(a.l1, g.Vh, p, cb, res);
    }
  }
  if (active) {
    if (a.c1 != 1.0) {
      const R c1 = (R)a.c1;
#pragma unroll
      for (int k = 0; k < 12; ++k) {
        nrm<R>(res[k]);
        res[k] = scl<R>(c1, res[k]);
      }
    }
    if (a.X) {
      V xv[12];
      load_spinor<P>(a.X, g.N, n, xv);
      if (LK != LOC_SMAT && a.l2.kind != LOC_NONE) {
        if constexpr (P == PDD) {
          if (a.l2.kind == LOC_CLOVER) clover_apply_dd_lowreg(a.l2.clov[p], g.Vh, cb, xv);
          else local_apply_thread<R>(a.l2, g.Vh, p, cb, xv);
        } else {
          local_apply_thread<R>(a.l2, g.Vh, p, cb, xv);
        }
      }
      const R c2 = (R)a.c2;
#pragma unroll
      for (int k = 0; k < 12; ++k) res[k] = mk<R>(fma(c2, xv[k].x, res[k].x), fma(c2, xv[k].y, res[k].y));
    }
    store_spinor<P>(a.out, g.N, n, res);
  }
  if (a.red && active) {
    double vr = 0, vi = 0;
    if (a.red == 1) {
      V yv[12];
      load_spinor<P>(a.Y, g.N, n, yv);
      site_dot<R>(yv, res, vr, vi);
    } else {
      vr = site_norm2<R>(res);
    }
    red_re += vr;
    red_im += vi;
  }
}

template <int P, int LS, int LK, bool LOOP>
__global__ void __launch_bounds__(256, (P == P64 ? 1 : P == PDD ? GBF_DSLASH_MINB_DD : GBF_DSLASH_MINB)) dslash_kernel(const DslashArgs a) {
  using R = typename SpinorT<P>::R;
  using V = cplx<R>;
  extern __shared__ __align__(16) double smem_d[];
  const Geo& g = a.g;
  if (a.check_done && a.ra.st->all_done) return;
  const int p = a.out_parity, q = 1 - p;
  double red_re = 0, red_im = 0;
  // block-uniform loop over tiles of blockDim sites; LOOP = false when the
  // grid covers every tile (one tile per block, no loop is compiled)
  const long long ntiles = (g.N + blockDim.x - 1) / blockDim.x;
  long long tile = blockIdx.x;
  do {
  const long long n = tile * blockDim.x + threadIdx.x;
  const bool active = n < g.N;
  V res[12];
#pragma unroll
  for (int k = 0; k < 12; ++k) res[k] = cz<R>();
  int cb = 0;
  if constexpr (P == PDD) {
    if (active) {
      // double-float, rolled direction loop (one iteration is about 1.5k
      // instructions; unrolled eight times the kernel would not fit the
      // instruction cache).  The 12 accumulators live in shared memory
      // ([component][thread], 16 B each) during the loop, which frees 48
      // registers per thread for more resident warps.
      cb = (int)g.fN5.div((unsigned)n);
      const unsigned i5 = (unsigned)n - (unsigned)cb * (unsigned)g.N5;
      const Coord c = cb_coords(g, cb, p);
      float4* acc = reinterpret_cast<float4*>(smem_d) + dd_acc_offset16(LK, blockDim.x) + threadIdx.x;
      const unsigned bs = blockDim.x;
#pragma unroll
      for (int k = 0; k < 12; ++k) acc[k * bs] = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll 1
      for (int d = 0; d < 8; ++d) {
        const int mu = d >> 1;
        const bool fwd = (d & 1) == 0;
        int y[4];
#pragma unroll
        for (int m = 0; m < 4; ++m) {
          const int xm = c.x[m], Lm = g.L[m];
          y[m] = (m != mu) ? xm : fwd ? (xm == Lm - 1 ? 0 : xm + 1) : (xm == 0 ? Lm - 1 : xm - 1);
        }
        const int ycb = cb_index(g, y);
        const unsigned site = (unsigned)ycb * (unsigned)g.N5 + i5;
        const float s = fwd ? a.sgn : -a.sgn;
#ifndef GBF_DD_SCALAR
        // lane-paired form (pdd): u h = Re(u) h + Im(u) (i h), and the
        // backward term's conj(u) negates Im(u)
        {
          const float4* sp = reinterpret_cast<const float4*>(a.in);
          const unsigned N = (unsigned)g.N;
          pdd h[2][3];
#pragma unroll
          for (int r = 0; r < 2; ++r) {
            const int pr = gperm(mu, r), cr = gcoef(mu, r);
#pragma unroll
            for (int col = 0; col < 3; ++col) {
              const pdd up = pdd_ld(__ldg(sp + (site + (unsigned)(3 * r + col) * N)));
              const pdd lo = pdd_ld(__ldg(sp + (site + (unsigned)(3 * pr + col) * N)));
              h[r][col] = pdd_coefmadd_rt(cr, s, lo, up);
            }
          }
          const float4* L = reinterpret_cast<const float4*>(a.links) +
                            (unsigned)(((fwd ? p : q) * 4 + mu) * 9) * (unsigned)g.Vh + (unsigned)(fwd ? cb : ycb);
          const float cs = fwd ? 1.f : -1.f;
          pdd uh[2][3];
#pragma unroll
          for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) {
              const unsigned k = fwd ? (unsigned)(3 * i + j) : (unsigned)(3 * j + i);
              const float4 qv = __ldg(L + k * (unsigned)g.Vh);
              const dd ux(qv.x, qv.z), uy = dd_scale2(cs, dd(qv.y, qv.w));
#pragma unroll
              for (int r = 0; r < 2; ++r) {
                uh[r][i] = j == 0 ? pdd_mul_s(ux, h[r][j]) : pdd_fma_s(ux, h[r][j], uh[r][i]);
                uh[r][i] = pdd_fma_s(uy, pdd_i(h[r][j]), uh[r][i]);
              }
            }
#pragma unroll
          for (int r = 0; r < 2; ++r)
#pragma unroll
            for (int i = 0; i < 3; ++i) {
              float4& m = acc[(3 * r + i) * bs];
              m = pdd_st(pdd_add(pdd_ld(m), uh[r][i]));
            }
#pragma unroll
          for (int r = 2; r < 4; ++r) {
            const bool first = gperm(mu, r) == 0;
            const int cr = gcoef(mu, r);
#pragma unroll
            for (int i = 0; i < 3; ++i) {
              float4& m = acc[(3 * r + i) * bs];
              m = pdd_st(pdd_coefmadd_rt(cr, s, first ? uh[0][i] : uh[1][i], pdd_ld(m)));
            }
          }
        }
#else
        cplx<dd> h[2][3];
#pragma unroll
        for (int r = 0; r < 2; ++r) {
          cplx<dd> up[3], lo[3];
          load_spin_dd(a.in, g.N, site, r, up);
          load_spin_dd(a.in, g.N, site, gperm(mu, r), lo);
          const int cr = gcoef(mu, r);
#pragma unroll
          for (int col = 0; col < 3; ++col) h[r][col] = coefmadd_rt(cr, s, lo[col], up[col]);
        }
        cplx<dd> u[9];
        load_link<LDD, dd>(a.links, g.Vh, fwd ? p : q, mu, fwd ? cb : ycb, u);
        cplx<dd> uh[2][3];
#pragma unroll
        for (int r = 0; r < 2; ++r)
#pragma unroll
          for (int i = 0; i < 3; ++i) {
            cplx<dd> t = cz<dd>();
#pragma unroll
            for (int j = 0; j < 3; ++j) t = fwd ? cmadd<dd>(t, u[3 * i + j], h[r][j]) : cmaddc<dd>(t, u[3 * j + i], h[r][j]);
            uh[r][i] = t;
          }
#pragma unroll
        for (int r = 0; r < 2; ++r)
#pragma unroll
          for (int i = 0; i < 3; ++i) {
            float4& m = acc[(3 * r + i) * bs];
            const cplx<dd> v = add<dd>(mk<dd>(dd(m.x, m.z), dd(m.y, m.w)), uh[r][i]);
            m = make_float4(v.x.h, v.y.h, v.x.l, v.y.l);
          }
#pragma unroll
        for (int r = 2; r < 4; ++r) {
          const bool first = gperm(mu, r) == 0;
          const int cr = gcoef(mu, r);
#pragma unroll
          for (int i = 0; i < 3; ++i) {
            float4& m = acc[(3 * r + i) * bs];
            const cplx<dd> v = coefmadd_rt(cr, s, first ? uh[0][i] : uh[1][i], mk<dd>(dd(m.x, m.z), dd(m.y, m.w)));
            m = make_float4(v.x.h, v.y.h, v.x.l, v.y.l);
          }
        }
#endif
      }
#pragma unroll
      for (int k = 0; k < 12; ++k) {
        const float4 m = acc[k * bs];
        res[k] = mk<dd>(dd(m.x, m.z), dd(m.y, m.w));
      }
    }
  } else if (active) {
    cb = (int)g.fN5.div((unsigned)n);
    const unsigned i5 = (unsigned)n - (unsigned)cb * (unsigned)g.N5;
    const Coord c = cb_coords(g, cb, p);
    const R sf = (R)a.sgn;
#pragma unroll
    for (int mu = 0; mu < 4; ++mu) {
#pragma unroll
      for (int dir = 0; dir < 2; ++dir) {
        int y[4] = {c.x[0], c.x[1], c.x[2], c.x[3]};
        const bool fwd = dir == 0;
        bool wrap;
        if (fwd) {
          wrap = (y[mu] == g.L[mu] - 1);
          y[mu] = wrap ? 0 : y[mu] + 1;
        } else {
          wrap = (y[mu] == 0);
          y[mu] = wrap ? g.L[mu] - 1 : y[mu] - 1;
        }
        const int ycb = cb_index(g, y);
        V psi[12];
        load_spinor<P>(a.in, g.N, (unsigned)ycb * (unsigned)g.N5 + i5, psi);
        // project: h_r = psi_r + s * coef_r * psi_perm(r), r = 0, 1
        const R s = fwd ? sf : -sf;
        V h[2][3];
#pragma unroll
        for (int r = 0; r < 2; ++r)
#pragma unroll
          for (int col = 0; col < 3; ++col)
            h[r][col] = coefmadd<R>(gcoef(mu, r), s, psi[3 * gperm(mu, r) + col], psi[3 * r + col]);
        V u[9];
        load_link<LS, R>(a.links, g.Vh, fwd ? p : q, mu, fwd ? cb : ycb, u);
        V uh[2][3];
#pragma unroll
        for (int r = 0; r < 2; ++r)
#pragma unroll
          for (int i = 0; i < 3; ++i) {
            V acc = cz<R>();
#pragma unroll
            for (int j = 0; j < 3; ++j) acc = fwd ? cmadd<R>(acc, u[3 * i + j], h[r][j]) : cmaddc<R>(acc, u[3 * j + i], h[r][j]);
            uh[r][i] = acc;
          }
        if (LS == L32R) {
          // lambda = -cc/2 times the boundary phase (conjugated for the backward link)
          const R lam = (R)g.lam[mu];
          V ph = mk<R>(lam, (R)0);
          if (wrap) ph = mk<R>(lam * (R)g.ph_re[mu], (fwd ? lam : -lam) * (R)g.ph_im[mu]);
#pragma unroll
          for (int r = 0; r < 2; ++r)
#pragma unroll
            for (int i = 0; i < 3; ++i) uh[r][i] = cmul<R>(ph, uh[r][i]);
        }
#pragma unroll
        for (int r = 0; r < 2; ++r)
#pragma unroll
          for (int i = 0; i < 3; ++i) res[3 * r + i] = add<R>(res[3 * r + i], uh[r][i]);
#pragma unroll
        for (int r = 2; r < 4; ++r)
#pragma unroll
          for (int i = 0; i < 3; ++i) res[3 * r + i] = coefmadd<R>(gcoef(mu, r), s, uh[gperm(mu, r)][i], res[3 * r + i]);
      }
    }
  }
  hop_epilogue<P, LK>(a, active, n, cb, res, red_re, red_im, smem_d);
  tile += gridDim.x;
  } while (LOOP && tile < ntiles);
  if (a.red) {
    double* sm = smem_d + (LK == LOC_SMAT ? (24 * blockDim.x + kSmatWords) * sizeof(R) / sizeof(double) + 1 : 0);
    block_reduce_finalize(a.ra, red_re, red_im, g.N5, g.Ls, g.nrhs, sm);
  }
}

// ---------------------------------------------------------------------------
// The hop for fields with an inner extent N5 = Ls * n_rhs >= 8 (Mobius 5D
// fields, packed right-hand sides), FP32 or FP16 spinors, 18-real FP32 links.
// A block covers S = blockDim / N5 consecutive 4D sites with all their N5
// inner sites (the same site -> thread mapping as dslash_kernel).  The N5
// threads of a 4D site share its 8 neighbour indices and 8 links, so the
// block computes them once into shared memory:
//   nbs[j][d]  checkerboard index of the neighbour of site j in direction d
//              (d = 2 mu + {0 forward, 1 backward});
//   lsm[j][d]  the link of that term as a row-major 3x3 complex matrix with
//              the boundary phase and -cc/2 folded in (the stored links),
//              conjugate-transposed for the backward terms, so every term is
//              the same matvec;
// loaded coalesced (consecutive threads take consecutive sites of one link
// component).  Each thread then streams its 8 neighbour spinors (coalesced
// 16-byte loads along the inner index) and runs the projected matvecs.
// Per 4D site the index arithmetic and the link loads are done once instead
// of N5 times, and no link registers stay live across the loads.
// ---------------------------------------------------------------------------
constexpr int kHop5LinkStride = 41;  // float4 per site (8 links x 5, +1 pad: site rows 4 banks apart)

// links, neighbour indices and (hop5_kernel) the link offsets of the S sites
__host__ __device__ inline size_t hop5_extra_smem(int S) {
  return (size_t)S * kHop5LinkStride * 16 + (size_t)S * 16 * 4;
}

// Resident blocks per SM the hop5 kernels are compiled for: 3 (80
// registers) with the s-matrix epilogue or a looping reduction, 4 (64
// registers) otherwise, the faster of each measured on GB300 (more warps
// hide the neighbour loads; the other two spill at 64)
#ifndef GBF_HOP5_MINB
#define GBF_HOP5_MINB 3
#endif
#ifndef GBF_HOP5_MINB_THREAD
#define GBF_HOP5_MINB_THREAD 4
#endif

// Order of the hop5 tiles.  lbx < 0: a tile is S consecutive checkerboard
// sites, and with slabT > 0 the (x2, x3) planes are visited slab by slab
// (slabT planes in x2, x3 slowest within a slab), so that a plane's x3
// neighbours are read while they are still in L2.  lbx >= 0: a tile is a
// brick of 2^lbx x 2^lby x 2^lbz x 2^lbt sites (x0/2, x1, x2, x3), whose
// neighbours in all four directions largely coincide (L1 reuse inside the
// block), and the bricks run x0 fastest within slabs of slabT planes in x2.
struct Hop5Order {
  int lbx, lby, lbz, lbt, slabT;
};

template <int P, int LK, bool LOOP>
__global__ void __launch_bounds__(256, (LK == LOC_SMAT || LOOP) ? GBF_HOP5_MINB : GBF_HOP5_MINB_THREAD)
    hop5_kernel(const DslashArgs a, unsigned epi_off16, int log2S,
                                                                   const Hop5Order ord) {
  using R = float;
  using V = float2;
  extern __shared__ __align__(16) double smem_d[];
  const Geo& g = a.g;
  if (a.check_done && a.ra.st->all_done) return;
  const int p = a.out_parity, q = 1 - p;
  const unsigned t = threadIdx.x, bd = blockDim.x;
  const unsigned S = 1u << log2S;
  constexpr unsigned kStride = kHop5LinkStride;
  float4* lsm = reinterpret_cast<float4*>(smem_d) + epi_off16;
  int* nbs = reinterpret_cast<int*>(lsm + S * kStride);
  const unsigned j = g.fN5.div(t);  // 4D site of this thread within the tile
  const unsigned i5 = t - j * (unsigned)g.N5;
  double red_re = 0, red_im = 0;
  const long long ntiles = (g.N + bd - 1) / bd;
  long long tile = blockIdx.x;
  do {
    int cb0 = (int)(tile << log2S);
    unsigned o0 = 0, o1 = 0, o2 = 0, o3 = 0;  // brick origin
    if (ord.lbx >= 0) {
      unsigned r = (unsigned)tile, qq;
      const unsigned n0 = (unsigned)g.Lh0 >> ord.lbx, n1 = (unsigned)g.L[1] >> ord.lby;
      const unsigned n2 = (unsigned)ord.slabT >> ord.lbz, n3 = (unsigned)g.L[3] >> ord.lbt;
      qq = r / n0; o0 = (r - qq * n0) << ord.lbx; r = qq;
      qq = r / n1; o1 = (r - qq * n1) << ord.lby; r = qq;
      qq = r / n2; o2 = (r - qq * n2) << ord.lbz; r = qq;
      qq = r / n3; o3 = (r - qq * n3) << ord.lbt;
      o2 += qq * (unsigned)ord.slabT;
    } else if (ord.slabT) {
      const unsigned pt = (unsigned)(g.Lh0 * g.L[1]) >> log2S;  // tiles per (x2, x3) plane
      const unsigned tp = (unsigned)tile / pt, w = (unsigned)tile - tp * pt;
      const unsigned r = tp / (unsigned)ord.slabT, x2 = tp - r * (unsigned)ord.slabT;
      const unsigned b = r / (unsigned)g.L[3], x3 = r - b * (unsigned)g.L[3];
      cb0 = (int)(((b * (unsigned)ord.slabT + x2 + (unsigned)g.L[2] * x3) * pt + w) << log2S);
    }
    auto site_of = [&](unsigned jj) -> int {
      if (ord.lbx < 0) return cb0 + (int)jj;
      const unsigned j0 = jj & ((1u << ord.lbx) - 1u);
      jj >>= ord.lbx;
      const unsigned j1 = jj & ((1u << ord.lby) - 1u);
      jj >>= ord.lby;
      const unsigned j2 = jj & ((1u << ord.lbz) - 1u), j3 = jj >> ord.lbz;
      return (int)((o0 + j0) + (unsigned)g.Lh0 * ((o1 + j1) + (unsigned)g.L[1] * ((o2 + j2) + (unsigned)g.L[2] * (o3 + j3))));
    };
    // ---- neighbour indices of the S sites, and the offset of each site's
    // link d in the link planes (fwd: U_mu(x) of parity p, bwd: U_mu(x - mu)
    // of parity q; ~0u for a site past the end) ----
    unsigned* loff = reinterpret_cast<unsigned*>(nbs + 8 * S);
    for (unsigned idx = t; idx < 8 * S; idx += bd) {
      const int jj = idx >> 3, d = idx & 7, cbj = site_of(jj);
      int ycb = 0;
      unsigned lo = ~0u;
      if (cbj < g.Vh) {
        const Coord c = cb_coords(g, cbj, p);
        const int mu = d >> 1;
        int y[4] = {c.x[0], c.x[1], c.x[2], c.x[3]};
        if ((d & 1) == 0) y[mu] = (y[mu] == g.L[mu] - 1) ? 0 : y[mu] + 1;
        else y[mu] = (y[mu] == 0) ? g.L[mu] - 1 : y[mu] - 1;
        ycb = cb_index(g, y);
        const bool fwd = (d & 1) == 0;
        lo = (unsigned)(((fwd ? p : q) * 4 + mu) * 9) * (unsigned)g.Vh + (unsigned)(fwd ? cbj : ycb);
      }
      nbs[idx] = ycb;
      loff[idx] = lo;
    }
    __syncthreads();
    const int cb = site_of(j);
    const long long n = (long long)cb * g.N5 + i5;
    const bool active = cb < g.Vh;
    // ---- links: component k of link d of site jj, jj fastest (coalesced).
    // Each thread's link entries (at most 9: 72 S entries over S N5 >= 8 S
    // threads) are requested, then (one-pass launches with a per-thread
    // epilogue) its first neighbour spinor, and only then are the links
    // stored, so the spinor load overlaps the link latency.  The looping and
    // s-matrix launches skip the early load (measured slower there).
    constexpr bool kEarly = !LOOP && LK != LOC_SMAT;
    V psi0[12];
    {
      const float2* L2 = reinterpret_cast<const float2*>(a.links);
      float* lf = reinterpret_cast<float*>(lsm);
      const unsigned total = 72u * S;
      auto link_src = [&](unsigned idx, unsigned& jj, unsigned& d, unsigned& k) -> const float2* {
        jj = idx & (S - 1);
        const unsigned dk = idx >> log2S;
        d = dk / 9u;
        k = dk - 9u * d;
        const unsigned lo = loff[jj * 8 + d];
        return lo == ~0u ? nullptr : L2 + (lo + k * (unsigned)g.Vh);
      };
      auto link_store = [&](unsigned jj, unsigned d, unsigned k, float2 v) {
        unsigned kk = k;
        if (d & 1) {  // U^dagger: (i, j) <- conj (j, i)
          kk = (k % 3u) * 3u + k / 3u;
          v.y = -v.y;
        }
        *reinterpret_cast<float2*>(lf + (jj * kStride + d * 5u) * 4u + 2u * kk) = v;
      };
      if constexpr (kEarly) {
        float2 lv[9];
#pragma unroll
        for (int c = 0; c < 9; ++c) {
          unsigned jj, d, k;
          const unsigned idx = t + (unsigned)c * bd;
          const float2* src = idx < total ? link_src(idx, jj, d, k) : nullptr;
          lv[c] = src ? __ldg(src) : make_float2(0.f, 0.f);
        }
        if (active) load_spinor<P>(a.in, g.N, (unsigned)nbs[j * 8] * (unsigned)g.N5 + i5, psi0);
        // (a site past the end gets zero links; it is inactive)
#pragma unroll
        for (int c = 0; c < 9; ++c) {
          const unsigned idx = t + (unsigned)c * bd;
          if (idx < total) {
            const unsigned jj = idx & (S - 1), dk = idx >> log2S, d = dk / 9u;
            link_store(jj, d, dk - 9u * d, lv[c]);
          }
        }
      } else {
        for (unsigned idx = t; idx < total; idx += bd) {
          unsigned jj, d, k;
          const float2* src = link_src(idx, jj, d, k);
          if (src) link_store(jj, d, k, __ldg(src));
        }
      }
    }
    __syncthreads();
    V res[12];
#pragma unroll
    for (int k = 0; k < 12; ++k) res[k] = cz<R>();
    if (active) {
      const R sf = (R)a.sgn;
      const int* nbj = nbs + j * 8;
      const float4* lj = lsm + j * kStride;
#pragma unroll
      for (int mu = 0; mu < 4; ++mu) {
#pragma unroll
        for (int dir = 0; dir < 2; ++dir) {
          const int d = 2 * mu + dir;
          const bool fwd = dir == 0;
          V psi[12];
          if (kEarly && d == 0) {
#pragma unroll
            for (int k = 0; k < 12; ++k) psi[k] = psi0[k];
          } else {
            load_spinor<P>(a.in, g.N, (unsigned)nbj[d] * (unsigned)g.N5 + i5, psi);
          }
          const R s = fwd ? sf : -sf;
          V h[2][3];
#pragma unroll
          for (int r = 0; r < 2; ++r)
#pragma unroll
            for (int col = 0; col < 3; ++col)
              h[r][col] = coefmadd<R>(gcoef(mu, r), s, psi[3 * gperm(mu, r) + col], psi[3 * r + col]);
          V u[10];
#pragma unroll
          for (int c = 0; c < 5; ++c) {
            const float4 w = lj[d * 5 + c];
            u[2 * c] = make_float2(w.x, w.y);
            u[2 * c + 1] = make_float2(w.z, w.w);
          }
          V uh[2][3];
#pragma unroll
          for (int r = 0; r < 2; ++r)
#pragma unroll
            for (int i = 0; i < 3; ++i) {
              V acc = cmul<R>(u[3 * i], h[r][0]);
              acc = cmadd<R>(acc, u[3 * i + 1], h[r][1]);
              uh[r][i] = cmadd<R>(acc, u[3 * i + 2], h[r][2]);
            }
#pragma unroll
          for (int r = 0; r < 2; ++r)
#pragma unroll
            for (int i = 0; i < 3; ++i) res[3 * r + i] = add<R>(res[3 * r + i], uh[r][i]);
#pragma unroll
          for (int r = 2; r < 4; ++r)
#pragma unroll
            for (int i = 0; i < 3; ++i) res[3 * r + i] = coefmadd<R>(gcoef(mu, r), s, uh[gperm(mu, r)][i], res[3 * r + i]);
        }
      }
    }
    hop_epilogue<P, LK>(a, active, n, cb, res, red_re, red_im, smem_d);
    tile += gridDim.x;
    if (LOOP) __syncthreads();  // the next tile overwrites nbs and lsm
  } while (LOOP && tile < ntiles);
  if (a.red) {
    double* sm = smem_d + (LK == LOC_SMAT ? (24 * blockDim.x + kSmatWords) * sizeof(R) / sizeof(double) + 1 : 0);
    block_reduce_finalize(a.ra, red_re, red_im, g.N5, g.Ls, g.nrhs, sm);
  }
}

// ---------------------------------------------------------------------------
// The hop of hop5_kernel with the neighbour spinors staged in shared memory
// by 1D bulk copies (cp.async.bulk, global -> shared, completion counted in
// bytes on an mbarrier), FP32 spinors.  For a tile of S 4D sites and
// direction d, the N5 inner sites of site j's neighbour are, in each of the
// 6 16-byte component planes of the FP32 layout, one contiguous run of
// N5 * 16 bytes; 6 S copies move them into a ring slot laid out
// [plane][site j][i5], i.e. [plane][thread].  A ring of kRing direction
// slots keeps kRing - 1 directions in flight while one is computed; thread 0
// waits for a slot's barrier (bounded) and a block barrier publishes the data
// and frees the slot used before, which the copy threads then refill.  The
// ring doubles as the epilogue's shared memory once the 8 directions are
// done.  A wait that runs out sets st->kernel_error and the block returns
// (all its threads together, after any copy still in flight has landed).
// ---------------------------------------------------------------------------
constexpr int kRing = 4;

__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
// bounded wait for the phase of `parity` to complete: about 1 s of SM clocks
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long* bar, unsigned parity) {
  const unsigned addr = smem_u32(bar);
  const long long t0 = clock64();
  while (true) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(addr), "r"(parity)
        : "memory");
    if (ok) return true;
    if (clock64() - t0 > 2000000000LL) return false;
  }
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, unsigned long long* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}

__host__ __device__ inline size_t hop5t_ring_bytes(int bd) { return (size_t)kRing * 6 * 16 * bd; }

template <int LK, bool LOOP>
__global__ void __launch_bounds__(256, GBF_HOP5_MINB) hop5t_kernel(const DslashArgs a, int log2S, unsigned links_off16) {
  using R = float;
  using V = float2;
  extern __shared__ __align__(128) double smem_d[];
  const Geo& g = a.g;
  if (a.check_done && a.ra.st->all_done) return;
  const int p = a.out_parity, q = 1 - p;
  const unsigned t = threadIdx.x, bd = blockDim.x;
  const unsigned S = 1u << log2S;
  const unsigned N = (unsigned)g.N, N5 = (unsigned)g.N5;
  float4* ring = reinterpret_cast<float4*>(smem_d);  // [kRing][6][bd], later the epilogue's region
  float4* lsm = reinterpret_cast<float4*>(smem_d) + links_off16;  // after max(ring, epilogue)
  int* nbs = reinterpret_cast<int*>(lsm + S * kHop5LinkStride);
  unsigned long long* full = reinterpret_cast<unsigned long long*>(nbs + 8 * S);
  __shared__ int s_ok;
  if (t == 0) {
    for (int r = 0; r < kRing; ++r) mbar_init(&full[r], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  unsigned par_bits = 0;  // completion parity of each slot, the same in every thread
  const unsigned j = g.fN5.div(t);
  const unsigned i5 = t - j * N5;
  double red_re = 0, red_im = 0;
  const long long ntiles = (g.N + bd - 1) / bd;
  long long tile = blockIdx.x;
  do {
    const int cb0 = (int)(tile << log2S);
    const unsigned s_act = (unsigned)min((long long)S, (long long)g.Vh - cb0);  // sites of this tile
    for (unsigned idx = t; idx < 8 * S; idx += bd) {
      const int jj = idx >> 3, d = idx & 7, cbj = cb0 + jj;
      int ycb = 0;
      if (cbj < g.Vh) {
        const Coord c = cb_coords(g, cbj, p);
        const int mu = d >> 1;
        int y[4] = {c.x[0], c.x[1], c.x[2], c.x[3]};
        if ((d & 1) == 0) y[mu] = (y[mu] == g.L[mu] - 1) ? 0 : y[mu] + 1;
        else y[mu] = (y[mu] == 0) ? g.L[mu] - 1 : y[mu] - 1;
        ycb = cb_index(g, y);
      }
      nbs[idx] = ycb;
    }
    __syncthreads();
    // issue direction d into its slot: thread 0 posts the expected bytes,
    // threads 0 .. 6 s_act - 1 each copy one plane run of one site
    auto issue = [&](int d) {
      const int slot = d % kRing;
      if (t < 6 * s_act) {
        if (t == 0) mbar_arrive_expect_tx(&full[slot], 6 * s_act * N5 * 16);
        const unsigned jj = t / 6, k = t - 6 * jj;
        const unsigned ycb = (unsigned)nbs[jj * 8 + d];
        const float4* src = reinterpret_cast<const float4*>(a.in) + (k * N + ycb * N5);
        float4* dst = ring + ((unsigned)slot * 6 + k) * bd + jj * N5;
        bulk_g2s(dst, src, N5 * 16, &full[slot]);
      }
    };
    // the ring was last written by the generic proxy (previous epilogue)
    if (t < 6 * s_act) asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
#pragma unroll
    for (int d = 0; d < kRing; ++d) issue(d);
    {
      const float2* L2 = reinterpret_cast<const float2*>(a.links);
      float* lf = reinterpret_cast<float*>(lsm);
      for (unsigned idx = t; idx < 72u * S; idx += bd) {
        const unsigned jj = idx & (S - 1), dk = idx >> log2S;
        const unsigned d = dk / 9u, k = dk - 9u * d;
        const int cbj = cb0 + (int)jj;
        if (cbj >= g.Vh) continue;
        const int mu = d >> 1;
        const bool fwd = (d & 1) == 0;
        const int site = fwd ? cbj : nbs[jj * 8 + d];
        const int par = fwd ? p : q;
        float2 v = __ldg(L2 + ((unsigned)((par * 4 + mu) * 9) + k) * (unsigned)g.Vh + (unsigned)site);
        unsigned kk = k;
        if (!fwd) {
          kk = (k % 3u) * 3u + k / 3u;
          v.y = -v.y;
        }
        *reinterpret_cast<float2*>(lf + (jj * kHop5LinkStride + d * 5u) * 4u + 2u * kk) = v;
      }
    }
    const long long n = tile * bd + t;
    const int cb = cb0 + (int)j;
    const bool active = cb < g.Vh;
    V res[12];
#pragma unroll
    for (int k = 0; k < 12; ++k) res[k] = cz<R>();
    const R sf = (R)a.sgn;
    const float4* lj = lsm + j * kHop5LinkStride;
#pragma unroll
    for (int mu = 0; mu < 4; ++mu) {
#pragma unroll
      for (int dir = 0; dir < 2; ++dir) {
        const int d = 2 * mu + dir;
        const int slot = d % kRing;
        if (t == 0) s_ok = mbar_wait_bounded(&full[slot], (par_bits >> slot) & 1u) ? 1 : 0;
        par_bits ^= 1u << slot;
        __syncthreads();  // slot d published (and the links); every thread is done with direction d - 1
        if (!s_ok) {
          if (t == 0) {
            atomicExch(&a.ra.st->kernel_error, 1);
            // let any copy of this block still in flight land before the
            // block's shared memory is released (about 0.1 s)
            for (int w = 0; w < 100000; ++w) __nanosleep(1000);
          }
          __syncthreads();
          return;
        }
        if (d >= 1 && d - 1 + kRing < 8) issue(d - 1 + kRing);
        if (active) {
          const bool fwd = dir == 0;
          V psi[12];
          const float4* src = ring + (unsigned)slot * 6 * bd + t;
#pragma unroll
          for (int k = 0; k < 6; ++k) {
            const float4 w = src[k * bd];
            psi[2 * k] = make_float2(w.x, w.y);
            psi[2 * k + 1] = make_float2(w.z, w.w);
          }
          const R s = fwd ? sf : -sf;
          V h[2][3];
#pragma unroll
          for (int r = 0; r < 2; ++r)
#pragma unroll
            for (int col = 0; col < 3; ++col)
              h[r][col] = coefmadd<R>(gcoef(mu, r), s, psi[3 * gperm(mu, r) + col], psi[3 * r + col]);
          V u[10];
#pragma unroll
          for (int c = 0; c < 5; ++c) {
            const float4 w = lj[d * 5 + c];
            u[2 * c] = make_float2(w.x, w.y);
            u[2 * c + 1] = make_float2(w.z, w.w);
          }
          V uh[2][3];
#pragma unroll
          for (int r = 0; r < 2; ++r)
#pragma unroll
            for (int i = 0; i < 3; ++i) {
              V acc = cmul<R>(u[3 * i], h[r][0]);
              acc = cmadd<R>(acc, u[3 * i + 1], h[r][1]);
              uh[r][i] = cmadd<R>(acc, u[3 * i + 2], h[r][2]);
            }
#pragma unroll
          for (int r = 0; r < 2; ++r)
#pragma unroll
            for (int i = 0; i < 3; ++i) res[3 * r + i] = add<R>(res[3 * r + i], uh[r][i]);
#pragma unroll
          for (int r = 2; r < 4; ++r)
#pragma unroll
            for (int i = 0; i < 3; ++i) res[3 * r + i] = coefmadd<R>(gcoef(mu, r), s, uh[gperm(mu, r)][i], res[3 * r + i]);
        }
      }
    }
    __syncthreads();  // the ring becomes the epilogue's shared memory
    hop_epilogue<P32, LK>(a, active, n, cb, res, red_re, red_im, smem_d);
    tile += gridDim.x;
    __syncthreads();  // the next tile refills the ring and the indices
  } while (LOOP && tile < ntiles);
  if (a.red) {
    double* sm = smem_d + (LK == LOC_SMAT ? (24 * blockDim.x + kSmatWords) * sizeof(R) / sizeof(double) + 1 : 0);
    block_reduce_finalize(a.ra, red_re, red_im, g.N5, g.Ls, g.nrhs, sm);
  }
}

// ---------------------------------------------------------------------------
// The double-float hop with two threads per 5D site (one right-hand side,
// per-thread epilogue).  Thread r = 0, 1 of a site projects the half spinor
// h_r = psi_r + s coef psi_perm(r) of every direction, multiplies it by the
// link and accumulates it into upper spin r and into the lower spin that
// takes h_r in that direction; its accumulators (upper spin r, both lower
// spins: 9 double-float complex numbers) live in shared memory.  After the 8
// directions the pair exchanges partial sums through shared memory and
// thread r owns chiral half r (spins 2r, 2r+1; the clover term is
// block-diagonal in the chiral basis) for the epilogue: its 6x6 clover or
// twisted-mass block, the X term, the store and its share of the
// reduction.  Against dslash_kernel<PDD> this halves the registers a thread
// needs (same arithmetic per site), so about twice the warps are resident to
// cover the latency of the double-float operation chains.  The lower spins
// are summed as thread 0's directions plus thread 1's (a fixed order).
// ---------------------------------------------------------------------------
#ifndef GBF_DD2_MINB
#define GBF_DD2_MINB 3
#endif
constexpr int kDD2Acc = 9;  // accumulators per thread: upper spin r (3), lower spins 2, 3 (6)

__device__ __forceinline__ cplx<dd> f4dd(const float4 q) { return mk<dd>(dd(q.x, q.z), dd(q.y, q.w)); }
__device__ __forceinline__ float4 ddf4(cplx<dd> v) {
  nrm<dd>(v);
  return make_float4(v.x.h, v.y.h, v.x.l, v.y.l);
}

// one chiral 6x6 block b of the double-float clover storage applied to w
__device__ __forceinline__ void clover_block_dd(const void* base, int Vh, int cb, int b, ddc (&w)[6]) {
  const float4* pb = reinterpret_cast<const float4*>(base) + cb + 18u * (unsigned)b * (unsigned)Vh;
  ddc o[6];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float4 q = __ldg(pb + (unsigned)k * (unsigned)Vh);
    o[2 * k] = scl<dd>(dd(q.x, q.z), w[2 * k]);
    o[2 * k + 1] = scl<dd>(dd(q.y, q.w), w[2 * k + 1]);
  }
#pragma unroll
  for (int i = 1; i < 6; ++i)
#pragma unroll
    for (int j = 0; j < i; ++j) {
      const float4 q = __ldg(pb + (unsigned)(3 + tri(i, j)) * (unsigned)Vh);
      const ddc cij = mk<dd>(dd(q.x, q.z), dd(q.y, q.w));
      o[i] = cmadd<dd>(o[i], cij, w[j]);
      o[j] = cmaddc<dd>(o[j], cij, w[i]);
    }
#pragma unroll
  for (int i = 0; i < 6; ++i) w[i] = o[i];
}
// site-local op restricted to chiral half b
__device__ __forceinline__ void local_half_dd(const LocalOp& l, int Vh, int parity, int cb, int b, ddc (&w)[6]) {
  if (l.kind == LOC_CLOVER) {
    clover_block_dd(l.clov[parity], Vh, cb, b, w);
  } else if (l.kind == LOC_TWIST) {
    const ddc z = mk<dd>(dd(l.z[2 * b]), dd(l.z[2 * b + 1]));
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      nrm<dd>(w[k]);
      w[k] = cmul<dd>(z, w[k]);
    }
  } else if (l.kind == LOC_SCALAR) {
    const dd sc(l.scalar);
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      nrm<dd>(w[k]);
      w[k] = scl<dd>(sc, w[k]);
    }
  }
}

template <bool LOOP>
__global__ void __launch_bounds__(256, GBF_DD2_MINB) dslash_dd2_kernel(const DslashArgs a) {
  extern __shared__ __align__(16) double smem_d[];
  const Geo& g = a.g;
  if (a.check_done && a.ra.st->all_done) return;
  const int p = a.out_parity, q = 1 - p;
  const unsigned t = threadIdx.x, bs = blockDim.x;
  const unsigned r = t & 1u;
  const unsigned sites = bs >> 1;
  float4* acc = reinterpret_cast<float4*>(smem_d) + t;  // [kDD2Acc][bs]
  const unsigned N = (unsigned)g.N;
  const float4* sp = reinterpret_cast<const float4*>(a.in);
  const float4* lk = reinterpret_cast<const float4*>(a.links);
  double red_re = 0, red_im = 0;
  const long long ntiles = (g.N + sites - 1) / sites;
  long long tile = blockIdx.x;
  do {
    const long long n = tile * sites + (t >> 1);
    const bool active = n < g.N;
    int cb = 0;
    if (active) {
      cb = (int)g.fN5.div((unsigned)n);
      const unsigned i5 = (unsigned)n - (unsigned)cb * (unsigned)g.N5;
      const Coord c = cb_coords(g, cb, p);
#pragma unroll
      for (int k = 0; k < kDD2Acc; ++k) acc[k * bs] = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll 1
      for (int d = 0; d < 8; ++d) {
        const int mu = d >> 1;
        const bool fwd = (d & 1) == 0;
        int y[4];
#pragma unroll
        for (int m = 0; m < 4; ++m) {
          const int xm = c.x[m], Lm = g.L[m];
          y[m] = (m != mu) ? xm : fwd ? (xm == Lm - 1 ? 0 : xm + 1) : (xm == 0 ? Lm - 1 : xm - 1);
        }
        const int ycb = cb_index(g, y);
        const unsigned site = (unsigned)ycb * (unsigned)g.N5 + i5;
        const float s = fwd ? a.sgn : -a.sgn;
        const int pr = gperm(mu, (int)r), cr = gcoef(mu, (int)r);
#ifndef GBF_DD_SCALAR
        {
          // lane-paired form: a complex double-float is one pdd, u h is
          // Re(u) h + Im(u) (i h), two lane-wise fmas per link entry
          pdd h[3], ih[3];
#pragma unroll
          for (int col = 0; col < 3; ++col) {
            const pdd up = pdd_ld(__ldg(sp + (site + (3u * r + col) * N)));
            const pdd lo = pdd_ld(__ldg(sp + (site + (unsigned)(3 * pr + col) * N)));
            h[col] = pdd_coefmadd_rt(cr, s, lo, up);
            ih[col] = pdd_i(h[col]);
          }
          const int rl = (gperm(mu, 2) == (int)r) ? 2 : 3;
          const int cl = gcoef(mu, rl);
          const float4* L = lk + (unsigned)(((fwd ? p : q) * 4 + mu) * 9) * (unsigned)g.Vh + (unsigned)(fwd ? cb : ycb);
          const float cs = fwd ? 1.f : -1.f;
#pragma unroll
          for (int i = 0; i < 3; ++i) {
            pdd uh;
#pragma unroll
            for (int j = 0; j < 3; ++j) {
              const unsigned k = fwd ? (unsigned)(3 * i + j) : (unsigned)(3 * j + i);
              const float4 qv = __ldg(L + k * (unsigned)g.Vh);
              const dd ux(qv.x, qv.z), uy = dd_scale2(cs, dd(qv.y, qv.w));  // U or U^dagger entry
              uh = j == 0 ? pdd_mul_s(ux, h[j]) : pdd_fma_s(ux, h[j], uh);
              uh = pdd_fma_s(uy, ih[j], uh);
            }
            // (the sums leave pdd_add normalised)
            float4& m = acc[i * bs];
            m = pdd_st(pdd_add(pdd_ld(m), uh));
            float4& ml = acc[(3 + 3 * (rl - 2) + i) * bs];
            ml = pdd_st(pdd_coefmadd_rt(cl, s, uh, pdd_ld(ml)));
          }
        }
#else
        cplx<dd> h[3];
#pragma unroll
        for (int col = 0; col < 3; ++col) {
          const cplx<dd> up = f4dd(__ldg(sp + (site + (3u * r + col) * N)));
          const cplx<dd> lo = f4dd(__ldg(sp + (site + (unsigned)(3 * pr + col) * N)));
          h[col] = coefmadd_rt(cr, s, lo, up);
        }
        // the lower spin that takes h_r in this direction, and its coefficient
        const int rl = (gperm(mu, 2) == (int)r) ? 2 : 3;
        const int cl = gcoef(mu, rl);
        const float4* L = lk + (unsigned)(((fwd ? p : q) * 4 + mu) * 9) * (unsigned)g.Vh + (unsigned)(fwd ? cb : ycb);
        const float cs = fwd ? 1.f : -1.f;
#pragma unroll
        for (int i = 0; i < 3; ++i) {
          cplx<dd> u[3];
#pragma unroll
          for (int j = 0; j < 3; ++j) {
            const unsigned k = fwd ? (unsigned)(3 * i + j) : (unsigned)(3 * j + i);
            const float4 qv = __ldg(L + k * (unsigned)g.Vh);
            u[j] = mk<dd>(dd(qv.x, qv.z), dd_scale2(cs, dd(qv.y, qv.w)));  // U or U^dagger entry
          }
          cplx<dd> uh = cmul<dd>(u[0], h[0]);
          uh = cmadd<dd>(uh, u[1], h[1]);
          uh = cmadd<dd>(uh, u[2], h[2]);
          float4& m = acc[i * bs];
          m = ddf4(add<dd>(f4dd(m), uh));
          float4& ml = acc[(3 + 3 * (rl - 2) + i) * bs];
          ml = ddf4(coefmadd_rt(cl, s, uh, f4dd(ml)));
        }
#endif
      }
    }
    __syncwarp();  // the partner's accumulators are visible
    ddc w[6];
    if (active) {
      const float4* mine = reinterpret_cast<const float4*>(smem_d) + t;
      const float4* other = reinterpret_cast<const float4*>(smem_d) + (t ^ 1u);
      if (r == 0) {  // spins 0 and 1: own upper sums and the partner's
#pragma unroll
        for (int i = 0; i < 3; ++i) {
          w[i] = f4dd(mine[i * bs]);
          w[3 + i] = f4dd(other[i * bs]);
        }
      } else {  // spins 2 and 3: thread 0's partial plus thread 1's
#pragma unroll
        for (int k = 0; k < 6; ++k) w[k] = add<dd>(f4dd(other[(3 + k) * bs]), f4dd(mine[(3 + k) * bs]));
      }
    }
    __syncwarp();  // both halves read before the next tile overwrites
    if (active) {
      const unsigned b = r;
      if (a.l1.kind != LOC_NONE) local_half_dd(a.l1, g.Vh, p, cb, (int)b, w);
      if (a.c1 != 1.0) {
        const dd c1(a.c1);
#pragma unroll
        for (int k = 0; k < 6; ++k) {
          nrm<dd>(w[k]);
          w[k] = scl<dd>(c1, w[k]);
        }
      }
      const float4* Xp = reinterpret_cast<const float4*>(a.X);
      if (Xp) {
        ddc xv[6];
#pragma unroll
        for (int k = 0; k < 6; ++k) xv[k] = f4dd(__ldg(Xp + ((unsigned)n + (6u * b + k) * N)));
        if (a.l2.kind != LOC_NONE) local_half_dd(a.l2, g.Vh, p, cb, (int)b, xv);
        const dd c2(a.c2);
#pragma unroll
        for (int k = 0; k < 6; ++k) w[k] = mk<dd>(fma(c2, xv[k].x, w[k].x), fma(c2, xv[k].y, w[k].y));
      }
      float4* out = reinterpret_cast<float4*>(a.out);
#pragma unroll
      for (int k = 0; k < 6; ++k) out[(unsigned)n + (6u * b + k) * N] = ddf4(w[k]);
      if (a.red) {
        double vr = 0, vi = 0;
        dd sr = rzero<dd>(), si = rzero<dd>();
        if (a.red == 1) {
          const float4* Yp = reinterpret_cast<const float4*>(a.Y);
#pragma unroll
          for (int k = 0; k < 6; ++k) {
            ddc yv = f4dd(__ldg(Yp + ((unsigned)n + (6u * b + k) * N)));
            ddc wk = w[k];
            nrm<dd>(yv);
            nrm<dd>(wk);
            sr = fma(yv.x, wk.x, sr);
            sr = fma(yv.y, wk.y, sr);
            si = fma(yv.x, wk.y, si);
            si = fma(-yv.y, wk.x, si);
          }
        } else {
#pragma unroll
          for (int k = 0; k < 6; ++k) {
            ddc wk = w[k];
            nrm<dd>(wk);
            sr = fma(wk.x, wk.x, sr);
            sr = fma(wk.y, wk.y, sr);
          }
        }
        vr = (double)sr;
        vi = (double)si;
        red_re += vr;
        red_im += vi;
      }
    }
    tile += gridDim.x;
    if (LOOP) __syncthreads();
  } while (LOOP && tile < ntiles);
  if (a.red) {
    double* sm = smem_d + (size_t)kDD2Acc * bs * 2;  // after the accumulators
    block_reduce_finalize(a.ra, red_re, red_im, 1, 1, 1, sm);
  }
}

// ---------------------------------------------------------------------------
// host-side launcher
// ---------------------------------------------------------------------------
static int sm_count() {
  static const int sms = [] {
    int d = 0, c = 152;
    if (cudaGetDevice(&d) == cudaSuccess) cudaDeviceGetAttribute(&c, cudaDevAttrMultiProcessorCount, d);
    return c;
  }();
  return sms;
}

// Blocks of `kernel` resident per SM at block size bd and dynamic shared
// memory smem; cached per (kernel, bd, smem).  Also raises the kernel's
// dynamic shared-memory limit to the largest smem requested so far (the limit
// only grows, so every cached configuration stays launchable).
int resident_blocks(const void* kernel, int bd, size_t smem) {
  static std::mutex mu;
  static std::map<std::tuple<const void*, int, size_t>, int> cache;
  static std::map<const void*, size_t> limit;
  const auto key = std::make_tuple(kernel, bd, smem);
  std::lock_guard<std::mutex> lock(mu);
  auto it = cache.find(key);
  if (it != cache.end()) return it->second;
  // (raised for every size above the current limit: a kernel's static shared
  // memory counts against the same 48 KB default as the dynamic request)
  if (smem > limit[kernel]) {
    cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    limit[kernel] = smem;
  }
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kernel, bd, smem) != cudaSuccess || nb < 1) {
    cudaGetLastError();
    nb = 1;
  }
  cache[key] = nb;
  return nb;
}

// Grid of a reducing launch: one full wave of resident blocks (every block
// then loops over an equal share of the tiles, with no partial last wave),
// and no more blocks than tiles.  The [block][rhs] partials stay few.
// min_partials > 0 allows more blocks, up to min_partials / nrhs, before the
// grid is capped (for kernels whose looping variant is slower).
long long reduce_grid(long long ntiles, int nrhs, int resident, long long min_partials) {
  long long cap = (long long)sm_count() * (resident > 0 ? resident : 1);
  const long long alt = min_partials / (nrhs > 0 ? nrhs : 1);
  if (alt > cap) cap = alt;
  return ntiles < cap ? ntiles : cap;
}

int block_size_for(int N5, int LK) {
  // blockDim = S * N5 with S a power of two and blockDim <= 256
  int S = 1;
  while (S * 2 * N5 <= 256) S *= 2;
  (void)LK;
  return N5 > 256 ? -1 : S * N5;
}

int pick_bd(int requested, int N5) {
  if (requested > 0 && requested <= 256 && requested % N5 == 0) {
    const int S = requested / N5;
    if ((S & (S - 1)) == 0) return requested;
  }
  return block_size_for(N5, 0);
}

size_t dslash_smem_bytes(int P, int LK, int bd) {
  size_t rb = (P == P64 || P == PDD) ? 8 : 4;
  size_t s = 0;
  if (LK == LOC_SMAT) s += (24 * (size_t)bd + kSmatWords) * rb + 8;
  s += 2 * (size_t)bd * 8;
  if (P == PDD) s = 16 * (size_t)dd_acc_offset16(LK, bd) + 12 * 16 * (size_t)bd;  // + accumulators
  return s;
}

// The double-float kernel's looping variant needs more registers (spills):
// its reducing launches keep one tile per block up to 4096 blocks.
static long long dslash_min_partials(int P) { return P == PDD ? 4096 : 0; }

template <int P, int LS, int LK, bool LOOP>
static cudaError_t launch_tl(const DslashArgs& a, cudaStream_t st) {
  const int bd = pick_bd(a.bd, a.g.N5);
  if (bd <= 0) return cudaErrorInvalidValue;
  const long long ntiles = (a.g.N + bd - 1) / bd;
  const size_t sm = dslash_smem_bytes(P, LK, bd);
  auto k = dslash_kernel<P, LS, LK, LOOP>;
  const int res = resident_blocks((const void*)k, bd, sm);
  const long long nb = a.red ? reduce_grid(ntiles, a.g.nrhs, res, dslash_min_partials(P)) : ntiles;
  k<<<(unsigned)nb, bd, sm, st>>>(a);
  return cudaGetLastError();
}

// hop5: the epilogue's shared memory first, then the links and indices
// Order of the hop5 tiles for tiles of S 4D sites.  The brick is
// min(S, 4) sites in x0/2 by the rest in x1 where those divide the lattice,
// else S consecutive sites.  The slab depth T (x2 planes) is the largest
// divisor of L2 below L2 (a multiple of the brick's x2 extent) whose three x3
// steps (T planes each; input, output and X term) stay within 64 MB of L2;
// no slabs when the whole field fits in 64 MB.  GBF_HOP5_SLAB=<T> forces T
// (0: none); GBF_HOP5_BRICK=<b0,b1,b2,b3> forces the brick (0: consecutive
// sites).
static Hop5Order hop5_order(const DslashArgs& a, int S) {
  static const int forced_slab = [] {
    const char* e = std::getenv("GBF_HOP5_SLAB");
    return e ? std::atoi(e) : -1;
  }();
  static const std::array<int, 4> forced_brick = [] {
    std::array<int, 4> b{-1, -1, -1, -1};
    const char* e = std::getenv("GBF_HOP5_BRICK");
    if (e) {
      if (std::sscanf(e, "%d,%d,%d,%d", &b[0], &b[1], &b[2], &b[3]) != 4) b = {0, 0, 0, 0};
    }
    return b;
  }();
  const Geo& g = a.g;
  Hop5Order o{-1, 0, 0, 0, 0};
  int br[4] = {S < 4 ? S : 4, S < 4 ? 1 : S / 4, 1, 1};
  if (forced_brick[0] >= 0) {
    for (int i = 0; i < 4; ++i) br[i] = forced_brick[i];
  }
  const int ext[4] = {g.Lh0, g.L[1], g.L[2], g.L[3]};
  bool brick = br[0] > 0 && (long long)br[0] * br[1] * br[2] * br[3] == S;
  for (int i = 0; i < 4 && brick; ++i) brick = br[i] > 0 && (br[i] & (br[i] - 1)) == 0 && ext[i] % br[i] == 0;
  const long long P = (long long)g.Lh0 * g.L[1];
  if (!brick && P % S) return o;
  const int bz = brick ? br[2] : 1;
  const double step = (double)P * g.N5 * 96.0 * (a.X ? 3 : 2);
  int T = 0;
  if (forced_slab >= 0) {
    T = (forced_slab > 0 && forced_slab < g.L[2] && g.L[2] % forced_slab == 0 && forced_slab % bz == 0) ? forced_slab : 0;
  } else if ((double)g.L[2] * g.L[3] * step > 64e6) {
    for (int t = bz; t < g.L[2]; t += bz)
      if (g.L[2] % t == 0 && 3.0 * t * step <= 64e6) T = t;
  }
  if (brick) {
    int l[4];
    for (int i = 0; i < 4; ++i) {
      l[i] = 0;
      while ((1 << l[i]) < br[i]) ++l[i];
    }
    o = Hop5Order{l[0], l[1], l[2], l[3], T ? T : g.L[2]};
  } else {
    o.slabT = T;
  }
  return o;
}

template <int P, int LK, bool LOOP>
static cudaError_t launch_hop5_tl(const DslashArgs& a, int bd, cudaStream_t st) {
  const int S = bd / a.g.N5;
  int log2S = 0;
  while ((1 << log2S) < S) ++log2S;
  const size_t epi = dslash_smem_bytes(P, LK, bd);
  const unsigned off16 = (unsigned)((epi + 15) / 16);
  const size_t sm = 16 * (size_t)off16 + hop5_extra_smem(S);
  const long long ntiles = (a.g.N + bd - 1) / bd;
  auto k = hop5_kernel<P, LK, LOOP>;
  const int res = resident_blocks((const void*)k, bd, sm);
  const long long nb = a.red ? reduce_grid(ntiles, a.g.nrhs, res) : ntiles;
  k<<<(unsigned)nb, bd, sm, st>>>(a, off16, log2S, hop5_order(a, S));
  return cudaGetLastError();
}

template <int P, int LK>
static cudaError_t launch_hop5(const DslashArgs& a, cudaStream_t st) {
  const int bd = pick_bd(a.bd, a.g.N5);
  if (bd <= 0) return cudaErrorInvalidValue;
  const int S = bd / a.g.N5;
  const size_t sm = 16 * ((dslash_smem_bytes(P, LK, bd) + 15) / 16) + hop5_extra_smem(S);
  const long long ntiles = (a.g.N + bd - 1) / bd;
  const int res = resident_blocks((const void*)hop5_kernel<P, LK, true>, bd, sm);
  const bool loop = a.red && reduce_grid(ntiles, a.g.nrhs, res) < ntiles;
  return loop ? launch_hop5_tl<P, LK, true>(a, bd, st) : launch_hop5_tl<P, LK, false>(a, bd, st);
}

// the bulk-copy hop: ring (also the epilogue's region), links, indices, barriers
static size_t hop5t_links_off(int LK, int bd) {
  const size_t ring = hop5t_ring_bytes(bd), epi = dslash_smem_bytes(P32, LK, bd);
  return ((ring > epi ? ring : epi) + 15) / 16 * 16;
}
static size_t hop5t_smem(int LK, int bd, int S) { return hop5t_links_off(LK, bd) + hop5_extra_smem(S) + kRing * 8; }
template <int LK, bool LOOP>
static cudaError_t launch_hop5t_tl(const DslashArgs& a, int bd, cudaStream_t st) {
  const int S = bd / a.g.N5;
  int log2S = 0;
  while ((1 << log2S) < S) ++log2S;
  const size_t sm = hop5t_smem(LK, bd, S);
  const long long ntiles = (a.g.N + bd - 1) / bd;
  auto k = hop5t_kernel<LK, LOOP>;
  const int res = resident_blocks((const void*)k, bd, sm);
  const long long nb = a.red ? reduce_grid(ntiles, a.g.nrhs, res) : ntiles;
  k<<<(unsigned)nb, bd, sm, st>>>(a, log2S, (unsigned)(hop5t_links_off(LK, bd) / 16));
  return cudaGetLastError();
}
template <int LK>
static cudaError_t launch_hop5t(const DslashArgs& a, cudaStream_t st) {
  const int bd = pick_bd(a.bd, a.g.N5);
  if (bd <= 0) return cudaErrorInvalidValue;
  const int S = bd / a.g.N5;
  const long long ntiles = (a.g.N + bd - 1) / bd;
  const int res = resident_blocks((const void*)hop5t_kernel<LK, true>, bd, hop5t_smem(LK, bd, S));
  const bool loop = a.red && reduce_grid(ntiles, a.g.nrhs, res) < ntiles;
  return loop ? launch_hop5t_tl<LK, true>(a, bd, st) : launch_hop5t_tl<LK, false>(a, bd, st);
}

// the two-threads-per-site double-float hop (one rhs, per-thread epilogue)
static size_t dd2_smem(int bd) { return (size_t)kDD2Acc * 16 * bd + 2 * 8 * (size_t)bd; }
template <bool LOOP>
static cudaError_t launch_dd2_tl(const DslashArgs& a, cudaStream_t st) {
  const int bd = 256, sites = bd / 2;
  const long long ntiles = (a.g.N + sites - 1) / sites;
  const size_t sm = dd2_smem(bd);
  auto k = dslash_dd2_kernel<LOOP>;
  const int res = resident_blocks((const void*)k, bd, sm);
  const long long nb = a.red ? reduce_grid(ntiles, 1, res) : ntiles;
  k<<<(unsigned)nb, bd, sm, st>>>(a);
  return cudaGetLastError();
}
static cudaError_t launch_dd2(const DslashArgs& a, cudaStream_t st) {
  const long long ntiles = (a.g.N + 127) / 128;
  const int res = resident_blocks((const void*)dslash_dd2_kernel<true>, 256, dd2_smem(256));
  const bool loop = a.red && reduce_grid(ntiles, 1, res) < ntiles;
  return loop ? launch_dd2_tl<true>(a, st) : launch_dd2_tl<false>(a, st);
}
static bool dd2_enabled();

template <int P, int LS, int LK>
static cudaError_t launch_t(const DslashArgs& a, cudaStream_t st) {
  // the pure hop (no site-local term, no X, no reduction) of one rhs: two
  // threads per site measured faster there (12.34 -> 11.55 ms on the
  // reference's Dhop benchmark); with the clover epilogue it was slower
  // (0.328 -> 0.345 ms per launch at 32^4), so the CG launches keep one thread
  if (P == PDD && LK != LOC_SMAT && a.g.nrhs == 1 && a.l1.kind == LOC_NONE && !a.X && !a.red && dd2_enabled())
    return launch_dd2(a, st);
  const int bd = pick_bd(a.bd, a.g.N5);
  if (bd <= 0) return cudaErrorInvalidValue;
  const long long ntiles = (a.g.N + bd - 1) / bd;
  const int res = resident_blocks((const void*)dslash_kernel<P, LS, LK, true>, bd, dslash_smem_bytes(P, LK, bd));
  const bool loop = a.red && reduce_grid(ntiles, a.g.nrhs, res, dslash_min_partials(P)) < ntiles;
  return loop ? launch_tl<P, LS, LK, true>(a, st) : launch_tl<P, LS, LK, false>(a, st);
}

// GBF_HOP5 in the environment selects the hop of FP32/FP16 fields with an
// inner extent >= 8: unset or 1 the shared-memory link hop (hop5_kernel),
// 0 the per-thread hop, 2 the bulk-copy staged hop (hop5t_kernel, FP32);
// results are bitwise equal, the default is the fastest measured
static bool hop5_enabled() {
  static const bool on = [] {
    const char* e = std::getenv("GBF_HOP5");
    return !(e && e[0] == '0');
  }();
  return on;
}
// GBF_DD2=0 selects the one-thread-per-site double-float hop everywhere
static bool dd2_enabled() {
  static const bool on = [] {
    const char* e = std::getenv("GBF_DD2");
    return !(e && e[0] == '0');
  }();
  return on;
}
static bool hop5_bulk() {
  static const bool on = [] {
    const char* e = std::getenv("GBF_HOP5");
    return e && e[0] == '2';
  }();
  return on;
}

cudaError_t launch_dslash(int P, int LS, const DslashArgs& a, cudaStream_t st) {
  const int LK = (a.l1.kind == LOC_SMAT || a.l2.kind == LOC_SMAT) ? LOC_SMAT : LOC_CLOVER;
  // FP32 fields with an inner extent of 8 or more: the bulk-copy hop when
  // selected (GBF_HOP5=2), otherwise the shared-memory link hop
  if (hop5_bulk() && a.g.N5 >= 8 && LS == L32 && P == P32)
    return LK == LOC_SMAT ? launch_hop5t<LOC_SMAT>(a, st) : launch_hop5t<LOC_CLOVER>(a, st);
  if (hop5_enabled() && a.g.N5 >= 8 && LS == L32 && (P == P32 || P == P16)) {
    if (P == P32) return LK == LOC_SMAT ? launch_hop5<P32, LOC_SMAT>(a, st) : launch_hop5<P32, LOC_CLOVER>(a, st);
    return LK == LOC_SMAT ? launch_hop5<P16, LOC_SMAT>(a, st) : launch_hop5<P16, LOC_CLOVER>(a, st);
  }
#define GBF_D(PP, LL)                                                     \
  if (P == PP && LS == LL) {                                             \
    if (LK == LOC_SMAT) return launch_t<PP, LL, LOC_SMAT>(a, st);        \
    return launch_t<PP, LL, LOC_CLOVER>(a, st);                          \
  }
  GBF_D(P64, L64)
  GBF_D(P32, L32)
  GBF_D(P32, L32R)
  GBF_D(P16, L32)
  GBF_D(P16, L32R)
  GBF_D(PDD, LDD)
#undef GBF_D
  return cudaErrorInvalidValue;
}

// number of blocks a launch uses (reduction partial buffers are sized by it)
long long dslash_blocks(const Geo& g, int LK) {
  const int bd = block_size_for(g.N5, LK);
  return (g.N + bd - 1) / bd;
}

}  // namespace gbf
