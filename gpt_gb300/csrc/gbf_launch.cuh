// gbf_launch.cuh -- argument blocks and host launchers of the device kernels.
#pragma once
#include "gbf_kernels.cuh"

namespace gbf {

// Even-odd hopping kernel (gbf_dslash.cu):
//   out = c1 * L1(Dhop_{p <- 1-p}(in)) + c2 * L2(X)  [+ reduction of <Y,out> or |out|^2]
struct DslashArgs {
  Geo g;
  int out_parity;
  float sgn;  // projector sign on the forward term: -1 Dhop, +1 Dhop^dag
  const void* in;
  void* out;
  const void* links;
  LocalOp l1, l2;  // l2 may not be LOC_SMAT
  double c1, c2;
  const void* X;
  int red;  // 0 none, 1 <Y,out>, 2 |out|^2
  const void* Y;
  RedArgs ra;
  int check_done;
  int bd;  // block size (0: default); a multiple of N5 with a power-of-two quotient, <= 256
};
cudaError_t launch_dslash(int P, int LS, const DslashArgs& a, cudaStream_t st);
int block_size_for(int N5, int LK);
// requested block size if valid for N5, else the default
int pick_bd(int requested, int N5);
long long reduce_grid(long long ntiles, int nrhs, int resident, long long min_partials = 0);
int resident_blocks(const void* kernel, int bd, size_t smem);
long long dslash_blocks(const Geo& g, int LK);

// Site-local kernel on one parity (gbf_local.cu):
//   if (pre):  W = A + beta_rhs * W   (beta from the CG state; written back)
//   out = c1 * L(W or A) + c2 * X       [+ reduction as above on `out`]
struct LocalArgs {
  Geo g;
  int parity;
  const void* A;
  void* W;       // pre-step target (p in CG), may be null
  int pre;       // 1: W = A + beta*W before the op
  LocalOp l;
  void* out;
  double c1, c2;
  const void* X;
  int red;
  const void* Y;
  RedArgs ra;
  int check_done;
  int bd;
};
cudaError_t launch_local(int P, const LocalArgs& a, cudaStream_t st);

// CG update (gbf_local.cu): r -= alpha*mmp; x += alpha*p; reduce |r|^2 -> FIN_BETA
struct CGUpdateArgs {
  Geo g;
  void* r;
  const void* mmp;
  void* x;
  const void* p;
  RedArgs ra;
  int bd;
};
cudaError_t launch_cg_update(int P, const CGUpdateArgs& a, cudaStream_t st);

// Generic BLAS over one half field (gbf_local.cu):
//   out = a_rhs * x + b_rhs * y  (a, b per rhs, from host arrays in the args)
//   then optional reduction: 1 <Y,out>, 2 |out|^2, 3 <x, y> (no write)
struct BlasArgs {
  Geo g;
  void* out;
  const void* x;
  const void* y;
  double a_re[kMaxRhs], a_im[kMaxRhs], b_re[kMaxRhs];
  int write;
  int red;
  RedArgs ra;
};
cudaError_t launch_blas(int P, const BlasArgs& a, cudaStream_t st);

// precision conversion of a half field
cudaError_t launch_convert(int Pout, void* out, int Pin, const void* in, long long N, double scale, cudaStream_t st);

// CG state initialisation from the FIN_STORE result: rsq = eps^2 * last, cp = last
cudaError_t launch_cg_init(CGState* st, int nrhs, double eps, int maxiter, cudaStream_t s);

// natural <-> internal field transfer; natural = complex128 [V][Ls][12] of one rhs
cudaError_t launch_import(int P, const Geo& g, const double2* nat, void* full, int rhs, int to_natural, cudaStream_t st);

// gauge packing: natural complex128 [4][V][9] on the device -> internal links
cudaError_t launch_pack_links(int LS, const Geo& g, const double2* U, void* links, const double* lam_mu, const double* ph,
                              unsigned* err_bits, cudaStream_t st);
// clover: natural gauge -> per parity clover and inverse (FP64 double2[36][Vh] and FP32 float4[18][Vh])
cudaError_t launch_clover(const Geo& g, const double2* U, double diag, double csw_r, double csw_t, void* c64, void* ci64,
                          void* c32, void* ci32, unsigned* err_bits, cudaStream_t st);

// set_mass of a clover operator: clover diagonal += shift (both parities and
// blocks, in place, in the operator's storage precision) and the inverse
// blocks rebuilt; err receives a large value for a singular block
cudaError_t launch_clover_shift(int prec, void* clov, void* clov_inv, int Vh, double shift, unsigned* err, cudaStream_t st);

// FP64 clover storage (double2 [2*nrows32][Vh]) -> FP32 (float4 [nrows32][Vh]);
// nrows32 is a row count (18 per parity block), not an element count
cudaError_t launch_clover_narrow(const void* src64, void* dst32, long long nrows32, int Vh, cudaStream_t st);
// the same from double-float storage (float4 (x.h, y.h, x.l, y.l) per double2)
cudaError_t launch_clover_narrow_dd(const void* srcdd, void* dst32, long long nrows32, int Vh, cudaStream_t st);
// FP64 complex array -> double-float (float4 per complex), n_complex elements
cudaError_t launch_split_dd(const void* src64, void* dst, long long n_complex, cudaStream_t st);

// block CG (gbf_block.cu): Gram matrix out[i k + j] = sum conj(A_i) . B_j of the
// k = nrhs packed vectors (partial: max_blocks x k x k entries; counter zero
// on entry, restored), and out_i = beta Y_i + sum_j X_j W[j k + i]
cudaError_t launch_gram(int P, const Geo& g, const void* A, const void* B, double2* partial, long long max_blocks,
                        unsigned* counter, double2* out, cudaStream_t st);
int gram_launches(int P, const Geo& g);
cudaError_t launch_lincomb(int P, const Geo& g, void* out, const void* Y, double beta, const void* X, const double2* W,
                           cudaStream_t st);
// multi-shift CG update over the active shifts: x_j += a_j p_j ; p_j = b_j p_j + g_j r
constexpr int kMaxShifts = 32;
struct MultiShiftArgs {
  const void* r;
  void* x[kMaxShifts];
  void* p[kMaxShifts];
  double a[kMaxShifts], b[kMaxShifts], g[kMaxShifts];
  int n;
};
cudaError_t launch_multishift(int P, const Geo& g, const MultiShiftArgs& a, cudaStream_t st);

// out1 = b1 Y1 + X1 W1 ; out2 = b2 Y2 + c out1 + X2 W2 in one pass
cudaError_t launch_lincomb2(int P, const Geo& g, void* out1, const void* Y1, double b1, const void* X1, const double2* W1,
                            void* out2, const void* Y2, double b2, double c, const void* X2, const double2* W2,
                            cudaStream_t st);

// mode representation (gbf_block.cu): inner products of a block of separate
// fields with one field, and their linear combination
constexpr int kModeBlock = 8;
struct ModeDotArgs {
  const void* v[kModeBlock];
  int n;
  const void* src;
  double2* partial;   // [gridDim][n]
  unsigned* counter;  // zero on entry, restored
  double2* out;       // out[j] = sum conj(v_j) . src
};
struct ModeAxpyArgs {
  const void* v[kModeBlock];
  double2 w[kModeBlock];
  int n;
  void* out;       // out = (accumulate ? out : 0) + sum_j w_j v_j
  int accumulate;
};
cudaError_t launch_mode_dot(int P, const Geo& g, const ModeDotArgs& a, long long max_partials, cudaStream_t st);
cudaError_t launch_mode_axpy(int P, const Geo& g, const ModeAxpyArgs& a, cudaStream_t st);

// fifth-dimension moves of the MADWF preconditioner (gbf_local.cu):
// dst_s = P- src_s + P+ src_{s + offset}, and a slice copy between fields of
// possibly different Ls (same 4D geometry and nrhs, one half)
cudaError_t launch_chiral_shift(int P, const Geo& g, const void* src, void* dst, int offset, cudaStream_t st);
cudaError_t launch_copy_slices(int P, const Geo& gd, void* dst, int d0, const Geo& gs, const void* src, int s0, int count,
                               double scale, cudaStream_t st);

}  // namespace gbf
