/*
 * gbferm.h -- C ABI of the GB300 fermion-matrix library (libgbferm.so).
 *
 * This is the drop-in boundary for gpt's fermion hot path.  The reference
 * reaches Grid through the cgpt CPython functions of
 * lib/cgpt/lib/operators.cc:34-133 (create / update / set_mass / delete /
 * apply_fermion_operator) with the opcode numbers generated from
 * lib/cgpt/lib/operators/types.h:26-65; the entry points below take their
 * place, with plain pointers and sizes instead of Python objects.
 *
 * Conventions
 *  - All field pointers are DEVICE pointers in the library's internal layout
 *    unless a function says otherwise.  A half (checkerboard) field holds
 *    N = V/2 * Ls * n_rhs "5D sites"; its size is gbf_field_bytes(op, 0).
 *    A full field is [even half][odd half].
 *  - "natural" layout (host interface, as in gpt's numpy views):
 *    complex128 [V][Ls][4 spin][3 colour], site = x0 + L0*(x1 + L1*(x2 + L2*x3));
 *    the gauge field is complex128 [4][V][3][3].
 *  - Every call returns 0 on success or a positive error class
 *    (GBF_E_*); gbf_last_error() gives the message of the calling thread.
 *    No exception crosses this boundary.
 *  - `stream` is a cudaStream_t (NULL = legacy default stream).  Calls are
 *    stream-ordered; functions that return host values synchronise the stream.
 *  - Distinct operators may be used from distinct threads concurrently; one
 *    operator must not be used by two threads at once.
 */
#ifndef GBFERM_H
#define GBFERM_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct gbf_op gbf_op;

/* precision (cgpt: "single" / "double", operators.cc:36-57).  GBF_HALF: FP16
 * spinors with a per-site FP32 scale, FP32 arithmetic.  GBF_DOUBLE_FLOAT (no
 * counterpart in the reference): spinors, links, clover and arithmetic in
 * double-float numbers, value = h + l of two FP32 words (48-bit significand,
 * relative rounding ~2^-48 per operation), the same 8 bytes per real as FP64;
 * FP64-class results computed on the FP32 pipe. */
enum { GBF_DOUBLE = 0, GBF_SINGLE = 1, GBF_HALF = 2, GBF_DOUBLE_FLOAT = 3 };
/* checkerboards (lib/gpt/core/checkerboard.py:22-25) */
enum { GBF_EVEN = 0, GBF_ODD = 1, GBF_FULL = 2 };
/* error classes */
enum { GBF_OK = 0, GBF_E_ARG = 1, GBF_E_OOM = 2, GBF_E_CUDA = 3, GBF_E_NOCONV = 4, GBF_E_UNSUPPORTED = 5 };

/* opcodes: same numbers as lib/cgpt/lib/operators/types.h via lib/gpt/qcd/fermion/register.py */
enum {
  GBF_M = 2001, GBF_MDAG = 2002, GBF_MEOOE = 2003, GBF_MEOOE_DAG = 2004,
  GBF_MOOEE = 2005, GBF_MOOEE_DAG = 2006, GBF_MOOEE_INV = 2007, GBF_MOOEE_INV_DAG = 2008,
  GBF_MDIAG = 2009, GBF_DMINUS = 2010, GBF_DMINUS_DAG = 2011,
  GBF_IMPORT_PHYSICAL_FERMION_SOURCE = 2012, GBF_IMPORT_UNPHYSICAL_FERMION = 2013,
  GBF_EXPORT_PHYSICAL_FERMION_SOLUTION = 2014, GBF_EXPORT_PHYSICAL_FERMION_SOURCE = 2015,
  GBF_DHOP = 3001, GBF_DHOP_EO = 3002, GBF_DHOP_DAG = 4001, GBF_DHOP_EO_DAG = 4002
};

/* Operator parameters: the keys of the reference's params dict
 * (lib/cgpt/lib/operators/wilson_clover.h:28-39, mobius.h:42-51). */
typedef struct {
  int dims[4];                /* L0..L3, L0 even */
  int Ls;                     /* mobius 5th dimension; 1 for wilson_clover */
  int n_rhs;                  /* right-hand sides packed into one field (1..16) */
  double mass;                /* wilson_clover m0 (kappa converted by the caller) */
  double csw_r, csw_t, xi_0, nu;
  int isAnisotropic;
  double boundary_phases[8];  /* 4 complex numbers (re, im) */
  double mass_plus, mass_minus, b, c, M5;
  int reconstruct;            /* -1 auto, 0: 18 reals per link, 1: 12 reals (SU(3), FP32/FP16) */
  double mu;                  /* wilson_twisted_mass: Mooee = (4 + mass) + i mu gamma5 */
  const double* omega;        /* zmobius: Ls complex omega_s as (re, im) pairs (read by gbf_create only) */
} gbf_params;

/* cgpt create_fermion_operator (operators.cc:34-57): name is "wilson_clover",
 * "wilson_twisted_mass" (operators/wilson_twisted_mass.h:19-45: isotropic
 * Wilson hop, no clover), "mobius" or "zmobius" (operators/zmobius.h: complex
 * per-slice b_s, c_s from omega, lib/gpt/qcd/fermion/zmobius.py:31-34).  Allocates device storage; the gauge field is set by
 * gbf_update_gauge before first use. */
int gbf_create(const char* name, int precision, const gbf_params* params, gbf_op** out);

/* cgpt update_fermion_operator (operators.cc:59-72): import the gauge field,
 * natural layout complex128 [4][V][3][3], host (on_device = 0) or device
 * memory.  Builds links, the clover term and its inverse on the device. */
int gbf_update_gauge(gbf_op* op, const void* U, int on_device, void* stream);

/* gbf_update_gauge for an operator that differs from `clover_from` only in
 * precision (base.py:230-231 `converted`): the links are packed from U and
 * the clover term and its inverse are converted from `clover_from` instead
 * of being rebuilt.  Falls back to the full build when the two operators'
 * geometry or clover parameters differ. */
int gbf_update_gauge_from(gbf_op* op, const void* U, int on_device, const gbf_op* clover_from, void* stream);

/* cgpt set_mass_fermion_operator (operators.cc:74-83; the per-action
 * semantics of lib/cgpt/lib/operators/implementation.h:21-45).  Mobius /
 * zmobius: the two wall masses.  Wilson-clover and twisted mass: mass_plus is
 * the new mass m (mass_minus is ignored); the diagonal term follows and a
 * clover operator's clover term and inverse are updated on the device. */
int gbf_set_mass(gbf_op* op, double mass_plus, double mass_minus);

/* cgpt delete_fermion_operator (operators.cc:85-94). */
int gbf_delete(gbf_op* op);

/* cgpt apply_fermion_operator (operators.cc:96-107, unary.h:20-48): apply
 * `opcode` to n fields.  Even-odd opcodes (Meooe, Mooee, MooeeInv, DhopEO and
 * daggers) take half fields of checkerboard src_parity (Meooe/DhopEO write
 * the other parity); all others take full fields.  Import/Export take a 4D
 * field (Ls = 1 layout) on one side. */
int gbf_apply(gbf_op* op, int opcode, const void* const* src, void* const* dst, int n, int src_parity, void* stream);

/* Size in bytes of a field: which = 0 half field, 1 full field, 2 full 4D
 * field of a mobius operator (import source / export solution). */
int gbf_field_bytes(const gbf_op* op, int which, size_t* bytes);

/* Natural <-> internal transfer of one right-hand side.  `natural` is a
 * DEVICE pointer to complex128 [V][Ls'][12] with Ls' = Ls (five_d = 1) or 1. */
int gbf_field_import(gbf_op* op, const void* natural, void* full, int rhs, int five_d, void* stream);
int gbf_field_export(gbf_op* op, const void* full, void* natural, int rhs, int five_d, void* stream);

/* Vector algebra on internal fields of this operator's layout
 * (lib/gpt/core/transform.py:101-153 -> cgpt transform.cc:143-247).
 * nhalves = 1 (half field) or 2 (full field); results per rhs, accumulated in
 * double precision with a fixed summation order (bitwise reproducible). */
int gbf_norm2(gbf_op* op, const void* x, int nhalves, double* out, void* stream);
int gbf_inner(gbf_op* op, const void* x, const void* y, int nhalves, double* out_re, double* out_im, void* stream);
/* out = a*x + b*y per rhs (a complex as a_re/a_im, b real; y may be NULL) */
int gbf_axpby(gbf_op* op, void* out, const double* a_re, const double* a_im, const void* x, const double* b, const void* y,
              int nhalves, void* stream);
/* out = a*x + y and |out|^2 per rhs in one pass (the fused form of
 * lib/gpt/core/transform.py:139-153 axpy then norm2, the CG's axpy_norm2,
 * cg.py:88); out may equal x or y. */
int gbf_axpy_norm2(gbf_op* op, void* out, const double* a_re, const double* a_im, const void* x, const void* y,
                   int nhalves, double* out_norm2, void* stream);
/* dst = scale * src between two operators' layouts (same geometry), the
 * precision change of mixed-precision solvers (cgpt transform.cc:128-141). */
int gbf_convert(gbf_op* dst_op, void* dst, gbf_op* src_op, const void* src, double scale, int nhalves, void* stream);

/* preconditioned(eo2_ne(), cg(eps, maxiter)) on device
 * (lib/gpt/algorithms/inverter/preconditioned.py:32-54, cg.py:47-105,
 * lib/gpt/qcd/fermion/preconditioner/even_odd_sites.py:61-72): solves
 * M x = src for all packed right-hand sides with zero initial guess.  The CG
 * loop runs in CUDA graphs with device-resident scalars (see
 * iterations_per_graph). */
typedef struct {
  double eps;
  int maxiter;
  int iterations_per_graph; /* K > 0: the CG loop runs as CUDA graphs of K iterations, the host
                               checks convergence between graph launches (kernels of iterations
                               past convergence return at once); 0: K = 16; -1: the whole loop
                               on the device, one CUDA graph with a conditional while node and no
                               host round trip.  Bitwise equal solutions in all modes. */
  int profile;              /* 1: no graphs; CUDA events time every kernel class (diagnostic run) */
} gbf_cg_params;
typedef struct {
  int iterations;
  int converged;            /* all right-hand sides reached |r|^2 <= eps^2 |b|^2 */
  int breakdown;            /* <p, A p> <= 0 or non-finite */
  double residual_sq[16];   /* final |r|^2 / |b|^2 of the eo2_ne system, per rhs */
  /* profile = 1 only: summed CUDA-event time (ms) and launch count per kernel
   * class inside the CG loop: [0] hopping kernel, [1] site-local kernel,
   * [2] CG update kernel */
  double kernel_ms[3];
  int kernel_launches[3];
} gbf_cg_result;
int gbf_solve_eo2ne_cg(gbf_op* op, const void* src, void* x, const gbf_cg_params* p, gbf_cg_result* res, void* stream);

/* preconditioned(eo2_ne(), block_cg(eps, maxiter)) on device
 * (lib/gpt/algorithms/inverter/block_cg.py:36-149): the n_rhs packed
 * right-hand sides share one Krylov space (block CG with a Cholesky QR of the
 * residual block).  Gram matrices are reduced on the device and the k x k
 * algebra runs on the host, two reads per iteration; zero initial guess.
 * Converged when max_b (C^H C)_bb / |b_b|^2 <= eps^2 (the reference's test).
 * All right-hand sides must be non-zero and linearly independent (otherwise
 * the QR breaks down: breakdown = 1).  iterations_per_graph and profile are
 * ignored; residual_sq[b] is the block recursion's (C^H C)_bb / |b_b|^2. */
int gbf_solve_eo2ne_block_cg(gbf_op* op, const void* src, void* x, const gbf_cg_params* p, gbf_cg_result* res,
                             void* stream);

/* The eo2_ne normal operator Mpc^+ Mpc on odd-site half fields (the matrix
 * the eo2_ne CG inverts, lib/gpt/algorithms/preconditioner/normal_equation.py
 * over schur_complement_two.py), and multi-shift CG on it
 * (lib/gpt/algorithms/inverter/multi_shift_cg.py:24-144): x[j] (n half
 * fields) receive the solutions of (Mpc^+ Mpc + shifts[j]) x_j = src for
 * n <= 32 shifts >= 0, n_rhs = 1.  Converged when every shift's recursive
 * residual satisfies |r_j|^2 <= eps^2 |src|^2; residual_sq[j] (j < 16) gets
 * that ratio. */
int gbf_apply_eo2ne_normal(gbf_op* op, const void* in, void* out, void* stream);
int gbf_solve_eo2ne_multishift(gbf_op* op, const void* src, void* const* x, const double* shifts, int n,
                               const gbf_cg_params* p, gbf_cg_result* res, void* stream);

/* cg(eps, maxiter) applied to the eo2_ne normal operator itself
 * (lib/gpt/algorithms/inverter/cg.py:47-105 with the guess the reference
 * takes from dst, :48-68): solves Mpc^+ Mpc x = b on odd-site half fields,
 * starting from x as passed in (zero allowed) and overwriting it with the
 * solution; b = 0 gives x = 0.  Converged when |r|^2 <= eps^2 |b|^2 (checked
 * before the first iteration too); residual_sq = |r|^2 / |b|^2.  The loop
 * is the one of gbf_solve_eo2ne_cg (graphs, iterations_per_graph,
 * profile).  This is the inner solve of inverter.sequence(deflate(...), cg)
 * (lib/gpt/algorithms/inverter/sequence.py:23-42). */
int gbf_solve_normal_cg(gbf_op* op, const void* b, void* x, const gbf_cg_params* p, gbf_cg_result* res, void* stream);

/* The two halves of preconditioned(eo2_ne(), inverter) around an arbitrary
 * inverter of the normal operator (lib/gpt/algorithms/inverter/
 * preconditioned.py:36-44): prepare writes the odd-site right-hand side
 * b = Mpc^+ (src_D - Dhop G_C src_C) of the full field src
 * (normal_equation.py:47-48, schur_complement_two.py:87-104); reconstruct
 * writes the full solution x from the odd-site solution y
 * (schur_complement_two.py:106-148). */
int gbf_eo2ne_prepare(gbf_op* op, const void* src, void* b, void* stream);
int gbf_eo2ne_reconstruct(gbf_op* op, const void* src, const void* y, void* x, void* stream);

/* The fifth-dimension moves of the MADWF preconditioner
 * (lib/gpt/qcd/fermion/preconditioner/mixed_dwf.py:43-98) on fields of a
 * mobius/zmobius layout.  gbf_chiral_shift: dst_s = P- src_s + P+ src_{s+offset}
 * (s + offset mod Ls, P+- = (1 +- gamma5)/2), the operator P of mixed_dwf.py
 * for offset = 1 and its inverse P^+ for offset = -1; src != dst.
 * gbf_copy_slices: dst slices [dst_s0, dst_s0 + count) = scale * src slices
 * [src_s0, src_s0 + count) for every 4D site and rhs (g.separate / g.merge
 * along the fifth dimension); the operators may differ in Ls, not in
 * precision, 4D geometry or n_rhs.  nhalves: 1 one checkerboard, 2 full. */
int gbf_chiral_shift(gbf_op* op, const void* src, void* dst, int offset, int nhalves, void* stream);
int gbf_copy_slices(gbf_op* dst_op, void* dst, int dst_s0, gbf_op* src_op, const void* src, int src_s0, int count,
                    double scale, int nhalves, void* stream);

/* Mode representation dst = sum_n left[n] <right[n], src> f[n]
 * (lib/gpt/algorithms/modes/matrix.py:31-56; the deflation inverter
 * lib/gpt/algorithms/inverter/deflate.py is left = right = eigenvectors,
 * f = 1 / eigenvalue).  left/right: n device fields of op's layout with
 * nhalves halves (1: one checkerboard, 2: full), n_rhs = 1; f: n complex
 * numbers as 2n doubles (re, im).  Inner products are reduced
 * deterministically in FP64 (blocks of 8 modes per pass over the sites);
 * src must differ from dst, and dst from every left mode. */
int gbf_modes_apply(gbf_op* op, const void* const* left, const void* const* right, const double* f, int n,
                    const void* src, void* dst, int nhalves, void* stream);

/* Autotuner (the role of lib/gpt/core/auto_tune.py for this library): times
 * the block-size candidates of the four kernel classes -- [0] hopping kernel
 * with a per-thread epilogue, [1] hopping kernel with the Mobius s-matrix
 * epilogue, [2] site-local kernel, [3] CG update -- on scratch fields of
 * `op` and keeps the fastest for all later launches of `op`.  out_bd[4]
 * receives the chosen block sizes (0 = class not used), out_us[4] (optional)
 * the time per launch.  gbf_set_tuning applies block sizes found earlier
 * (for example from a cache file) without timing. */
int gbf_tune(gbf_op* op, void* stream, int* out_bd, double* out_us);
int gbf_set_tuning(gbf_op* op, const int* bd);

/* Thread-local message of the last error (exception.h:21-39 analogue). */
const char* gbf_last_error(void);

/* Device synchronisation helper for callers without a CUDA runtime binding. */
int gbf_stream_sync(void* stream);

/* Number of kernels this library has launched in the process so far
 * (a graph launch counts every kernel node it runs). */
unsigned long long gbf_launch_count(void);

/* Bytes per stored gauge link chosen by gbf_update_gauge: 144 (FP64, 18
 * reals), 72 (FP32, 18 reals) or 48 (FP32, 12 reals, SU(3) links). */
int gbf_link_bytes(const gbf_op* op);

/* Synthetic inputs on the device, natural layout (benchmarks and serving;
 * the reference's g.qcd.gauge.random / rng.cnormal use gpt's CPU RNG,
 * lib/gpt/core/random.py:103-148): U = exp(i eps H) per link with H
 * Hermitian traceless from complex-Gaussian entries, complex128 [4][V][3][3];
 * and n_complex standard complex-Gaussian numbers.  Counter-based
 * (Philox4x32-10), so the output depends only on (seed, index). */
int gbf_random_gauge(const int* dims, double eps, unsigned long long seed, void* U, void* stream);
int gbf_random_spinor(long long n_complex, unsigned long long seed, void* out, void* stream);

/* |x|^2 of a field, allocating nothing (no counterpart in the reference).
 * For callers that cannot call cudaMalloc: a process whose free HBM belongs
 * to its own pool, or a latency-critical loop that must not take cudaMalloc's
 * device-wide synchronisation (gbf_norm2 allocates its workspace on first
 * use).  x: device field of `precision` with n_sites 5D sites per half and
 * nhalves halves (the layout of gbf_field_bytes); the sum over all sites is
 * written to the host double *out after the stream is synchronised.
 * The reduction scratch is a static device array of about 263 KB, held on
 * every GPU where it is loaded until the process exits; at most 4194304
 * sites per half (larger sizes return GBF_E_ARG).  CUDA loads the library's
 * modules lazily, so the first call on a device loads this one (taking the
 * array's memory) and looks up the array's address for that device: make
 * that first call before any stream capture and before the caller's own pool
 * takes the free HBM; a call with n_sites = 0 does only this set-up.  All
 * calls share the array: calls that overlap on the GPU race.  Errors:
 * gbf_norm2_noalloc_error(). */
int gbf_norm2_noalloc(int precision, const void* x, long long n_sites, int nhalves, double* out, void* stream);
const char* gbf_norm2_noalloc_error(void);

#ifdef __cplusplus
}
#endif
#endif /* GBFERM_H */
