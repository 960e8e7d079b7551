// gbf_api.cu -- the C ABI of include/gbferm.h: operator objects, opcode
// dispatch onto the kernels, vector algebra and the device-resident
// eo2_ne-preconditioned CG.
//
// Reference interfaces replaced here (paths relative to the gpt project root):
//   create/update/set_mass/delete/apply  lib/cgpt/lib/operators.cc:34-133
//   opcode dispatch                       lib/cgpt/lib/operators/unary.h:20-64
//   Wilson-clover factory                 lib/cgpt/lib/operators/wilson_clover.h:19-71
//   Mobius factory                        lib/cgpt/lib/operators/mobius.h:34-87
//   eo2_ne + CG                           lib/gpt/algorithms/preconditioner/schur_complement_two.py:58-152,
//                                         normal_equation.py:35-65, inverter/cg.py:24-117
#include <cstdio>
#include <cstring>
#include <algorithm>
#include <cmath>
#include <complex>
#include <string>
#include <vector>
#include <stdexcept>
#include "gbf_launch.cuh"
#include "../../include/gbferm.h"

using namespace gbf;

#include <atomic>

static thread_local std::string g_err;
static std::atomic<unsigned long long> g_launches{0};
static inline void count_launch(unsigned long long n = 1) { g_launches.fetch_add(n, std::memory_order_relaxed); }
// CG iterations per host-checked graph launch when the caller passes 0
static constexpr int kDefaultGraphIterations = 16;

namespace {

struct Fail : std::runtime_error {
  int code;
  Fail(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

#define CK(x)                                                                                       \
  do {                                                                                              \
    cudaError_t e_ = (x);                                                                           \
    if (e_ != cudaSuccess) throw Fail(GBF_E_CUDA, std::string(#x) + ": " + cudaGetErrorString(e_)); \
  } while (0)

template <typename F> int guarded(F&& f) {
  try {
    f();
    return GBF_OK;
  } catch (const Fail& e) {
    g_err = e.what();
    return e.code;
  } catch (const std::bad_alloc&) {
    g_err = "host allocation failed";
    return GBF_E_OOM;
  } catch (const std::exception& e) {
    g_err = e.what();
    return GBF_E_ARG;
  }
}

void* dmalloc(size_t bytes) {
  void* p = nullptr;
  cudaError_t e = cudaMalloc(&p, bytes ? bytes : 16);
  if (e != cudaSuccess) {
    cudaGetLastError();
    throw Fail(GBF_E_OOM, "cudaMalloc of " + std::to_string(bytes) + " bytes failed: " + cudaGetErrorString(e));
  }
  return p;
}

// Mobius s-matrix slots (real Ls x Ls per chirality)
// (DM1, DMC: the diagonal parts of Dminus = DM1 + DMC Dhop, per-slice
//  1 - c_s (4 - M5) and -c_s, used when c_s varies with s)
enum { S_A = 0, S_ADAG, S_AINV, S_AINVDAG, S_B, S_BDAG, S_G, S_GDAG, S_DM1, S_DM1DAG, S_DMC, S_DMCDAG, S_COUNT };

}  // namespace

struct gbf_op {
  std::string name;
  bool mobius = false;
  int prec = P64;   // spinor storage precision
  int LS = L64;     // link storage
  gbf_params par;
  Geo g;            // fields of this operator (N5 = Ls * nrhs)
  Geo g4;           // 4D fields of a mobius operator (N5 = nrhs)
  double cc[4];
  double diag = 0;  // 1/(2 kappa) for wilson_clover
  bool has_clover = false;
  bool twisted = false;  // wilson_twisted_mass: Mooee = diag + i mu g5
  double mu = 0;
  bool gauge_set = false;
  void* links = nullptr;
  void* clov_mem = nullptr;      // clover + inverse, both parities, op precision
  void* clov[2] = {nullptr, nullptr};
  void* clov_inv[2] = {nullptr, nullptr};
  void* smat = nullptr;          // [S_COUNT][2][Ls][Ls] in the arithmetic precision ((re, im) pairs if complex)
  bool smat_cplx = false;        // zmobius: complex per-slice coefficients
  bool zmobius = false;
  std::vector<std::complex<double>> bs, cs;  // Cayley coefficients per slice
  // workspace
  void* pair_mem[6] = {};        // workspace: full fields allocated on first use
  void* tmp[12] = {};
  double2* partial = nullptr;
  unsigned* counter = nullptr;
  CGState* st = nullptr;
  CGState* hst = nullptr;        // pinned, 2 buffers
  unsigned* errbits = nullptr;
  cudaStream_t stream = nullptr; // internal stream for graph capture
  cudaEvent_t ev_in = nullptr, ev_out = nullptr, ev_chk[2] = {nullptr, nullptr};
  cudaGraphExec_t graph = nullptr;   // K CG iterations (host-checked loop)
  int graph_K = 0;
  cudaGraphExec_t cgraph = nullptr;  // the whole CG loop: a conditional while node
  unsigned long long cond = 0;       // its loop condition
  bool cond_active = false;          // set while the loop body is captured
  void drop_graphs() {
    if (graph) { cudaGraphExecDestroy(graph); graph = nullptr; }
    if (cgraph) { cudaGraphExecDestroy(cgraph); cgraph = nullptr; }
  }
  // block sizes chosen by gbf_tune (0: default): hop with a per-thread
  // epilogue, hop with the s-matrix epilogue, site-local kernel, CG update
  int tuned_bd[4] = {0, 0, 0, 0};
  // block CG workspace: Gram partials [max_blocks][k*k], device results and
  // coefficient matrices (k*k Gram + 4 x k*k), pinned host mirror
  double2* blk_partial = nullptr;
  double2* blk_dev = nullptr;
  double2* blk_host = nullptr;
  long long blk_max_blocks = 0;
  // multi-shift CG: search directions of the shifts
  void* ms_mem = nullptr;
  int ms_count = 0;
  // reduction partials: capacity of `partial` in double2 entries
  long long partial_cap = 0;
  // mode representation: inner products of the modes (device), capacity
  double2* mode_dev = nullptr;
  int mode_cap = 0;

  size_t half() const { return (size_t)half_bytes(prec, g.N); }
  // workspace half field i; halves 2k and 2k+1 are one contiguous full field,
  // allocated when first used (an operator that only applies M never holds
  // the CG's vectors)
  void* T(int i);
  size_t half4() const { return (size_t)half_bytes(prec, g4.N); }
  size_t rb() const { return (prec == P64 || prec == PDD) ? 8 : 4; }

  // ---- site-local operators ----
  LocalOp none() const { LocalOp l{}; l.kind = LOC_NONE; return l; }
  LocalOp smat_slot(int s) const {
    LocalOp l{};
    l.kind = LOC_SMAT;
    l.cplx = smat_cplx ? 1 : 0;
    l.smat = (const char*)smat + (size_t)s * 2 * g.Ls * g.Ls * (smat_cplx ? 2 : 1) * rb();
    return l;
  }
  LocalOp clover(bool inv) const {
    LocalOp l{};
    if (has_clover) {
      l.kind = LOC_CLOVER;
      l.clov[0] = inv ? clov_inv[0] : clov[0];
      l.clov[1] = inv ? clov_inv[1] : clov[1];
    } else {
      l.kind = LOC_SCALAR;
      l.scalar = inv ? 1.0 / diag : diag;
    }
    return l;
  }
  // twisted mass: (a + i mu g5), inverse (a - i mu g5) / (a^2 + mu^2), adjoints conjugate
  LocalOp twist(bool inv, bool dag) const {
    LocalOp l{};
    l.kind = LOC_TWIST;
    const double a = diag, den = inv ? a * a + mu * mu : 1.0;
    double b = (inv ? -mu : mu) / den;
    if (dag) b = -b;
    l.z[0] = a / den;
    l.z[1] = b;   // spins 0, 1 (g5 = +1)
    l.z[2] = a / den;
    l.z[3] = -b;  // spins 2, 3 (g5 = -1)
    return l;
  }
  LocalOp G() const { return mobius ? smat_slot(S_G) : twisted ? twist(true, false) : clover(true); }
  LocalOp Gdag() const { return mobius ? smat_slot(S_GDAG) : twisted ? twist(true, true) : clover(true); }
  LocalOp A(bool dag) const { return mobius ? smat_slot(dag ? S_ADAG : S_A) : twisted ? twist(false, dag) : clover(false); }
  LocalOp Ainv(bool dag) const {
    return mobius ? smat_slot(dag ? S_AINVDAG : S_AINV) : twisted ? twist(true, dag) : clover(true);
  }
  LocalOp B(bool dag) const { return smat_slot(dag ? S_BDAG : S_B); }

  RedArgs red(int fin) const { RedArgs r; r.fin = fin; r.partial = partial; r.counter = counter; r.st = st; return r; }

  // ---- kernel wrappers ----
  // out(parity p) = c1 * L1(Dhop[^dag](in)) + c2 * L2(X)  [+ reduction]
  void dslash(cudaStream_t s, int p, bool dag, const void* in, void* out, LocalOp l1, double c1 = 1.0, const void* X = nullptr,
              double c2 = 0.0, LocalOp l2 = LocalOp{}, int redmode = 0, const void* Y = nullptr, int fin = FIN_STORE,
              int check_done = 0, const Geo* geo = nullptr) const {
    DslashArgs a{};
    a.g = geo ? *geo : g;
    a.out_parity = p;
    a.sgn = dag ? 1.f : -1.f;
    a.in = in;
    a.out = out;
    a.links = links;
    a.l1 = l1;
    a.l2 = l2;
    a.c1 = c1;
    a.c2 = c2;
    a.X = X;
    a.red = redmode;
    a.Y = Y;
    a.ra = red(fin);
    a.check_done = check_done;
    a.bd = tuned_bd[(l1.kind == LOC_SMAT) ? 1 : 0];
    if (l2.kind == LOC_SMAT) throw Fail(GBF_E_ARG, "internal: smat on the X term");
    CK(launch_dslash(prec, LS, a, s));
    count_launch();
  }
  void local(cudaStream_t s, int p, const void* A_, void* out, LocalOp l, double c1 = 1.0, const void* X = nullptr, double c2 = 0.0,
             void* W = nullptr, int pre = 0, int redmode = 0, const void* Y = nullptr, int fin = FIN_STORE, int check_done = 0,
             const Geo* geo = nullptr) const {
    LocalArgs a{};
    a.g = geo ? *geo : g;
    a.parity = p;
    a.A = A_;
    a.W = W;
    a.pre = pre;
    a.l = l;
    a.out = out;
    a.c1 = c1;
    a.c2 = c2;
    a.X = X;
    a.red = redmode;
    a.Y = Y;
    a.ra = red(fin);
    a.check_done = check_done;
    a.bd = tuned_bd[2];
    CK(launch_local(prec, a, s));
    count_launch();
  }
  void cg_update(cudaStream_t s, void* r, const void* mmp, void* x, const void* p) const {
    CGUpdateArgs a{};
    a.g = g;
    a.r = r;
    a.mmp = mmp;
    a.x = x;
    a.p = p;
    a.ra = red(FIN_BETA);
    a.ra.cond = cond;
    a.ra.use_cond = cond_active ? 1 : 0;
    a.bd = tuned_bd[3];
    CK(launch_cg_update(prec, a, s));
    count_launch();
  }
};

void* gbf_op::T(int i) {
  if (i < 0 || i >= 12) throw Fail(GBF_E_ARG, "internal: workspace index");
  const int pr = i / 2;
  if (!pair_mem[pr]) {
    pair_mem[pr] = dmalloc(2 * half());
    tmp[2 * pr] = pair_mem[pr];
    tmp[2 * pr + 1] = (char*)pair_mem[pr] + half();
  }
  return tmp[i];
}

namespace {

void setup_geo(gbf_op* op) {
  const gbf_params& p = op->par;
  Geo& g = op->g;
  for (int m = 0; m < 4; ++m) g.L[m] = p.dims[m];
  g.Lh0 = p.dims[0] / 2;
  long long V = (long long)p.dims[0] * p.dims[1] * p.dims[2] * p.dims[3];
  g.Vh = (int)(V / 2);
  g.Ls = op->mobius ? p.Ls : 1;
  g.nrhs = p.n_rhs;
  g.N5 = g.Ls * g.nrhs;
  g.N = (long long)g.Vh * g.N5;
  for (int m = 0; m < 4; ++m) {
    g.lam[m] = (float)(-0.5 * op->cc[m]);
    g.ph_re[m] = (float)p.boundary_phases[2 * m];
    g.ph_im[m] = (float)p.boundary_phases[2 * m + 1];
  }
  g.fLh0 = FastDiv((unsigned)g.Lh0);
  g.fL1 = FastDiv((unsigned)g.L[1]);
  g.fL2 = FastDiv((unsigned)g.L[2]);
  g.fN5 = FastDiv((unsigned)g.N5);
  g.fLs = FastDiv((unsigned)g.Ls);
  op->g4 = g;
  op->g4.Ls = 1;
  op->g4.N5 = g.nrhs;
  op->g4.N = (long long)g.Vh * g.nrhs;
  op->g4.fN5 = FastDiv((unsigned)g.nrhs);
  op->g4.fLs = FastDiv(1u);
}

// Host -> device copy that has completed when it returns, on a stream of its
// own (a plain cudaMemcpy from pageable memory may still be in flight on the
// legacy default stream, which the operators' non-blocking streams do not
// wait for)
void upload(void* dst, const void* src, size_t bytes) {
  cudaStream_t t;
  CK(cudaStreamCreateWithFlags(&t, cudaStreamNonBlocking));
  const cudaError_t e1 = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, t);
  const cudaError_t e2 = cudaStreamSynchronize(t);
  cudaStreamDestroy(t);
  CK(e1);
  CK(e2);
}

// Cayley s-matrices of the Mobius / zmobius operator with per-slice b_s, c_s
// (mobius: b, c for every s, lib/gpt/qcd/fermion/mobius.py:29-46; zmobius:
// b_s = ((b + c) / omega_s + (b - c)) / 2, c_s = ((b + c) / omega_s - (b - c)) / 2,
// lib/gpt/qcd/fermion/zmobius.py:31-34).  With K+ the s-1 -> s hop with the
// wall term -m+ at (0, Ls-1) and K- the s+1 -> s hop with -m- at (Ls-1, 0),
// c_s scaling the output slice (the convention that reproduces the
// reference's zmobius fingerprint):
//   B = diag(b) + diag(c) K,  A = (4 - M5) B + 1 - K  (Mooee),  G = B A^-1.
// Adjoint slots hold conjugate transposes.
void build_smat(gbf_op* op) {
  using zc = std::complex<double>;
  const int Ls = op->g.Ls;
  const gbf_params& p = op->par;
  const int L2 = Ls * Ls;
  std::vector<zc> all((size_t)S_COUNT * 2 * L2, zc(0.0, 0.0));
  auto slot = [&](int sl, int ch) { return all.data() + ((size_t)sl * 2 + ch) * L2; };
  for (int ch = 0; ch < 2; ++ch) {
    std::vector<double> K(L2, 0.0);
    for (int s = 0; s < Ls; ++s) {
      if (ch == 0) {
        if (s >= 1) K[s * Ls + s - 1] = 1.0;
        else K[Ls - 1] = -p.mass_plus;
      } else {
        if (s <= Ls - 2) K[s * Ls + s + 1] = 1.0;
        else K[(Ls - 1) * Ls] = -p.mass_minus;
      }
    }
    std::vector<zc> A(L2), B(L2), Ai(L2, zc(0.0, 0.0)), G(L2, zc(0.0, 0.0));
    for (int s = 0; s < Ls; ++s)
      for (int t = 0; t < Ls; ++t) {
        const double k = K[s * Ls + t];
        const zc bv = (s == t ? op->bs[s] : zc(0.0, 0.0)) + k * op->cs[s];
        B[s * Ls + t] = bv;
        A[s * Ls + t] = (4.0 - p.M5) * bv + (s == t ? 1.0 : 0.0) - k;
      }
    // Gauss-Jordan inverse of A with partial pivoting
    std::vector<zc> a = A;
    for (int i = 0; i < Ls; ++i) Ai[i * Ls + i] = 1.0;
    for (int c = 0; c < Ls; ++c) {
      int piv = c;
      for (int r = c + 1; r < Ls; ++r)
        if (std::abs(a[r * Ls + c]) > std::abs(a[piv * Ls + c])) piv = r;
      if (std::abs(a[piv * Ls + c]) == 0.0) throw Fail(GBF_E_ARG, "singular Mooee (check M5, b, c, omega, masses)");
      for (int k = 0; k < Ls; ++k) {
        std::swap(a[c * Ls + k], a[piv * Ls + k]);
        std::swap(Ai[c * Ls + k], Ai[piv * Ls + k]);
      }
      const zc d = 1.0 / a[c * Ls + c];
      for (int k = 0; k < Ls; ++k) {
        a[c * Ls + k] *= d;
        Ai[c * Ls + k] *= d;
      }
      for (int r = 0; r < Ls; ++r) {
        if (r == c) continue;
        const zc f = a[r * Ls + c];
        if (f == zc(0.0, 0.0)) continue;
        for (int k = 0; k < Ls; ++k) {
          a[r * Ls + k] -= f * a[c * Ls + k];
          Ai[r * Ls + k] -= f * Ai[c * Ls + k];
        }
      }
    }
    for (int i = 0; i < Ls; ++i)
      for (int j = 0; j < Ls; ++j) {
        zc acc(0.0, 0.0);
        for (int k = 0; k < Ls; ++k) acc += B[i * Ls + k] * Ai[k * Ls + j];
        G[i * Ls + j] = acc;
      }
    std::vector<zc> DM1(L2, zc(0.0, 0.0)), DMC(L2, zc(0.0, 0.0));
    for (int s = 0; s < Ls; ++s) {
      DM1[s * Ls + s] = 1.0 - op->cs[s] * (4.0 - p.M5);
      DMC[s * Ls + s] = -op->cs[s];
    }
    auto put = [&](int sl, const std::vector<zc>& M, bool adj) {
      zc* d = slot(sl, ch);
      for (int i = 0; i < Ls; ++i)
        for (int j = 0; j < Ls; ++j) d[i * Ls + j] = adj ? std::conj(M[j * Ls + i]) : M[i * Ls + j];
    };
    put(S_A, A, false); put(S_ADAG, A, true);
    put(S_AINV, Ai, false); put(S_AINVDAG, Ai, true);
    put(S_B, B, false); put(S_BDAG, B, true);
    put(S_G, G, false); put(S_GDAG, G, true);
    put(S_DM1, DM1, false); put(S_DM1DAG, DM1, true);
    put(S_DMC, DMC, false); put(S_DMCDAG, DMC, true);
  }
  // real storage unless a coefficient is complex
  op->smat_cplx = false;
  for (const zc& v : all)
    if (v.imag() != 0.0) op->smat_cplx = true;
  std::vector<double> flat;
  flat.reserve(all.size() * 2);
  for (const zc& v : all) {
    flat.push_back(v.real());
    if (op->smat_cplx) flat.push_back(v.imag());
  }
  const size_t bytes = all.size() * 2 * op->rb();  // room for the complex layout
  if (!op->smat) op->smat = dmalloc(bytes);
  if (op->prec == P64) {
    upload(op->smat, flat.data(), flat.size() * 8);
  } else if (op->prec == PDD) {
    std::vector<float> f(2 * flat.size());
    for (size_t i = 0; i < flat.size(); ++i) {
      const dd v(flat[i]);
      f[2 * i] = v.h;
      f[2 * i + 1] = v.l;
    }
    upload(op->smat, f.data(), f.size() * 4);
  } else {
    std::vector<float> f(flat.begin(), flat.end());
    upload(op->smat, f.data(), f.size() * 4);
  }
}

void ensure_ws(gbf_op* op) {
  if (op->partial) return;
  // reducing launches use at most one wave of resident blocks (<= 32 per SM)
  // or, for the double-float hop, up to 4096 blocks (reduce_grid)
  int dev = 0, sms = 152;
  if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const long long maxblocks = std::min<long long>(op->g.Vh + 1, (long long)sms * 32 + 4096);
  op->partial = (double2*)dmalloc((size_t)maxblocks * op->g.nrhs * sizeof(double2));
  op->partial_cap = maxblocks * op->g.nrhs;
  op->counter = (unsigned*)dmalloc(sizeof(unsigned) * 4);
  op->st = (CGState*)dmalloc(sizeof(CGState));
  CK(cudaMallocHost(&op->hst, 2 * sizeof(CGState)));
  CK(cudaStreamCreateWithFlags(&op->stream, cudaStreamNonBlocking));
  // zero the counter and the CG state on the op's own stream and wait: a
  // cudaMemset would go to the legacy default stream, which non-blocking
  // streams do not wait for, so it could land after this op's first kernels
  // (seen as CG states reset between cg_init and the loop)
  CK(cudaMemsetAsync(op->counter, 0, sizeof(unsigned) * 4, op->stream));
  CK(cudaMemsetAsync(op->st, 0, sizeof(CGState), op->stream));
  CK(cudaStreamSynchronize(op->stream));
  CK(cudaEventCreateWithFlags(&op->ev_in, cudaEventDisableTiming));
  CK(cudaEventCreateWithFlags(&op->ev_out, cudaEventDisableTiming));
  CK(cudaEventCreateWithFlags(&op->ev_chk[0], cudaEventDisableTiming));
  CK(cudaEventCreateWithFlags(&op->ev_chk[1], cudaEventDisableTiming));
}

void free_op(gbf_op* op) {
  op->drop_graphs();
  cudaFree(op->links);
  cudaFree(op->clov_mem);
  cudaFree(op->smat);
  for (void* m : op->pair_mem) cudaFree(m);
  cudaFree(op->partial);
  cudaFree(op->blk_partial);
  cudaFree(op->blk_dev);
  cudaFree(op->ms_mem);
  cudaFree(op->mode_dev);
  if (op->blk_host) cudaFreeHost(op->blk_host);
  cudaFree(op->counter);
  cudaFree(op->st);
  cudaFree(op->errbits);
  if (op->hst) cudaFreeHost(op->hst);
  if (op->stream) cudaStreamDestroy(op->stream);
  for (cudaEvent_t e : {op->ev_in, op->ev_out, op->ev_chk[0], op->ev_chk[1]})
    if (e) cudaEventDestroy(e);
  delete op;
}

// read one reduction result (all rhs) into host memory; synchronises s
void read_last(gbf_op* op, cudaStream_t s, double* re, double* im) {
  CK(cudaMemcpyAsync(op->hst, op->st, sizeof(CGState), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  for (int r = 0; r < op->g.nrhs; ++r) {
    if (re) re[r] = op->hst->last[r];
    if (im) im[r] = op->hst->last_im[r];
  }
}

}  // namespace

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

const char* gbf_last_error(void) { return g_err.c_str(); }

unsigned long long gbf_launch_count(void) { return g_launches.load(); }

int gbf_link_bytes(const gbf_op* op) {
  if (!op) return 0;
  return (op->LS == L64 || op->LS == LDD) ? 144 : (op->LS == L32 ? 72 : 48);
}

int gbf_stream_sync(void* stream) {
  return guarded([&] { CK(cudaStreamSynchronize((cudaStream_t)stream)); });
}

int gbf_create(const char* name, int precision, const gbf_params* params, gbf_op** out) {
  return guarded([&] {
    if (!name || !params || !out) throw Fail(GBF_E_ARG, "null argument");
    *out = nullptr;
    std::string nm(name);
    if (nm != "wilson_clover" && nm != "mobius" && nm != "wilson_twisted_mass" && nm != "zmobius")
      throw Fail(GBF_E_UNSUPPORTED, "unknown fermion operator " + nm);
    if (precision < GBF_DOUBLE || precision > GBF_DOUBLE_FLOAT) throw Fail(GBF_E_ARG, "bad precision");
    const gbf_params& p = *params;
    for (int m = 0; m < 4; ++m)
      if (p.dims[m] < 2 || p.dims[m] % 2) throw Fail(GBF_E_ARG, "lattice dimensions must be even and >= 2");
    if (p.n_rhs < 1 || p.n_rhs > kMaxRhs) throw Fail(GBF_E_ARG, "n_rhs must be in [1, 16]");
    const bool zmob = nm == "zmobius";
    const bool mob = nm == "mobius" || zmob;
    if (mob && (p.Ls < 1 || p.Ls > kMaxLs)) throw Fail(GBF_E_ARG, "Ls must be in [1, 32]");
    if (zmob && !p.omega) throw Fail(GBF_E_ARG, "zmobius needs omega (2 Ls doubles)");
    const int N5 = (mob ? p.Ls : 1) * p.n_rhs;
    if (N5 > 256) throw Fail(GBF_E_ARG, "Ls * n_rhs must be <= 256");
    long long V = (long long)p.dims[0] * p.dims[1] * p.dims[2] * p.dims[3];
    if (V / 2 * N5 > (1LL << 31) / 12) throw Fail(GBF_E_ARG, "field too large for 32-bit component indexing");
    if (V / 2 * 80 >= (1LL << 31)) throw Fail(GBF_E_ARG, "lattice too large for 32-bit link and clover indexing");
    auto* op = new gbf_op;
    op->name = nm;
    op->mobius = mob;
    op->par = p;
    op->prec = precision == GBF_DOUBLE ? P64 : precision == GBF_SINGLE ? P32 : precision == GBF_HALF ? P16 : PDD;
    if (mob) {
      for (int m = 0; m < 4; ++m) op->cc[m] = 1.0;
      op->diag = 4.0 - p.M5;
      op->zmobius = zmob;
      op->bs.assign(p.Ls, std::complex<double>(p.b, 0.0));
      op->cs.assign(p.Ls, std::complex<double>(p.c, 0.0));
      if (zmob) {
        // lib/gpt/qcd/fermion/zmobius.py:31-34
        for (int s = 0; s < p.Ls; ++s) {
          const std::complex<double> w(p.omega[2 * s], p.omega[2 * s + 1]);
          if (std::abs(w) == 0.0) {
            delete op;
            throw Fail(GBF_E_ARG, "omega must be non-zero");
          }
          op->bs[s] = 0.5 * ((p.b + p.c) / w + (p.b - p.c));
          op->cs[s] = 0.5 * ((p.b + p.c) / w - (p.b - p.c));
        }
      }
      op->par.omega = nullptr;  // not kept: the caller owns the array
    } else {
      const double xi0 = p.xi_0 != 0.0 ? p.xi_0 : 1.0;
      const double nu = p.nu != 0.0 ? p.nu : 1.0;
      for (int m = 0; m < 3; ++m) op->cc[m] = nu / xi0;
      op->cc[3] = 1.0;
      op->diag = p.mass + 1.0 + 3.0 * nu / xi0;
      op->has_clover = (p.csw_r != 0.0 || p.csw_t != 0.0);
      if (nm == "wilson_twisted_mass") {
        if (op->has_clover || xi0 != 1.0 || nu != 1.0) {
          delete op;
          throw Fail(GBF_E_UNSUPPORTED, "wilson_twisted_mass is isotropic and has no clover term");
        }
        op->twisted = true;
        op->mu = p.mu;
      }
    }
    setup_geo(op);
    try {
      if (mob) build_smat(op);
      op->errbits = (unsigned*)dmalloc(sizeof(unsigned) * 2);
    } catch (...) {
      free_op(op);
      throw;
    }
    *out = op;
  });
}

int gbf_delete(gbf_op* op) {
  return guarded([&] {
    if (op) free_op(op);
  });
}

int gbf_set_mass(gbf_op* op, double mass_plus, double mass_minus) {
  return guarded([&] {
    if (!op) throw Fail(GBF_E_ARG, "null operator");
    if (op->mobius) {
      op->par.mass_plus = mass_plus;
      op->par.mass_minus = mass_minus;
      build_smat(op);
      op->drop_graphs();
      return;
    }
    // Wilson-type operators (lib/cgpt/lib/operators/implementation.h:21-29):
    // mass_plus is the new mass; the diagonal 4 + m (anisotropic:
    // m + 1 + 3 nu / xi_0) moves by the difference, and a clover operator's
    // stored clover term and its inverse are shifted and re-inverted on the
    // device on the operator's stream
    const double xi0 = op->par.xi_0 != 0.0 ? op->par.xi_0 : 1.0;
    const double nu = op->par.nu != 0.0 ? op->par.nu : 1.0;
    const double diag = mass_plus + 1.0 + 3.0 * nu / xi0;
    const double shift = diag - op->diag;
    if (op->has_clover && op->gauge_set && shift != 0.0) {
      ensure_ws(op);
      cudaStream_t s = op->stream;
      CK(cudaMemsetAsync(op->errbits + 1, 0, sizeof(unsigned), s));
      CK(launch_clover_shift(op->prec, op->clov[0], op->clov_inv[0], op->g.Vh, shift, op->errbits + 1, s));
      count_launch();
      unsigned eb = 0;
      CK(cudaMemcpyAsync(&eb, op->errbits + 1, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
      CK(cudaStreamSynchronize(s));
      if (eb != 0) throw Fail(GBF_E_ARG, "singular clover block after set_mass");
    }
    op->par.mass = mass_plus;
    op->diag = diag;
    op->drop_graphs();
  });
}

static void update_gauge_impl(gbf_op* op, const void* U, int on_device, const gbf_op* from, void* stream);

int gbf_update_gauge(gbf_op* op, const void* U, int on_device, void* stream) {
  return guarded([&] { update_gauge_impl(op, U, on_device, nullptr, stream); });
}

int gbf_update_gauge_from(gbf_op* op, const void* U, int on_device, const gbf_op* clover_from, void* stream) {
  return guarded([&] { update_gauge_impl(op, U, on_device, clover_from, stream); });
}

}  // extern "C"

static bool clover_compatible(const gbf_op* a, const gbf_op* b) {
  if (!a || !b || a->mobius || b->mobius || !a->has_clover || !b->has_clover || !b->gauge_set) return false;
  for (int m = 0; m < 4; ++m)
    if (a->par.dims[m] != b->par.dims[m]) return false;
  return a->par.mass == b->par.mass && a->par.csw_r == b->par.csw_r && a->par.csw_t == b->par.csw_t &&
         a->par.xi_0 == b->par.xi_0 && a->par.nu == b->par.nu && (b->prec == P64 || b->prec == PDD) &&
         (b->prec == P64 || a->prec != P64);
}

static void update_gauge_impl(gbf_op* op, const void* U, int on_device, const gbf_op* from, void* stream) {
  {
    if (!op || !U) throw Fail(GBF_E_ARG, "null argument");
    cudaStream_t s = (cudaStream_t)stream;
    const Geo& g = op->g;
    const size_t ubytes = (size_t)8 * g.Vh * 9 * sizeof(double2);
    const double2* Ud = (const double2*)U;
    void* tmpU = nullptr;
    if (!on_device) {
      tmpU = dmalloc(ubytes);
      CK(cudaMemcpyAsync(tmpU, U, ubytes, cudaMemcpyHostToDevice, s));
      Ud = (const double2*)tmpU;
    }
    double lam[4], ph[8];
    for (int m = 0; m < 4; ++m) lam[m] = -0.5 * op->cc[m];
    for (int k = 0; k < 8; ++k) ph[k] = op->par.boundary_phases[k];
    const bool wide = op->prec == P64 || op->prec == PDD;  // 8 bytes per real
    if (!op->links) op->links = dmalloc((size_t)8 * link_bytes_per_parity_mu(wide ? L64 : L32, g.Vh));
    int LS = op->prec == P64 ? L64 : (op->prec == PDD ? LDD : L32);
    // 12-real links save 24 B per link per output site, but cost a
    // reconstruction and a run-time phase in every thread.  When Ls * n_rhs
    // threads share each link (5D / multi-rhs fields) the link bytes are
    // already amortised and those flops would dominate: keep 18 reals.
    const bool try_r12 = op->par.reconstruct == 1 || (op->par.reconstruct != 0 && op->g.N5 < 4);
    if (!wide && try_r12) {
      CK(cudaMemsetAsync(op->errbits, 0, sizeof(unsigned), s));
      CK(launch_pack_links(L32R, g, Ud, op->links, lam, ph, op->errbits, s));
      unsigned eb = 0;
      CK(cudaMemcpyAsync(&eb, op->errbits, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
      CK(cudaStreamSynchronize(s));
      float err;
      std::memcpy(&err, &eb, sizeof(float));
      if (err < 1e-6f) LS = L32R;
      else if (op->par.reconstruct == 1) throw Fail(GBF_E_ARG, "links are not SU(3) to 1e-6: 12-real storage impossible");
    }
    if (LS != L32R) CK(launch_pack_links(LS, g, Ud, op->links, lam, ph, op->errbits, s));
    op->LS = LS;
    if (op->has_clover && clover_compatible(op, from)) {
      // convert the source operator's clover and inverse instead of rebuilding
      const size_t c64 = (size_t)2 * 36 * g.Vh * sizeof(double2);
      const size_t c32 = (size_t)2 * 18 * g.Vh * sizeof(float4);
      const size_t mine = wide ? c64 : c32;
      if (!op->clov_mem) op->clov_mem = dmalloc(2 * mine);
      if (op->prec == from->prec) {
        CK(cudaMemcpyAsync(op->clov_mem, from->clov_mem, 2 * mine, cudaMemcpyDeviceToDevice, s));
      } else if (op->prec == PDD) {
        // FP64 -> double-float, 4 x 36 complex per site pair
        CK(launch_split_dd(from->clov_mem, op->clov_mem, 4LL * 36 * g.Vh, s));
        count_launch();
      } else {
        // 4 blocks (clover, inverse) x (even, odd) of 18 float4 rows of Vh sites
        if (from->prec == PDD) CK(launch_clover_narrow_dd(from->clov_mem, op->clov_mem, 4LL * 18, g.Vh, s));
        else CK(launch_clover_narrow(from->clov_mem, op->clov_mem, 4LL * 18, g.Vh, s));
        count_launch();
      }
      const size_t perpar = mine / 2;
      op->clov[0] = op->clov_mem;
      op->clov[1] = (char*)op->clov_mem + perpar;
      op->clov_inv[0] = (char*)op->clov_mem + mine;
      op->clov_inv[1] = (char*)op->clov_mem + mine + perpar;
    } else if (op->has_clover) {
      const size_t c64 = (size_t)2 * 36 * g.Vh * sizeof(double2);  // one of clover / inverse, both parities
      const size_t c32 = (size_t)2 * 18 * g.Vh * sizeof(float4);
      const size_t mine = wide ? c64 : c32;
      if (!op->clov_mem) op->clov_mem = dmalloc(2 * mine);
      // the build writes FP64 and FP32 copies; a double-float operator builds
      // both into scratch and splits the FP64 copy
      void* other = dmalloc(2 * (op->prec == P64 ? c32 : op->prec == PDD ? c32 + c64 : c64));
      void *C64, *CI64, *C32, *CI32;
      if (op->prec == P64) { C64 = op->clov_mem; CI64 = (char*)op->clov_mem + c64; C32 = other; CI32 = (char*)other + c32; }
      else if (op->prec == PDD) { C64 = other; CI64 = (char*)other + c64; C32 = (char*)other + 2 * c64; CI32 = (char*)other + 2 * c64 + c32; }
      else { C32 = op->clov_mem; CI32 = (char*)op->clov_mem + c32; C64 = other; CI64 = (char*)other + c64; }
      CK(cudaMemsetAsync(op->errbits + 1, 0, sizeof(unsigned), s));
      const double xi0 = op->par.xi_0 != 0.0 ? op->par.xi_0 : 1.0;
      CK(launch_clover(g, Ud, op->diag, op->par.csw_r / xi0, op->par.csw_t, C64, CI64, C32, CI32, op->errbits + 1, s));
      if (op->prec == PDD) {
        CK(launch_split_dd(C64, op->clov_mem, 4LL * 36 * g.Vh, s));  // C64 and CI64 are contiguous
        count_launch();
      }
      unsigned eb = 0;
      CK(cudaMemcpyAsync(&eb, op->errbits + 1, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
      CK(cudaStreamSynchronize(s));
      cudaFree(other);
      if (eb != 0) throw Fail(GBF_E_ARG, "singular clover block");
      const size_t perpar = mine / 2;
      op->clov[0] = op->clov_mem;
      op->clov[1] = (char*)op->clov_mem + perpar;
      op->clov_inv[0] = (char*)op->clov_mem + mine;
      op->clov_inv[1] = (char*)op->clov_mem + mine + perpar;
    }
    if (tmpU) {
      CK(cudaStreamSynchronize(s));
      cudaFree(tmpU);
    }
    op->gauge_set = true;
    op->drop_graphs();
  }
}

extern "C" {

int gbf_field_bytes(const gbf_op* op, int which, size_t* bytes) {
  return guarded([&] {
    if (!op || !bytes) throw Fail(GBF_E_ARG, "null argument");
    if (which == 0) *bytes = op->half();
    else if (which == 1) *bytes = 2 * op->half();
    else if (which == 2) *bytes = 2 * op->half4();
    else throw Fail(GBF_E_ARG, "bad field kind");
  });
}

int gbf_field_import(gbf_op* op, const void* natural, void* full, int rhs, int five_d, void* stream) {
  return guarded([&] {
    if (!op || !natural || !full) throw Fail(GBF_E_ARG, "null argument");
    if (rhs < 0 || rhs >= op->g.nrhs) throw Fail(GBF_E_ARG, "rhs out of range");
    const Geo& g = (op->mobius && !five_d) ? op->g4 : op->g;
    CK(launch_import(op->prec, g, (const double2*)natural, full, rhs, 0, (cudaStream_t)stream));
    count_launch();
  });
}

int gbf_field_export(gbf_op* op, const void* full, void* natural, int rhs, int five_d, void* stream) {
  return guarded([&] {
    if (!op || !natural || !full) throw Fail(GBF_E_ARG, "null argument");
    if (rhs < 0 || rhs >= op->g.nrhs) throw Fail(GBF_E_ARG, "rhs out of range");
    const Geo& g = (op->mobius && !five_d) ? op->g4 : op->g;
    CK(launch_import(op->prec, g, (const double2*)natural, const_cast<void*>(full), rhs, 1, (cudaStream_t)stream));
    count_launch();
  });
}

int gbf_norm2(gbf_op* op, const void* x, int nhalves, double* out, void* stream) {
  double im[kMaxRhs];
  return gbf_inner(op, x, x, nhalves, out, im, stream);
}

int gbf_inner(gbf_op* op, const void* x, const void* y, int nhalves, double* out_re, double* out_im, void* stream) {
  return guarded([&] {
    if (!op || !x || !y) throw Fail(GBF_E_ARG, "null argument");
    if (nhalves != 1 && nhalves != 2) throw Fail(GBF_E_ARG, "nhalves must be 1 or 2");
    ensure_ws(op);
    cudaStream_t s = (cudaStream_t)stream;
    double re[kMaxRhs] = {0}, imv[kMaxRhs] = {0};
    for (int h = 0; h < nhalves; ++h) {
      BlasArgs a{};
      a.g = op->g;
      a.x = (const char*)x + h * op->half();
      a.y = (const char*)y + h * op->half();
      a.red = 3;
      a.ra = op->red(FIN_STORE);
      CK(launch_blas(op->prec, a, s));
      count_launch();
      double r1[kMaxRhs], i1[kMaxRhs];
      read_last(op, s, r1, i1);
      for (int r = 0; r < op->g.nrhs; ++r) { re[r] += r1[r]; imv[r] += i1[r]; }
    }
    for (int r = 0; r < op->g.nrhs; ++r) {
      if (out_re) out_re[r] = re[r];
      if (out_im) out_im[r] = imv[r];
    }
  });
}

int gbf_axpby(gbf_op* op, void* out, const double* a_re, const double* a_im, const void* x, const double* b, const void* y,
              int nhalves, void* stream) {
  return guarded([&] {
    if (!op || !out || !x || !a_re) throw Fail(GBF_E_ARG, "null argument");
    ensure_ws(op);
    for (int h = 0; h < nhalves; ++h) {
      BlasArgs a{};
      a.g = op->g;
      a.out = (char*)out + h * op->half();
      a.x = (const char*)x + h * op->half();
      a.y = y ? (const char*)y + h * op->half() : nullptr;
      for (int r = 0; r < op->g.nrhs; ++r) {
        a.a_re[r] = a_re[r];
        a.a_im[r] = a_im ? a_im[r] : 0.0;
        a.b_re[r] = b ? b[r] : 0.0;
      }
      a.write = 1;
      a.red = 0;
      a.ra = op->red(FIN_STORE);
      CK(launch_blas(op->prec, a, (cudaStream_t)stream));
      count_launch();
    }
  });
}

int gbf_axpy_norm2(gbf_op* op, void* out, const double* a_re, const double* a_im, const void* x, const void* y,
                   int nhalves, double* out_norm2, void* stream) {
  return guarded([&] {
    if (!op || !out || !x || !y || !a_re || !out_norm2) throw Fail(GBF_E_ARG, "null argument");
    if (nhalves != 1 && nhalves != 2) throw Fail(GBF_E_ARG, "nhalves must be 1 or 2");
    ensure_ws(op);
    cudaStream_t s = (cudaStream_t)stream;
    double acc[kMaxRhs] = {0};
    for (int h = 0; h < nhalves; ++h) {
      BlasArgs a{};
      a.g = op->g;
      a.out = (char*)out + h * op->half();
      a.x = (const char*)x + h * op->half();
      a.y = (const char*)y + h * op->half();
      for (int r = 0; r < op->g.nrhs; ++r) {
        a.a_re[r] = a_re[r];
        a.a_im[r] = a_im ? a_im[r] : 0.0;
        a.b_re[r] = 1.0;
      }
      a.write = 1;
      a.red = 2;
      a.ra = op->red(FIN_STORE);
      CK(launch_blas(op->prec, a, s));
      count_launch();
      double r1[kMaxRhs];
      read_last(op, s, r1, nullptr);
      for (int r = 0; r < op->g.nrhs; ++r) acc[r] += r1[r];
    }
    for (int r = 0; r < op->g.nrhs; ++r) out_norm2[r] = acc[r];
  });
}

int gbf_convert(gbf_op* dst_op, void* dst, gbf_op* src_op, const void* src, double scale, int nhalves, void* stream) {
  return guarded([&] {
    if (!dst_op || !src_op || !dst || !src) throw Fail(GBF_E_ARG, "null argument");
    if (dst_op->g.N != src_op->g.N) throw Fail(GBF_E_ARG, "operators have different field geometry");
    for (int h = 0; h < nhalves; ++h)
      CK(launch_convert(dst_op->prec, (char*)dst + h * dst_op->half(), src_op->prec, (const char*)src + h * src_op->half(),
                        dst_op->g.N, scale, (cudaStream_t)stream));
    count_launch(nhalves);
  });
}

}  // extern "C"

// ---------------------------------------------------------------------------
// opcode dispatch (lib/cgpt/lib/operators/unary.h:20-48 analogue)
// ---------------------------------------------------------------------------
static void apply_one(gbf_op* op, int opcode, const void* src, void* dst, int sp, cudaStream_t s) {
  const size_t h = op->half();
  auto H = [&](const void* f, int p) { return (const void*)((const char*)f + p * h); };
  auto HW = [&](void* f, int p) { return (void*)((char*)f + p * h); };
  const bool mob = op->mobius;
  switch (opcode) {
    case GBF_MEOOE:
    case GBF_MEOOE_DAG:
    case GBF_DHOP_EO:
    case GBF_DHOP_EO_DAG: {
      if (sp != GBF_EVEN && sp != GBF_ODD) throw Fail(GBF_E_ARG, "even-odd opcode needs src_parity 0 or 1");
      const bool dag = opcode == GBF_MEOOE_DAG || opcode == GBF_DHOP_EO_DAG;
      const bool meo = opcode == GBF_MEOOE || opcode == GBF_MEOOE_DAG;
      if (mob && meo && !dag) {
        op->local(s, sp, src, op->T(0), op->B(false));
        op->dslash(s, 1 - sp, false, op->T(0), dst, op->none());
      } else {
        op->dslash(s, 1 - sp, dag, src, dst, (mob && meo) ? op->B(true) : op->none());
      }
      break;
    }
    case GBF_MOOEE:
    case GBF_MOOEE_DAG:
      op->local(s, sp, src, dst, op->A(opcode == GBF_MOOEE_DAG));
      break;
    case GBF_MOOEE_INV:
    case GBF_MOOEE_INV_DAG:
      op->local(s, sp, src, dst, op->Ainv(opcode == GBF_MOOEE_INV_DAG));
      break;
    case GBF_MDIAG:
      for (int p = 0; p < 2; ++p) op->local(s, p, H(src, p), HW(dst, p), op->A(false));
      break;
    case GBF_DHOP:
    case GBF_DHOP_DAG:
      for (int p = 0; p < 2; ++p) op->dslash(s, p, opcode == GBF_DHOP_DAG, H(src, 1 - p), HW(dst, p), op->none());
      break;
    case GBF_M:
    case GBF_MDAG: {
      const bool dag = opcode == GBF_MDAG;
      for (int p = 0; p < 2; ++p) {
        if (!mob) {
          op->dslash(s, p, dag, H(src, 1 - p), HW(dst, p), op->none(), 1.0, H(src, p), 1.0, op->A(dag));
        } else {
          op->local(s, p, H(src, p), op->T(1), op->A(dag));
          if (!dag) {
            op->local(s, 1 - p, H(src, 1 - p), op->T(0), op->B(false));
            op->dslash(s, p, false, op->T(0), HW(dst, p), op->none(), 1.0, op->T(1), 1.0);
          } else {
            op->dslash(s, p, true, H(src, 1 - p), HW(dst, p), op->B(true), 1.0, op->T(1), 1.0);
          }
        }
      }
      break;
    }
    case GBF_DMINUS:
    case GBF_DMINUS_DAG: {
      if (!mob) {  // Wilson: Dminus is the identity (reference/wilson_clover.py:174-176)
        CK(cudaMemcpyAsync(dst, src, 2 * h, cudaMemcpyDeviceToDevice, s));
        break;
      }
      if (op->zmobius) {
        // per-slice c_s: Dminus = diag(1 - c_s (4 - M5)) + diag(-c_s) Dhop
        // (diag(c_s) and Dhop commute; the adjoint conjugates c_s)
        const bool dag = opcode == GBF_DMINUS_DAG;
        for (int p = 0; p < 2; ++p) {
          op->local(s, p, H(src, p), op->T(8), op->smat_slot(dag ? S_DM1DAG : S_DM1));
          op->dslash(s, p, dag, H(src, 1 - p), HW(dst, p), op->smat_slot(dag ? S_DMCDAG : S_DMC), 1.0, op->T(8), 1.0);
        }
        break;
      }
      // psi - c D_W psi, D_W = (4 - M5) + Dhop, slice by slice
      const double c = op->par.c, d = 1.0 - c * (4.0 - op->par.M5);
      for (int p = 0; p < 2; ++p)
        op->dslash(s, p, opcode == GBF_DMINUS_DAG, H(src, 1 - p), HW(dst, p), op->none(), -c, H(src, p), d);
      break;
    }
    default:
      throw Fail(GBF_E_UNSUPPORTED, "opcode " + std::to_string(opcode) + " not supported");
  }
}

// Mobius wall transfer (4D <-> 5D) on one parity of internal fields.
//   WALL_IMPORT          s = 0 <- P+ eta, s = Ls-1 <- P- eta (ImportUnphysicalFermion;
//                        ImportPhysicalFermionSource applies Dminus after it)
//   WALL_EXPORT_SOLUTION q = P- psi_0 + P+ psi_{Ls-1} (ExportPhysicalFermionSolution)
//   WALL_EXPORT_SOURCE   q = P+ psi_0 + P- psi_{Ls-1} (ExportPhysicalFermionSource,
//                        the adjoint of WALL_IMPORT)
enum { WALL_EXPORT_SOLUTION = 0, WALL_IMPORT = 1, WALL_EXPORT_SOURCE = 2 };
template <int P>
__global__ void wall_kernel(Geo g, Geo g4, const void* in, void* out, int mode) {
  using R = typename SpinorT<P>::R;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= g4.N) return;  // one thread per (4D site, rhs)
  const long long cb = t / g4.N5;
  const int rhs = (int)(t - cb * g4.N5);
  const long long n0 = cb * g.N5 + (long long)rhs * g.Ls, nl = n0 + g.Ls - 1;
  cplx<R> v[12], w[12];
  if (mode == WALL_IMPORT) {
    // s = 0 gets P+ eta, s = Ls-1 gets P- eta (the convention that reproduces
    // the reference's ImportPhysicalFermionSource fingerprint)
    load_spinor<P>(in, g4.N, t, v);
    for (int k = 0; k < 12; ++k) w[k] = (k < 6) ? v[k] : cz<R>();
    store_spinor<P>(out, g.N, n0, w);
    for (int k = 0; k < 12; ++k) w[k] = (k < 6) ? cz<R>() : v[k];
    store_spinor<P>(out, g.N, nl, w);
  } else {
    // solution: q = P- psi_0 + P+ psi_{Ls-1}  (lib/gpt/qcd/fermion/mobius.py:162);
    // source: q = P+ psi_0 + P- psi_{Ls-1}
    const bool sol = mode == WALL_EXPORT_SOLUTION;
    load_spinor<P>(in, g.N, sol ? n0 : nl, v);
    load_spinor<P>(in, g.N, sol ? nl : n0, w);
    for (int k = 0; k < 6; ++k) v[k] = w[k];
    store_spinor<P>(out, g4.N, t, v);
  }
}

static void wall(gbf_op* op, const void* in, void* out, int mode, cudaStream_t s) {
  const unsigned nb = (unsigned)((op->g4.N + 255) / 256);
  const bool to5d = mode == WALL_IMPORT;
  for (int p = 0; p < 2; ++p) {
    const void* i = (const char*)in + p * (to5d ? op->half4() : op->half());
    void* o = (char*)out + p * (to5d ? op->half() : op->half4());
    if (op->prec == P64) wall_kernel<P64><<<nb, 256, 0, s>>>(op->g, op->g4, i, o, mode);
    else if (op->prec == P32) wall_kernel<P32><<<nb, 256, 0, s>>>(op->g, op->g4, i, o, mode);
    else if (op->prec == PDD) wall_kernel<PDD><<<nb, 256, 0, s>>>(op->g, op->g4, i, o, mode);
    else wall_kernel<P16><<<nb, 256, 0, s>>>(op->g, op->g4, i, o, mode);
    CK(cudaGetLastError());
    count_launch();
  }
}

// ---------------------------------------------------------------------------
// eo2_ne CG iteration.  D = odd sites (the reference default parity), C = even.
//   G = C_C^-1 / C_D^-1 (Wilson-clover) or B A^-1 (Mobius), so that
//   Mpc = 1 - Dhop G Dhop G and Mpc^+ = 1 - G^+ Dhop^+ G^+ Dhop^+.
// Workspace: tmp[0..1] t, z ; tmp[2..3] w, u ; tmp[4] p ; tmp[5] r ; tmp[6] mmp ;
//            tmp[7] y (CG solution) ; tmp[8..9] prepare/reconstruct scratch.
// ---------------------------------------------------------------------------
static constexpr int kKernelsPerIteration = 6;

// ev (optional, profile mode): 7 events recorded around the six launches
static void cg_iteration(gbf_op* op, cudaStream_t s, cudaEvent_t* ev = nullptr) {
  const int D = GBF_ODD, C = GBF_EVEN;
  void *t = op->T(0), *z = op->T(1), *w = op->T(2), *u = op->T(3);
  void *p = op->T(4), *r = op->T(5), *mmp = op->T(6), *y = op->T(7);
  auto mark = [&](int i) {
    if (ev) CK(cudaEventRecord(ev[i], s));
  };
  mark(0);
  // p = r + beta p ; t = G_D p
  op->local(s, D, r, t, op->G(), 1.0, nullptr, 0.0, p, 1, 0, nullptr, FIN_STORE, 1);
  mark(1);
  // z = G_C Dhop t
  op->dslash(s, C, false, t, z, op->G(), 1.0, nullptr, 0.0, op->none(), 0, nullptr, FIN_STORE, 1);
  mark(2);
  // w = p - Dhop z
  op->dslash(s, D, false, z, w, op->none(), -1.0, p, 1.0, op->none(), 0, nullptr, FIN_STORE, 1);
  mark(3);
  // u = G_C^+ Dhop^+ w
  op->dslash(s, C, true, w, u, op->Gdag(), 1.0, nullptr, 0.0, op->none(), 0, nullptr, FIN_STORE, 1);
  mark(4);
  // mmp = w - G_D^+ Dhop^+ u ; d = Re <p, mmp> -> alpha
  op->dslash(s, D, true, u, mmp, op->Gdag(), -1.0, w, 1.0, op->none(), 1, p, FIN_ALPHA, 1);
  mark(5);
  // r -= alpha mmp ; y += alpha p ; |r|^2 -> beta, convergence
  op->cg_update(s, r, mmp, y, p);
  mark(6);
}

extern "C" {

int gbf_apply(gbf_op* op, int opcode, const void* const* src, void* const* dst, int n, int src_parity, void* stream) {
  return guarded([&] {
    if (!op || !src || !dst || n < 0) throw Fail(GBF_E_ARG, "null argument");
    if (!op->gauge_set) throw Fail(GBF_E_ARG, "gauge field not set (gbf_update_gauge)");
    ensure_ws(op);
    cudaStream_t s = (cudaStream_t)stream;
    for (int i = 0; i < n; ++i) {
      if (!src[i] || !dst[i]) throw Fail(GBF_E_ARG, "null field");
      if (src[i] == dst[i]) throw Fail(GBF_E_ARG, "src and dst must differ (as in the reference)");
      if (opcode == GBF_IMPORT_PHYSICAL_FERMION_SOURCE || opcode == GBF_IMPORT_UNPHYSICAL_FERMION ||
          opcode == GBF_EXPORT_PHYSICAL_FERMION_SOLUTION || opcode == GBF_EXPORT_PHYSICAL_FERMION_SOURCE) {
        if (!op->mobius) {
          // Wilson: every import and export is a copy (reference/wilson_clover.py:165-173)
          CK(cudaMemcpyAsync(dst[i], src[i], 2 * op->half(), cudaMemcpyDeviceToDevice, s));
        } else if (opcode == GBF_IMPORT_PHYSICAL_FERMION_SOURCE) {
          // walls, then Dminus
          void* t = op->T(2);  // tmp[2], tmp[3] form one contiguous full field
          CK(cudaMemsetAsync(t, 0, 2 * op->half(), s));
          wall(op, src[i], t, WALL_IMPORT, s);
          apply_one(op, GBF_DMINUS, t, dst[i], GBF_FULL, s);
        } else if (opcode == GBF_IMPORT_UNPHYSICAL_FERMION) {
          // the walls alone
          CK(cudaMemsetAsync(dst[i], 0, 2 * op->half(), s));
          wall(op, src[i], dst[i], WALL_IMPORT, s);
        } else {
          wall(op, src[i], dst[i], opcode == GBF_EXPORT_PHYSICAL_FERMION_SOLUTION ? WALL_EXPORT_SOLUTION : WALL_EXPORT_SOURCE, s);
        }
        continue;
      }
      apply_one(op, opcode, src[i], dst[i], src_parity, s);
    }
  });
}

}  // extern "C"

namespace {

void apply_ne(gbf_op* op, cudaStream_t s, const void* in, void* out);

// R_ne of the eo2_ne system: b = Mpc^+ (src_D - Dhop G_C src_C) on the odd
// sites (normal_equation.py:47-48, schur_complement_two.py:87-104); with
// norm = true |b|^2 goes to the CG state (FIN_STORE, the `last` slot)
void eo2ne_prepare(gbf_op* op, cudaStream_t s, const void* src, void* b, bool norm) {
  const int D = GBF_ODD, C = GBF_EVEN;
  const size_t h = op->half();
  const void* srcC = (const char*)src + C * h;
  const void* srcD = (const char*)src + D * h;
  void *s1 = op->T(8), *tC = op->T(9), *u = op->T(3);
  op->local(s, C, srcC, tC, op->G());
  op->dslash(s, D, false, tC, s1, op->none(), -1.0, srcD, 1.0);
  op->dslash(s, C, true, s1, u, op->Gdag());
  op->dslash(s, D, true, u, b, op->Gdag(), -1.0, s1, 1.0, op->none(), norm ? 2 : 0, nullptr, FIN_STORE);
}

// The solution from the odd-site solution y: x_D = A_D^-1 y,
// x_C = A_C^-1 (src_C - Dhop G_D y)  (schur_complement_two.py:106-148)
void eo2ne_reconstruct(gbf_op* op, cudaStream_t s, const void* src, const void* y, void* x) {
  const int D = GBF_ODD, C = GBF_EVEN;
  const size_t h = op->half();
  const void* srcC = (const char*)src + C * h;
  void* xC = (char*)x + C * h;
  void* xD = (char*)x + D * h;
  void *s1 = op->T(8), *tC = op->T(9);
  op->local(s, D, y, xD, op->Ainv(false));
  op->local(s, D, y, tC, op->G());
  op->dslash(s, C, false, tC, s1, op->none(), -1.0, srcC, 1.0);
  op->local(s, C, s1, xC, op->Ainv(false));
}

// The CG loop on the device state prepared in op->st (cp, rsq, done, p, r,
// y = T(4), T(5), T(7)); returns whether the device loop ran and fills the
// profile timings (cg.py:73-105)
bool cg_loop(gbf_op* op, cudaStream_t s, const gbf_cg_params* prm, double* kms, int* kcount) {
  if (prm->profile) {
    // diagnostic: plain launches with CUDA events around each kernel class
    cudaEvent_t ev[7];
    for (int i = 0; i < 7; ++i) CK(cudaEventCreate(&ev[i]));
    for (int it = 0; it < prm->maxiter; ++it) {
      cg_iteration(op, s, ev);
      CK(cudaEventSynchronize(ev[6]));
      float ms;
      CK(cudaEventElapsedTime(&ms, ev[0], ev[1]));
      kms[1] += ms;
      for (int i = 1; i < 5; ++i) {
        CK(cudaEventElapsedTime(&ms, ev[i], ev[i + 1]));
        kms[0] += ms;
      }
      CK(cudaEventElapsedTime(&ms, ev[5], ev[6]));
      kms[2] += ms;
      kcount[0] += 4;
      kcount[1] += 1;
      kcount[2] += 1;
      CK(cudaMemcpyAsync(op->hst, op->st, sizeof(CGState), cudaMemcpyDeviceToHost, s));
      CK(cudaStreamSynchronize(s));
      if (op->hst->all_done) break;
    }
    for (int i = 0; i < 7; ++i) cudaEventDestroy(ev[i]);
  }
  bool device_loop = false;
  if (!prm->profile && prm->iterations_per_graph < 0) {
    // ---- the whole CG loop on the device: a conditional while node whose
    // body is one iteration; the CG update kernel sets the loop condition to
    // !all_done (converged, maxiter reached or every rhs broken down), and
    // its early exit sets it to 0, so the loop ends within maxiter + 1
    // bodies.  No host round trip and no iteration past convergence. ----
    device_loop = true;
    if (!op->cgraph) {
      cudaGraph_t gr;
      CK(cudaGraphCreate(&gr, 0));
      try {
        cudaGraphConditionalHandle h;
        CK(cudaGraphConditionalHandleCreate(&h, gr, 1, cudaGraphCondAssignDefault));
        cudaGraphNodeParams np{};
        np.type = cudaGraphNodeTypeConditional;
        np.conditional.handle = h;
        np.conditional.type = cudaGraphCondTypeWhile;
        np.conditional.size = 1;
        cudaGraphNode_t node;
        CK(cudaGraphAddNode(&node, gr, nullptr, nullptr, 0, &np));
        cudaGraph_t body = np.conditional.phGraph_out[0];
        CK(cudaStreamBeginCaptureToGraph(s, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
        op->cond = h;
        op->cond_active = true;
        try {
          cg_iteration(op, s);
        } catch (...) {
          op->cond_active = false;
          cudaGraph_t t;
          cudaStreamEndCapture(s, &t);
          throw;
        }
        op->cond_active = false;
        cudaGraph_t t;
        CK(cudaStreamEndCapture(s, &t));
        CK(cudaGraphInstantiate(&op->cgraph, gr, 0));
      } catch (...) {
        cudaGraphDestroy(gr);
        throw;
      }
      cudaGraphDestroy(gr);
    }
    CK(cudaGraphLaunch(op->cgraph, s));
    CK(cudaStreamSynchronize(s));
  }
  // ---- CG loop in graphs of K iterations, convergence checked by the host ----
  const int K = prm->iterations_per_graph > 0 ? prm->iterations_per_graph : kDefaultGraphIterations;
  if (!prm->profile && !device_loop && (!op->graph || op->graph_K != K)) {
    op->drop_graphs();
    cudaGraph_t gr;
    CK(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    try {
      for (int k = 0; k < K; ++k) cg_iteration(op, s);
    } catch (...) {
      cudaStreamEndCapture(s, &gr);
      throw;
    }
    CK(cudaStreamEndCapture(s, &gr));
    CK(cudaGraphInstantiate(&op->graph, gr, 0));
    cudaGraphDestroy(gr);
    op->graph_K = K;
  }
  const int max_launches = (prm->profile || device_loop) ? 0 : (prm->maxiter + K - 1) / K;
  bool done = false;
  int launched = 0;
  for (; launched < max_launches && !done; ++launched) {
    CK(cudaGraphLaunch(op->graph, s));
    count_launch((unsigned long long)K * kKernelsPerIteration);
    CK(cudaMemcpyAsync(op->hst + (launched & 1), op->st, sizeof(CGState), cudaMemcpyDeviceToHost, s));
    CK(cudaEventRecord(op->ev_chk[launched & 1], s));
    if (launched > 0) {
      CK(cudaEventSynchronize(op->ev_chk[(launched - 1) & 1]));
      done = op->hst[(launched - 1) & 1].all_done != 0;
    }
  }
  CK(cudaStreamSynchronize(s));
  return device_loop;
}

// Results of a CG run from the final device state (synchronised)
void cg_results(gbf_op* op, cudaStream_t s, cudaStream_t user, bool device_loop, const double* kms, const int* kcount,
                gbf_cg_result* res) {
  CK(cudaMemcpyAsync(op->hst, op->st, sizeof(CGState), cudaMemcpyDeviceToHost, s));
  CK(cudaEventRecord(op->ev_out, s));
  CK(cudaStreamWaitEvent(user, op->ev_out, 0));
  CK(cudaEventSynchronize(op->ev_out));
  const CGState& st = op->hst[0];
  if (st.kernel_error)
    throw Fail(GBF_E_CUDA, "a hopping kernel's wait for its bulk copies timed out (code " +
                               std::to_string(st.kernel_error) + ")");
  if (device_loop) count_launch((unsigned long long)(st.iter > 0 ? st.iter : 1) * kKernelsPerIteration);
  if (res) {
    res->iterations = st.iter;
    int conv = 1;
    for (int k = 0; k < op->g.nrhs; ++k) {
      const double b2 = st.last[k];  // |b|^2 of the system (FIN_STORE before the loop)
      res->residual_sq[k] = b2 > 0 ? st.cp[k] / b2 : 0.0;
      conv &= (st.cp[k] <= st.rsq[k]) ? 1 : 0;
    }
    res->converged = conv;
    res->breakdown = st.breakdown;
    for (int i = 0; i < 3; ++i) {
      res->kernel_ms[i] = kms[i];
      res->kernel_launches[i] = kcount[i];
    }
  }
}

void check_solve_args(gbf_op* op, const void* a, const void* b, const gbf_cg_params* prm) {
  if (!op || !a || !b || !prm) throw Fail(GBF_E_ARG, "null argument");
  if (!op->gauge_set) throw Fail(GBF_E_ARG, "gauge field not set (gbf_update_gauge)");
  ensure_ws(op);
  for (int i = 0; i < 10; ++i) op->T(i);  // allocate before any graph capture
}

}  // namespace

extern "C" {

int gbf_solve_eo2ne_cg(gbf_op* op, const void* src, void* x, const gbf_cg_params* prm, gbf_cg_result* res, void* stream) {
  return guarded([&] {
    check_solve_args(op, src, x, prm);
    cudaStream_t user = (cudaStream_t)stream;
    cudaStream_t s = op->stream;
    CK(cudaEventRecord(op->ev_in, user));
    CK(cudaStreamWaitEvent(s, op->ev_in, 0));
    const size_t h = op->half();
    void *p = op->T(4), *r = op->T(5), *y = op->T(7);
    // ---- prepare: r = R_ne src, |r|^2 -> state; CG from y = 0 ----
    eo2ne_prepare(op, s, src, r, true);
    CK(launch_cg_init(op->st, op->g.nrhs, prm->eps, prm->maxiter, s));
    count_launch();
    CK(cudaMemsetAsync(p, 0, h, s));
    CK(cudaMemsetAsync(y, 0, h, s));
    double kms[3] = {0, 0, 0};
    int kcount[3] = {0, 0, 0};
    const bool device_loop = cg_loop(op, s, prm, kms, kcount);
    // ---- reconstruct: x_D = A^-1 y ; x_C = A_C^-1 (src_C - Dhop G y) ----
    eo2ne_reconstruct(op, s, src, y, x);
    cg_results(op, s, user, device_loop, kms, kcount, res);
  });
}

int gbf_solve_normal_cg(gbf_op* op, const void* b, void* x, const gbf_cg_params* prm, gbf_cg_result* res, void* stream) {
  return guarded([&] {
    check_solve_args(op, b, x, prm);
    if (b == x) throw Fail(GBF_E_ARG, "source and solution must differ");
    cudaStream_t user = (cudaStream_t)stream;
    cudaStream_t s = op->stream;
    CK(cudaEventRecord(op->ev_in, user));
    CK(cudaStreamWaitEvent(s, op->ev_in, 0));
    const size_t h = op->half();
    void *p = op->T(4), *r = op->T(5), *mmp = op->T(6), *y = op->T(7);
    const int nr = op->g.nrhs;
    // |b|^2 -> state (FIN_STORE), then rsq = eps^2 |b|^2
    BlasArgs nb{};
    nb.g = op->g;
    nb.x = b;
    nb.y = b;
    nb.red = 3;
    nb.ra = op->red(FIN_STORE);
    CK(launch_blas(op->prec, nb, s));
    count_launch();
    double b2[kMaxRhs];
    read_last(op, s, b2, nullptr);
    bool zero = true;
    for (int k = 0; k < nr; ++k) zero = zero && b2[k] == 0.0;
    if (zero) {
      // cg.py:66-68: a zero source has the zero solution
      CK(cudaMemsetAsync(x, 0, h, s));
      CK(cudaEventRecord(op->ev_out, s));
      CK(cudaStreamWaitEvent(user, op->ev_out, 0));
      CK(cudaStreamSynchronize(s));
      if (res) {
        std::memset(res, 0, sizeof(*res));
        res->converged = 1;
      }
      return;
    }
    CK(launch_cg_init(op->st, nr, prm->eps, prm->maxiter, s));
    count_launch();
    // r = b - A x (the guess), |r|^2 -> cp and the done flags (FIN_INIT)
    apply_ne(op, s, x, mmp);
    BlasArgs ra{};
    ra.g = op->g;
    ra.out = r;
    ra.x = mmp;
    ra.y = b;
    for (int k = 0; k < nr; ++k) {
      ra.a_re[k] = -1.0;
      ra.b_re[k] = 1.0;
    }
    ra.write = 1;
    ra.red = 2;
    ra.ra = op->red(FIN_INIT);
    CK(launch_blas(op->prec, ra, s));
    count_launch();
    CK(cudaMemcpyAsync(y, x, h, cudaMemcpyDeviceToDevice, s));
    CK(cudaMemsetAsync(p, 0, h, s));
    double kms[3] = {0, 0, 0};
    int kcount[3] = {0, 0, 0};
    const bool device_loop = cg_loop(op, s, prm, kms, kcount);
    CK(cudaMemcpyAsync(x, y, h, cudaMemcpyDeviceToDevice, s));
    cg_results(op, s, user, device_loop, kms, kcount, res);
  });
}

// MADWF fifth-dimension moves (lib/gpt/qcd/fermion/preconditioner/mixed_dwf.py:43-98)
int gbf_chiral_shift(gbf_op* op, const void* src, void* dst, int offset, int nhalves, void* stream) {
  return guarded([&] {
    if (!op || !src || !dst) throw Fail(GBF_E_ARG, "null argument");
    if (nhalves != 1 && nhalves != 2) throw Fail(GBF_E_ARG, "nhalves must be 1 or 2");
    if (src == dst) throw Fail(GBF_E_ARG, "src and dst must differ");
    const size_t h = op->half();
    for (int hf = 0; hf < nhalves; ++hf) {
      CK(launch_chiral_shift(op->prec, op->g, (const char*)src + hf * h, (char*)dst + hf * h, offset,
                             (cudaStream_t)stream));
      count_launch();
    }
  });
}

int gbf_copy_slices(gbf_op* dst_op, void* dst, int dst_s0, gbf_op* src_op, const void* src, int src_s0, int count,
                    double scale, int nhalves, void* stream) {
  return guarded([&] {
    if (!dst_op || !src_op || !dst || !src) throw Fail(GBF_E_ARG, "null argument");
    if (nhalves != 1 && nhalves != 2) throw Fail(GBF_E_ARG, "nhalves must be 1 or 2");
    const Geo &gd = dst_op->g, &gs = src_op->g;
    if (dst_op->prec != src_op->prec) throw Fail(GBF_E_ARG, "fields of different precision");
    for (int m = 0; m < 4; ++m)
      if (gd.L[m] != gs.L[m]) throw Fail(GBF_E_ARG, "fields of different 4D geometry");
    if (gd.nrhs != gs.nrhs) throw Fail(GBF_E_ARG, "fields with different n_rhs");
    if (count < 0 || dst_s0 < 0 || src_s0 < 0 || dst_s0 + count > gd.Ls || src_s0 + count > gs.Ls)
      throw Fail(GBF_E_ARG, "slice range outside the fifth dimension");
    if (src == dst && dst_s0 != src_s0) throw Fail(GBF_E_ARG, "overlapping slice copy");
    const size_t hd = dst_op->half(), hs = src_op->half();
    for (int hf = 0; hf < nhalves; ++hf) {
      CK(launch_copy_slices(dst_op->prec, gd, (char*)dst + hf * hd, dst_s0, gs, (const char*)src + hf * hs, src_s0,
                            count, scale, (cudaStream_t)stream));
      count_launch();
    }
  });
}

int gbf_eo2ne_prepare(gbf_op* op, const void* src, void* b, void* stream) {
  return guarded([&] {
    if (!op || !src || !b) throw Fail(GBF_E_ARG, "null argument");
    if (!op->gauge_set) throw Fail(GBF_E_ARG, "gauge field not set (gbf_update_gauge)");
    ensure_ws(op);
    eo2ne_prepare(op, (cudaStream_t)stream, src, b, false);
  });
}

int gbf_eo2ne_reconstruct(gbf_op* op, const void* src, const void* y, void* x, void* stream) {
  return guarded([&] {
    if (!op || !src || !y || !x) throw Fail(GBF_E_ARG, "null argument");
    if (!op->gauge_set) throw Fail(GBF_E_ARG, "gauge field not set (gbf_update_gauge)");
    if (x == src || x == y) throw Fail(GBF_E_ARG, "the solution must not alias the inputs");
    ensure_ws(op);
    eo2ne_reconstruct(op, (cudaStream_t)stream, src, y, x);
  });
}

// dst = sum_n left_n <right_n, src> f_n  (lib/gpt/algorithms/modes/matrix.py:31-56)
int gbf_modes_apply(gbf_op* op, const void* const* left, const void* const* right, const double* f, int n,
                    const void* src, void* dst, int nhalves, void* stream) {
  return guarded([&] {
    if (!op || !left || !right || !f || !src || !dst) throw Fail(GBF_E_ARG, "null argument");
    if (n < 1) throw Fail(GBF_E_ARG, "at least one mode");
    if (nhalves != 1 && nhalves != 2) throw Fail(GBF_E_ARG, "nhalves must be 1 or 2");
    if (src == dst) throw Fail(GBF_E_ARG, "src and dst must differ (as in the reference)");
    if (op->g.nrhs != 1) throw Fail(GBF_E_UNSUPPORTED, "mode representations act on fields with one right-hand side");
    for (int i = 0; i < n; ++i) {
      if (!left[i] || !right[i]) throw Fail(GBF_E_ARG, "null mode");
      if (left[i] == dst) throw Fail(GBF_E_ARG, "dst must not be a mode");
    }
    ensure_ws(op);
    if (op->mode_cap < 2 * n) {
      cudaFree(op->mode_dev);
      op->mode_dev = nullptr;
      op->mode_dev = (double2*)dmalloc((size_t)2 * n * sizeof(double2));
      op->mode_cap = 2 * n;
    }
    cudaStream_t s = (cudaStream_t)stream;
    const size_t h = op->half();
    // <right_n, src> per half, every block of modes on the stream, one read back
    for (int hf = 0; hf < nhalves; ++hf) {
      for (int i0 = 0; i0 < n; i0 += kModeBlock) {
        const int m = std::min(kModeBlock, n - i0);
        ModeDotArgs a{};
        for (int j = 0; j < m; ++j) a.v[j] = (const char*)right[i0 + j] + hf * h;
        a.n = m;
        a.src = (const char*)src + hf * h;
        a.partial = op->partial;
        a.counter = op->counter;
        a.out = op->mode_dev + (size_t)hf * n + i0;
        CK(launch_mode_dot(op->prec, op->g, a, op->partial_cap, s));
        count_launch();
      }
    }
    std::vector<double2> c((size_t)nhalves * n);
    CK(cudaMemcpyAsync(c.data(), op->mode_dev, c.size() * sizeof(double2), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    // w_n = f_n <right_n, src>, the halves summed in order
    std::vector<std::complex<double>> w(n, 0.0);
    for (int hf = 0; hf < nhalves; ++hf)
      for (int i = 0; i < n; ++i) w[i] += std::complex<double>(c[(size_t)hf * n + i].x, c[(size_t)hf * n + i].y);
    for (int i = 0; i < n; ++i) w[i] *= std::complex<double>(f[2 * i], f[2 * i + 1]);
    // dst = sum_n w_n left_n, kModeBlock modes per pass
    for (int hf = 0; hf < nhalves; ++hf) {
      for (int i0 = 0; i0 < n; i0 += kModeBlock) {
        const int m = std::min(kModeBlock, n - i0);
        ModeAxpyArgs a{};
        for (int j = 0; j < m; ++j) {
          a.v[j] = (const char*)left[i0 + j] + hf * h;
          a.w[j] = make_double2(w[i0 + j].real(), w[i0 + j].imag());
        }
        a.n = m;
        a.out = (char*)dst + hf * h;
        a.accumulate = i0 > 0;
        CK(launch_mode_axpy(op->prec, op->g, a, s));
        count_launch();
      }
    }
  });
}

// ---------------------------------------------------------------------------
// autotuner: time each block-size candidate of the four kernel classes on
// scratch fields of this operator (CUDA events on the caller's stream) and
// keep the fastest.  Candidates: blockDim = S * N5, S a power of two,
// 32 <= blockDim <= 256 (or N5 itself when N5 > 128).
// ---------------------------------------------------------------------------
int gbf_tune(gbf_op* op, void* stream, int* out_bd, double* out_us) {
  return guarded([&] {
    if (!op || !out_bd) throw Fail(GBF_E_ARG, "null argument");
    if (!op->gauge_set) throw Fail(GBF_E_ARG, "gauge field not set (gbf_update_gauge)");
    ensure_ws(op);
    cudaStream_t s = (cudaStream_t)stream;
    for (int i = 0; i < 4; ++i) CK(cudaMemsetAsync(op->T(i), 0, op->half(), s));
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    const int N5 = op->g.N5;
    std::vector<int> cand;
    for (int S = 1; S * N5 <= 256; S *= 2)
      if (S * N5 >= 32 || N5 > 128) cand.push_back(S * N5);
    if (cand.empty()) cand.push_back(pick_bd(0, N5));
    // CG update timing: a state whose right-hand sides never converge, so
    // that no launch returns early on the all-done flag
    CGState* cgs = op->hst + 1;
    std::memset(cgs, 0, sizeof(CGState));
    cgs->nrhs = op->g.nrhs;
    cgs->maxiter = 1 << 30;
    for (int r = 0; r < op->g.nrhs; ++r) {
      cgs->cp[r] = 1.0;
      cgs->rsq[r] = -1.0;
    }
    auto run = [&](int cls) {
      if (cls == 3) CK(cudaMemcpyAsync(op->st, cgs, sizeof(CGState), cudaMemcpyHostToDevice, s));
      switch (cls) {
        case 0: op->dslash(s, 0, false, op->T(0), op->T(1), op->mobius ? op->none() : op->G()); break;
        case 1: op->dslash(s, 0, false, op->T(0), op->T(1), op->G()); break;
        case 2: op->local(s, 0, op->T(0), op->T(1), op->G()); break;
        default: op->cg_update(s, op->T(0), op->T(1), op->T(2), op->T(3)); break;
      }
    };
    for (int cls = 0; cls < 4; ++cls) {
      out_bd[cls] = 0;
      if (out_us) out_us[cls] = 0.0;
      if (cls == 1 && !op->mobius) continue;
      int best = cand[0];
      float best_ms = 1e30f;
      for (int bd : cand) {
        op->tuned_bd[cls] = bd;
        run(cls);  // warm-up
        CK(cudaEventRecord(e0, s));
        for (int r = 0; r < 3; ++r) run(cls);
        CK(cudaEventRecord(e1, s));
        CK(cudaEventSynchronize(e1));
        float ms = 0;
        CK(cudaEventElapsedTime(&ms, e0, e1));
        if (ms < best_ms) {
          best_ms = ms;
          best = bd;
        }
      }
      op->tuned_bd[cls] = best;
      out_bd[cls] = best;
      if (out_us) out_us[cls] = 1000.0 * best_ms / 3.0;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    op->drop_graphs();
  });
}

int gbf_set_tuning(gbf_op* op, const int* bd) {
  return guarded([&] {
    if (!op || !bd) throw Fail(GBF_E_ARG, "null argument");
    for (int i = 0; i < 4; ++i) op->tuned_bd[i] = bd[i] > 0 ? pick_bd(bd[i], op->g.N5) : 0;
    op->drop_graphs();
  });
}

}  // extern "C"

// ---------------------------------------------------------------------------
// block CG (lib/gpt/algorithms/inverter/block_cg.py:36-149, after Grid's
// BlockConjugateGradient with a Cholesky QR): the k = n_rhs packed right-hand
// sides of the eo2_ne normal equations share one Krylov space.  Vectors and
// Gram matrices live on the device; the k x k algebra (inverse, Cholesky)
// runs on the host in complex128, as in the reference, with one Gram read
// back per half iteration.
// ---------------------------------------------------------------------------
namespace {

using zc = std::complex<double>;
using zmat = std::vector<zc>;  // k x k, row-major

zmat zmul(int k, const zmat& a, const zmat& b) {
  zmat c((size_t)k * k, zc(0.0, 0.0));
  for (int i = 0; i < k; ++i)
    for (int l = 0; l < k; ++l) {
      const zc ail = a[(size_t)i * k + l];
      for (int j = 0; j < k; ++j) c[(size_t)i * k + j] += ail * b[(size_t)l * k + j];
    }
  return c;
}
zmat zadj(int k, const zmat& a) {
  zmat c((size_t)k * k);
  for (int i = 0; i < k; ++i)
    for (int j = 0; j < k; ++j) c[(size_t)j * k + i] = std::conj(a[(size_t)i * k + j]);
  return c;
}
// Cholesky of the Hermitian part of A: A = L L^H, L lower; false if A is not
// positive definite or numerically rank deficient (a pivot below 1e-13 of
// its diagonal entry: linearly dependent block vectors)
bool zcholesky(int k, const zmat& A, zmat& L) {
  L.assign((size_t)k * k, zc(0.0, 0.0));
  for (int j = 0; j < k; ++j) {
    const double ajj = A[(size_t)j * k + j].real();
    double d = ajj;
    for (int l = 0; l < j; ++l) d -= std::norm(L[(size_t)j * k + l]);
    if (!(d > 1e-13 * ajj) || !std::isfinite(d)) return false;
    const double ljj = std::sqrt(d);
    L[(size_t)j * k + j] = ljj;
    for (int i = j + 1; i < k; ++i) {
      zc v = 0.5 * (A[(size_t)i * k + j] + std::conj(A[(size_t)j * k + i]));
      for (int l = 0; l < j; ++l) v -= L[(size_t)i * k + l] * std::conj(L[(size_t)j * k + l]);
      L[(size_t)i * k + j] = v / ljj;
    }
  }
  return true;
}
// inverse of an upper-triangular U
zmat zinv_upper(int k, const zmat& U) {
  zmat X((size_t)k * k, zc(0.0, 0.0));
  for (int c = 0; c < k; ++c) {
    for (int i = c; i >= 0; --i) {
      zc v = (i == c) ? zc(1.0, 0.0) : zc(0.0, 0.0);
      for (int l = i + 1; l <= c; ++l) v -= U[(size_t)i * k + l] * X[(size_t)l * k + c];
      X[(size_t)i * k + c] = v / U[(size_t)i * k + i];
    }
  }
  return X;
}
// general inverse, Gauss-Jordan with partial pivoting; false if singular
bool zinv(int k, zmat A, zmat& X) {
  X.assign((size_t)k * k, zc(0.0, 0.0));
  for (int i = 0; i < k; ++i) X[(size_t)i * k + i] = 1.0;
  for (int c = 0; c < k; ++c) {
    int piv = c;
    for (int r = c + 1; r < k; ++r)
      if (std::abs(A[(size_t)r * k + c]) > std::abs(A[(size_t)piv * k + c])) piv = r;
    if (std::abs(A[(size_t)piv * k + c]) == 0.0 || !std::isfinite(std::abs(A[(size_t)piv * k + c]))) return false;
    for (int l = 0; l < k; ++l) {
      std::swap(A[(size_t)c * k + l], A[(size_t)piv * k + l]);
      std::swap(X[(size_t)c * k + l], X[(size_t)piv * k + l]);
    }
    const zc d = 1.0 / A[(size_t)c * k + c];
    for (int l = 0; l < k; ++l) {
      A[(size_t)c * k + l] *= d;
      X[(size_t)c * k + l] *= d;
    }
    for (int r = 0; r < k; ++r) {
      if (r == c) continue;
      const zc f = A[(size_t)r * k + c];
      if (f == zc(0.0, 0.0)) continue;
      for (int l = 0; l < k; ++l) {
        A[(size_t)r * k + l] -= f * A[(size_t)c * k + l];
        X[(size_t)r * k + l] -= f * X[(size_t)c * k + l];
      }
    }
  }
  return true;
}

void ensure_block_ws(gbf_op* op) {
  if (op->blk_partial) return;
  int dev = 0, sms = 152;
  if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int k = op->g.nrhs;
  op->blk_max_blocks = (long long)sms * 32;
  op->blk_partial = (double2*)dmalloc((size_t)op->blk_max_blocks * k * k * sizeof(double2));
  op->blk_dev = (double2*)dmalloc((size_t)5 * k * k * sizeof(double2));
  CK(cudaMallocHost(&op->blk_host, (size_t)5 * k * k * sizeof(double2)));
}

// Z = Mpc^+ Mpc D on the odd sites (the CG iteration's kernel sequence)
void apply_ne(gbf_op* op, cudaStream_t s, const void* in, void* out) {
  const int D = GBF_ODD, C = GBF_EVEN;
  void *t = op->T(0), *z = op->T(1), *w = op->T(2), *u = op->T(3);
  op->local(s, D, in, t, op->G());
  op->dslash(s, C, false, t, z, op->G());
  op->dslash(s, D, false, z, w, op->none(), -1.0, in, 1.0);
  op->dslash(s, C, true, w, u, op->Gdag());
  op->dslash(s, D, true, u, out, op->Gdag(), -1.0, w, 1.0);
}

// Gram matrix <A_i, B_j> of two packed half fields, read back (synchronises s)
zmat gram(gbf_op* op, cudaStream_t s, const void* A, const void* B) {
  const int k = op->g.nrhs;
  CK(launch_gram(op->prec, op->g, A, B, op->blk_partial, op->blk_max_blocks, op->counter, op->blk_dev, s));
  count_launch(gram_launches(op->prec, op->g));
  CK(cudaMemcpyAsync(op->blk_host, op->blk_dev, (size_t)k * k * sizeof(double2), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  zmat m((size_t)k * k);
  for (int q = 0; q < k * k; ++q) m[q] = zc(op->blk_host[q].x, op->blk_host[q].y);
  return m;
}

double2* upload(gbf_op* op, cudaStream_t s, int slot, const zmat& W) {
  const int k = op->g.nrhs;
  double2* h = op->blk_host + (size_t)slot * k * k;
  for (int q = 0; q < k * k; ++q) h[q] = make_double2(W[q].real(), W[q].imag());
  double2* d = op->blk_dev + (size_t)slot * k * k;
  CK(cudaMemcpyAsync(d, h, (size_t)k * k * sizeof(double2), cudaMemcpyHostToDevice, s));
  return d;
}

// out1 = b1 Y1 + X1 W1 ; out2 = b2 Y2 + c out1 + X2 W2 (coefficient slots 1, 2 or 3, 4)
void lincomb2(gbf_op* op, cudaStream_t s, int slot, void* out1, const void* Y1, double b1, const void* X1, const zmat& W1,
              void* out2, const void* Y2, double b2, double c, const void* X2, const zmat& W2) {
  double2* d1 = upload(op, s, slot, W1);
  double2* d2 = upload(op, s, slot + 1, W2);
  CK(launch_lincomb2(op->prec, op->g, out1, Y1, b1, X1, d1, out2, Y2, b2, c, X2, d2, s));
  count_launch();
}

// out = beta Y + X W with W uploaded into coefficient slot `slot` (1..4)
void lincomb(gbf_op* op, cudaStream_t s, int slot, void* out, const void* Y, double beta, const void* X, const zmat& W) {
  const int k = op->g.nrhs;
  double2* h = op->blk_host + (size_t)slot * k * k;
  for (int q = 0; q < k * k; ++q) h[q] = make_double2(W[q].real(), W[q].imag());
  double2* d = op->blk_dev + (size_t)slot * k * k;
  CK(cudaMemcpyAsync(d, h, (size_t)k * k * sizeof(double2), cudaMemcpyHostToDevice, s));
  CK(launch_lincomb(op->prec, op->g, out, Y, beta, X, d, s));
  count_launch();
}

}  // namespace

extern "C" int gbf_solve_eo2ne_block_cg(gbf_op* op, const void* src, void* x, const gbf_cg_params* prm,
                                        gbf_cg_result* res, void* stream) {
  return guarded([&] {
    if (!op || !src || !x || !prm) throw Fail(GBF_E_ARG, "null argument");
    if (!op->gauge_set) throw Fail(GBF_E_ARG, "gauge field not set (gbf_update_gauge)");
    ensure_ws(op);
    ensure_block_ws(op);
    for (int i = 0; i < 12; ++i) op->T(i);
    cudaStream_t s = (cudaStream_t)stream;
    const int k = op->g.nrhs;
    const int D = GBF_ODD, C = GBF_EVEN;
    const size_t h = op->half();
    const void* srcC = (const char*)src + C * h;
    const void* srcD = (const char*)src + D * h;
    void* xC = (char*)x + C * h;
    void* xD = (char*)x + D * h;
    void *Dv = op->T(4), *B = op->T(5), *Z = op->T(6), *X = op->T(7), *s1 = op->T(8), *tC = op->T(9);
    void *Q = op->T(10), *tmp = op->T(11), *u = op->T(3);
    // ---- prepare B = Mpc^+ (src_D - Dhop G_C src_C), |B_b|^2 ----
    op->local(s, C, srcC, tC, op->G());
    op->dslash(s, D, false, tC, s1, op->none(), -1.0, srcD, 1.0);
    op->dslash(s, C, true, s1, u, op->Gdag());
    op->dslash(s, D, true, u, B, op->Gdag(), -1.0, s1, 1.0, op->none(), 2, nullptr, FIN_STORE);
    double ssq[kMaxRhs];
    read_last(op, s, ssq, nullptr);
    CK(cudaMemsetAsync(X, 0, h, s));
    int iters = 0, converged = 0, breakdown = 0;
    std::vector<double> rel(k, 0.0);
    double total = 0.0;
    for (int b = 0; b < k; ++b) total += ssq[b];
    if (total > 0.0) {
      // QR of R = B (X = 0): Q C = B, D = Q
      zmat L, Cm;
      if (!zcholesky(k, gram(op, s, B, B), L)) {
        breakdown = 1;
      } else {
        Cm = zadj(k, L);
        lincomb(op, s, 1, Q, nullptr, 0.0, B, zinv_upper(k, Cm));
        CK(cudaMemcpyAsync(Dv, Q, h, cudaMemcpyDeviceToDevice, s));
        void* Dn = s1;  // free until the reconstruction
        for (int it = 0; it < prm->maxiter; ++it) {
          apply_ne(op, s, Dv, Z);
          zmat M;
          if (!zinv(k, gram(op, s, Dv, Z), M)) {
            breakdown = 1;
            break;
          }
          // X += D (M C) ; tmp = Q - Z M
          zmat mM = M;
          for (auto& v : mM) v = -v;
          lincomb2(op, s, 1, X, X, 1.0, Dv, zmul(k, M, Cm), tmp, Q, 1.0, 0.0, Z, mM);
          // QR: Q S = tmp
          if (!zcholesky(k, gram(op, s, tmp, tmp), L)) {
            breakdown = 1;
            break;
          }
          const zmat S = zadj(k, L);
          // Q = tmp S^-1 ; D = Q + D S^H
          lincomb2(op, s, 3, Q, nullptr, 0.0, tmp, zinv_upper(k, S), Dn, nullptr, 0.0, 1.0, Dv, zadj(k, S));
          std::swap(Dv, Dn);
          Cm = zmul(k, S, Cm);
          const zmat rr = zmul(k, zadj(k, Cm), Cm);
          double worst = 0.0;
          for (int b = 0; b < k; ++b) {
            rel[b] = ssq[b] > 0.0 ? rr[(size_t)b * k + b].real() / ssq[b] : 0.0;
            worst = std::max(worst, rel[b]);
          }
          iters = it + 1;
          if (worst <= prm->eps * prm->eps) {
            converged = 1;
            break;
          }
        }
      }
    } else {
      converged = 1;
    }
    // ---- reconstruct: x_D = A^-1 X ; x_C = A_C^-1 (src_C - Dhop G X) ----
    op->local(s, D, X, xD, op->Ainv(false));
    op->local(s, D, X, tC, op->G());
    op->dslash(s, C, false, tC, s1, op->none(), -1.0, srcC, 1.0);
    op->local(s, C, s1, xC, op->Ainv(false));
    CK(cudaStreamSynchronize(s));
    if (res) {
      std::memset(res, 0, sizeof(*res));
      res->iterations = iters;
      res->converged = converged;
      res->breakdown = breakdown;
      for (int b = 0; b < k; ++b) res->residual_sq[b] = rel[b];
    }
  });
}

// ---------------------------------------------------------------------------
// The eo2_ne normal operator and multi-shift CG on it
// (lib/gpt/algorithms/inverter/multi_shift_cg.py:24-144): solves
// (Mpc^+ Mpc + s_j) x_j = src on the odd sites for every shift s_j with one
// Krylov space.  The vector updates run on the device (one fused pass for all
// shifts); the per-shift scalar recurrences run on the host in double, two
// reductions read back per iteration, as in the reference.
// ---------------------------------------------------------------------------
namespace {

// out = a x + b y on one half field (nrhs 1), then red: 0 none, 2 |out|^2,
// 3 <x, y> without writing; synchronises s when red != 0 and returns the value
double blas_half(gbf_op* op, cudaStream_t s, void* out, double a, const void* x, double b, const void* y, int red) {
  BlasArgs ba{};
  ba.g = op->g;
  ba.out = out;
  ba.x = x;
  ba.y = y;
  ba.a_re[0] = a;
  ba.b_re[0] = b;
  ba.write = red == 3 ? 0 : 1;
  ba.red = red;
  ba.ra = op->red(FIN_STORE);
  CK(launch_blas(op->prec, ba, s));
  count_launch();
  if (!red) return 0.0;
  double re[kMaxRhs], im[kMaxRhs];
  read_last(op, s, re, im);
  return re[0];
}

}  // namespace

extern "C" int gbf_apply_eo2ne_normal(gbf_op* op, const void* in, void* out, void* stream) {
  return guarded([&] {
    if (!op || !in || !out) throw Fail(GBF_E_ARG, "null argument");
    if (!op->gauge_set) throw Fail(GBF_E_ARG, "gauge field not set (gbf_update_gauge)");
    if (in == out) throw Fail(GBF_E_ARG, "source and destination must differ");
    ensure_ws(op);
    apply_ne(op, (cudaStream_t)stream, in, out);
  });
}

extern "C" int gbf_solve_eo2ne_multishift(gbf_op* op, const void* src, void* const* x, const double* shifts, int n,
                                          const gbf_cg_params* prm, gbf_cg_result* res, void* stream) {
  return guarded([&] {
    if (!op || !src || !x || !shifts || !prm) throw Fail(GBF_E_ARG, "null argument");
    if (!op->gauge_set) throw Fail(GBF_E_ARG, "gauge field not set (gbf_update_gauge)");
    if (n < 1 || n > kMaxShifts) throw Fail(GBF_E_ARG, "1 to 32 shifts");
    if (op->g.nrhs != 1) throw Fail(GBF_E_UNSUPPORTED, "multi-shift CG takes one right-hand side (n_rhs = 1)");
    ensure_ws(op);
    for (int i = 0; i < 8; ++i) op->T(i);
    const size_t h = op->half();
    if (op->ms_count < n) {
      cudaFree(op->ms_mem);
      op->ms_mem = nullptr;
      op->ms_mem = dmalloc((size_t)n * h);
      op->ms_count = n;
    }
    cudaStream_t s = (cudaStream_t)stream;
    const int D = GBF_ODD;
    void *p = op->T(4), *r = op->T(5), *mmp = op->T(6);
    std::vector<void*> pj(n);
    for (int j = 0; j < n; ++j) {
      pj[j] = (char*)op->ms_mem + (size_t)j * h;
      CK(cudaMemcpyAsync(pj[j], src, h, cudaMemcpyDeviceToDevice, s));
      CK(cudaMemsetAsync(x[j], 0, h, s));
    }
    CK(cudaMemcpyAsync(p, src, h, cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(r, src, h, cudaMemcpyDeviceToDevice, s));
    std::vector<double> rh(n, 1.0), aj(n, 1.0), bj(n, 0.0), gh(n, 1.0);
    std::vector<int> conv(n, 0);
    double b = 0.0, a = blas_half(op, s, nullptr, 1.0, src, 0.0, src, 3);
    if (!(a > 0.0)) throw Fail(GBF_E_ARG, "multi-shift CG needs a non-zero source");
    const double src2 = a, rsq = prm->eps * prm->eps * a;
    double cp = a;
    int iters = 0, breakdown = 0, all = 0;
    for (int k = 0; k < prm->maxiter && !all; ++k) {
      const double c = cp;
      // mmp = Mpc^+ Mpc p, d = Re <p, mmp>
      void *t = op->T(0), *z = op->T(1), *w = op->T(2), *u = op->T(3);
      op->local(s, D, p, t, op->G());
      op->dslash(s, GBF_EVEN, false, t, z, op->G());
      op->dslash(s, D, false, z, w, op->none(), -1.0, p, 1.0);
      op->dslash(s, GBF_EVEN, true, w, u, op->Gdag());
      op->dslash(s, D, true, u, mmp, op->Gdag(), -1.0, w, 1.0, op->none(), 1, p, FIN_STORE);
      double dre[kMaxRhs], dim[kMaxRhs];
      read_last(op, s, dre, dim);
      const double d = dre[0];
      if (!(d > 0.0) || !std::isfinite(d)) {
        breakdown = 1;
        break;
      }
      double om = b / a;
      a = c / d;
      om *= a;
      cp = blas_half(op, s, r, -a, mmp, 1.0, r, 2);  // r -= a mmp ; |r|^2
      b = cp / c;
      MultiShiftArgs ms{};
      ms.r = r;
      for (int j = 0; j < n; ++j) {
        if (conv[j]) continue;
        const double q = 1.0 / (1.0 + shifts[j] * a + (1.0 - rh[j]) * om);
        rh[j] = q;
        aj[j] = q * a;
        bj[j] = q * q * b;
        gh[j] *= q;
        ms.x[ms.n] = x[j];
        ms.p[ms.n] = pj[j];
        ms.a[ms.n] = aj[j];
        ms.b[ms.n] = bj[j];
        ms.g[ms.n] = gh[j];
        ++ms.n;
      }
      CK(launch_multishift(op->prec, op->g, ms, s));
      count_launch();
      blas_half(op, s, p, b, p, 1.0, r, 0);  // p = b p + r
      iters = k + 1;
      all = 1;
      for (int j = 0; j < n; ++j) {
        if (!conv[j] && gh[j] * gh[j] * cp <= rsq) conv[j] = 1;
        all &= conv[j];
      }
    }
    CK(cudaStreamSynchronize(s));
    if (res) {
      std::memset(res, 0, sizeof(*res));
      res->iterations = iters;
      res->converged = all;
      res->breakdown = breakdown;
      for (int j = 0; j < n && j < 16; ++j) res->residual_sq[j] = gh[j] * gh[j] * cp / src2;
    }
  });
}
