// oracle.cpp -- CPU restatement of the gpt fermion-matrix hot path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the oracle for the CUDA path in
// gpt_gb300/csrc: tests/, __graft_entry__.smoke() and the cpu_baseline /
// reference leg of bench.py may load it; the product never does.
//
// What is restated here, each block citing the reference file it follows
// (paths relative to the lehner/gpt project root):
//   * SHA-256 (FIPS 180-4), as used for seeding in lib/cgpt/lib/random/vector.h:38-58
//   * ranlux24 subtract-with-borrow with luxury skip, lib/cgpt/lib/random/ranlux.h:33-114
//   * the 64-lane vector generator, lib/cgpt/lib/random/vector.h:19-114
//   * bit pool / uniform / Box-Muller / cnormal, lib/cgpt/lib/random/distribution.h:20-159
//   * per-grid block-parallel streams, lib/cgpt/lib/random/engine.h:88-99,
//     lib/cgpt/lib/random/parallel.h:20-126,132-180
//   * random SU(3) links, lib/gpt/core/random.py:103-148 with the generators of
//     lib/gpt/core/object_type/su_n.py:208-239 and the matrix exponential of
//     lib/gpt/core/foundation/lattice/matrix/exp.py:167-219
//   * plaquette, lib/gpt/qcd/gauge/stencil/plaquette.py:25-47
//   * Wilson-clover operator, lib/gpt/qcd/fermion/reference/wilson_clover.py:42-262
//     (field strength lib/gpt/qcd/gauge/loops.py:162-174, gamma basis
//     lib/gpt/core/gamma.py:28-41, boundary phases lib/gpt/core/covariant.py:22-60)
//   * Mobius domain-wall operator, tests/qcd/domain_wall.py:309-340 and
//     lib/gpt/qcd/fermion/mobius.py:29-46
//   * eo2_ne preconditioned CG, lib/gpt/algorithms/preconditioner/schur_complement_two.py:87-148,
//     lib/gpt/algorithms/preconditioner/normal_equation.py:44-51,
//     lib/gpt/algorithms/inverter/cg.py:47-105
//   * defect correction with a reduced-precision inner solve,
//     lib/gpt/algorithms/inverter/defect_correcting.py:85-130
//
// Field layouts ("natural" layout, shared with the product's host interface):
//   4D site index  = x0 + L0*(x1 + L1*(x2 + L2*x3))
//   spinor         = [site][spin 4][colour 3] complex (re, im interleaved)
//   5D spinor      = [site][s][spin][colour]   (s fastest, as in gpt's F_grid)
//   gauge field    = [mu][site][row][col]
#include <cstdint>
#include <cstring>
#include <cmath>
#include <cfloat>
#include <vector>
#include <map>
#include <string>
#include <memory>
#include <stdexcept>
#include <algorithm>
#include <omp.h>

extern "C" {
static thread_local std::string g_err;
const char* orc_last_error() { return g_err.c_str(); }
}

template <typename F> static int guarded(F&& f) {
  try {
    f();
    return 0;
  } catch (const std::exception& e) {
    g_err = e.what();
    return 1;
  }
}

// ---------------------------------------------------------------------------
// complex helpers
// ---------------------------------------------------------------------------
template <typename T> struct cx {
  T re, im;
};
template <typename T> static inline cx<T> cmul(cx<T> a, cx<T> b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
template <typename T> static inline cx<T> cmulc(cx<T> a, cx<T> b) { return {a.re * b.re + a.im * b.im, a.re * b.im - a.im * b.re}; }  // conj(a)*b
template <typename T> static inline cx<T> cadd(cx<T> a, cx<T> b) { return {a.re + b.re, a.im + b.im}; }
template <typename T> static inline cx<T> csub(cx<T> a, cx<T> b) { return {a.re - b.re, a.im - b.im}; }
template <typename T> static inline cx<T> cscale(T s, cx<T> a) { return {s * a.re, s * a.im}; }

// ---------------------------------------------------------------------------
// SHA-256, FIPS 180-4.  Output: the eight 32-bit state words H0..H7.
// ---------------------------------------------------------------------------
static const uint32_t kSha[64] = {
    0x428a2f98, 0x71374491, 0xb5c0fbcf, 0xe9b5dba5, 0x3956c25b, 0x59f111f1, 0x923f82a4, 0xab1c5ed5, 0xd807aa98, 0x12835b01, 0x243185be,
    0x550c7dc3, 0x72be5d74, 0x80deb1fe, 0x9bdc06a7, 0xc19bf174, 0xe49b69c1, 0xefbe4786, 0x0fc19dc6, 0x240ca1cc, 0x2de92c6f, 0x4a7484aa,
    0x5cb0a9dc, 0x76f988da, 0x983e5152, 0xa831c66d, 0xb00327c8, 0xbf597fc7, 0xc6e00bf3, 0xd5a79147, 0x06ca6351, 0x14292967, 0x27b70a85,
    0x2e1b2138, 0x4d2c6dfc, 0x53380d13, 0x650a7354, 0x766a0abb, 0x81c2c92e, 0x92722c85, 0xa2bfe8a1, 0xa81a664b, 0xc24b8b70, 0xc76c51a3,
    0xd192e819, 0xd6990624, 0xf40e3585, 0x106aa070, 0x19a4c116, 0x1e376c08, 0x2748774c, 0x34b0bcb5, 0x391c0cb3, 0x4ed8aa4a, 0x5b9cca4f,
    0x682e6ff3, 0x748f82ee, 0x78a5636f, 0x84c87814, 0x8cc70208, 0x90befffa, 0xa4506ceb, 0xbef9a3f7, 0xc67178f2};

static inline uint32_t rotr(uint32_t x, int n) { return (x >> n) | (x << (32 - n)); }

static void sha256_block(uint32_t h[8], const uint8_t* blk) {
  uint32_t w[64];
  for (int i = 0; i < 16; ++i)
    w[i] = (uint32_t)blk[4 * i] << 24 | (uint32_t)blk[4 * i + 1] << 16 | (uint32_t)blk[4 * i + 2] << 8 | (uint32_t)blk[4 * i + 3];
  for (int i = 16; i < 64; ++i) {
    uint32_t s0 = rotr(w[i - 15], 7) ^ rotr(w[i - 15], 18) ^ (w[i - 15] >> 3);
    uint32_t s1 = rotr(w[i - 2], 17) ^ rotr(w[i - 2], 19) ^ (w[i - 2] >> 10);
    w[i] = w[i - 16] + s0 + w[i - 7] + s1;
  }
  uint32_t a = h[0], b = h[1], c = h[2], d = h[3], e = h[4], f = h[5], g = h[6], hh = h[7];
  for (int i = 0; i < 64; ++i) {
    uint32_t S1 = rotr(e, 6) ^ rotr(e, 11) ^ rotr(e, 25);
    uint32_t ch = (e & f) ^ (~e & g);
    uint32_t t1 = hh + S1 + ch + kSha[i] + w[i];
    uint32_t S0 = rotr(a, 2) ^ rotr(a, 13) ^ rotr(a, 22);
    uint32_t mj = (a & b) ^ (a & c) ^ (b & c);
    uint32_t t2 = S0 + mj;
    hh = g; g = f; f = e; e = d + t1; d = c; c = b; b = a; a = t1 + t2;
  }
  h[0] += a; h[1] += b; h[2] += c; h[3] += d; h[4] += e; h[5] += f; h[6] += g; h[7] += hh;
}

static void sha256_words(const uint8_t* data, size_t n, uint32_t out[8]) {
  uint32_t h[8] = {0x6a09e667, 0xbb67ae85, 0x3c6ef372, 0xa54ff53a, 0x510e527f, 0x9b05688c, 0x1f83d9ab, 0x5be0cd19};
  size_t full = n / 64;
  for (size_t i = 0; i < full; ++i) sha256_block(h, data + 64 * i);
  uint8_t tail[128];
  size_t rem = n - 64 * full;
  std::memset(tail, 0, sizeof(tail));
  std::memcpy(tail, data + 64 * full, rem);
  tail[rem] = 0x80;
  size_t tl = (rem + 1 + 8 <= 64) ? 64 : 128;
  uint64_t bits = (uint64_t)n * 8;
  for (int i = 0; i < 8; ++i) tail[tl - 1 - i] = (uint8_t)(bits >> (8 * i));
  sha256_block(h, tail);
  if (tl == 128) sha256_block(h, tail + 64);
  for (int i = 0; i < 8; ++i) out[i] = h[i];
}

extern "C" int orc_sha256(const uint8_t* data, size_t n, uint32_t* out) {
  sha256_words(data, n, out);
  return 0;
}

// ---------------------------------------------------------------------------
// ranlux24: x_n = (x_{n-10} - x_{n-24} - c) mod 2^24 with borrow c, and after
// every 24 returned values p-24 further values are skipped (luxury p=389).
// Ring indexing follows lib/cgpt/lib/random/ranlux.h:36-43,74-93 so that the
// seed words land on the same lags as in the reference.
// ---------------------------------------------------------------------------
struct Ranlux24 {
  uint32_t x[24];
  uint32_t carry = 0;
  int off = 0;
  int discard = 23;
  int p = 389;
  void seed(const uint32_t* s) {
    for (int i = 0; i < 24; ++i) x[i] = s[i] & 0xFFFFFFu;
    carry = (s[0] == 0);
    off = 0;
    discard = 23;
  }
  inline uint32_t step() {
    off = (off + 1) % 24;
    uint32_t& lag24 = x[(23 - off + 24) % 24];
    uint32_t lag10 = x[(9 - off + 24) % 24];
    uint32_t d = lag10 - lag24 - carry;  // unsigned wraparound
    carry = (d >= (1u << 24));
    d += (1u << 24);
    lag24 = d & 0xFFFFFFu;
    return lag24;
  }
  inline uint32_t operator()() {
    if (++discard == 24) {
      discard = 0;
      for (int i = 0; i < p - 24; ++i) step();
    }
    return step();
  }
};

// 64 independent ranlux24 lanes; lane k is seeded with outputs [24k, 24k+24)
// of a scalar ranlux24 that is itself seeded from SHA-256 words
// (lib/cgpt/lib/random/vector.h:33-101).
struct VectorRng {
  Ranlux24 lanes[64];
  uint32_t buffer[64];
  int nbuffer = 0;
  explicit VectorRng(const std::vector<uint64_t>& s) {
    uint32_t words[24];
    int nw = 0;
    uint64_t idx = 0;
    while (nw < 24) {
      std::vector<uint64_t> tmp = s;
      tmp.push_back(idx++);
      uint32_t hw[8];
      sha256_words(reinterpret_cast<const uint8_t*>(tmp.data()), tmp.size() * sizeof(uint64_t), hw);
      for (int w = 0; w < 8 && nw < 24; ++w) words[nw++] = hw[w];
    }
    Ranlux24 scalar;
    scalar.seed(words);
    for (int k = 0; k < 64; ++k) {
      uint32_t ls[24];
      for (int j = 0; j < 24; ++j) ls[j] = scalar();
      lanes[k].seed(ls);
    }
    populate();
  }
  void populate() {
    for (int k = 0; k < 64; ++k) buffer[k] = lanes[k]();
    nbuffer = 0;
  }
  uint32_t operator()() {
    if (nbuffer == 64) populate();
    return buffer[nbuffer++];
  }
};

// Bit pool and distributions, lib/cgpt/lib/random/distribution.h:20-137.
struct Dist {
  VectorRng rng;
  uint64_t state = 0;
  int nbits = 0;
  std::vector<double> stack;
  explicit Dist(const std::vector<uint64_t>& s) : rng(s) { populate(); }
  void populate() {
    state = state * (uint64_t)(1u << 24) + rng();
    nbits += 24;
    if (nbits > 64) nbits = 64;
  }
  uint64_t get_bits(int bits) {
    while (bits > nbits) populate();
    uint64_t base = (uint64_t)1 << bits;
    uint64_t res = state & (base - 1);
    state /= base;
    nbits -= bits;
    return res;
  }
  double get_double() { return (double)get_bits(53) / (double)((uint64_t)1 << 53); }
  static int ilog2(uint64_t n) { return (n > 1) ? 1 + ilog2(n >> 1) : 0; }
  uint64_t get_uniform_int(uint64_t max) {
    if (max == 0) return 0;
    int bits = ilog2(max) + 1;
    while (true) {
      uint64_t r = get_bits(bits);
      if (r <= max) return r;
    }
  }
  double get_normal() {
    if (!stack.empty()) {
      double r = stack.back();
      stack.pop_back();
      return r;
    }
    const double two_pi = 2.0 * 3.14159265358979323846;
    double u1, u2;
    do {
      u1 = get_double();
      u2 = get_double();
    } while (u1 <= DBL_MIN);
    double z0 = std::sqrt(-2.0 * std::log(u1)) * std::cos(two_pi * u2);
    double z1 = std::sqrt(-2.0 * std::log(u1)) * std::sin(two_pi * u2);
    stack.push_back(z1);
    return z0;
  }
};

enum { DIST_NORMAL = 0, DIST_CNORMAL = 1, DIST_UNIFORM_REAL = 2, DIST_UNIFORM_INT = 3, DIST_ZN = 4 };

static void draw(Dist& d, int dist, double p0, double p1, double* re, double* im) {
  switch (dist) {
    case DIST_NORMAL: *re = d.get_normal() * p1 + p0; *im = 0; break;
    case DIST_CNORMAL: {
      double i = d.get_normal() * p1 + p0;  // imaginary part is drawn first
      double r = d.get_normal() * p1 + p0;
      *re = r; *im = i;
      break;
    }
    case DIST_UNIFORM_REAL: *re = d.get_double() * (p1 - p0) + p0; *im = 0; break;
    case DIST_UNIFORM_INT: *re = (double)((int64_t)d.get_uniform_int((uint64_t)((int)p1 - (int)p0)) + (int)p0); *im = 0; break;
    case DIST_ZN: {
      int n = (int)p0;
      double k = (double)d.get_uniform_int((uint64_t)(n - 1));
      double ang = k * (2.0 * M_PI / (double)n);
      *re = std::cos(ang); *im = std::sin(ang);
      break;
    }
    default: throw std::runtime_error("unknown distribution");
  }
}

// Per-grid parallel streams: 2^nd-site blocks (s not blocked for 5D grids),
// block seed = seed string ++ fdims ++ gdims ++ [block hash],
// lib/cgpt/lib/random/engine.h:88-99 and parallel.h:20-126.
struct Prng {
  int nd;
  std::vector<long> dims, block_dim, reduced_dim;
  std::vector<std::unique_ptr<Dist>> blocks;
  long sites_per_block;
};

struct Engine {
  std::string seed_str;
  Dist srng;
  std::map<std::string, std::unique_ptr<Prng>> prng;
  static std::vector<uint64_t> str_seed(const std::string& s) {
    std::vector<uint64_t> r;
    for (char c : s) r.push_back((uint64_t)(int64_t)c);
    return r;
  }
  explicit Engine(const std::string& s) : seed_str(s), srng(str_seed(s)) {}
  Prng& get(const std::string& key, int nd, const long* dims) {
    auto it = prng.find(key);
    if (it != prng.end()) return *it->second;
    auto p = std::make_unique<Prng>();
    p->nd = nd;
    p->dims.assign(dims, dims + nd);
    p->block_dim.resize(nd);
    p->reduced_dim.resize(nd);
    std::vector<bool> blocked(nd, true);
    if (nd == 5) blocked[0] = false;
    if (nd > 5) throw std::runtime_error("nd > 5 not supported");
    long nblocks = 1;
    for (int j = 0; j < nd; ++j) {
      if (blocked[j]) {
        if (dims[j] % 2) throw std::runtime_error("dimension not divisible by 2");
        p->block_dim[j] = dims[j] / 2;
        p->reduced_dim[j] = 2;
      } else {
        p->block_dim[j] = 1;
        p->reduced_dim[j] = dims[j];
      }
      nblocks *= p->block_dim[j];
    }
    long sites = 1;
    for (int j = 0; j < nd; ++j) sites *= dims[j];
    p->sites_per_block = sites / nblocks;
    std::vector<uint64_t> base = str_seed(seed_str);
    for (int j = 0; j < nd; ++j) base.push_back((uint64_t)dims[j]);  // fdimensions
    for (int j = 0; j < nd; ++j) base.push_back((uint64_t)dims[j]);  // gdimensions (full grid)
    p->blocks.resize(nblocks);
#pragma omp parallel for schedule(dynamic)
    for (long idx = 0; idx < nblocks; ++idx) {
      // block coordinate, dim 0 fastest
      long r = idx;
      std::vector<long> bc(nd);
      for (int j = 0; j < nd; ++j) {
        bc[j] = r % p->block_dim[j];
        r /= p->block_dim[j];
      }
      // hash: blocked dims, dim 0 slowest
      long t = 0;
      for (int j = 0; j < nd; ++j)
        if (blocked[j]) t = t * (dims[j] / 2) + bc[j];
      std::vector<uint64_t> s = base;
      s.push_back((uint64_t)t);
      p->blocks[idx] = std::make_unique<Dist>(s);
    }
    Prng& ref = *p;
    prng[key] = std::move(p);
    return ref;
  }
};

extern "C" {
void* orc_rng_new(const char* seed) { return new Engine(seed); }
void orc_rng_free(void* e) { delete (Engine*)e; }

// One scalar draw from the engine-level stream (used when no lattice is given).
int orc_rng_scalar(void* e, int dist, double p0, double p1, double* out2) {
  return guarded([&] { draw(((Engine*)e)->srng, dist, p0, p1, out2, out2 + 1); });
}

// Fill one lattice with n_per_site complex numbers per site (natural layout).
int orc_rng_sample(void* e, const char* key, int nd, const long* dims, int dist, double p0, double p1, int n_per_site, double* out) {
  return guarded([&] {
    Engine& eng = *(Engine*)e;
    Prng& pr = eng.get(key, nd, dims);
    long nblocks = (long)pr.blocks.size();
    long spb = pr.sites_per_block;
#pragma omp parallel for schedule(dynamic)
    for (long idx = 0; idx < nblocks; ++idx) {
      Dist& d = *pr.blocks[idx];
      std::vector<long> bc(nd), rc(nd);
      long r = idx;
      for (int j = 0; j < nd; ++j) {
        bc[j] = r % pr.block_dim[j];
        r /= pr.block_dim[j];
      }
      for (long i = 0; i < spb; ++i) {
        long q = i;
        for (int j = 0; j < nd; ++j) {
          rc[j] = q % pr.reduced_dim[j];
          q /= pr.reduced_dim[j];
        }
        long site = 0;
        for (int j = nd - 1; j >= 0; --j) site = site * pr.dims[j] + bc[j] * pr.reduced_dim[j] + rc[j];
        for (int c = 0; c < n_per_site; ++c) {
          double re, im;
          draw(d, dist, p0, p1, &re, &im);
          out[2 * (site * n_per_site + c)] = re;
          out[2 * (site * n_per_site + c) + 1] = im;
        }
      }
    }
  });
}
}

// ---------------------------------------------------------------------------
// SU(3) algebra, exponential, random links
// ---------------------------------------------------------------------------
typedef cx<double> cd;

// Generators in the order of lib/gpt/core/object_type/su_n.py:211-235,
// normalised to Tr(T_a T_b) = delta_ab / 2.
static void su3_generators(cd T[8][9]) {
  int n = 0;
  for (int i = 0; i < 3; ++i)
    for (int j = i + 1; j < 3; ++j) {
      cd a[9] = {}, b[9] = {};
      a[3 * i + j] = {1, 0}; a[3 * j + i] = {1, 0};
      b[3 * i + j] = {0, -1}; b[3 * j + i] = {0, 1};
      std::memcpy(T[n++], a, sizeof(a));
      std::memcpy(T[n++], b, sizeof(b));
      if (j == i + 1) {
        cd c[9] = {};
        for (int l = 0; l < j; ++l) c[4 * l] = {1, 0};
        c[4 * j] = {(double)-j, 0};
        std::memcpy(T[n++], c, sizeof(c));
      }
    }
  for (int k = 0; k < 8; ++k) {
    double tr = 0;
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c) tr += cmul(T[k][3 * r + c], T[k][3 * c + r]).re;
    double nrm = std::sqrt(tr * 2.0);
    for (int e = 0; e < 9; ++e) T[k][e] = cscale(1.0 / nrm, T[k][e]);
  }
}

static inline void mat3_mul(const cd* a, const cd* b, cd* c) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      cd s = {0, 0};
      for (int k = 0; k < 3; ++k) s = cadd(s, cmul(a[3 * i + k], b[3 * k + j]));
      c[3 * i + j] = s;
    }
}
static inline void mat3_adj(const cd* a, cd* c) {
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) c[3 * i + j] = {a[3 * j + i].re, -a[3 * j + i].im};
}

// exp(X) for a whole field of 3x3 matrices: one global scaling 2^-ns chosen
// from the field norm, 19th-order Taylor series, ns squarings
// (lib/gpt/core/foundation/lattice/matrix/exp.py:167-219).
static void field_exp(cd* X, long V) {
  double n2 = 0;
#pragma omp parallel for reduction(+ : n2)
  for (long i = 0; i < V * 9; ++i) n2 += X[i].re * X[i].re + X[i].im * X[i].im;
  double n = std::sqrt(n2) / (double)V;
  const double maxn = 0.01;
  int ns = 0;
  if (n > maxn) ns = (int)std::log2(n / maxn);
  double sc = 1.0 / std::pow(2.0, ns);
#pragma omp parallel for
  for (long s = 0; s < V; ++s) {
    cd x[9], o[9], xn[9], t[9];
    for (int e = 0; e < 9; ++e) x[e] = ns ? cscale(sc, X[9 * s + e]) : X[9 * s + e];
    for (int e = 0; e < 9; ++e) o[e] = {(e % 4 == 0) ? 1.0 : 0.0, 0.0};
    std::memcpy(xn, x, sizeof(xn));
    for (int e = 0; e < 9; ++e) o[e] = cadd(o[e], xn[e]);
    double nfac = 1.0;
    for (int j = 2; j <= 19; ++j) {
      nfac /= j;
      mat3_mul(xn, x, t);
      std::memcpy(xn, t, sizeof(xn));
      for (int e = 0; e < 9; ++e) o[e] = cadd(o[e], cscale(nfac, xn[e]));
    }
    for (int k = 0; k < ns; ++k) {
      mat3_mul(o, o, t);
      std::memcpy(o, t, sizeof(o));
    }
    std::memcpy(X + 9 * s, o, sizeof(o));
  }
}

extern "C" {
// g.qcd.gauge.random(grid, rng, scale): for each mu, for each generator a,
// one uniform_real[-0.5,0.5] draw per site; X = sum_a scale*c_a*T_a; U = exp(iX)
// (lib/gpt/qcd/gauge/create.py:66-70, lib/gpt/core/random.py:117-148).
int orc_gauge_random(void* e, const char* key, const long* dims, double scale, double* Uout) {
  return guarded([&] {
    long V = dims[0] * dims[1] * dims[2] * dims[3];
    cd T[8][9];
    su3_generators(T);
    std::vector<double> c(2 * V);
    for (int mu = 0; mu < 4; ++mu) {
      cd* X = reinterpret_cast<cd*>(Uout) + (size_t)mu * V * 9;
      for (long i = 0; i < V * 9; ++i) X[i] = {0, 0};
      for (int a = 0; a < 8; ++a) {
        if (orc_rng_sample(e, key, 4, dims, DIST_UNIFORM_REAL, -0.5, 0.5, 1, c.data())) throw std::runtime_error(g_err);
#pragma omp parallel for
        for (long s = 0; s < V; ++s) {
          cd ca = {scale * c[2 * s], scale * c[2 * s + 1]};
          for (int el = 0; el < 9; ++el) X[9 * s + el] = cadd(X[9 * s + el], cmul(ca, T[a][el]));
        }
      }
      // exp(i X)
#pragma omp parallel for
      for (long i = 0; i < V * 9; ++i) X[i] = {-X[i].im, X[i].re};
      field_exp(X, V);
    }
  });
}

// exp(i*X) of a field of 3x3 matrices (same algorithm as above).
int orc_field_exp_i(double* X, long V) {
  return guarded([&] {
    cd* x = reinterpret_cast<cd*>(X);
#pragma omp parallel for
    for (long i = 0; i < V * 9; ++i) x[i] = {-x[i].im, x[i].re};
    field_exp(x, V);
  });
}
}

// ---------------------------------------------------------------------------
// Lattice geometry
// ---------------------------------------------------------------------------
struct Geom {
  long L[4];
  long V;
  std::vector<int32_t> fwd[4], bwd[4];
  std::vector<int32_t> par_sites[2];  // sites of each parity, ascending
  std::vector<uint8_t> parity;
  explicit Geom(const long* dims) {
    V = 1;
    for (int m = 0; m < 4; ++m) { L[m] = dims[m]; V *= L[m]; }
    for (int m = 0; m < 4; ++m) { fwd[m].resize(V); bwd[m].resize(V); }
    parity.resize(V);
    for (long s = 0; s < V; ++s) {
      long x[4], r = s;
      for (int m = 0; m < 4; ++m) { x[m] = r % L[m]; r /= L[m]; }
      parity[s] = (uint8_t)((x[0] + x[1] + x[2] + x[3]) & 1);
      for (int m = 0; m < 4; ++m) {
        long y[4] = {x[0], x[1], x[2], x[3]};
        y[m] = (x[m] + 1) % L[m];
        fwd[m][s] = (int32_t)(y[0] + L[0] * (y[1] + L[1] * (y[2] + L[2] * y[3])));
        y[m] = (x[m] + L[m] - 1) % L[m];
        bwd[m][s] = (int32_t)(y[0] + L[0] * (y[1] + L[1] * (y[2] + L[2] * y[3])));
      }
    }
    for (long s = 0; s < V; ++s) par_sites[parity[s]].push_back((int32_t)s);
  }
  long coord(long s, int m) const {
    for (int k = 0; k < m; ++k) s /= L[k];
    return s % L[m];
  }
};

extern "C" double orc_plaquette(const double* Uin, const long* dims) {
  Geom G(dims);
  const cd* U = reinterpret_cast<const cd*>(Uin);
  long V = G.V;
  double sum = 0;
#pragma omp parallel for reduction(+ : sum)
  for (long s = 0; s < V; ++s) {
    for (int mu = 0; mu < 4; ++mu)
      for (int nu = 0; nu < mu; ++nu) {
        // U_mu(x) U_nu(x+mu) U_mu(x+nu)^+ U_nu(x)^+
        cd a[9], b[9], t[9], t2[9];
        mat3_mul(U + 9 * ((size_t)mu * V + s), U + 9 * ((size_t)nu * V + G.fwd[mu][s]), t);
        mat3_adj(U + 9 * ((size_t)mu * V + G.fwd[nu][s]), a);
        mat3_mul(t, a, t2);
        mat3_adj(U + 9 * ((size_t)nu * V + s), b);
        mat3_mul(t2, b, t);
        sum += t[0].re + t[4].re + t[8].re;
      }
  }
  return 2.0 * sum / (double)V / 4.0 / 3.0 / 3.0;
}

// ---------------------------------------------------------------------------
// Gamma matrices (lib/gpt/core/gamma.py:28-41) in sparse form:
// gamma_mu[row][perm[row]] = coef[row]; every row has exactly one entry.
// ---------------------------------------------------------------------------
struct GammaSparse {
  int perm[4];
  cd coef[4];
};
static const GammaSparse kGamma[4] = {
    {{3, 2, 1, 0}, {{0, 1}, {0, 1}, {0, -1}, {0, -1}}},
    {{3, 2, 1, 0}, {{-1, 0}, {1, 0}, {1, 0}, {-1, 0}}},
    {{2, 3, 0, 1}, {{0, 1}, {0, -1}, {0, -1}, {0, 1}}},
    {{2, 3, 0, 1}, {{1, 0}, {1, 0}, {1, 0}, {1, 0}}},
};
static void gamma_dense(int mu, cd g[16]) {
  for (int i = 0; i < 16; ++i) g[i] = {0, 0};
  for (int r = 0; r < 4; ++r) g[4 * r + kGamma[mu].perm[r]] = kGamma[mu].coef[r];
}

// ---------------------------------------------------------------------------
// Wilson hopping term with anisotropy and boundary phases:
//   Dhop psi(x) = -sum_mu cc_mu/2 [ (1 - g_mu) U_mu(x) psi(x+mu)
//                                  + (1 + g_mu) U_mu(x-mu)^+ psi(x-mu) ]
// (lib/gpt/qcd/fermion/reference/wilson_clover.py:182-200, written there as
// cc/2 (g_mu - 1) fwd - cc/2 (g_mu + 1) bwd), cc = nu/xi_0 for spatial mu and
// 1 for mu = 3.  The adjoint swaps (1 -+ g_mu).  Links carry the boundary phase
// on the slice x_mu = L_mu - 1 (lib/gpt/core/covariant.py:27-36).
// Spin projection: rows 2,3 of (1 + s g)psi equal s*coef[row]*row perm[row].
// ---------------------------------------------------------------------------
template <typename T>
struct Hop {
  const Geom* G;
  std::vector<cx<T>> U;  // [mu][site][9], boundary phases applied
  T cc[4];
  void load(const Geom* g, const double* Uin, const double* phases, double aniso) {
    G = g;
    long V = G->V;
    U.resize((size_t)4 * V * 9);
    const cd* u = reinterpret_cast<const cd*>(Uin);
    for (int mu = 0; mu < 4; ++mu) {
      cd ph = {phases[2 * mu], phases[2 * mu + 1]};
#pragma omp parallel for
      for (long s = 0; s < V; ++s) {
        bool last = G->coord(s, mu) == G->L[mu] - 1;
        for (int e = 0; e < 9; ++e) {
          cd v = u[9 * ((size_t)mu * V + s) + e];
          if (last) v = cmul(v, ph);
          U[9 * ((size_t)mu * V + s) + e] = {(T)v.re, (T)v.im};
        }
      }
      cc[mu] = (T)((mu == 3) ? 1.0 : aniso);
    }
  }
  // out(x) for every x of `out_parity` (0, 1, or 2 = all sites).
  // n5: number of 5th-dimension entries per site (spinors [site][n5][12]).
  void apply(cx<T>* out, const cx<T>* in, int out_parity, bool dag, int n5) const {
    const long V = G->V;
    const std::vector<int32_t>* list = out_parity < 2 ? &G->par_sites[out_parity] : nullptr;
    const long n = list ? (long)list->size() : V;
    const T sf = dag ? (T)1 : (T)-1;  // (1 + sf g) on the forward term
#pragma omp parallel for schedule(static)
    for (long i = 0; i < n; ++i) {
      const long x = list ? (*list)[i] : i;
      for (int s5 = 0; s5 < n5; ++s5) {
        cx<T> acc[4][3];
        for (int a = 0; a < 4; ++a)
          for (int c = 0; c < 3; ++c) acc[a][c] = {0, 0};
        for (int mu = 0; mu < 4; ++mu) {
          const GammaSparse& gm = kGamma[mu];
          for (int dir = 0; dir < 2; ++dir) {
            const long y = dir == 0 ? G->fwd[mu][x] : G->bwd[mu][x];
            const T sg = dir == 0 ? sf : -sf;
            const cx<T>* psi = in + ((size_t)y * n5 + s5) * 12;
            const cx<T>* u = dir == 0 ? &U[9 * ((size_t)mu * V + x)] : &U[9 * ((size_t)mu * V + y)];
            // h_r = psi_r + sg*coef_r*psi_perm(r), r = 0,1
            cx<T> h[2][3], uh[2][3];
            for (int r = 0; r < 2; ++r) {
              cx<T> cf = {(T)gm.coef[r].re * sg, (T)gm.coef[r].im * sg};
              for (int c = 0; c < 3; ++c) h[r][c] = cadd(psi[3 * r + c], cmul(cf, psi[3 * gm.perm[r] + c]));
            }
            for (int r = 0; r < 2; ++r)
              for (int a = 0; a < 3; ++a) {
                cx<T> sacc = {0, 0};
                for (int b = 0; b < 3; ++b)
                  sacc = cadd(sacc, dir == 0 ? cmul(u[3 * a + b], h[r][b]) : cmulc(u[3 * b + a], h[r][b]));
                uh[r][a] = sacc;
              }
            const T w = cc[mu];
            for (int r = 0; r < 2; ++r)
              for (int c = 0; c < 3; ++c) acc[r][c] = cadd(acc[r][c], cscale(w, uh[r][c]));
            for (int r = 2; r < 4; ++r) {
              cx<T> cf = {(T)gm.coef[r].re * sg, (T)gm.coef[r].im * sg};
              for (int c = 0; c < 3; ++c) acc[r][c] = cadd(acc[r][c], cscale(w, cmul(cf, uh[gm.perm[r]][c])));
            }
          }
        }
        cx<T>* o = out + ((size_t)x * n5 + s5) * 12;
        for (int a = 0; a < 4; ++a)
          for (int c = 0; c < 3; ++c) o[3 * a + c] = cscale((T)-0.5, acc[a][c]);
      }
    }
  }
};

// ---------------------------------------------------------------------------
// Clover term (lib/gpt/qcd/fermion/reference/wilson_clover.py:91-127):
//   C(x) = sum_{mu<nu} -1/2 c_p sigma_munu (x) F_munu(x) + 1/(2 kappa),
//   c_p = csw_t if nu = 3 else csw_r/xi_0, 1/(2 kappa) = m0 + 1 + 3 nu/xi_0,
//   F_munu = 1/8 (Q - Q^+) from the clover leaves (lib/gpt/qcd/gauge/loops.py:162-174).
// sigma_munu commutes with gamma_5 = diag(1,1,-1,-1), so C(x) is two 6x6
// blocks (spins {0,1} and {2,3}) stored as [site][block][6][6].
// ---------------------------------------------------------------------------
static void field_strength_site(const Geom& G, const cd* U, long V, int mu, int nu, long x, cd F[9]) {
  auto L = [&](int m, long s) { return U + 9 * ((size_t)m * V + s); };
  cd t1[9], t2[9], a[9], b[9];
  // staple_up(y) = U_nu(y+mu) U_mu(y+nu)^+ U_nu(y)^+
  auto staple_up = [&](long y, cd* out) {
    cd p[9], q[9];
    mat3_adj(L(mu, G.fwd[nu][y]), p);
    mat3_mul(L(nu, G.fwd[mu][y]), p, q);
    mat3_adj(L(nu, y), p);
    mat3_mul(q, p, out);
  };
  // staple_down(y) = [U_nu(z+mu)^+ U_mu(z)^+ U_nu(z)] at z = y - nu
  auto staple_down = [&](long y, cd* out) {
    long z = G.bwd[nu][y];
    cd p[9], q[9], r[9];
    mat3_adj(L(nu, G.fwd[mu][z]), p);
    mat3_adj(L(mu, z), q);
    mat3_mul(p, q, r);
    mat3_mul(r, L(nu, z), out);
  };
  auto vfield = [&](long y, cd* out) {
    cd su[9], sd[9];
    staple_up(y, su);
    staple_down(y, sd);
    for (int e = 0; e < 9; ++e) out[e] = csub(su[e], sd[e]);
  };
  vfield(x, a);
  mat3_mul(L(mu, x), a, t1);
  long xm = G.bwd[mu][x];
  vfield(xm, b);
  mat3_mul(b, L(mu, xm), t2);
  cd Fr[9];
  for (int e = 0; e < 9; ++e) Fr[e] = cadd(t1[e], t2[e]);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 3; ++j) {
      cd d = {Fr[3 * j + i].re, -Fr[3 * j + i].im};
      F[3 * i + j] = cscale(0.125, csub(Fr[3 * i + j], d));
    }
}

static bool invert_cmat(int n, const cd* A, cd* Ainv) {
  std::vector<cd> M(A, A + n * n), I(n * n, cd{0, 0});
  for (int i = 0; i < n; ++i) I[i * n + i] = {1, 0};
  for (int col = 0; col < n; ++col) {
    int piv = col;
    double best = -1;
    for (int r = col; r < n; ++r) {
      double m = M[r * n + col].re * M[r * n + col].re + M[r * n + col].im * M[r * n + col].im;
      if (m > best) { best = m; piv = r; }
    }
    if (best <= 0) return false;
    if (piv != col)
      for (int k = 0; k < n; ++k) { std::swap(M[col * n + k], M[piv * n + k]); std::swap(I[col * n + k], I[piv * n + k]); }
    cd p = M[col * n + col];
    double pn = p.re * p.re + p.im * p.im;
    cd pinv = {p.re / pn, -p.im / pn};
    for (int k = 0; k < n; ++k) { M[col * n + k] = cmul(M[col * n + k], pinv); I[col * n + k] = cmul(I[col * n + k], pinv); }
    for (int r = 0; r < n; ++r) {
      if (r == col) continue;
      cd f = M[r * n + col];
      if (f.re == 0 && f.im == 0) continue;
      for (int k = 0; k < n; ++k) {
        M[r * n + k] = csub(M[r * n + k], cmul(f, M[col * n + k]));
        I[r * n + k] = csub(I[r * n + k], cmul(f, I[col * n + k]));
      }
    }
  }
  std::memcpy(Ainv, I.data(), sizeof(cd) * n * n);
  return true;
}

// ---------------------------------------------------------------------------
// Operators
// ---------------------------------------------------------------------------
enum {
  OP_M = 2001, OP_MDAG = 2002, OP_MEOOE = 2003, OP_MEOOE_DAG = 2004, OP_MOOEE = 2005, OP_MOOEE_DAG = 2006,
  OP_MOOEE_INV = 2007, OP_MOOEE_INV_DAG = 2008, OP_MDIAG = 2009, OP_DMINUS = 2010, OP_DMINUS_DAG = 2011,
  OP_IMPORT_PHYS_SRC = 2012, OP_IMPORT_UNPHYS = 2013, OP_EXPORT_PHYS_SOL = 2014, OP_EXPORT_PHYS_SRC = 2015,
  OP_DHOP = 3001, OP_DHOP_DAG = 4001
};

// Common interface used by the even-odd solver: all fields are natural
// full-lattice arrays; "parity" restricts the sites written.
template <typename T>
struct OpBase {
  const Geom* G = nullptr;
  int n5 = 1;  // 5th-dimension entries per 4D site
  virtual ~OpBase() {}
  virtual void Meooe(cx<T>* out, const cx<T>* in, int out_parity, bool dag) const = 0;
  // the hopping term alone (Grid's Dhop/DhopEO: for the 5D operator the 4D hop on every s-slice)
  virtual void Dhop(cx<T>* out, const cx<T>* in, int out_parity, bool dag) const = 0;
  virtual void Mooee(cx<T>* out, const cx<T>* in, int parity, bool dag, bool inv) const = 0;
  size_t site_len() const { return (size_t)n5 * 12; }
};

template <typename T>
struct WilsonClover : OpBase<T> {
  Hop<T> hop;
  bool has_clover = false;
  T diag = 0;                     // 1/(2 kappa)
  // twisted mass: Mooee = diag + i mu g5, g5 = diag(1, 1, -1, -1) in the gpt
  // basis (lib/cgpt/lib/operators/wilson_twisted_mass.h:19-45 -> Grid's
  // WilsonTMFermion, statement of the fingerprint in
  // tests/qcd/fermion_operators.py:366-386)
  double mu = 0.0;
  std::vector<cx<T>> clov, clov_inv;  // [site][2][36]
  using OpBase<T>::G;
  void build(const Geom* g, const double* Uin, double m0, double csw_r, double csw_t, double xi_0, double nu,
             const double* phases) {
    G = g;
    double aniso = nu / xi_0;
    hop.load(G, Uin, phases, aniso);
    double d = m0 + 1.0 + 3.0 * nu / xi_0;
    diag = (T)d;
    double cr = csw_r / xi_0, ct = csw_t;
    has_clover = (cr != 0.0 || ct != 0.0);
    if (!has_clover) return;
    long V = G->V;
    clov.resize((size_t)V * 72);
    clov_inv.resize((size_t)V * 72);
    cd sig[4][4][16];
    for (int mu = 0; mu < 4; ++mu)
      for (int nuu = 0; nuu < 4; ++nuu) {
        cd gm[16], gn[16];
        gamma_dense(mu, gm);
        gamma_dense(nuu, gn);
        for (int i = 0; i < 4; ++i)
          for (int j = 0; j < 4; ++j) {
            cd s = {0, 0};
            for (int k = 0; k < 4; ++k) s = cadd(s, csub(cmul(gm[4 * i + k], gn[4 * k + j]), cmul(gn[4 * i + k], gm[4 * k + j])));
            sig[mu][nuu][4 * i + j] = cscale(0.5, s);
          }
        for (int i = 0; i < 4; ++i)
          for (int j = 0; j < 4; ++j)
            if ((i < 2) != (j < 2) && (sig[mu][nuu][4 * i + j].re != 0 || sig[mu][nuu][4 * i + j].im != 0))
              throw std::runtime_error("sigma_munu is not chirally block diagonal");
      }
    const cd* U = reinterpret_cast<const cd*>(Uin);
    bool ok = true;
#pragma omp parallel for reduction(&& : ok)
    for (long x = 0; x < V; ++x) {
      cd blk[2][36];
      for (int b = 0; b < 2; ++b)
        for (int e = 0; e < 36; ++e) blk[b][e] = {0, 0};
      for (int mu = 0; mu < 4; ++mu)
        for (int nuu = mu + 1; nuu < 4; ++nuu) {
          double cp = (mu == 3 || nuu == 3) ? ct : cr;
          cd F[9];
          field_strength_site(*G, U, V, mu, nuu, x, F);
          for (int b = 0; b < 2; ++b)
            for (int s1 = 0; s1 < 2; ++s1)
              for (int s2 = 0; s2 < 2; ++s2) {
                cd sg = sig[mu][nuu][4 * (2 * b + s1) + (2 * b + s2)];
                if (sg.re == 0 && sg.im == 0) continue;
                cd f = cscale(-0.5 * cp, sg);
                for (int a = 0; a < 3; ++a)
                  for (int c = 0; c < 3; ++c)
                    blk[b][6 * (3 * s1 + a) + (3 * s2 + c)] = cadd(blk[b][6 * (3 * s1 + a) + (3 * s2 + c)], cmul(f, F[3 * a + c]));
              }
        }
      for (int b = 0; b < 2; ++b) {
        for (int i = 0; i < 6; ++i) blk[b][7 * i].re += d;
        cd inv[36];
        if (!invert_cmat(6, blk[b], inv)) ok = false;
        for (int e = 0; e < 36; ++e) {
          clov[(size_t)x * 72 + 36 * b + e] = {(T)blk[b][e].re, (T)blk[b][e].im};
          clov_inv[(size_t)x * 72 + 36 * b + e] = {(T)inv[e].re, (T)inv[e].im};
        }
      }
    }
    if (!ok) throw std::runtime_error("singular clover block");
  }
  void Meooe(cx<T>* out, const cx<T>* in, int out_parity, bool dag) const override { hop.apply(out, in, out_parity, dag, 1); }
  void Dhop(cx<T>* out, const cx<T>* in, int out_parity, bool dag) const override { hop.apply(out, in, out_parity, dag, 1); }
  void Mooee(cx<T>* out, const cx<T>* in, int parity, bool dag, bool inv) const override {
    const long V = G->V;
    const std::vector<int32_t>* list = parity < 2 ? &G->par_sites[parity] : nullptr;
    const long n = list ? (long)list->size() : V;
#pragma omp parallel for schedule(static)
    for (long i = 0; i < n; ++i) {
      const long x = list ? (*list)[i] : i;
      const cx<T>* p = in + (size_t)x * 12;
      cx<T>* o = out + (size_t)x * 12;
      if (!has_clover && mu != 0.0) {
        // (a + i mu g5), its inverse (a - i mu g5) / (a^2 + mu^2), adjoints conjugate
        const double a = (double)diag, den = inv ? a * a + mu * mu : 1.0;
        for (int k = 0; k < 12; ++k) {
          const double g5 = k < 6 ? 1.0 : -1.0;
          double zi = (inv ? -mu : mu) * g5 / den;
          if (dag) zi = -zi;
          const cx<T> z = {(T)(a / den), (T)zi};
          o[k] = cmul(z, p[k]);
        }
        continue;
      }
      if (!has_clover) {
        const T f = inv ? (T)(1.0 / (double)diag) : diag;  // 2 kappa for the inverse
        for (int k = 0; k < 12; ++k) o[k] = cscale(f, p[k]);
        continue;
      }
      const cx<T>* C = &(inv ? clov_inv : clov)[(size_t)x * 72];
      cx<T> r[12];
      for (int b = 0; b < 2; ++b)
        for (int i2 = 0; i2 < 6; ++i2) {
          cx<T> s = {0, 0};
          for (int j = 0; j < 6; ++j) {
            cx<T> m = dag ? cx<T>{C[36 * b + 6 * j + i2].re, -C[36 * b + 6 * j + i2].im} : C[36 * b + 6 * i2 + j];
            s = cadd(s, cmul(m, p[6 * b + j]));
          }
          r[6 * b + i2] = s;
        }
      for (int k = 0; k < 12; ++k) o[k] = r[k];
    }
  }
};

// Mobius domain-wall operator.  With D_W the 4D Wilson operator at mass -M5
// (diagonal 4 - M5) and P+- = (1 +- g5)/2, tests/qcd/domain_wall.py:309-340
// states  M psi_s = (b D_W + 1) psi_s + (c D_W - 1)(P+ psi_{s-1} + P- psi_{s+1})
// with the wall terms -m+ (c D_W - 1) P+ psi_{Ls-1} at s = 0 and
// -m- (c D_W - 1) P- psi_0 at s = Ls-1.  Writing K for the s-hop with those
// wall terms,  M = Dhop (b + cK) + [(4-M5)(b + cK) + 1 - K],  so
//   Meooe = Dhop (b + cK),   Mooee = (4-M5)(b + cK) + 1 - K.
// Mooee acts on chiralities separately as an Ls x Ls matrix A+/A-.
template <typename T>
struct Mobius : OpBase<T> {
  Hop<T> hop;
  int Ls;
  double b, c, M5, mp, mm;
  // per-slice Cayley coefficients (zmobius: complex, from omega; mobius: b, c)
  // and the dense per-chirality matrices B = diag(bs) + diag(cs) K (cs scales
  // the output slice; col_scale: K diag(cs), the input slice)
  std::vector<cd> bs, cs;
  bool col_scale = false;
  std::vector<cd> Ainv[2], A[2], B[2];  // [chirality][Ls*Ls], chirality 0 = P+ (spins 0,1)
  using OpBase<T>::G;
  using OpBase<T>::n5;
  void build(const Geom* g, const double* Uin, int Ls_, double b_, double c_, double M5_, double mp_, double mm_,
             const double* phases) {
    std::vector<cd> vb(Ls_, cd{b_, 0}), vc(Ls_, cd{c_, 0});
    build_z(g, Uin, Ls_, vb, vc, M5_, mp_, mm_, phases, false);
    b = b_;
    c = c_;
  }
  void build_z(const Geom* g, const double* Uin, int Ls_, const std::vector<cd>& bs_, const std::vector<cd>& cs_,
               double M5_, double mp_, double mm_, const double* phases, bool col) {
    G = g;
    Ls = Ls_; n5 = Ls; M5 = M5_; mp = mp_; mm = mm_;
    bs = bs_; cs = cs_; col_scale = col;
    b = bs[0].re; c = cs[0].re;
    hop.load(G, Uin, phases, 1.0);
    for (int ch = 0; ch < 2; ++ch) {
      std::vector<double> K(Ls * Ls, 0.0);
      for (int s = 0; s < Ls; ++s) {
        if (ch == 0) {  // P+: couples s to s-1, wall term at s=0 from Ls-1
          if (s >= 1) K[s * Ls + s - 1] = 1.0;
          else K[Ls - 1] = -mp;
        } else {  // P-: couples s to s+1, wall term at s=Ls-1 from 0
          if (s <= Ls - 2) K[s * Ls + s + 1] = 1.0;
          else K[(Ls - 1) * Ls] = -mm;
        }
      }
      B[ch].assign(Ls * Ls, cd{0, 0});
      A[ch].assign(Ls * Ls, cd{0, 0});
      for (int s = 0; s < Ls; ++s)
        for (int t = 0; t < Ls; ++t) {
          const double k = K[s * Ls + t];
          cd v = (s == t) ? bs[s] : cd{0, 0};
          if (k != 0.0) v = cadd(v, cscale(k, col_scale ? cs[t] : cs[s]));
          B[ch][s * Ls + t] = v;
          cd a = cscale(4.0 - M5, v);
          if (s == t) a.re += 1.0;
          a.re -= k;
          A[ch][s * Ls + t] = a;
        }
      Ainv[ch].resize(Ls * Ls);
      if (!invert_cmat(Ls, A[ch].data(), Ainv[ch].data())) throw std::runtime_error("singular Mooee");
    }
  }
  // B psi or B^+ psi, per 4D site of the given parity
  void mix(cx<T>* out, const cx<T>* in, int parity, bool dag) const {
    const std::vector<int32_t>* list = parity < 2 ? &G->par_sites[parity] : nullptr;
    const long n = list ? (long)list->size() : G->V;
#pragma omp parallel for schedule(static)
    for (long i = 0; i < n; ++i) {
      const long x = list ? (*list)[i] : i;
      const cx<T>* p = in + (size_t)x * Ls * 12;
      cx<T>* o = out + (size_t)x * Ls * 12;
      std::vector<cx<T>> r((size_t)Ls * 12);
      for (int ch = 0; ch < 2; ++ch)
        for (int s = 0; s < Ls; ++s)
          for (int k = 6 * ch; k < 6 * ch + 6; ++k) {
            cx<T> acc = {0, 0};
            for (int t = 0; t < Ls; ++t) {
              const cd m = dag ? cd{B[ch][t * Ls + s].re, -B[ch][t * Ls + s].im} : B[ch][s * Ls + t];
              if (m.re == 0.0 && m.im == 0.0) continue;
              acc = cadd(acc, cmul(cx<T>{(T)m.re, (T)m.im}, p[t * 12 + k]));
            }
            r[s * 12 + k] = acc;
          }
      for (size_t k = 0; k < r.size(); ++k) o[k] = r[k];
    }
  }
  void Dhop(cx<T>* out, const cx<T>* in, int out_parity, bool dag) const override { hop.apply(out, in, out_parity, dag, Ls); }
  void Meooe(cx<T>* out, const cx<T>* in, int out_parity, bool dag) const override {
    // out = Dhop B in  (dag: B^+ Dhop^+ in); B acts on the source parity
    size_t len = (size_t)G->V * Ls * 12;
    std::vector<cx<T>> tmp(len);
    if (!dag) {
      int src_par = out_parity < 2 ? 1 - out_parity : 2;
      mix(tmp.data(), in, src_par, false);
      hop.apply(out, tmp.data(), out_parity, false, Ls);
    } else {
      hop.apply(tmp.data(), in, out_parity, true, Ls);
      mix(out, tmp.data(), out_parity, true);
    }
  }
  void Mooee(cx<T>* out, const cx<T>* in, int parity, bool dag, bool inv) const override {
    const std::vector<int32_t>* list = parity < 2 ? &G->par_sites[parity] : nullptr;
    const long n = list ? (long)list->size() : G->V;
#pragma omp parallel for schedule(static)
    for (long i = 0; i < n; ++i) {
      const long x = list ? (*list)[i] : i;
      const cx<T>* p = in + (size_t)x * Ls * 12;
      cx<T>* o = out + (size_t)x * Ls * 12;
      std::vector<cx<T>> r((size_t)Ls * 12);
      for (int ch = 0; ch < 2; ++ch) {
        const std::vector<cd>& Mx = inv ? Ainv[ch] : A[ch];
        for (int s = 0; s < Ls; ++s)
          for (int k = 6 * ch; k < 6 * ch + 6; ++k) {
            cx<T> acc = {0, 0};
            for (int sp = 0; sp < Ls; ++sp) {
              cd m = dag ? cd{Mx[sp * Ls + s].re, -Mx[sp * Ls + s].im} : Mx[s * Ls + sp];
              acc = cadd(acc, cmul(cx<T>{(T)m.re, (T)m.im}, p[sp * 12 + k]));
            }
            r[s * 12 + k] = acc;
          }
      }
      for (size_t k = 0; k < r.size(); ++k) o[k] = r[k];
    }
  }
};

// ---------------------------------------------------------------------------
// BLAS over the sites of one parity (or all sites), double accumulation
// (lib/cgpt/lib/foundation/reduce.h accumulates in ComplexD for both precisions)
// ---------------------------------------------------------------------------
template <typename T>
struct Blas {
  const Geom* G;
  size_t slen;
  int parity;
  long count() const { return parity < 2 ? (long)G->par_sites[parity].size() : G->V; }
  long site(long i) const { return parity < 2 ? G->par_sites[parity][i] : i; }
  double norm2(const cx<T>* a) const {
    double s = 0;
    long n = count();
#pragma omp parallel for reduction(+ : s) schedule(static)
    for (long i = 0; i < n; ++i) {
      const cx<T>* p = a + site(i) * slen;
      for (size_t k = 0; k < slen; ++k) s += (double)p[k].re * p[k].re + (double)p[k].im * p[k].im;
    }
    return s;
  }
  cd inner(const cx<T>* a, const cx<T>* b) const {
    double sr = 0, si = 0;
    long n = count();
#pragma omp parallel for reduction(+ : sr, si) schedule(static)
    for (long i = 0; i < n; ++i) {
      const cx<T>* p = a + site(i) * slen;
      const cx<T>* q = b + site(i) * slen;
      for (size_t k = 0; k < slen; ++k) {
        sr += (double)p[k].re * q[k].re + (double)p[k].im * q[k].im;
        si += (double)p[k].re * q[k].im - (double)p[k].im * q[k].re;
      }
    }
    return {sr, si};
  }
  // out = a*x + y
  void axpy(cx<T>* out, T a, const cx<T>* x, const cx<T>* y) const {
    long n = count();
#pragma omp parallel for schedule(static)
    for (long i = 0; i < n; ++i) {
      size_t o = site(i) * slen;
      for (size_t k = 0; k < slen; ++k) out[o + k] = {a * x[o + k].re + y[o + k].re, a * x[o + k].im + y[o + k].im};
    }
  }
  void zero(cx<T>* out) const {
    long n = count();
#pragma omp parallel for schedule(static)
    for (long i = 0; i < n; ++i) std::memset(out + site(i) * slen, 0, sizeof(cx<T>) * slen);
  }
  void copy(cx<T>* out, const cx<T>* in) const {
    long n = count();
#pragma omp parallel for schedule(static)
    for (long i = 0; i < n; ++i) std::memcpy(out + site(i) * slen, in + site(i) * slen, sizeof(cx<T>) * slen);
  }
};

// eo2_ne: D = odd (default parity), C = even.
//   Mpc   x = x - DC CC^-1 CD DD^-1 x         (schur_complement_two.py:87-95)
//   Mpc^+ x = x - DD^-1+ CD^+ CC^-1+ DC^+ x    (schur_complement_two.py:101-109)
template <typename T>
struct Eo2Ne {
  const OpBase<T>* op;
  int D, C;
  mutable std::vector<cx<T>> td, tc0, tc1;
  Blas<T> bd;
  Eo2Ne(const OpBase<T>* o, int parityD) : op(o), D(parityD), C(1 - parityD) {
    size_t len = (size_t)op->G->V * op->site_len();
    td.assign(len, {0, 0}); tc0.assign(len, {0, 0}); tc1.assign(len, {0, 0});
    bd = Blas<T>{op->G, op->site_len(), D};
  }
  void Mpc(cx<T>* o, const cx<T>* i) const {
    op->Mooee(td.data(), i, D, false, true);
    op->Meooe(tc0.data(), td.data(), C, false);
    op->Mooee(tc1.data(), tc0.data(), C, false, true);
    op->Meooe(o, tc1.data(), D, false);
    bd.axpy(o, (T)-1, o, i);
  }
  void MpcDag(cx<T>* o, const cx<T>* i) const {
    op->Meooe(tc0.data(), i, C, true);
    op->Mooee(tc1.data(), tc0.data(), C, true, true);
    op->Meooe(td.data(), tc1.data(), D, true);
    op->Mooee(o, td.data(), D, true, true);
    bd.axpy(o, (T)-1, o, i);
  }
};

// CG on Mpc^+ Mpc, cg.py:47-105 (no preconditioner branch).
template <typename T>
static int cg_solve(const Eo2Ne<T>& N, cx<T>* psi, const cx<T>* src, double eps, int maxiter, double* res_out) {
  const Blas<T>& B = N.bd;
  size_t len = (size_t)N.op->G->V * N.op->site_len();
  std::vector<cx<T>> p(len, {0, 0}), mmp(len, {0, 0}), r(len, {0, 0}), w(len, {0, 0});
  N.Mpc(w.data(), psi);
  N.MpcDag(mmp.data(), w.data());
  B.axpy(r.data(), (T)-1, mmp.data(), src);
  B.copy(p.data(), r.data());
  double cp = B.norm2(p.data());
  double ssq = B.norm2(src);
  if (ssq == 0.0) {
    B.zero(psi);
    *res_out = 0;
    return 0;
  }
  double rsq = eps * eps * ssq;
  int k;
  for (k = 0; k < maxiter; ++k) {
    double c = cp;
    N.Mpc(w.data(), p.data());
    N.MpcDag(mmp.data(), w.data());
    double d = B.inner(p.data(), mmp.data()).re;
    double a = c / d;
    B.axpy(r.data(), (T)(-a), mmp.data(), r.data());
    cp = B.norm2(r.data());
    double bb = cp / c;
    B.axpy(psi, (T)a, p.data(), psi);
    B.axpy(p.data(), (T)bb, p.data(), r.data());
    if (cp <= rsq) {
      *res_out = cp;
      return k + 1;
    }
  }
  *res_out = cp;
  return -k;
}

// preconditioned(eo2_ne, cg): preconditioned.py:36-44 with
//   R_ne src = Mpc^+ (src_D - DC CC^-1 src_C)   (normal_equation.py:47-48, schur_complement_two.py:131-132)
//   x_D = DD^-1 y,  x_C = CC^-1 (src_C - CD x_D)  (schur_complement_two.py:114-119, 143-148)
template <typename T>
static int eo2ne_solve(const OpBase<T>* op, cx<T>* x, const cx<T>* src, double eps, int maxiter, double* res) {
  const int D = 1, C = 0;
  Eo2Ne<T> N(op, D);
  size_t len = (size_t)op->G->V * op->site_len();
  std::vector<cx<T>> t1(len, {0, 0}), t2(len, {0, 0}), pc_src(len, {0, 0}), y(len, {0, 0});
  Blas<T> bc{op->G, op->site_len(), C};
  op->Mooee(t1.data(), src, C, false, true);
  op->Meooe(t2.data(), t1.data(), D, false);
  N.bd.axpy(t2.data(), (T)-1, t2.data(), src);
  N.MpcDag(pc_src.data(), t2.data());
  int it = cg_solve(N, y.data(), pc_src.data(), eps, maxiter, res);
  op->Mooee(x, y.data(), D, false, true);
  op->Meooe(t1.data(), x, C, false);
  bc.axpy(t1.data(), (T)-1, t1.data(), src);
  op->Mooee(x, t1.data(), C, false, true);
  return it;
}

// Full-lattice application of the operator family.
template <typename T>
static void apply_full(const OpBase<T>* op, int opcode, cx<T>* out, const cx<T>* in, int parity) {
  size_t len = (size_t)op->G->V * op->site_len();
  switch (opcode) {
    case OP_M:
    case OP_MDAG: {
      bool dag = opcode == OP_MDAG;
      std::vector<cx<T>> t(len);
      for (int p = 0; p < 2; ++p) {
        op->Meooe(out, in, p, dag);
        op->Mooee(t.data(), in, p, dag, false);
        Blas<T> b{op->G, op->site_len(), p};
        b.axpy(out, (T)1, t.data(), out);
      }
      break;
    }
    case OP_MEOOE: op->Meooe(out, in, parity, false); break;
    case OP_MEOOE_DAG: op->Meooe(out, in, parity, true); break;
    case OP_MOOEE: op->Mooee(out, in, parity, false, false); break;
    case OP_MOOEE_DAG: op->Mooee(out, in, parity, true, false); break;
    case OP_MOOEE_INV: op->Mooee(out, in, parity, false, true); break;
    case OP_MOOEE_INV_DAG: op->Mooee(out, in, parity, true, true); break;
    case OP_MDIAG: op->Mooee(out, in, 2, false, false); break;
    case OP_DHOP: op->Dhop(out, in, 2, false); break;
    case OP_DHOP_DAG: op->Dhop(out, in, 2, true); break;
    default: throw std::runtime_error("opcode not supported by this operator");
  }
}

// ---------------------------------------------------------------------------
// C interface
// ---------------------------------------------------------------------------
struct OracleOp {
  std::unique_ptr<Geom> G;
  std::unique_ptr<OpBase<double>> d;
  std::unique_ptr<OpBase<float>> f;
  bool mobius = false;
  Mobius<double>* mob() const { return static_cast<Mobius<double>*>(d.get()); }
};

extern "C" {

// phases: 4 complex numbers (re, im interleaved)
void* orc_wilson_clover_new(const double* U, const long* dims, double m0, double csw_r, double csw_t, double xi_0, double nu,
                            const double* phases, int with_single) {
  try {
    auto o = new OracleOp;
    o->G = std::make_unique<Geom>(dims);
    auto w = std::make_unique<WilsonClover<double>>();
    w->build(o->G.get(), U, m0, csw_r, csw_t, xi_0, nu, phases);
    o->d = std::move(w);
    if (with_single) {
      auto ws = std::make_unique<WilsonClover<float>>();
      ws->build(o->G.get(), U, m0, csw_r, csw_t, xi_0, nu, phases);
      o->f = std::move(ws);
    }
    return o;
  } catch (const std::exception& e) {
    g_err = e.what();
    return nullptr;
  }
}

// twisted-mass Wilson operator (isotropic, no clover)
void* orc_wilson_twisted_mass_new(const double* U, const long* dims, double m0, double mu, const double* phases,
                                  int with_single) {
  try {
    auto o = new OracleOp;
    o->G = std::make_unique<Geom>(dims);
    auto w = std::make_unique<WilsonClover<double>>();
    w->build(o->G.get(), U, m0, 0.0, 0.0, 1.0, 1.0, phases);
    w->mu = mu;
    o->d = std::move(w);
    if (with_single) {
      auto ws = std::make_unique<WilsonClover<float>>();
      ws->build(o->G.get(), U, m0, 0.0, 0.0, 1.0, 1.0, phases);
      ws->mu = mu;
      o->f = std::move(ws);
    }
    return o;
  } catch (const std::exception& e) {
    g_err = e.what();
    return nullptr;
  }
}

void* orc_mobius_new(const double* U, const long* dims, int Ls, double b, double c, double M5, double mass_plus,
                     double mass_minus, const double* phases, int with_single) {
  try {
    auto o = new OracleOp;
    o->mobius = true;
    o->G = std::make_unique<Geom>(dims);
    auto m = std::make_unique<Mobius<double>>();
    m->build(o->G.get(), U, Ls, b, c, M5, mass_plus, mass_minus, phases);
    o->d = std::move(m);
    if (with_single) {
      auto ms = std::make_unique<Mobius<float>>();
      ms->build(o->G.get(), U, Ls, b, c, M5, mass_plus, mass_minus, phases);
      o->f = std::move(ms);
    }
    return o;
  } catch (const std::exception& e) {
    g_err = e.what();
    return nullptr;
  }
}

void orc_op_free(void* o) { delete (OracleOp*)o; }

int orc_op_apply(void* o, int opcode, const double* in, double* out, int parity) {
  return guarded([&] {
    OracleOp& op = *(OracleOp*)o;
    auto* i = reinterpret_cast<const cd*>(in);
    auto* out_ = reinterpret_cast<cd*>(out);
    if (op.mobius) {
      Mobius<double>& m = *op.mob();
      const Geom& G = *op.G;
      int Ls = m.Ls;
      size_t len = (size_t)G.V * Ls * 12;
      if (opcode == OP_DMINUS || opcode == OP_DMINUS_DAG) {
        // Dminus psi_s = psi_s - c_s D_W psi_s, D_W = (4 - M5) + Dhop (slice-wise);
        // the adjoint takes conj(c_s)
        std::vector<cd> t(len);
        m.hop.apply(t.data(), i, 2, opcode == OP_DMINUS_DAG, Ls);
#pragma omp parallel for
        for (long k = 0; k < (long)len; ++k) {
          const int sl = (int)((k / 12) % Ls);
          cd cc = m.cs[sl];
          if (opcode == OP_DMINUS_DAG) cc.im = -cc.im;
          cd dw = cadd(t[k], cscale(4.0 - m.M5, i[k]));
          out_[k] = csub(i[k], cmul(cc, dw));
        }
        return;
      }
      if (opcode == OP_EXPORT_PHYS_SOL || opcode == OP_EXPORT_PHYS_SRC) {
        // solution: q = P- psi_0 + P+ psi_{Ls-1} (lib/gpt/qcd/fermion/mobius.py:162);
        // source (opcode 2015, lib/gpt/qcd/fermion/operator/base.py:159-164):
        // q = P+ psi_0 + P- psi_{Ls-1}, the adjoint of the wall placement of
        // the import (lib/gpt/qcd/fermion/preconditioner/physical.py:36-39
        // composes it with Dminus^+ as the adjoint of the physical import)
        const bool sol = opcode == OP_EXPORT_PHYS_SOL;
#pragma omp parallel for
        for (long x = 0; x < G.V; ++x)
          for (int k = 0; k < 12; ++k) {
            const bool from_last = (k < 6) == sol;
            out_[x * 12 + k] = i[((size_t)x * Ls + (from_last ? Ls - 1 : 0)) * 12 + k];
          }
        return;
      }
      if (opcode == OP_IMPORT_PHYS_SRC || opcode == OP_IMPORT_UNPHYS) throw std::runtime_error("use orc_mobius_import");
    } else if (opcode >= OP_IMPORT_PHYS_SRC && opcode <= OP_EXPORT_PHYS_SRC) {
      // Wilson: every import and export is a copy (lib/gpt/qcd/fermion/reference/wilson_clover.py:165-173)
      std::memcpy(out_, i, (size_t)op.G->V * 12 * sizeof(cd));
      return;
    }
    apply_full(op.d.get(), opcode, out_, i, parity);
  });
}

// zmobius: per-slice complex b_s, c_s (2 Ls doubles each, re/im pairs);
// col_scale selects K diag(c) instead of diag(c) K
void* orc_zmobius_new(const double* U, const long* dims, int Ls, const double* bs, const double* cs, double M5,
                      double mass_plus, double mass_minus, const double* phases, int with_single, int col_scale) {
  try {
    auto o = new OracleOp;
    o->mobius = true;
    o->G = std::make_unique<Geom>(dims);
    std::vector<cd> vb(Ls), vc(Ls);
    for (int s = 0; s < Ls; ++s) {
      vb[s] = {bs[2 * s], bs[2 * s + 1]};
      vc[s] = {cs[2 * s], cs[2 * s + 1]};
    }
    auto m = std::make_unique<Mobius<double>>();
    m->build_z(o->G.get(), U, Ls, vb, vc, M5, mass_plus, mass_minus, phases, col_scale != 0);
    o->d = std::move(m);
    if (with_single) {
      auto ms = std::make_unique<Mobius<float>>();
      ms->build_z(o->G.get(), U, Ls, vb, vc, M5, mass_plus, mass_minus, phases, col_scale != 0);
      o->f = std::move(ms);
    }
    return o;
  } catch (const std::exception& e) {
    g_err = e.what();
    return nullptr;
  }
}

// Mobius source import: the 4D source is placed on the walls with the chiral
// projections selected by `variant` (bit 0: P+ on s=0 and P- on s=Ls-1 when
// set, the opposite when clear) and then multiplied by Dminus when bit 1 is set.
int orc_mobius_import(void* o, const double* in4, double* out5, int variant) {
  return guarded([&] {
    OracleOp& op = *(OracleOp*)o;
    if (!op.mobius) throw std::runtime_error("not a mobius operator");
    Mobius<double>& m = *op.mob();
    const Geom& G = *op.G;
    int Ls = m.Ls;
    size_t len = (size_t)G.V * Ls * 12;
    std::vector<cd> tmp(len, cd{0, 0});
    auto* i = reinterpret_cast<const cd*>(in4);
    bool plus_first = variant & 1;
    for (long x = 0; x < G.V; ++x)
      for (int k = 0; k < 12; ++k) {
        bool upper = k < 6;
        if (upper == plus_first) tmp[((size_t)x * Ls) * 12 + k] = i[x * 12 + k];
        else tmp[((size_t)x * Ls + Ls - 1) * 12 + k] = i[x * 12 + k];
      }
    if (variant & 2) {
      if (orc_op_apply(o, OP_DMINUS, reinterpret_cast<double*>(tmp.data()), out5, 2)) throw std::runtime_error(g_err);
    } else {
      std::memcpy(out5, tmp.data(), len * sizeof(cd));
    }
  });
}

// Plain eo2_ne CG in double precision.  Returns iterations (negative if not converged).
int orc_eo2ne_cg(void* o, const double* src, double* x, double eps, int maxiter, double* res) {
  try {
    OracleOp& op = *(OracleOp*)o;
    return eo2ne_solve<double>(op.d.get(), reinterpret_cast<cd*>(x), reinterpret_cast<const cd*>(src), eps, maxiter, res);
  } catch (const std::exception& e) {
    g_err = e.what();
    return -1000000000;
  }
}

// eo2_ne CG of the single-precision operator (inner solve of the mixed method).
int orc_eo2ne_cg_single(void* o, const double* src, double* x, double eps, int maxiter, double* res) {
  try {
    OracleOp& op = *(OracleOp*)o;
    if (!op.f) throw std::runtime_error("single-precision operator not built");
    size_t len = (size_t)op.G->V * op.d->site_len();
    std::vector<cx<float>> sf(len), xf(len, cx<float>{0, 0});
    for (size_t k = 0; k < len; ++k) sf[k] = {(float)src[2 * k], (float)src[2 * k + 1]};
    int it = eo2ne_solve<float>(op.f.get(), xf.data(), sf.data(), eps, maxiter, res);
    for (size_t k = 0; k < len; ++k) { x[2 * k] = xf[k].re; x[2 * k + 1] = xf[k].im; }
    return it;
  } catch (const std::exception& e) {
    g_err = e.what();
    return -1000000000;
  }
}

// Defect correction (defect_correcting.py:85-130) around a single-precision
// eo2_ne CG (mixed_precision.py:23-32): outer residual s = src - M x in double,
// inner solve of M d = s/|s_ref| in single precision, x += d*|src|.
// Returns the total number of inner CG iterations; outer count in *n_outer.
int orc_defect_correcting(void* o, const double* src, double* x, double eps_outer, int maxouter, double eps_inner, int maxinner,
                          double* true_res, int* n_outer) {
  try {
    OracleOp& op = *(OracleOp*)o;
    if (!op.f) throw std::runtime_error("single-precision operator not built");
    const Geom& G = *op.G;
    size_t len = (size_t)G.V * op.d->site_len();
    std::vector<cd> s(len), t(len);
    std::vector<cx<float>> sf(len), df(len);
    Blas<double> all{&G, op.d->site_len(), 2};
    auto* srcc = reinterpret_cast<const cd*>(src);
    auto* xc = reinterpret_cast<cd*>(x);
    double nsrc = std::sqrt(all.norm2(srcc));
    int total = 0, i;
    for (i = 0; i < maxouter; ++i) {
      apply_full<double>(op.d.get(), OP_M, t.data(), xc, 2);
      all.axpy(s.data(), -1.0, t.data(), srcc);
      double r = std::sqrt(all.norm2(s.data())) / nsrc;
      *true_res = r;
      if (r < eps_outer) break;
      double inv = 1.0 / nsrc;
#pragma omp parallel for
      for (long k = 0; k < (long)len; ++k) { sf[k] = {(float)(s[k].re * inv), (float)(s[k].im * inv)}; df[k] = {0, 0}; }
      double res;
      int it = eo2ne_solve<float>(op.f.get(), df.data(), sf.data(), eps_inner, maxinner, &res);
      total += it < 0 ? -it : it;
#pragma omp parallel for
      for (long k = 0; k < (long)len; ++k) { xc[k].re += (double)df[k].re * nsrc; xc[k].im += (double)df[k].im * nsrc; }
    }
    *n_outer = i;
    return total;
  } catch (const std::exception& e) {
    g_err = e.what();
    return -1;
  }
}

int orc_num_threads() { return omp_get_max_threads(); }
}
