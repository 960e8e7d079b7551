// gbf_noalloc.cu -- |x|^2 of a field with no device allocation at all.
//
// gbf_norm2 keeps its reduction scratch (per-block partial sums, a block
// counter and the result word) in workspace that the operator allocates with
// cudaMalloc on first use.  Some callers cannot allow that: a serving process
// that has handed all free HBM to its own memory pool, or a latency-critical
// loop that must not take the device-wide synchronisation of cudaMalloc /
// cudaFree.  gbf_norm2_noalloc computes the same sum with the scratch in a
// file-scope __device__ array instead.
//
// Limits and rules (also stated in include/gbferm.h):
//   * at most kNoAllocMaxSites 5D sites per checkerboard half (16384 blocks
//     of 256 sites); larger fields are rejected with GBF_E_ARG;
//   * the array (about 263 KB) is held on every GPU where the library's
//     module is loaded, for the life of the process.  CUDA loads modules
//     lazily (the default since CUDA 12.2), so the module holding this array
//     and its kernels is loaded, and the array's memory taken, on the first
//     call on a device, when cudaGetSymbolAddress looks up the array's
//     device address (once per device, with that device current);
//   * so make that first call early: before any stream capture, and before
//     a memory pool of the caller takes the device's free HBM (otherwise the
//     module load itself can fail with out-of-memory).  A call with
//     n_sites = 0 does only this set-up and launches nothing;
//   * every call shares the one array: calls whose kernels overlap on the GPU
//     (different streams, or concurrent host threads) race and give wrong sums.
//     The block counter is cleared at the start of each call.
#include <mutex>
#include <string>

#include "gbf_launch.cuh"
#include "../../include/gbferm.h"

namespace {

constexpr int kNoAllocBlock = 256;
constexpr int kNoAllocMaxBlocks = 16384;
constexpr long long kNoAllocMaxSites = (long long)kNoAllocMaxBlocks * kNoAllocBlock;

struct NoAllocScratch {
  gbf::CGState st;   // st.last[0] receives the sum
  unsigned counter;  // blocks finished; must be zero when a launch starts
  unsigned pad[63];
  double2 partial[kNoAllocMaxBlocks];
};

}  // namespace

static __device__ __align__(256) NoAllocScratch g_noalloc_scratch;

namespace {

template <int P>
__global__ void __launch_bounds__(kNoAllocBlock) norm2_noalloc_kernel(const void* x, long long N, NoAllocScratch* s) {
  using R = typename gbf::SpinorT<P>::R;
  __shared__ double sm[2 * kNoAllocBlock];
  const long long n = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double v = 0.0;
  if (n < N) {
    gbf::cplx<R> a[12];
    gbf::load_spinor<P>(x, N, n, a);
    v = gbf::site_norm2<R>(a);
  }
  gbf::RedArgs ra;
  ra.fin = gbf::FIN_STORE;
  ra.partial = s->partial;
  ra.counter = &s->counter;
  ra.st = &s->st;
  gbf::block_reduce_finalize(ra, v, 0.0, 1, 1, 1, sm);
}

std::mutex g_setup_mutex;
void* g_scratch_addr[64] = {};  // device address of g_noalloc_scratch per device
thread_local std::string g_noalloc_err;

}  // namespace

extern "C" int gbf_norm2_noalloc(int precision, const void* x, long long n_sites, int nhalves, double* out, void* stream) {
  if (!x || !out || n_sites < 0 || (nhalves != 1 && nhalves != 2) || precision < GBF_DOUBLE || precision > GBF_DOUBLE_FLOAT) {
    g_noalloc_err = "gbf_norm2_noalloc: bad argument";
    return GBF_E_ARG;
  }
  if (n_sites > kNoAllocMaxSites) {
    g_noalloc_err = "gbf_norm2_noalloc: " + std::to_string(n_sites) + " sites per half exceed the maximum of " +
                    std::to_string(kNoAllocMaxSites) + " (static scratch of " + std::to_string(kNoAllocMaxBlocks) +
                    " blocks); use gbf_norm2";
    return GBF_E_ARG;
  }
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= 64) {
    g_noalloc_err = std::string("gbf_norm2_noalloc: cudaGetDevice: ") + cudaGetErrorString(e);
    return GBF_E_CUDA;
  }
  void* addr = nullptr;
  {
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_addr[dev]) {
      e = cudaGetSymbolAddress(&g_scratch_addr[dev], g_noalloc_scratch);
      if (e != cudaSuccess) {
        g_scratch_addr[dev] = nullptr;
        g_noalloc_err = std::string("gbf_norm2_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e);
        return GBF_E_CUDA;
      }
    }
    addr = g_scratch_addr[dev];
  }
  NoAllocScratch* s = reinterpret_cast<NoAllocScratch*>(addr);
  cudaStream_t st = (cudaStream_t)stream;
  const int P = precision == GBF_DOUBLE ? gbf::P64
              : precision == GBF_SINGLE ? gbf::P32
              : precision == GBF_HALF ? gbf::P16 : gbf::PDD;
  const long long half = gbf::half_bytes(P, n_sites);
  double total = 0.0;
  for (int h = 0; h < nhalves; ++h) {
    double part = 0.0;
    if (n_sites > 0) {
      e = cudaMemsetAsync(&s->counter, 0, sizeof(unsigned), st);
      if (e == cudaSuccess) {
        const unsigned nb = (unsigned)((n_sites + kNoAllocBlock - 1) / kNoAllocBlock);
        const void* xh = (const char*)x + h * half;
        if (P == gbf::P64) norm2_noalloc_kernel<gbf::P64><<<nb, kNoAllocBlock, 0, st>>>(xh, n_sites, s);
        else if (P == gbf::P32) norm2_noalloc_kernel<gbf::P32><<<nb, kNoAllocBlock, 0, st>>>(xh, n_sites, s);
        else if (P == gbf::PDD) norm2_noalloc_kernel<gbf::PDD><<<nb, kNoAllocBlock, 0, st>>>(xh, n_sites, s);
        else norm2_noalloc_kernel<gbf::P16><<<nb, kNoAllocBlock, 0, st>>>(xh, n_sites, s);
        e = cudaGetLastError();
      }
      if (e == cudaSuccess) e = cudaMemcpyAsync(&part, &s->st.last[0], sizeof(double), cudaMemcpyDeviceToHost, st);
      if (e == cudaSuccess) e = cudaStreamSynchronize(st);
      if (e != cudaSuccess) {
        g_noalloc_err = std::string("gbf_norm2_noalloc: ") + cudaGetErrorString(e);
        return GBF_E_CUDA;
      }
    }
    total += part;
  }
  *out = total;
  return GBF_OK;
}

extern "C" const char* gbf_norm2_noalloc_error(void) { return g_noalloc_err.c_str(); }
