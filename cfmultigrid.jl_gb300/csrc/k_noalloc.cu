// cfmg_norm_noalloc: the masked sum of squares of a caller-owned device
// field, computed without allocating any memory.
//
// Some callers of this library cannot allocate GPU memory at the point
// where they need a norm: a host application whose device memory pool is
// owned by another allocator (a Julia CuArray pool or a PyTorch caching
// allocator that must not see foreign cudaMalloc calls), code running
// where a cudaMalloc would synchronise the device at a bad time, or
// deployments with a fixed device-memory budget. They already hold the
// field and the mask on the device and want the reduction only.
//
// The reduction's scratch (its per-chunk partial sums and nothing else) is
// a file-scope static __device__ array of kStaticChunks doubles (32 KB). Every
// GPU that loads the library holds it until the process exits. Its size
// bounds the input: at most kStaticChunks * kChunk = 268,435,456 elements;
// larger sizes are rejected with CFMG_ERR_ARG. The caller passes the inputs
// and a device (or mapped host) address that receives the result.
//
// In host code the symbol g_noalloc_partials is only a host-side stand-in,
// not a device address. The device address is obtained once per device, with
// that device current, by cudaGetSymbolAddress (on the entry point's first
// call on that device; make that first call before any stream capture).
// The cached address belongs to the CUDA context it was taken in: a device
// reset (cudaDeviceReset, CUDA.device_reset! in Julia) destroys that context,
// and the module, with its static array, is loaded again into the next one,
// possibly at another address. Each call therefore compares the current
// context's unique id (cuCtxGetId) with the one the address was taken under
// and repeats the set-up when they differ; the first call after a reset is
// then a set-up call too, and belongs before any stream capture as well.
//
// Every call shares the one array. Each chunk's partial is written before
// it is read and only the chunks of the current call are read, so nothing
// has to be cleared between calls. Calls whose kernels overlap on the GPU
// (the same device, different streams, not ordered) race on the array.
#include <mutex>

#include "cfmg_internal.h"

namespace cfmg {
namespace {

constexpr int kStaticChunks = 4096;
constexpr long long kChunk = 1LL << 16;
constexpr long long kMaxElems = kStaticChunks * kChunk;
constexpr int kMaxDevices = 64;
constexpr int kThreadsNA = 256;

static __device__ __align__(256) double g_noalloc_partials[kStaticChunks];

std::mutex g_mu;
double* g_addr[kMaxDevices] = {nullptr};
unsigned long long g_ctx_id[kMaxDevices] = {0};

// Driver entry points reached through the runtime, so that the library does
// not link libcuda itself (it must load on machines without a driver).
typedef int (*PFN_ctxGetCurrent)(void**);
typedef int (*PFN_ctxGetId)(void*, unsigned long long*);
PFN_ctxGetCurrent g_ctx_get_current = nullptr;
PFN_ctxGetId g_ctx_get_id = nullptr;

// Block c sums msk*x^2 over elements [c*kChunk, min(n, (c+1)*kChunk)).
__global__ void __launch_bounds__(kThreadsNA) k_chunk_partials(const double* __restrict__ x,
                                                               const uint8_t* __restrict__ m, long long n,
                                                               double* __restrict__ partials) {
  const long long lo = (long long)blockIdx.x * kChunk;
  const long long hi = lo + kChunk < n ? lo + kChunk : n;
  double s = 0.0;
  for (long long I = lo + threadIdx.x; I < hi; I += kThreadsNA) {
    const uint8_t mm = m[I];
    if (mm) {
      const double v = x[I];
      s = (mm == 1) ? __fma_rn(v, v, s) : __dadd_rn(s, __dmul_rn((double)mm, __dmul_rn(v, v)));
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s = __dadd_rn(s, __shfl_down_sync(0xffffffffu, s, o));
  __shared__ double ws[kThreadsNA / 32];
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    s = threadIdx.x < kThreadsNA / 32 ? ws[threadIdx.x] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s = __dadd_rn(s, __shfl_down_sync(0xffffffffu, s, o));
    if (threadIdx.x == 0) partials[blockIdx.x] = s;
  }
}

// Fixed-order sum of the nchunks partials; 0 -> 1 as in the reference's
// norm (src/operators_at_level.jl:21-23).
__global__ void __launch_bounds__(1024) k_chunk_final(const double* __restrict__ partials, int nchunks,
                                                      double* out) {
  __shared__ double sh[1024];
  double s = 0.0;
  for (int c = threadIdx.x; c < nchunks; c += 1024) s = __dadd_rn(s, partials[c]);
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int w = 512; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) sh[threadIdx.x] = __dadd_rn(sh[threadIdx.x], sh[threadIdx.x + w]);
    __syncthreads();
  }
  if (threadIdx.x == 0) out[0] = (sh[0] == 0.0) ? 1.0 : sh[0];
}

int fail_na(int code, const std::string& msg) {
  set_global_error(msg);  // read back with cfmg_last_error(NULL)
  return code;
}

// Unique id of the current CUDA context (0 when none is current yet).
int current_context_id(unsigned long long* id) {
  *id = 0;
  if (!g_ctx_get_current || !g_ctx_get_id) {
    cudaDriverEntryPointQueryResult q1, q2;
    void *f1 = nullptr, *f2 = nullptr;
    cudaError_t e1 = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1);
    cudaError_t e2 = cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2);
    if (e1 != cudaSuccess || e2 != cudaSuccess || q1 != cudaDriverEntryPointSuccess ||
        q2 != cudaDriverEntryPointSuccess || !f1 || !f2)
      return fail_na(CFMG_ERR_CUDA, "cfmg_norm_noalloc: cuCtxGetCurrent/cuCtxGetId are not available");
    g_ctx_get_current = (PFN_ctxGetCurrent)f1;
    g_ctx_get_id = (PFN_ctxGetId)f2;
  }
  void* ctx = nullptr;
  if (g_ctx_get_current(&ctx) != 0)
    return fail_na(CFMG_ERR_CUDA, "cfmg_norm_noalloc: cuCtxGetCurrent failed");
  if (ctx && g_ctx_get_id(ctx, id) != 0) return fail_na(CFMG_ERR_CUDA, "cfmg_norm_noalloc: cuCtxGetId failed");
  return CFMG_OK;
}

// Device address of the static scratch on the current device. Set up once
// per device and context: repeated only when the context has changed.
int scratch_address(double** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail_na(CFMG_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return fail_na(CFMG_ERR_UNSUPPORTED, "device index beyond 63");
  std::lock_guard<std::mutex> lk(g_mu);
  unsigned long long ctx = 0;
  int rc = current_context_id(&ctx);
  if (rc != CFMG_OK) return rc;
  if (!g_addr[dev] || ctx == 0 || ctx != g_ctx_id[dev]) {
    double* p = nullptr;
    e = cudaGetSymbolAddress((void**)&p, g_noalloc_partials);
    if (e != cudaSuccess) {
      set_global_error(std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
      return CFMG_ERR_CUDA;
    }
    // cudaGetSymbolAddress made the runtime's context current if none was.
    rc = current_context_id(&ctx);
    if (rc != CFMG_OK) return rc;
    g_addr[dev] = p;
    g_ctx_id[dev] = ctx;
  }
  *out = g_addr[dev];
  return CFMG_OK;
}

}  // namespace

}  // namespace cfmg

using namespace cfmg;

extern "C" int cfmg_norm_noalloc(const double* x, const uint8_t* msk, long long n, double* out, void* stream) {
  if (!x || !msk || !out) return fail_na(CFMG_ERR_ARG, "cfmg_norm_noalloc: null pointer");
  if (n < 0) return fail_na(CFMG_ERR_ARG, "cfmg_norm_noalloc: negative n = " + std::to_string(n));
  if (n > kMaxElems)
    return fail_na(CFMG_ERR_ARG, "cfmg_norm_noalloc: n = " + std::to_string(n) + " exceeds the static scratch limit of " +
                                     std::to_string(kMaxElems) + " elements");
  double* partials = nullptr;
  int rc = scratch_address(&partials);
  if (rc != CFMG_OK) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  const int nchunks = (int)((n + kChunk - 1) / kChunk);
  if (nchunks > 0) k_chunk_partials<<<nchunks, kThreadsNA, 0, s>>>(x, msk, n, partials);
  k_chunk_final<<<1, 1024, 0, s>>>(partials, nchunks, out);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail_na(CFMG_ERR_CUDA, std::string("cfmg_norm_noalloc launch: ") + cudaGetErrorString(e));
  return CFMG_OK;
}
