// Issue-rate probe: FP64 DADD/DMUL/DFMA vs FP32 FFMA, and HBM copy bandwidth (design input for the FP64 form).
#include <cstdio>
#include <cuda_runtime.h>

#define CK(x) do { cudaError_t e = (x); if (e != cudaSuccess) { printf("err %s line %d\n", cudaGetErrorString(e), __LINE__); return 1; } } while (0)

template <int OP>
__global__ void k_fp64(double* out, double a, double b, int iters) {
  double x0 = threadIdx.x * 1e-3, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
  double x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
#define STEP(x) if (OP == 0) x = __dadd_rn(x, a); else if (OP == 1) x = __dmul_rn(x, b); else x = __fma_rn(x, b, a);
    STEP(x0) STEP(x1) STEP(x2) STEP(x3) STEP(x4) STEP(x5) STEP(x6) STEP(x7)
  }
  double s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
  if (s == 12345.678) out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void k_fp32(float* out, float a, float b, int iters) {
  float x0 = threadIdx.x * 1e-3f, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
  float x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
#define STEPF(x) x = __fmaf_rn(x, b, a);
    STEPF(x0) STEPF(x1) STEPF(x2) STEPF(x3) STEPF(x4) STEPF(x5) STEPF(x6) STEPF(x7)
  }
  float s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
  if (s == 12345.678f) out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void k_copy(const double2* __restrict__ a, double2* __restrict__ b, size_t n) {
  size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  size_t stride = (size_t)gridDim.x * blockDim.x;
  for (; i < n; i += stride) b[i] = a[i];
}

int main() {
  cudaDeviceProp p;
  CK(cudaGetDeviceProperties(&p, 0));
  printf("name %s sms %d l2 %d smem/blk optin %zu cc %d.%d\n", p.name, p.multiProcessorCount,
         p.l2CacheSize, p.sharedMemPerBlockOptin, p.major, p.minor);
  int sms = p.multiProcessorCount;
  double* out;
  CK(cudaMalloc(&out, 1 << 24));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  int iters = 4096;
  int blocks = sms * 8, threads = 256;
  const char* names[3] = {"dadd", "dmul", "dfma"};
  for (int op = 0; op < 3; ++op) {
    for (int rep = 0; rep < 2; ++rep) {
      cudaEventRecord(e0);
      if (op == 0) k_fp64<0><<<blocks, threads>>>(out, 1e-9, 1.0000001, iters);
      if (op == 1) k_fp64<1><<<blocks, threads>>>(out, 1e-9, 1.0000001, iters);
      if (op == 2) k_fp64<2><<<blocks, threads>>>(out, 1e-9, 1.0000001, iters);
      cudaEventRecord(e1);
      CK(cudaEventSynchronize(e1));
      float ms;
      cudaEventElapsedTime(&ms, e0, e1);
      double ops = (double)blocks * threads * iters * 8;
      if (rep == 1) printf("%s: %.3f ms  %.1f Gop/s  (%.2f lane-ops/clk/SM at 1.92GHz)\n", names[op], ms, ops / ms / 1e6,
                           ops / (ms * 1e-3) / sms / 1.92e9);
    }
  }
  for (int rep = 0; rep < 2; ++rep) {
    cudaEventRecord(e0);
    k_fp32<<<blocks, threads>>>((float*)out, 1e-9f, 1.0000001f, iters * 4);
    cudaEventRecord(e1);
    CK(cudaEventSynchronize(e1));
    float ms;
    cudaEventElapsedTime(&ms, e0, e1);
    double ops = (double)blocks * threads * iters * 4 * 8;
    if (rep == 1) printf("ffma: %.3f ms  %.1f Gop/s\n", ms, ops / ms / 1e6);
  }
  size_t n = (size_t)1 << 27;  // 2 GiB each as double2*16B
  double2 *a, *b;
  CK(cudaMalloc(&a, n * 16));
  CK(cudaMalloc(&b, n * 16));
  CK(cudaMemset(a, 0, n * 16));
  for (int rep = 0; rep < 3; ++rep) {
    cudaEventRecord(e0);
    k_copy<<<sms * 8, 512>>>(a, b, n);
    cudaEventRecord(e1);
    CK(cudaEventSynchronize(e1));
    float ms;
    cudaEventElapsedTime(&ms, e0, e1);
    printf("copy: %.3f ms %.1f GB/s\n", ms, 2.0 * n * 16 / ms / 1e6);
  }
  CK(cudaGetLastError());
  return 0;
}
