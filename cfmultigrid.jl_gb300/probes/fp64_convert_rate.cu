// Issue-rate probe: FP64 <-> FP32 / int64 conversions and int64 arithmetic on sm_103a (design input for the mixed form).
#include <cstdio>
#include <cstdint>
#include <cuda_runtime.h>

#define CK(x) do { cudaError_t e = (x); if (e != cudaSuccess) { printf("err %s line %d\n", cudaGetErrorString(e), __LINE__); return 1; } } while (0)

template <int OP>
__global__ void k(double* out, int iters) {
  double d0 = threadIdx.x * 1e-3 + 1.0, d1 = d0 + 1, d2 = d0 + 2, d3 = d0 + 3;
  float f0 = threadIdx.x * 1e-3f + 1.0f, f1 = f0 + 1, f2 = f0 + 2, f3 = f0 + 3;
  long long l0 = threadIdx.x, l1 = l0 + 1, l2 = l0 + 2, l3 = l0 + 3;
  for (int i = 0; i < iters; ++i) {
    if (OP == 0) {  // f32 -> f64 -> f32 round trip (F2F both ways)
      d0 = (double)f0 + 1e-30; f0 = (float)d0 * 1.0000001f;
      d1 = (double)f1 + 1e-30; f1 = (float)d1 * 1.0000001f;
      d2 = (double)f2 + 1e-30; f2 = (float)d2 * 1.0000001f;
      d3 = (double)f3 + 1e-30; f3 = (float)d3 * 1.0000001f;
    } else if (OP == 1) {  // i64 -> f64 (I2F.F64.S64) then bits back (integer)
      d0 = __ll2double_rn(l0); l0 = __double_as_longlong(d0) + 3;
      d1 = __ll2double_rn(l1); l1 = __double_as_longlong(d1) + 3;
      d2 = __ll2double_rn(l2); l2 = __double_as_longlong(d2) + 3;
      d3 = __ll2double_rn(l3); l3 = __double_as_longlong(d3) + 3;
    } else if (OP == 2) {  // f32 -> i64 (F2I.S64) and back via int ops
      l0 = __float2ll_rn(f0) + l0; f0 = __int_as_float((int)(l0 & 0x3fffffff) | 0x3f800000);
      l1 = __float2ll_rn(f1) + l1; f1 = __int_as_float((int)(l1 & 0x3fffffff) | 0x3f800000);
      l2 = __float2ll_rn(f2) + l2; f2 = __int_as_float((int)(l2 & 0x3fffffff) | 0x3f800000);
      l3 = __float2ll_rn(f3) + l3; f3 = __int_as_float((int)(l3 & 0x3fffffff) | 0x3f800000);
    } else if (OP == 3) {  // 64-bit integer add chain
      l0 = l0 + l1 * 2; l1 = l1 + l2 * 4; l2 = l2 + l3; l3 = l3 + l0;
    } else if (OP == 4) {  // f32 -> f64 only (F2F.F64.F32), with dadd
      d0 = __dadd_rn(d0, (double)f0); f0 = f0 * 1.0000001f;
      d1 = __dadd_rn(d1, (double)f1); f1 = f1 * 1.0000001f;
      d2 = __dadd_rn(d2, (double)f2); f2 = f2 * 1.0000001f;
      d3 = __dadd_rn(d3, (double)f3); f3 = f3 * 1.0000001f;
    }
  }
  double s = d0 + d1 + d2 + d3 + f0 + f1 + f2 + f3 + (double)(l0 + l1 + l2 + l3);
  if (s == 12345.678) out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

int main() {
  int sms;
  CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0));
  double* out;
  CK(cudaMalloc(&out, 1 << 24));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  int iters = 2048, blocks = sms * 8, threads = 256;
  const char* names[5] = {"f32<->f64 roundtrip (2 cvt + 1 dadd + 1 fmul)/elem", "i64->f64 (1 I2F.F64)/elem",
                          "f32->i64 (1 F2I.S64 + iops)/elem", "i64 add/mul chain (1 op-pair)/elem",
                          "f32->f64 + dadd (1 cvt + 1 dadd)/elem"};
  for (int op = 0; op < 5; ++op) {
    for (int rep = 0; rep < 2; ++rep) {
      cudaEventRecord(e0);
      switch (op) {
        case 0: k<0><<<blocks, threads>>>(out, iters); break;
        case 1: k<1><<<blocks, threads>>>(out, iters); break;
        case 2: k<2><<<blocks, threads>>>(out, iters); break;
        case 3: k<3><<<blocks, threads>>>(out, iters); break;
        case 4: k<4><<<blocks, threads>>>(out, iters); break;
      }
      cudaEventRecord(e1);
      CK(cudaEventSynchronize(e1));
      float ms;
      cudaEventElapsedTime(&ms, e0, e1);
      double el = (double)blocks * threads * iters * 4;
      if (rep == 1) printf("%-55s %8.3f ms  %8.1f G elem/s\n", names[op], ms, el / ms / 1e6);
    }
  }
  CK(cudaGetLastError());
  return 0;
}
