// Fused FP64 steps of the mixed-precision defect-correction loop.
//
// One pass over level 1 computes the FP64 residual r = b - A x with the
// same per-cell arithmetic as the residual operator, and in the same pass
//   * accumulates sum(msk r^2) and sum(msk r) per block (FP64; fixed
//     block-to-cell assignment, so the reduction is deterministic),
//   * writes the FP32 right-hand side of the correction equation,
//     (float)(r * scale), where scale is a power of two taken from the
//     previous residual norm (its only job is to keep FP32 far from
//     under- and overflow; exact in both directions).
// For the vertex-centred (Dirichlet) operator that is the whole FP64 work
// of an iteration besides the update x += e / scale. For the cell-centred
// (Neumann) operator the wet mean must come off first: the pass also keeps
// r in FP64 and a second pass writes the mean-free FP32 right-hand side.
#include "ops_dev.cuh"

namespace cfmg {

constexpr int kMxThreads = 256;
constexpr int kMxParts = 1024;  // blocks of the fused pass; two sums each
static_assert(2 * kMxParts <= kPartials, "the fused pass writes 2*kMxParts partial sums");

// per-block partial sums -> 2 * kMxParts doubles: [sum r^2 | sum r]. With
// NEUMANN the FP64 r is kept for the mean-removing pass and sum r is
// Neumaier-compensated per thread; else the scaled FP32 right-hand side is
// written here and r64 is not stored.
template <int KIND, bool NEUMANN>
__global__ void __launch_bounds__(kMxThreads) k_resid_fused(double* __restrict__ r, const double* __restrict__ x,
                                                            const double* __restrict__ b, const double* __restrict__ d,
                                                            const uint8_t* __restrict__ m, Geom g, Box bx,
                                                            long long lo, long long n, const double* __restrict__ ds,
                                                            float* __restrict__ b32, float* __restrict__ r32,
                                                            double* __restrict__ partials) {
  const double scale = ds[0];
  double s2 = 0.0, s1 = 0.0, c1 = 0.0;
  const long long ni = bx.i1 - bx.i0 + 1, nj = bx.j1 - bx.j0 + 1;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    long long I;
    if (KIND == OPK_RESID9 || KIND == OPK_RESID7 || KIND == OPK_RESID19) {
      const int i = bx.i0 + (int)(t % ni);
      const long long q = t / ni;
      const int j = bx.j0 + (int)(q % nj);
      const int k = bx.k0 + (int)(q / nj);
      I = lin(g, i, j, k);
    } else {
      I = lo + t;
    }
    double v;
    if (KIND == OPK_RESID5) v = v_resid5(x, b, d, m, g.n1, I);
    else if (KIND == OPK_RESID9) v = v_resid9(x, b, d, m, g.n1, I);
    else if (KIND == OPK_RESID7) v = v_resid7(x, b, d, m, g.n1, g.n2, I);
    else v = v_resid19(x, b, d, m, g.n1, g.n2, I);
    s2 = __fma_rn(v, v, s2);  // v is a signed zero on dry cells
    if (NEUMANN) {
      r[I] = v;
      const double tt = __dadd_rn(s1, v);
      c1 = __dadd_rn(c1, (fabs(s1) >= fabs(v)) ? __dadd_rn(__dsub_rn(s1, tt), v) : __dadd_rn(__dsub_rn(v, tt), s1));
      s1 = tt;
    } else {
      const float f = (float)(v * scale);
      b32[I] = f;
      r32[I] = f;
    }
  }
  s1 = __dadd_rn(s1, c1);
  __shared__ double sh2[kMxThreads / 32], sh1[kMxThreads / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    s2 += __shfl_down_sync(0xffffffffu, s2, o);
    s1 += __shfl_down_sync(0xffffffffu, s1, o);
  }
  if ((threadIdx.x & 31) == 0) {
    sh2[threadIdx.x >> 5] = s2;
    sh1[threadIdx.x >> 5] = s1;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, c = 0.0;
    for (int w = 0; w < kMxThreads / 32; ++w) {
      a += sh2[w];
      c += sh1[w];
    }
    partials[blockIdx.x] = a;
    partials[kMxParts + blockIdx.x] = c;
  }
}

// Final reduction into the handle's scalars: S_NORM = sum msk r^2 (0 -> 1
// for the reference rule), S_RES = the residual ratio against *normb,
// S_MEAN2 = wet mean of r (when nwet is given). The scale the pass just
// applied (S_NEXT on entry) becomes S_CUR / S_ICUR, and the next scale
// 2^-round(log2(rms)) goes to S_NEXT (powers of two, exact both ways).
__global__ void __launch_bounds__(kMxParts) k_fused_final(const double* __restrict__ partials, double* ds,
                                                          const double* normb, const double* nwet, int norm_kind) {
  __shared__ double a[kMxParts], c[kMxParts];
  a[threadIdx.x] = partials[threadIdx.x];
  c[threadIdx.x] = partials[kMxParts + threadIdx.x];
  __syncthreads();
  for (int w = kMxParts / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) {
      a[threadIdx.x] += a[threadIdx.x + w];
      c[threadIdx.x] += c[threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    double sum = a[0];
    const double raw = sum;
    if (norm_kind == CFMG_NORM_REF_SQUARED) {
      if (sum == 0.0) sum = 1.0;
      ds[S_NORM] = sum;
      ds[S_RES] = (*normb > 0.0) ? sum / *normb : 0.0;
    } else {
      ds[S_NORM] = sum;
      ds[S_RES] = (*normb > 0.0) ? sqrt(sum / *normb) : 0.0;
    }
    const double nw = (nwet && *nwet > 0) ? *nwet : 1.0;
    ds[S_MEAN2] = nwet ? c[0] / nw : 0.0;
    const double used = ds[S_NEXT];
    ds[S_CUR] = used;
    ds[S_ICUR] = 1.0 / used;
    const double rms = sqrt(raw / (nwet && *nwet > 0 ? *nwet : 1.0));
    int e = 0;
    if (rms > 0 && isfinite(rms)) frexp(rms, &e);
    ds[S_NEXT] = ldexp(1.0, -e);
  }
}

// Neumann second pass: b32 = r32 = msk ? (r - mean) * scale : 0, with
// ms[0] = S_MEAN2 and ms[1] = S_CUR (the scale of this right-hand side)
__global__ void k_rhs32_mean(const double* __restrict__ r, const uint8_t* __restrict__ m,
                             const double* __restrict__ ms, float* __restrict__ b32, float* __restrict__ r32,
                             long long n) {
  long long I = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (I >= n) return;
  const float f = m[I] ? (float)((r[I] - ms[0]) * ms[S_CUR - S_MEAN2]) : 0.f;
  b32[I] = f;
  r32[I] = f;
}

// x += e * iscale
__global__ void k_update_scaled(double* __restrict__ x, const float* __restrict__ e, const double* __restrict__ is,
                                long long n) {
  long long I = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (I < n) x[I] = __fma_rn((double)e[I], is[0], x[I]);
}

void launch_resid_fused(int kind, double* r, const double* x, const double* b, const double* d, const uint8_t* m,
                        const Geom& g, const Box& bx, long long lo, long long n, const double* scale, float* b32,
                        float* r32, bool neumann, double* partials, cudaStream_t s) {
#define CFMG_FUSED(K)                                                                                            \
  if (kind == K) {                                                                                               \
    if (neumann)                                                                                                 \
      k_resid_fused<K, true><<<kMxParts, kMxThreads, 0, s>>>(r, x, b, d, m, g, bx, lo, n, scale, b32, r32, partials); \
    else                                                                                                         \
      k_resid_fused<K, false><<<kMxParts, kMxThreads, 0, s>>>(r, x, b, d, m, g, bx, lo, n, scale, b32, r32, partials); \
    return;                                                                                                      \
  }
  CFMG_FUSED(OPK_RESID5)
  CFMG_FUSED(OPK_RESID9)
  CFMG_FUSED(OPK_RESID7)
  CFMG_FUSED(OPK_RESID19)
#undef CFMG_FUSED
}

void launch_fused_final(const double* partials, double* ds, const double* normb, const double* nwet, int norm_kind,
                        cudaStream_t s) {
  k_fused_final<<<1, kMxParts, 0, s>>>(partials, ds, normb, nwet, norm_kind);
}

void launch_rhs32_mean(const double* r, const uint8_t* m, const double* mean_scale, float* b32, float* r32,
                       long long n, cudaStream_t s) {
  k_rhs32_mean<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(r, m, mean_scale, b32, r32, n);
}

void launch_update_scaled(double* x, const float* e, const double* iscale, long long n, cudaStream_t s) {
  k_update_scaled<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(x, e, iscale, n);
}

}  // namespace cfmg
