// Batched solver: many independent 2D instances of uneven sizes advance
// through the mixed-precision solve loop in lockstep.
//
// An iteration is a fixed sequence of launches, each covering every
// instance at once: the fused FP64 residual pass over all level-1 grids,
// one reduction block per instance (residual ratio, history, stopping
// rule), the FP32 cycle as a sequence of level steps, and the FP64 update.
// The cycle's steps are aligned at the coarsest level: step "depth d" acts
// on level nlev_i - d + 1 of every instance with at least d levels, so all
// instances share one schedule while their level counts differ. Every
// launch is a grid-stride loop over fixed-size chunks of its work, and an
// instance that has converged drops out of all of them (its chunks are
// skipped). The host captures one iteration in the body of a graph `while`
// node whose condition the last kernel sets: the whole batch is one graph
// launch.
//
// Arithmetic per cell is the single-instance code (ops_dev.cuh); the
// reductions use a fixed chunk-to-thread assignment and fixed-order block
// sums, so a batch's results do not depend on the launch shape.
#include "exec_dev.cuh"

namespace cfmg {

__device__ __forceinline__ unsigned long long gtimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// last item i with cstart[i] <= c
__device__ __forceinline__ int find_item(const long long* __restrict__ cstart, int nitems, long long c) {
  int lo = 0, hi = nitems - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (cstart[mid] <= c) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// fixed-order block sum (kBThreads threads); valid in thread 0
__device__ __forceinline__ double bsum(double v, double* sh) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = __dadd_rn(v, __shfl_down_sync(0xffffffffu, v, o));
  __syncthreads();
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < kBThreads / 32; ++w) t = __dadd_rn(t, sh[w]);
  return t;
}

// ------------------------------------------------------------ cycle steps
// Generic step: the chunks of a list of Ops (any kinds, one per instance
// or more), each executed with the per-item code of the program engine.
__global__ void __launch_bounds__(kBThreads, 3) k_bstage(const Op* __restrict__ ops, const long long* __restrict__ cstart,
                                                      int nops, long long nchunks, const int* __restrict__ active) {
  __shared__ Op op;
  for (long long c = blockIdx.x; c < nchunks; c += gridDim.x) {
    const int o = find_item(cstart, nops, c);
    if (!active[ops[o].inst]) continue;
    __syncthreads();  // the previous chunk's readers of op are done
    if (threadIdx.x < sizeof(Op) / sizeof(int)) ((int*)&op)[threadIdx.x] = ((const int*)&ops[o])[threadIdx.x];
    __syncthreads();
    const long long t0 = (c - cstart[o]) * kBChunk;
    const long long e = t0 + kBChunk < op.n ? t0 + kBChunk : op.n;
    if (op.prec == 0) exec<double>(op, t0 + threadIdx.x, kBThreads, e);
    else exec<float>(op, t0 + threadIdx.x, kBThreads, e);
  }
}
static_assert(sizeof(Op) / sizeof(int) <= kBThreads, "one thread per word of an Op");

// ------------------------------------------------------- FP64 loop steps
// start of a solve: zero x when asked, normb = sum msk b^2 (0 -> 1 for the
// reference rule), the first right-hand-side scale from |b|, counters.
// One block per instance.
__global__ void __launch_bounds__(kBThreads) k_binit(const BInst* __restrict__ bi, int zero_x, int* active,
                                                     int* nactive) {
  __shared__ double sh[kBThreads / 32];
  const BInst& B = bi[blockIdx.x];
  double* sc = B.sc;
  const bool zx = zero_x != 0;
  double v = 0.0;
  for (long long t = threadIdx.x; t < B.len; t += kBThreads) {
    if (zx) B.x[t] = 0.0;
    const uint8_t mm = B.m[t];
    const double bb = B.b[t];
    if (mm) v = (mm == 1) ? __fma_rn(bb, bb, v) : __dadd_rn(v, __dmul_rn((double)mm, __dmul_rn(bb, bb)));
  }
  double tot = bsum(v, sh);
  if (threadIdx.x == 0) {
    if (B.norm_kind == CFMG_NORM_REF_SQUARED && tot == 0.0) tot = 1.0;
    sc[BS_NORMB] = tot;
    sc[BS_NITE] = 0.0;
    const double nw = sc[BS_NWET] > 0 ? sc[BS_NWET] : 1.0;
    const double rms = sqrt(tot / nw);
    int e = 0;
    if (rms > 0 && isfinite(rms)) frexp(rms, &e);
    sc[BS_NEXT] = ldexp(1.0, -e);
    sc[BS_T0] = (double)gtimer();
    active[blockIdx.x] = 1;
    if (blockIdx.x == 0) *nactive = 0;
  }
}

// Fused FP64 residual over the level-1 chunks of every active instance:
// r = b - A x per cell (the residual operator's arithmetic), the chunk's
// sum r^2 and sum r to partials[2c], partials[2c+1], and the scaled FP32
// right-hand side (vertex-centred) or the FP64 r (cell-centred, for the
// mean-removing pass).
template <int KIND, bool NEUMANN>
__global__ void __launch_bounds__(kBThreads) k_bres(const BInst* __restrict__ bi, const long long* __restrict__ cstart,
                                                    int ninst, long long nchunks, const int* __restrict__ active,
                                                    double* __restrict__ partials) {
  __shared__ double sh2[kBThreads / 32], sh1[kBThreads / 32];
  for (long long c = blockIdx.x; c < nchunks; c += gridDim.x) {
    const int i = find_item(cstart, ninst, c);
    if (!active[i]) continue;
    const BInst& B = bi[i];
    const double scale = B.sc[BS_NEXT];
    const long long t0 = (c - cstart[i]) * kBChunk;
    const long long e = t0 + kBChunk < B.n ? t0 + kBChunk : B.n;
    const long long ni = B.box.i1 - B.box.i0 + 1, nj = B.box.j1 - B.box.j0 + 1;
    double s2 = 0.0, s1 = 0.0, c1 = 0.0;
    for (long long t = t0 + threadIdx.x; t < e; t += kBThreads) {
      long long I;
      if (KIND == OPK_RESID9) {
        const int ii = B.box.i0 + (int)(t % ni);
        const long long q = t / ni;
        I = lin(B.g, ii, B.box.j0 + (int)(q % nj), B.box.k0 + (int)(q / nj));
      } else {
        I = B.lo + t;
      }
      const double v = (KIND == OPK_RESID9) ? v_resid9(B.x, B.b, B.d, B.m, B.g.n1, I)
                                            : v_resid5(B.x, B.b, B.d, B.m, B.g.n1, I);
      s2 = __fma_rn(v, v, s2);
      if (NEUMANN) {
        B.r[I] = v;
        const double tt = __dadd_rn(s1, v);
        c1 = __dadd_rn(c1, (fabs(s1) >= fabs(v)) ? __dadd_rn(__dsub_rn(s1, tt), v) : __dadd_rn(__dsub_rn(v, tt), s1));
        s1 = tt;
      } else {
        const float f = (float)(v * scale);
        B.b32[I] = f;
        B.r32[I] = f;
      }
    }
    s1 = __dadd_rn(s1, c1);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      s2 = __dadd_rn(s2, __shfl_down_sync(0xffffffffu, s2, o));
      s1 = __dadd_rn(s1, __shfl_down_sync(0xffffffffu, s1, o));
    }
    __syncthreads();
    if ((threadIdx.x & 31) == 0) {
      sh2[threadIdx.x >> 5] = s2;
      sh1[threadIdx.x >> 5] = s1;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      double a = 0.0, b = 0.0;
      for (int w = 0; w < kBThreads / 32; ++w) {
        a = __dadd_rn(a, sh2[w]);
        b = __dadd_rn(b, sh1[w]);
      }
      partials[2 * c] = a;
      partials[2 * c + 1] = b;
    }
  }
}

// One block per active instance: its chunks' partial sums in a fixed
// order, then the loop's bookkeeping.
//   res = sum/normb (reference rule, sum 0 -> 1) or sqrt(sum/normb) (L2);
//   hist[nite] = res; mean = sum r / nwet (cell-centred);
//   the scale the pass just applied (NEXT) becomes CUR / ICUR, and the
//   next one is 2^-round(log2(rms)) (exact both ways);
//   continue while res > tol && nite < maxite (src/gmg_solver.jl:29-39),
//   counting the cycle about to run; else the instance stops here.
__global__ void __launch_bounds__(kBThreads) k_bfinal(const BInst* __restrict__ bi,
                                                      const long long* __restrict__ cstart,
                                                      const double* __restrict__ partials, int* active,
                                                      int* nactive) {
  __shared__ double sh[kBThreads / 32];
  const int i = blockIdx.x;
  if (!active[i]) return;
  const BInst& B = bi[i];
  double a = 0.0, b = 0.0;
  for (long long c = cstart[i] + threadIdx.x; c < cstart[i + 1]; c += kBThreads) {
    a = __dadd_rn(a, partials[2 * c]);
    b = __dadd_rn(b, partials[2 * c + 1]);
  }
  const double s2 = bsum(a, sh);
  const double s1 = bsum(b, sh);
  if (threadIdx.x == 0) {
    double* sc = B.sc;
    double sum = s2;
    double res;
    const double normb = sc[BS_NORMB];
    if (B.norm_kind == CFMG_NORM_REF_SQUARED) {
      if (sum == 0.0) sum = 1.0;
      res = normb > 0.0 ? sum / normb : 0.0;
    } else {
      res = normb > 0.0 ? sqrt(sum / normb) : 0.0;
    }
    const int nite = (int)sc[BS_NITE];
    sc[BS_RES] = res;
    sc[BS_HIST + nite] = res;
    const double nw = sc[BS_NWET] > 0 ? sc[BS_NWET] : 1.0;
    sc[BS_MEAN] = s1 / nw;
    const double used = sc[BS_NEXT];
    sc[BS_CUR] = used;
    sc[BS_ICUR] = 1.0 / used;
    const double rms = sqrt(s2 / nw);
    int e = 0;
    if (rms > 0 && isfinite(rms)) frexp(rms, &e);
    sc[BS_NEXT] = ldexp(1.0, -e);
    if (res > B.tol && nite < B.maxite) {
      sc[BS_NITE] = (double)(nite + 1);
      atomicAdd(nactive, 1);
    } else {
      active[i] = 0;
      sc[BS_T1] = (double)gtimer();
    }
  }
}

// cell-centred: b32 = r32 = msk ? (r - mean) * CUR : 0 over the whole array
__global__ void __launch_bounds__(kBThreads) k_brhs(const BInst* __restrict__ bi, const long long* __restrict__ cstart,
                                                    int ninst, long long nchunks, const int* __restrict__ active) {
  for (long long c = blockIdx.x; c < nchunks; c += gridDim.x) {
    const int i = find_item(cstart, ninst, c);
    if (!active[i]) continue;
    const BInst& B = bi[i];
    const double mean = B.sc[BS_MEAN], scale = B.sc[BS_CUR];
    const long long t0 = (c - cstart[i]) * kBChunk;
    const long long e = t0 + kBChunk < B.len ? t0 + kBChunk : B.len;
    for (long long t = t0 + threadIdx.x; t < e; t += kBThreads) {
      const float f = B.m[t] ? (float)((B.r[t] - mean) * scale) : 0.f;
      B.b32[t] = f;
      B.r32[t] = f;
    }
  }
}

// x += e32 * ICUR over the whole array
__global__ void __launch_bounds__(kBThreads) k_bupdate(const BInst* __restrict__ bi,
                                                       const long long* __restrict__ cstart, int ninst,
                                                       long long nchunks, const int* __restrict__ active) {
  for (long long c = blockIdx.x; c < nchunks; c += gridDim.x) {
    const int i = find_item(cstart, ninst, c);
    if (!active[i]) continue;
    const BInst& B = bi[i];
    const double is = B.sc[BS_ICUR];
    const long long t0 = (c - cstart[i]) * kBChunk;
    const long long e = t0 + kBChunk < B.len ? t0 + kBChunk : B.len;
    for (long long t = t0 + threadIdx.x; t < e; t += kBThreads) B.x[t] = __fma_rn((double)B.e32[t], is, B.x[t]);
  }
}

// the `while` condition: another iteration while any instance continues
__global__ void k_bcond(cudaGraphConditionalHandle hc, int* nactive) {
  const int n = *nactive;
  *nactive = 0;
  cudaGraphSetConditional(hc, n > 0 ? 1u : 0u);
}

// ------------------------------------------------------------- launchers
static int g_nsm = 0;
static long long grid_for(long long nchunks, int per_sm) {
  if (!g_nsm) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&g_nsm, cudaDevAttrMultiProcessorCount, dev);
    if (g_nsm <= 0) g_nsm = 1;
  }
  const long long g = (long long)g_nsm * per_sm;
  return nchunks < g ? (nchunks > 0 ? nchunks : 1) : g;
}

void launch_bstage(const Op* ops, const long long* cstart, int nops, long long nchunks, const int* active,
                   cudaStream_t s) {
  if (nchunks <= 0) return;
  k_bstage<<<(unsigned)grid_for(nchunks, 8), kBThreads, 0, s>>>(ops, cstart, nops, nchunks, active);
}

void launch_binit(const BInst* bi, int ninst, int zero_x, int* active, int* nactive, cudaStream_t s) {
  k_binit<<<ninst, kBThreads, 0, s>>>(bi, zero_x, active, nactive);
}

void launch_bres(int kind, bool neumann, const BInst* bi, const long long* cstart, int ninst, long long nchunks,
                 const int* active, double* partials, cudaStream_t s) {
  const unsigned g = (unsigned)grid_for(nchunks, 8);
  if (kind == OPK_RESID9) {
    if (neumann) k_bres<OPK_RESID9, true><<<g, kBThreads, 0, s>>>(bi, cstart, ninst, nchunks, active, partials);
    else k_bres<OPK_RESID9, false><<<g, kBThreads, 0, s>>>(bi, cstart, ninst, nchunks, active, partials);
  } else {
    if (neumann) k_bres<OPK_RESID5, true><<<g, kBThreads, 0, s>>>(bi, cstart, ninst, nchunks, active, partials);
    else k_bres<OPK_RESID5, false><<<g, kBThreads, 0, s>>>(bi, cstart, ninst, nchunks, active, partials);
  }
}

void launch_bfinal(const BInst* bi, const long long* cstart, int ninst, const double* partials, int* active,
                   int* nactive, cudaStream_t s) {
  k_bfinal<<<ninst, kBThreads, 0, s>>>(bi, cstart, partials, active, nactive);
}

void launch_brhs(const BInst* bi, const long long* cstart, int ninst, long long nchunks, const int* active,
                 cudaStream_t s) {
  k_brhs<<<(unsigned)grid_for(nchunks, 8), kBThreads, 0, s>>>(bi, cstart, ninst, nchunks, active);
}

void launch_bupdate(const BInst* bi, const long long* cstart, int ninst, long long nchunks, const int* active,
                    cudaStream_t s) {
  k_bupdate<<<(unsigned)grid_for(nchunks, 8), kBThreads, 0, s>>>(bi, cstart, ninst, nchunks, active);
}

void launch_bcond(cudaGraphConditionalHandle hc, int* nactive, cudaStream_t s) {
  k_bcond<<<1, 1, 0, s>>>(hc, nactive);
}

}  // namespace cfmg
