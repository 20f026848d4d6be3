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
#include <algorithm>

#include "exec_dev.cuh"

namespace cfmg {

__device__ __forceinline__ unsigned long long gtimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Block-wide ordered compaction of a window of `win` (<= blockDim.x) table
// entries (base .. base+win-1): the entries whose instance is still active,
// as offsets from base in list[]; returns their count. wsum needs
// blockDim/32 + 1 ints.
__device__ __forceinline__ int active_window(const int4* __restrict__ tab, long long base, long long n, int win,
                                             const int* __restrict__ active, int* list, int* wsum) {
  const long long c = base + threadIdx.x;
  bool ok = false;
  if ((int)threadIdx.x < win && c < n) ok = active[tab[c].z] != 0;
  const unsigned bal = __ballot_sync(0xffffffffu, ok);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if (lane == 0) wsum[wid] = __popc(bal);
  __syncthreads();
  if (threadIdx.x == 0) {
    int a = 0;
    for (int w = 0; w < nw; ++w) {
      const int v = wsum[w];
      wsum[w] = a;
      a += v;
    }
    wsum[nw] = a;
  }
  __syncthreads();
  if (ok) list[wsum[wid] + __popc(bal & ((1u << lane) - 1u))] = threadIdx.x;
  const int cnt = wsum[nw];
  __syncthreads();
  return cnt;
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

// block maximum (kBThreads threads); valid in thread 0
__device__ __forceinline__ double bmax(double v, double* sh) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
  __syncthreads();
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < kBThreads / 32; ++w) t = fmax(t, sh[w]);
  return t;
}

// ------------------------------------------------------------ cycle steps
// Generic step: the active chunks (kBStageChunk items) of a list of Ops
// (tab[c] = {op, chunk of the op, instance}), each executed with the
// per-item code of the program engine, 4 (FP32) or 2 (FP64) items per
// thread in flight.
__global__ void __launch_bounds__(kBThreads, 2) k_bstage(const Op* __restrict__ ops, const int4* __restrict__ tab,
                                                         long long nchunks, int win, const int* __restrict__ active) {
  dep_wait();
  __shared__ Op op;
  __shared__ int list[kBThreads];
  __shared__ int wsum[kBThreads / 32 + 1];
  int cur = -1;
  for (long long base = (long long)blockIdx.x * win; base < nchunks; base += (long long)gridDim.x * win) {
    const int cnt = active_window(tab, base, nchunks, win, active, list, wsum);
    for (int q = 0; q < cnt; ++q) {
      const int4 en = tab[base + list[q]];
      if (en.x != cur) {
        __syncthreads();  // the previous Op's readers are done
        if (threadIdx.x < sizeof(Op) / sizeof(int)) ((int*)&op)[threadIdx.x] = ((const int*)&ops[en.x])[threadIdx.x];
        __syncthreads();
        cur = en.x;
      }
      const long long t0 = (long long)en.y * kBStageChunk;
      const long long e = t0 + kBStageChunk < op.n ? t0 + kBStageChunk : op.n;
      if (op.prec == 0) exec<double, 2>(op, t0 + threadIdx.x, kBThreads, e);
      else exec<float, 4>(op, t0 + threadIdx.x, kBThreads, e);
    }
    __syncthreads();  // list is rewritten by the next window
  }
}
static_assert(sizeof(Op) / sizeof(int) <= kBThreads, "one thread per word of an Op");

// ------------------------------------------------------- FP64 loop steps
// start of a solve: zero x when asked, normb = sum msk b^2 (0 -> 1 for the
// reference rule), the first right-hand-side scale from |b|, counters.
// One block per instance.
__global__ void __launch_bounds__(kBThreads) k_binit(const BInst* __restrict__ bi, int zero_x, int* active,
                                                     int* nactive) {
  dep_wait();
  __shared__ double sh[kBThreads / 32];
  const BInst& B = bi[blockIdx.x];
  double* sc = B.sc;
  const bool zx = zero_x != 0;
  double v = 0.0, mx = 0.0, mb = 0.0;
  for (long long t = threadIdx.x; t < B.len; t += kBThreads) {
    if (zx) B.x[t] = 0.0;
    const uint8_t mm = B.m[t];
    const double bb = B.b[t];
    if (mm) v = (mm == 1) ? __fma_rn(bb, bb, v) : __dadd_rn(v, __dmul_rn((double)mm, __dmul_rn(bb, bb)));
    mx = fmax(mx, fabs(B.x[t]));
    mb = fmax(mb, fabs(bb));
  }
  double tot = bsum(v, sh);
  __syncthreads();
  const double tmx = bmax(mx, sh), tmb = bmax(mb, sh);
  if (threadIdx.x == 0) {
    sc[BS_MAXX] = tmx;
    sc[BS_MAXB] = tmb;
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

// Fused FP64 residual over the active level-1 chunks (tab[c] = {instance,
// chunk of its level 1, instance, slot}): r = b - A x per cell (the
// residual operator's arithmetic), the chunk's sum r^2 and sum r to
// partials[2 slot], partials[2 slot + 1], and the scaled FP32 right-hand
// side (vertex-centred) or the FP64 r (cell-centred, for the mean-removing
// pass).
template <int KIND, bool NEUMANN>
__global__ void __launch_bounds__(kBThreads) k_bres(const BInst* __restrict__ bi, const int4* __restrict__ tab,
                                                    long long nchunks, int win, const int* __restrict__ active,
                                                    double* __restrict__ partials) {
  dep_wait();
  constexpr int U = kBChunk / kBThreads;
  __shared__ int list[kBThreads];
  __shared__ int wsum[kBThreads / 32 + 1];
  __shared__ double sh2[kBThreads / 32], sh1[kBThreads / 32];
  for (long long base = (long long)blockIdx.x * win; base < nchunks; base += (long long)gridDim.x * win) {
    const int cnt = active_window(tab, base, nchunks, win, active, list, wsum);
    for (int q = 0; q < cnt; ++q) {
      const int4 en = tab[base + list[q]];
      const long long c = en.w;  // the chunk's partial-sum slot (its instance's chunks are consecutive slots)
      const BInst& B = bi[en.x];
      const double scale = B.sc[BS_NEXT];
      const long long t0 = (long long)en.y * kBChunk;
      const long long ni = B.box.i1 - B.box.i0 + 1, nj = B.box.j1 - B.box.j0 + 1;
      double s2 = 0.0, s1 = 0.0, c1 = 0.0;
      double v[U];
      long long I[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const long long t = t0 + threadIdx.x + (long long)u * kBThreads;
        I[u] = -1;
        if (t < B.n) {
          if (KIND == OPK_RESID9) {
            const int ii = B.box.i0 + (int)(t % ni);
            const long long qq = t / ni;
            I[u] = lin(B.g, ii, B.box.j0 + (int)(qq % nj), B.box.k0 + (int)(qq / nj));
            v[u] = v_resid9(B.x, B.b, B.d, B.m, B.g.n1, I[u]);
          } else {
            I[u] = B.lo + t;
            v[u] = v_resid5(B.x, B.b, B.d, B.m, B.g.n1, I[u]);
          }
        }
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        if (I[u] < 0) continue;
        s2 = __fma_rn(v[u], v[u], s2);
        if (NEUMANN) {
          B.r[I[u]] = v[u];
          const double tt = __dadd_rn(s1, v[u]);
          c1 = __dadd_rn(c1, (fabs(s1) >= fabs(v[u])) ? __dadd_rn(__dsub_rn(s1, tt), v[u])
                                                       : __dadd_rn(__dsub_rn(v[u], tt), s1));
          s1 = tt;
        } else {
          const float f = (float)(v[u] * scale);
          B.b32[I[u]] = f;
          B.r32[I[u]] = f;
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
    __syncthreads();
  }
}

// Integer form of the fused residual (see k_resid_int2d in k_mixed.cu):
// one warp per task {instance, strip of 32 columns, chunk of kBIntRows
// rows}; the fixed-point exponent is the instance's own (BS_MAXX from its
// last update, BS_MAXB from the start of the solve). partials[2 task] =
// sum r^2 (from the FP32 right-hand-side values), partials[2 task + 1] =
// sum r (exact per task).
template <int KIND, bool NEUMANN>
__global__ void __launch_bounds__(kBThreads) k_bres_int(const BInst* __restrict__ bi, const int4* __restrict__ ttab,
                                                        long long ntasks, const int* __restrict__ active,
                                                        double* __restrict__ partials) {
  dep_wait();
  constexpr int q = (KIND == OPK_RESID9) ? 2 : 0;
  const int lane = threadIdx.x & 31;
  const long long warp0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long task = warp0; task < ntasks; task += nwarps) {
    const int4 en = ttab[task];
    if (!active[en.x]) continue;
    const BInst& B = bi[en.x];
    const double mx = fmax(B.sc[BS_MAXX], B.sc[BS_MAXB]);
    int ex = 0;
    if (mx > 0 && isfinite(mx)) frexp(mx, &ex);
    const int k = 58 - ex;
    const double scale = B.sc[BS_NEXT];
    const float fm = (float)ldexp(scale, -(k + q));
    const long long n1 = B.g.n1, len = B.len;
    const double* __restrict__ x = B.x;
    const int c = B.c0 + en.y * kBIntCols + lane - 1;  // lanes 1..30 own the strip
    const bool col_ok = lane >= 1 && lane <= kBIntCols && c < B.c0 + B.ncols;
    const int ra = en.z * kBIntRows, rb = min(ra + kBIntRows, B.nrows);
    auto at = [&](long long J) { return x[J < 0 ? 0 : (J >= len ? len - 1 : J)]; };
    auto conv_row = [&](double xc, long long& W, long long& C, long long& E) {
      C = to_fix(xc, k);
      W = __shfl_up_sync(0xffffffffu, C, 1);
      E = __shfl_down_sync(0xffffffffu, C, 1);
    };
    long long I = B.row0 + (long long)ra * n1 + c;
    long long Wm, Cm, Em, W0, C0, E0, Wp, Cp, Ep;
    conv_row(at(I - n1), Wm, Cm, Em);
    conv_row(at(I), W0, C0, E0);
    double nc = at(I + n1);  // one row of look-ahead (see k_resid_int2d)
    double nb = col_ok ? B.b[I] : 0.0;
    int nd = col_ok ? B.dq[I] : -1;
    float hi = 0.f, lo = 0.f;
    __int128 s1 = 0;
    for (int r = ra; r < rb; ++r, I += n1) {
      conv_row(nc, Wp, Cp, Ep);
      const double cb = nb;
      const int d = nd;
      if (r + 1 < rb) {
        nc = at(I + 2 * n1);
        nb = col_ok ? B.b[I + n1] : 0.0;
        nd = col_ok ? B.dq[I + n1] : -1;
      }
      if (col_ok) {
        long long R = 0;
        if (d >= 0) {
          const long long Bf = to_fix(cb, k);
          if (KIND == OPK_RESID9)
            R = (long long)d * C0 + 4 * Bf - 2 * (((W0 + E0) + Cm) + Cp) - (((Wm + Em) + Wp) + Ep);
          else
            R = (long long)d * C0 + Bf - (((W0 + E0) + Cm) + Cp);
        }
        const float f = __fmul_rn(__ll2float_rn(R), fm);
        B.b32[I] = f;
        if (NEUMANN) s1 += (__int128)R;
        else B.r32[I] = f;
        // p + e = f^2 exactly; (hi, lo) += p + e by TwoSum (explicit _rn
        // operations: a contracted hi + f*f would break the error terms)
        const float p = __fmul_rn(f, f), e = __fmaf_rn(f, f, -p);
        const float sn = __fadd_rn(hi, p), bp = __fsub_rn(sn, hi);
        lo = __fadd_rn(lo, __fadd_rn(__fadd_rn(__fsub_rn(hi, __fsub_rn(sn, bp)), __fsub_rn(p, bp)), e));
        hi = sn;
      }
      Wm = W0; Cm = C0; Em = E0;
      W0 = Wp; C0 = Cp; E0 = Ep;
    }
    double a2 = ((double)hi + (double)lo) / (scale * scale);
    double a1 = NEUMANN ? ldexp(__dadd_rn(__dmul_rn((double)(long long)(s1 >> 64), 18446744073709551616.0),
                                          (double)(unsigned long long)s1),
                                -(k + q))
                        : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      a2 = __dadd_rn(a2, __shfl_down_sync(0xffffffffu, a2, o));
      a1 = __dadd_rn(a1, __shfl_down_sync(0xffffffffu, a1, o));
    }
    if (lane == 0) {
      partials[2 * task] = a2;
      partials[2 * task + 1] = a1;
    }
  }
}

// cell-centred, integer form: b32 = r32 = msk ? b32 - mean * CUR : 0
__global__ void __launch_bounds__(kBThreads) k_brhs_shift(const BInst* __restrict__ bi, const int4* __restrict__ tab,
                                                          long long nchunks, int win, const int* __restrict__ active) {
  dep_wait();
  constexpr int U = kBChunk / kBThreads;
  __shared__ int list[kBThreads];
  __shared__ int wsum[kBThreads / 32 + 1];
  for (long long base = (long long)blockIdx.x * win; base < nchunks; base += (long long)gridDim.x * win) {
    const int cnt = active_window(tab, base, nchunks, win, active, list, wsum);
    for (int q = 0; q < cnt; ++q) {
      const int4 en = tab[base + list[q]];
      const BInst& B = bi[en.x];
      const float sh = *reinterpret_cast<const float*>(B.sc + BS_SHIFT);  // (float)(mean * scale)
      const long long t0 = (long long)en.y * kBChunk + threadIdx.x;
      float f[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const long long t = t0 + (long long)u * kBThreads;
        f[u] = 0.f;
        if (t < B.len && B.m[t]) f[u] = __fsub_rn(B.b32[t], sh);
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const long long t = t0 + (long long)u * kBThreads;
        if (t < B.len) {
          B.b32[t] = f[u];
          B.r32[t] = f[u];
        }
      }
    }
    __syncthreads();
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
  dep_wait();
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
    // a NaN or Inf |b| stops the instance with a NaN residual (reported as
    // non-finite), where the ratio alone would read as converged
    if (!isfinite(normb)) res = __longlong_as_double(0x7ff8000000000000LL);
    const int nite = (int)sc[BS_NITE];
    sc[BS_RES] = res;
    sc[BS_HIST + nite] = res;
    const double nw = sc[BS_NWET] > 0 ? sc[BS_NWET] : 1.0;
    sc[BS_MEAN] = s1 / nw;
    const double used = sc[BS_NEXT];
    sc[BS_CUR] = used;
    sc[BS_ICUR] = 1.0 / used;
    *reinterpret_cast<float*>(sc + BS_SHIFT) = (float)(sc[BS_MEAN] * used);
    const double rms = sqrt(s2 / nw);
    int e = 0;
    if (rms > 0 && isfinite(rms)) frexp(rms, &e);
    sc[BS_NEXT] = ldexp(1.0, -e);
    sc[BS_MAXX] = 0.0;  // the next update collects max |x| afresh
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
__global__ void __launch_bounds__(kBThreads) k_brhs(const BInst* __restrict__ bi, const int4* __restrict__ tab,
                                                    long long nchunks, int win, const int* __restrict__ active) {
  dep_wait();
  constexpr int U = kBChunk / kBThreads;
  __shared__ int list[kBThreads];
  __shared__ int wsum[kBThreads / 32 + 1];
  for (long long base = (long long)blockIdx.x * win; base < nchunks; base += (long long)gridDim.x * win) {
    const int cnt = active_window(tab, base, nchunks, win, active, list, wsum);
    for (int q = 0; q < cnt; ++q) {
      const int4 en = tab[base + list[q]];
      const BInst& B = bi[en.x];
      const double mean = B.sc[BS_MEAN], scale = B.sc[BS_CUR];
      const long long t0 = (long long)en.y * kBChunk + threadIdx.x;
      float f[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const long long t = t0 + (long long)u * kBThreads;
        f[u] = 0.f;
        if (t < B.len && B.m[t]) f[u] = (float)((B.r[t] - mean) * scale);
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const long long t = t0 + (long long)u * kBThreads;
        if (t < B.len) {
          B.b32[t] = f[u];
          B.r32[t] = f[u];
        }
      }
    }
    __syncthreads();
  }
}

// x += e32 * ICUR over the whole array
__global__ void __launch_bounds__(kBThreads) k_bupdate(const BInst* __restrict__ bi, const int4* __restrict__ tab,
                                                       long long nchunks, int win, const int* __restrict__ active) {
  dep_wait();
  constexpr int U = kBChunk / kBThreads;
  __shared__ int list[kBThreads];
  __shared__ int wsum[kBThreads / 32 + 1];
  for (long long base = (long long)blockIdx.x * win; base < nchunks; base += (long long)gridDim.x * win) {
    const int cnt = active_window(tab, base, nchunks, win, active, list, wsum);
    for (int q = 0; q < cnt; ++q) {
      const int4 en = tab[base + list[q]];
      const BInst& B = bi[en.x];
      const double is = B.sc[BS_ICUR];
      const int pe = pow2_exponent(is);  // iscale = 2^pe
      const long long t0 = (long long)en.y * kBChunk + threadIdx.x;
      double xn[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const long long t = t0 + (long long)u * kBThreads;
        if (t < B.len) xn[u] = __dadd_rn(B.x[t], f2d_pow2(B.e32[t], pe, is));
      }
      unsigned long long mx = 0;
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const long long t = t0 + (long long)u * kBThreads;
        if (t < B.len) {
          B.x[t] = xn[u];
          const unsigned long long ub = (unsigned long long)__double_as_longlong(xn[u]) & 0x7FFFFFFFFFFFFFFFULL;
          mx = ub > mx ? ub : mx;
        }
      }
      // max |x| of the chunk into the instance's BS_MAXX (one atomic per warp)
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long ox = __shfl_down_sync(0xffffffffu, mx, o);
        mx = ox > mx ? ox : mx;
      }
      if ((threadIdx.x & 31) == 0 && mx) atomicMax((unsigned long long*)(B.sc + BS_MAXX), mx);
    }
    __syncthreads();
  }
}

template <class T>
__device__ void bsmall_run(const BSmall& s, T* X, T* Y, T* B, T* W) {
  const long long len = s.g.len;
  for (long long t = threadIdx.x; t < len; t += blockDim.x) {
    X[t] = (T)s.x32[t];
    B[t] = (T)s.b32[t];
    W[t] = ((const T*)s.w)[t];
    Y[t] = ((const T*)s.y)[t];
  }
  __syncthreads();
  const T cff = (T)s.cff;
  const long long n1 = s.g.n1;
  for (int p = 0; p < s.npairs; ++p) {
    if (s.stencil == 5) {
      for (long long t = threadIdx.x; t < s.n; t += blockDim.x) Y[s.lo + t] = v_sweep5(X, B, W, cff, n1, s.lo + t);
      __syncthreads();
      for (long long t = threadIdx.x; t < s.n; t += blockDim.x) X[s.lo + t] = v_sweep5(Y, B, W, cff, n1, s.lo + t);
      __syncthreads();
    } else {
      int i, j, k;
      const long long ne = (long long)(s.ext.i1 - s.ext.i0 + 1) * (s.ext.j1 - s.ext.j0 + 1) * (s.ext.k1 - s.ext.k0 + 1);
      for (long long t = threadIdx.x; t < ne; t += blockDim.x) {
        box3(s.ext, t, i, j, k);
        const long long I = lin(s.g, i, j, k);
        Y[I] = v_sweep9(X, B, W, cff, n1, I);
      }
      __syncthreads();
      const long long ni = (long long)(s.in.i1 - s.in.i0 + 1) * (s.in.j1 - s.in.j0 + 1) * (s.in.k1 - s.in.k0 + 1);
      for (long long t = threadIdx.x; t < ni; t += blockDim.x) {
        box3(s.in, t, i, j, k);
        const long long I = lin(s.g, i, j, k);
        X[I] = v_sweep9(Y, B, W, cff, n1, I);
      }
      __syncthreads();
    }
  }
  for (long long t = threadIdx.x; t < len; t += blockDim.x) s.x32[t] = (float)X[t];
}

__global__ void __launch_bounds__(kBThreads) k_bsmall(const BSmall* __restrict__ sm, const int* __restrict__ active) {
  dep_wait();
  extern __shared__ double dsm[];
  const BSmall& s = sm[blockIdx.x];
  if (!active[s.inst]) return;
  const long long len = s.g.len;
  if (s.prec == 0) bsmall_run<double>(s, dsm, dsm + len, dsm + 2 * len, dsm + 3 * len);
  else {
    float* f = (float*)dsm;
    bsmall_run<float>(s, f, f + len, f + 2 * len, f + 3 * len);
  }
}

// Coarse runs: block b executes run runs[b] = {instance, first entry, end
// entry, 0} of the entry list, in order, with a block barrier after each
// entry: ent = {0, Op index} runs the Op over its whole index space,
// {1, BSmall index} a small-level smoothing in shared memory. Same per-item
// code as k_bstage and k_bsmall, so the same values.
__global__ void __launch_bounds__(kBRunThreads) k_brun(const Op* __restrict__ ops, const BSmall* __restrict__ sm,
                                                       const int2* __restrict__ ent, const int4* __restrict__ runs,
                                                       const int* __restrict__ active) {
  dep_wait();
  extern __shared__ double dsm[];
  __shared__ Op op;
  const int4 rn = runs[blockIdx.x];
  if (!active[rn.x]) return;
  for (int e = rn.y; e < rn.z; ++e) {
    const int2 en = ent[e];
    if (en.x == 1) {
      const BSmall& s = sm[en.y];
      const long long len = s.g.len;
      if (s.prec == 0) {
        bsmall_run<double>(s, dsm, dsm + len, dsm + 2 * len, dsm + 3 * len);
      } else {
        float* f = (float*)dsm;
        bsmall_run<float>(s, f, f + len, f + 2 * len, f + 3 * len);
      }
    } else {
      if (threadIdx.x < sizeof(Op) / sizeof(int)) ((int*)&op)[threadIdx.x] = ((const int*)&ops[en.y])[threadIdx.x];
      __syncthreads();
      if (op.prec == 0) exec<double, 2>(op, threadIdx.x, kBRunThreads, op.n);
      else exec<float, 4>(op, threadIdx.x, kBRunThreads, op.n);
    }
    __syncthreads();  // the next entry reads this one's output (and rewrites op)
  }
}
static_assert(sizeof(Op) / sizeof(int) <= kBRunThreads, "one thread per word of an Op");

// the `while` condition: another iteration while any instance continues
__global__ void k_bcond(cudaGraphConditionalHandle hc, int* nactive) {
  dep_wait();
  const int n = *nactive;
  *nactive = 0;
  cudaGraphSetConditional(hc, n > 0 ? 1u : 0u);
}

// ------------------------------------------------------------- launchers
static int g_nsm = 0;
// resident blocks (per_sm per SM), each taking windows of `win` entries so
// that every block has work while entries are few
static long long grid_for(long long nchunks, int per_sm, int* win) {
  if (!g_nsm) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&g_nsm, cudaDevAttrMultiProcessorCount, dev);
    if (g_nsm <= 0) g_nsm = 1;
  }
  const long long g = (long long)g_nsm * per_sm;
  long long w = (nchunks + g - 1) / g;
  w = w < 1 ? 1 : (w > kBThreads ? kBThreads : w);
  *win = (int)w;
  const long long windows = (nchunks + w - 1) / w;
  return windows < g ? (windows > 0 ? windows : 1) : g;
}

void launch_bstage(const Op* ops, const int4* tab, long long nchunks, const int* active, cudaStream_t s) {
  if (nchunks <= 0) return;
  int win;
  const unsigned g = (unsigned)grid_for(nchunks, 2, &win);
  launch_dep(k_bstage, g, kBThreads, 0, s, ops, tab, nchunks, win, active);
}

void launch_binit(const BInst* bi, int ninst, int zero_x, int* active, int* nactive, cudaStream_t s) {
  launch_dep(k_binit, ninst, kBThreads, 0, s, bi, zero_x, active, nactive);
}

void launch_bres(int kind, bool neumann, const BInst* bi, const int4* tab, long long nchunks, const int* active,
                 double* partials, cudaStream_t s) {
  int win;
  const unsigned g = (unsigned)grid_for(nchunks, 6, &win);
  if (kind == OPK_RESID9) {
    if (neumann) launch_dep(k_bres<OPK_RESID9, true>, g, kBThreads, 0, s, bi, tab, nchunks, win, active, partials);
    else launch_dep(k_bres<OPK_RESID9, false>, g, kBThreads, 0, s, bi, tab, nchunks, win, active, partials);
  } else {
    if (neumann) launch_dep(k_bres<OPK_RESID5, true>, g, kBThreads, 0, s, bi, tab, nchunks, win, active, partials);
    else launch_dep(k_bres<OPK_RESID5, false>, g, kBThreads, 0, s, bi, tab, nchunks, win, active, partials);
  }
}

void launch_bfinal(const BInst* bi, const long long* cstart, int ninst, const double* partials, int* active,
                   int* nactive, cudaStream_t s) {
  launch_dep(k_bfinal, ninst, kBThreads, 0, s, bi, cstart, partials, active, nactive);
}

void launch_brhs(const BInst* bi, const int4* tab, long long nchunks, const int* active, cudaStream_t s) {
  int win;
  const unsigned g = (unsigned)grid_for(nchunks, 6, &win);
  launch_dep(k_brhs, g, kBThreads, 0, s, bi, tab, nchunks, win, active);
}

void launch_bupdate(const BInst* bi, const int4* tab, long long nchunks, const int* active, cudaStream_t s) {
  int win;
  const unsigned g = (unsigned)grid_for(nchunks, 6, &win);
  launch_dep(k_bupdate, g, kBThreads, 0, s, bi, tab, nchunks, win, active);
}

void launch_bres_int(int kind, bool neumann, const BInst* bi, const int4* ttab, long long ntasks, const int* active,
                     double* partials, cudaStream_t s) {
  int win;
  grid_for(1, 1, &win);  // device SM count
  const long long want = (ntasks + kBThreads / 32 - 1) / (kBThreads / 32);  // one warp per task
  const unsigned grid = (unsigned)std::max(1LL, std::min(want, (long long)g_nsm * 8));
  if (kind == OPK_RESID9) {
    if (neumann) launch_dep(k_bres_int<OPK_RESID9, true>, grid, kBThreads, 0, s, bi, ttab, ntasks, active, partials);
    else launch_dep(k_bres_int<OPK_RESID9, false>, grid, kBThreads, 0, s, bi, ttab, ntasks, active, partials);
  } else {
    if (neumann) launch_dep(k_bres_int<OPK_RESID5, true>, grid, kBThreads, 0, s, bi, ttab, ntasks, active, partials);
    else launch_dep(k_bres_int<OPK_RESID5, false>, grid, kBThreads, 0, s, bi, ttab, ntasks, active, partials);
  }
}

void launch_brhs_shift(const BInst* bi, const int4* tab, long long nchunks, const int* active, cudaStream_t s) {
  int win;
  const unsigned g = (unsigned)grid_for(nchunks, 6, &win);
  launch_dep(k_brhs_shift, g, kBThreads, 0, s, bi, tab, nchunks, win, active);
}

void launch_bsmall(const BSmall* sm, int n, int smem, const int* active, cudaStream_t st) {
  if (n <= 0) return;
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_bsmall, cudaFuncAttributeMaxDynamicSharedMemorySize, kBSmallBytes);
    attr = true;
  }
  launch_dep(k_bsmall, n, kBThreads, smem, st, sm, active);
}

void launch_brun(const Op* ops, const BSmall* sm, const int2* ent, const int4* runs, int nruns, int smem,
                 const int* active, cudaStream_t st) {
  if (nruns <= 0) return;
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_brun, cudaFuncAttributeMaxDynamicSharedMemorySize, kBSmallBytes);
    attr = true;
  }
  launch_dep(k_brun, nruns, kBRunThreads, smem, st, ops, sm, ent, runs, active);
}

void launch_bcond(cudaGraphConditionalHandle hc, int* nactive, cudaStream_t s) {
  launch_dep(k_bcond, 1, 1, 0, s, hc, nactive);
}

}  // namespace cfmg
