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
  dep_wait();
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
  dep_wait();
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
    ds[S_MAXX] = ds[S_MAXO];  // the next update collects max |x| from max |x| outside U
    // the wet mean in units of the right-hand side, as an FP32 value
    *reinterpret_cast<float*>(ds + S_SHIFT) = (float)(ds[S_MEAN2] * used);
  }
}

// Neumann second pass: b32 = r32 = msk ? (r - mean) * scale : 0, with
// ms[0] = S_MEAN2 and ms[1] = S_CUR (the scale of this right-hand side)
__global__ void k_rhs32_mean(const double* __restrict__ r, const uint8_t* __restrict__ m,
                             const double* __restrict__ ms, float* __restrict__ b32, float* __restrict__ r32,
                             long long n) {
  dep_wait();
  long long I = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (I >= n) return;
  const float f = m[I] ? (float)((r[I] - ms[0]) * ms[S_CUR - S_MEAN2]) : 0.f;
  b32[I] = f;
  r32[I] = f;
}

// x += e * iscale
__global__ void k_update_scaled(double* __restrict__ x, const float* __restrict__ e, const double* __restrict__ is,
                                long long n) {
  dep_wait();
  long long I = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (I < n) x[I] = __fma_rn((double)e[I], is[0], x[I]);
}

// ----------------------------------------------------------------------
// Integer form of the fused pass. The FP64 pipe of a GB300 runs at 1/64 of
// the FP32 rate, and the FP64 stencil arithmetic above keeps it busy
// (about 13 FP64 operations a cell). Here x and b are read as FP64 but
// converted with integer operations to 64-bit fixed point, v * 2^k rounded
// to an integer, with k = 58 - E for max(|x|, |b|) < 2^E (S_MAXX, S_MAXB).
// The residual Q*r = Q*(diag*x + b) - (stencil sum), with Q = 4 for the
// 9-point weights 1/2 and 1/4 and Q = 1 otherwise, is then an exact
// integer (|Q r| 2^k < 2^63), so it carries no rounding at all: its error
// is that of representing x on the 2^-k grid, below 2^-58 max|x| per cell
// (FP64 arithmetic on the same x rounds at 2^-53 |x| per operation). The
// FP64 pipe is left with two conversions and one FMA a cell: sum r^2 in
// FP64 and the FP32 right-hand side. The cell-centred sum r is kept exact
// in 128-bit integers per thread.
//
// dq[I] = Q*diag[I] (an integer in 0..127) on wet cells, -128 on dry ones.

template <int KIND>
__device__ __forceinline__ long long fix_resid(const double* __restrict__ x, const double* __restrict__ b, int dq,
                                               int k, long long n1, long long n2, long long I) {
  if (dq < 0) return 0;
  const long long X = to_fix(x[I], k), B = to_fix(b[I], k);
  if (KIND == OPK_RESID9) {
    const long long F = to_fix(x[I - 1], k) + to_fix(x[I + 1], k) + to_fix(x[I - n1], k) + to_fix(x[I + n1], k);
    const long long D = to_fix(x[I - 1 - n1], k) + to_fix(x[I + 1 - n1], k) + to_fix(x[I - 1 + n1], k) +
                        to_fix(x[I + 1 + n1], k);
    return (long long)dq * X + 4 * B - 2 * F - D;
  } else if (KIND == OPK_RESID7) {
    const long long F = to_fix(x[I - 1], k) + to_fix(x[I + 1], k) + to_fix(x[I - n1], k) + to_fix(x[I + n1], k) +
                        to_fix(x[I - n2], k) + to_fix(x[I + n2], k);
    return (long long)dq * X + B - F;
  } else {
    const long long F = to_fix(x[I - 1], k) + to_fix(x[I + 1], k) + to_fix(x[I - n1], k) + to_fix(x[I + n1], k);
    return (long long)dq * X + B - F;
  }
}

// per-block partial sums: partials[blk] = sum r^2, partials[kMxParts + blk]
// = sum r. NEUMANN: b32 = (float)(r * scale) here, the mean comes off in a
// second pass (which also writes r32); else b32 and, when r32 != nullptr,
// r32 get the right-hand side.
template <int KIND, bool NEUMANN>
__global__ void __launch_bounds__(kMxThreads) k_resid_int(const double* __restrict__ x, const double* __restrict__ b,
                                                          const int8_t* __restrict__ dq, Geom g, Box bx, long long lo,
                                                          long long n, const double* __restrict__ ds,
                                                          float* __restrict__ b32, float* __restrict__ r32,
                                                          double* __restrict__ partials) {
  dep_wait();
  constexpr int q = (KIND == OPK_RESID9) ? 2 : 0;  // Q = 2^q
  const int k = fix_exponent(ds);
  const float fm = (float)ldexp(ds[S_NEXT], -(k + q));  // power of two: R -> r * scale
  double s2 = 0.0;
  __int128 s1 = 0;
  const long long ni = bx.i1 - bx.i0 + 1, nj = bx.j1 - bx.j0 + 1;
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
    long long I;
    if (KIND == OPK_RESID5) {
      I = lo + t;
    } else {
      const int i = bx.i0 + (int)(t % ni);
      const long long qq = t / ni;
      I = lin(g, i, bx.j0 + (int)(qq % nj), bx.k0 + (int)(qq / nj));
    }
    const long long R = fix_resid<KIND>(x, b, dq[I], k, g.n1, g.n2, I);
    const double rd = __ll2double_rn(R);
    s2 = __fma_rn(rd, rd, s2);
    const float f = __fmul_rn(__ll2float_rn(R), fm);
    b32[I] = f;
    if (NEUMANN) s1 += (__int128)R;
    else if (r32) r32[I] = f;
  }
  // per-thread exact sum r -> double (hi 2^64 + lo)
  const double s1d = NEUMANN ? __dadd_rn(__dmul_rn((double)(long long)(s1 >> 64), 18446744073709551616.0),
                                         (double)(unsigned long long)s1)
                             : 0.0;
  __shared__ double sh2[kMxThreads / 32], sh1[kMxThreads / 32];
  double a2 = s2, a1 = s1d;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a2 += __shfl_down_sync(0xffffffffu, a2, o);
    a1 += __shfl_down_sync(0xffffffffu, a1, o);
  }
  if ((threadIdx.x & 31) == 0) {
    sh2[threadIdx.x >> 5] = a2;
    sh1[threadIdx.x >> 5] = a1;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double u = 0.0, v = 0.0;
    for (int w = 0; w < kMxThreads / 32; ++w) {
      u += sh2[w];
      v += sh1[w];
    }
    partials[blockIdx.x] = ldexp(u, -2 * (k + q));
    partials[kMxParts + blockIdx.x] = ldexp(v, -(k + q));
  }
}

// Strips of rows (2D, and 3D plane by plane): the same residual with every
// x converted once. A warp owns 30 consecutive linear indices of a row
// (lanes 1..30; lanes 0 and 31 hold the values on either side, which at the
// ends of a row are the wrap-around neighbours of the linear 5-point range)
// and walks down `rows` rows, keeping each converted row's centre and
// west + east sum in registers; the west and east values come from the
// adjacent lanes. Integer sums are exact, so each row's west + east sum
// serves as the start of its faces (as centre row) and of the diagonals of
// the rows above and below. The loop body covers 6 rows, so the rotation of
// the row window (period 3) and of the load queue (period 2) costs no moves;
// x is loaded two rows ahead, b and dq one row ahead of their use. The
// residual norm is summed from the FP32 right-hand-side values f = r*scale
// (exact squares via FMA, double-float accumulation per thread, FP64
// across threads), so the FP64 pipe does one conversion a cell. The grid is
// one wave of warps, each taking several equal tasks.
//
// x is the level-1 array of the handle's arena. The lanes around the index
// space read up to 31 elements before its start and after its end, into the
// device scalars before it and into y after it; those values are not used.
constexpr int kIntCols = 30;  // output columns per warp strip
static_assert(kIntCols + 1 < kResidIntReach, "a warp reaches kIntCols + 1 columns beyond its strip's first");
constexpr int kIntUnroll = 6;  // rows per loop body; rows per task is a multiple

struct StripSpace {
  long long len;   // array length
  long long row0;  // linear index of column 0 of the first row (of the first plane)
  long long n2;    // plane stride (7-point: the k +- 1 neighbours)
  int nplanes;     // planes of the index space (1 in 2D)
  int c0, ncols;   // columns of the index space: c0 .. c0+ncols-1 (0-based linear offsets in a row)
  int nrows;       // rows of the index space
  int nstrips;     // ceil(ncols / kIntCols)
  int rows;        // rows per warp task (a multiple of kIntUnroll)
  long long n1;
};

// sflag (optional): 1 for each (plane, row, strip) whose 30 columns hold a
// wet cell; a task whose rows are all dry in its strip is skipped (its b32 is
// +0 already, its residuals would add exact zeros to the sums).
template <int KIND, bool NEUMANN>
__global__ void __launch_bounds__(kMxThreads) k_resid_int2d(const double* __restrict__ x, const double* __restrict__ b,
                                                            const int8_t* __restrict__ dq, StripSpace sp,
                                                            const double* __restrict__ ds, float* __restrict__ b32,
                                                            float* __restrict__ r32, double* __restrict__ partials,
                                                            const uint8_t* __restrict__ sflag) {
  dep_wait();
  constexpr int q = (KIND == OPK_RESID9) ? 2 : 0;  // Q = 2^q
  const int k = fix_exponent(ds);
  const double scale = ds[S_NEXT];
  const float fm = (float)ldexp(scale, -(k + q));  // power of two: R -> r * scale
  const int lane = threadIdx.x & 31;
  const long long warp0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
  const int nchunks = (sp.nrows + sp.rows - 1) / sp.rows;
  const long long per_plane = (long long)sp.nstrips * nchunks;
  const long long ntasks = per_plane * sp.nplanes;
  const long long n1 = sp.n1;
  float hi = 0.f, lo = 0.f;  // double-float sum of f^2
  __int128 s1 = 0;
  for (long long task = warp0; task < ntasks; task += nwarps) {
    const int plane = (int)(task / per_plane);
    const long long pt = task - plane * per_plane;
    const int strip = (int)(pt % sp.nstrips);
    const int chunk = (int)(pt / sp.nstrips);
    // lanes 1..30 own the strip's 30 columns; lanes 0 and 31 hold the
    // columns on either side, so every x is converted by exactly one lane
    const int c = sp.c0 + strip * kIntCols + lane - 1;  // this lane's column
    const bool col_ok = lane >= 1 && lane <= kIntCols && c < sp.c0 + sp.ncols;
    const int ra = chunk * sp.rows, rb = min(ra + sp.rows, sp.nrows);
    if (sflag) {  // warp-uniform: the task's rows of this strip, a lane a row
      unsigned any = 0;
      for (int r = ra + lane; r < rb; r += 32) any |= sflag[((long long)plane * sp.nrows + r) * sp.nstrips + strip];
      if (!__any_sync(0xffffffffu, any != 0)) continue;
    }
    const long long I0 = sp.row0 + plane * sp.n2 + (long long)ra * n1 + c;  // row ra, this lane
    const double* xp = x + I0;
    // rows ra-1 and ra converted; x of rows ra+1, ra+2 and b, dq of row ra in flight
    long long Cm = to_fix(xp[-n1], k), C0 = to_fix(xp[0], k);
    long long rsm = __shfl_up_sync(0xffffffffu, Cm, 1) + __shfl_down_sync(0xffffffffu, Cm, 1);
    long long rs0 = __shfl_up_sync(0xffffffffu, C0, 1) + __shfl_down_sync(0xffffffffu, C0, 1);
    double xa = xp[n1];
    double xb = ra + 2 <= rb ? xp[2 * n1] : 0.0;
    double ba = col_ok ? b[I0] : 0.0;
    int da = col_ok ? dq[I0] : -1;
    double za = 0.0, zb = 0.0;  // 7-point: x of the planes below and above, row ra
    if (KIND == OPK_RESID7 && col_ok) {
      za = xp[-sp.n2];
      zb = xp[sp.n2];
    }
    // one row of the strip (r < rb): the rotation of the row window is the
    // last step, so in the unguarded 6-row groups it costs no register moves
    auto row_step = [&](int r) {
      const long long I = I0 + (long long)(r - ra) * n1;
      // row r+1 converted; row r+3 of x and row r+1 of b, dq requested
      const long long Cp = to_fix(xa, k);
      const long long rsp = __shfl_up_sync(0xffffffffu, Cp, 1) + __shfl_down_sync(0xffffffffu, Cp, 1);
      const double cb = ba, clo = za, chi = zb;
      const int d = da;
      xa = xb;
      if (r + 3 <= rb) xb = x[I + 3 * n1];
      if (r + 1 < rb) {
        ba = col_ok ? b[I + n1] : 0.0;
        da = col_ok ? dq[I + n1] : -1;
        if (KIND == OPK_RESID7 && col_ok) {
          za = x[I + n1 - sp.n2];
          zb = x[I + n1 + sp.n2];
        }
      }
      const long long B = to_fix(cb, k);
      long long R;
      if (KIND == OPK_RESID9)
        R = (long long)d * C0 + 4 * B - 2 * (rs0 + Cm + Cp) - (rsm + rsp);
      else if (KIND == OPK_RESID7)
        R = (long long)d * C0 + B - (rs0 + Cm + Cp + to_fix(clo, k) + to_fix(chi, k));
      else
        R = (long long)d * C0 + B - (rs0 + Cm + Cp);
      R = d >= 0 ? R : 0LL;  // dry cells and lanes outside the strip
      const float f = __fmul_rn(__ll2float_rn(R), fm);
      if (col_ok) {
        b32[I] = f;
        if (!NEUMANN && r32) r32[I] = f;
      }
      if (NEUMANN) s1 += (__int128)R;
      // p + e = f^2 exactly; (hi, lo) += p + e by TwoSum (explicit _rn
      // operations: a contracted hi + f*f would break the error terms);
      // f = 0 outside the strip adds exactly nothing
      const float p = __fmul_rn(f, f), e = __fmaf_rn(f, f, -p);
      const float sn = __fadd_rn(hi, p), bp = __fsub_rn(sn, hi);
      lo = __fadd_rn(lo, __fadd_rn(__fadd_rn(__fsub_rn(hi, __fsub_rn(sn, bp)), __fsub_rn(p, bp)), e));
      hi = sn;
      Cm = C0; rsm = rs0;
      C0 = Cp; rs0 = rsp;
    };
    int r0 = ra;
    for (; r0 + kIntUnroll <= rb; r0 += kIntUnroll) {
#pragma unroll
      for (int u = 0; u < kIntUnroll; ++u) row_step(r0 + u);
    }
    for (; r0 < rb; ++r0) row_step(r0);
  }
  // sum f^2 -> sum r^2 = sum f^2 / scale^2 (exact power of two)
  const double s2d = ((double)hi + (double)lo) / (scale * scale);
  const double s1d = NEUMANN ? ldexp(__dadd_rn(__dmul_rn((double)(long long)(s1 >> 64), 18446744073709551616.0),
                                               (double)(unsigned long long)s1),
                                     -(k + q))
                             : 0.0;
  __shared__ double sh2[kMxThreads / 32], sh1[kMxThreads / 32];
  double a2 = s2d, a1 = s1d;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a2 += __shfl_down_sync(0xffffffffu, a2, o);
    a1 += __shfl_down_sync(0xffffffffu, a1, o);
  }
  if (lane == 0) {
    sh2[threadIdx.x >> 5] = a2;
    sh1[threadIdx.x >> 5] = a1;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double u = 0.0, v = 0.0;
    for (int w = 0; w < kMxThreads / 32; ++w) {
      u += sh2[w];
      v += sh1[w];
    }
    partials[blockIdx.x] = u;
    partials[kMxParts + blockIdx.x] = v;
    // the final pass reads kMxParts partials: the blocks clear the unused ones
    for (int i = gridDim.x + blockIdx.x; i < kMxParts; i += gridDim.x) partials[i] = partials[kMxParts + i] = 0.0;
  }
}

template <int KIND, bool NEUMANN>
static int int2d_grid() {
  static int blocks = 0;  // one wave: resident blocks per SM x SMs, at most kMxParts
  if (!blocks) {
    int dev = 0, nsm = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_resid_int2d<KIND, NEUMANN>, kMxThreads, 0);
    blocks = nsm * (per > 0 ? per : 1);
    if (blocks > kMxParts || blocks <= 0) blocks = kMxParts;
  }
  return blocks;
}

// the strips of the 2D (and 3D strip-form) residual: false when the form
// does not apply
static bool strip_space(int kind, const Geom& g, const Box& bx, StripSpace& sp) {
  sp.n1 = g.n1;
  sp.n2 = g.n2;
  sp.len = g.len;
  sp.nplanes = 1;
  if (kind == OPK_RESID7) {  // interior box ic x jc x kc (rloop3d!)
    sp.row0 = (long long)(bx.j0 - 1) * g.n1 + (long long)(bx.k0 - 1) * g.n2;
    sp.c0 = bx.i0 - 1;
    sp.ncols = bx.i1 - bx.i0 + 1;
    sp.nrows = bx.j1 - bx.j0 + 1;
    sp.nplanes = bx.k1 - bx.k0 + 1;
  } else if (g.tz != 1) {
    return false;
  } else if (kind == OPK_RESID5) {  // linear range 1+n1 .. len-n1: rows 2..ty-1, every column
    sp.row0 = g.n1;
    sp.c0 = 0;
    sp.ncols = g.tx;
    sp.nrows = g.ty - 2;
  } else if (kind == OPK_RESID9) {  // interior box of the single layer
    sp.row0 = (long long)(bx.j0 - 1) * g.n1;
    sp.c0 = bx.i0 - 1;
    sp.ncols = bx.i1 - bx.i0 + 1;
    sp.nrows = bx.j1 - bx.j0 + 1;
  } else {
    return false;
  }
  if (sp.nrows <= 0 || sp.ncols <= 0 || sp.nplanes <= 0) return false;
  sp.nstrips = (sp.ncols + kIntCols - 1) / kIntCols;
  return true;
}

bool launch_resid_int2d(int kind, const double* x, const double* b, const int8_t* dq, const Geom& g, const Box& bx,
                        const double* ds, float* b32, float* r32, bool neumann, double* partials, cudaStream_t s,
                        const uint8_t* sflag) {
  StripSpace sp;
  if (!strip_space(kind, g, bx, sp)) return false;
#define CFMG_INT2(K)                                                                                        \
  if (kind == K) {                                                                                          \
    const int grid = neumann ? int2d_grid<K, true>() : int2d_grid<K, false>();                             \
    /* about 4 tasks per warp of the wave, 6 to 96 rows each */                                             \
    const long long warp_rows = (long long)sp.nstrips * sp.nrows * sp.nplanes;                              \
    long long rows = warp_rows / (4LL * grid * (kMxThreads / 32));                                          \
    rows = rows < kIntUnroll ? kIntUnroll : (rows > 96 ? 96 : rows);                                        \
    sp.rows = (int)((rows + kIntUnroll - 1) / kIntUnroll * kIntUnroll);                                     \
    if (neumann)                                                                                            \
      launch_dep(k_resid_int2d<K, true>, grid, kMxThreads, 0, s, x, b, dq, sp, ds, b32, r32, partials, sflag);      \
    else                                                                                                    \
      launch_dep(k_resid_int2d<K, false>, grid, kMxThreads, 0, s, x, b, dq, sp, ds, b32, r32, partials, sflag);     \
    return true;                                                                                            \
  }
  CFMG_INT2(OPK_RESID5)
  CFMG_INT2(OPK_RESID9)
  CFMG_INT2(OPK_RESID7)
#undef CFMG_INT2
  return false;
}

// sflag[(plane * nrows + row) * nstrips + strip] = 1 when the strip's
// columns of that row hold a wet cell
__global__ void k_make_sflag(const uint8_t* __restrict__ m, uint8_t* __restrict__ sflag, StripSpace sp) {
  const long long T = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long n = (long long)sp.nplanes * sp.nrows * sp.nstrips;
  if (T >= n) return;
  const int strip = (int)(T % sp.nstrips);
  const long long pr = T / sp.nstrips;
  const int row = (int)(pr % sp.nrows), plane = (int)(pr / sp.nrows);
  const long long base = sp.row0 + plane * sp.n2 + (long long)row * sp.n1;
  const int c0 = sp.c0 + strip * kIntCols, c1 = min(c0 + kIntCols, sp.c0 + sp.ncols);
  unsigned any = 0;
  for (int c = c0; c < c1; ++c) any |= m[base + c];
  sflag[T] = any ? 1 : 0;
}

long long resid_sflag_size(int kind, const Geom& g, const Box& bx) {
  StripSpace sp;
  if (!strip_space(kind, g, bx, sp)) return 0;
  return (long long)sp.nplanes * sp.nrows * sp.nstrips;
}

void launch_make_sflag(int kind, const uint8_t* m, uint8_t* sflag, const Geom& g, const Box& bx, cudaStream_t s) {
  StripSpace sp;
  if (!strip_space(kind, g, bx, sp)) return;
  const long long n = (long long)sp.nplanes * sp.nrows * sp.nstrips;
  k_make_sflag<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(m, sflag, sp);
}

// cell-centred second pass: b32 = r32 = msk ? b32 - mean * scale : 0 with
// ms = ds + S_MEAN2 (the FP32 shift sits in S_SHIFT, made once by k_fused_final)
__global__ void k_rhs32_shift(const uint8_t* __restrict__ m, const double* __restrict__ ms, float* __restrict__ b32,
                              float* __restrict__ r32, long long n) {
  dep_wait();
  long long I = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (I >= n) return;
  const float sh = *reinterpret_cast<const float*>(ms + (S_SHIFT - S_MEAN2));  // (float)(mean * scale)
  const float f = m[I] ? __fsub_rn(b32[I], sh) : 0.f;
  b32[I] = f;
  if (r32) r32[I] = f;  // only the F-cycle restricts level 1's r before forming it
}

// the same, 16 cells a thread in 16-byte accesses (m, b32, r32 16-byte
// aligned); the last n % 16 cells by the scalar form in the final thread
template <bool SKIP>
__global__ void __launch_bounds__(256) k_rhs32_shift16(const uint8_t* __restrict__ m, const double* __restrict__ ms,
                                                       float* __restrict__ b32, float* __restrict__ r32,
                                                       long long n) {
  dep_wait();
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long ng = n >> 4;
  if (t > ng) return;
  const float sh = *reinterpret_cast<const float*>(ms + (S_SHIFT - S_MEAN2));
  if (t == ng) {
    for (long long I = ng << 4; I < n; ++I) {
      const float f = m[I] ? __fsub_rn(b32[I], sh) : 0.f;
      b32[I] = f;
      if (r32) r32[I] = f;
    }
    return;
  }
  const uint4 mv = reinterpret_cast<const uint4*>(m)[t];
  // SKIP: 16 dry cells hold b32 = +0 already (the residual pass writes 0 there)
  if (SKIP && (mv.x | mv.y | mv.z | mv.w) == 0u) return;
  float4* bp = reinterpret_cast<float4*>(b32) + 4 * t;
  float4 v[4];
#pragma unroll
  for (int u = 0; u < 4; ++u) v[u] = bp[u];
  const unsigned mw[4] = {mv.x, mv.y, mv.z, mv.w};
#pragma unroll
  for (int u = 0; u < 4; ++u) {  // mask bytes of cells 4u .. 4u+3, little-endian
    v[u].x = (mw[u] & 0xffu) ? __fsub_rn(v[u].x, sh) : 0.f;
    v[u].y = (mw[u] & 0xff00u) ? __fsub_rn(v[u].y, sh) : 0.f;
    v[u].z = (mw[u] & 0xff0000u) ? __fsub_rn(v[u].z, sh) : 0.f;
    v[u].w = (mw[u] & 0xff000000u) ? __fsub_rn(v[u].w, sh) : 0.f;
  }
#pragma unroll
  for (int u = 0; u < 4; ++u) bp[u] = v[u];
  if (r32) {
    float4* rp = reinterpret_cast<float4*>(r32) + 4 * t;
#pragma unroll
    for (int u = 0; u < 4; ++u) rp[u] = v[u];
  }
}

// dq from diag and msk; *ok is cleared when a wet cell's Q*diag is not an
// integer in 0..127 or a mask value is not 0/1
__global__ void k_make_dq(const double* __restrict__ diag, const uint8_t* __restrict__ m, double Q, int8_t* dq,
                          long long n, int* ok) {
  dep_wait();
  long long I = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (I >= n) return;
  int8_t v = -128;
  if (m[I] == 1) {
    const double qd = diag[I] * Q;
    if (qd >= 0.0 && qd <= 127.0 && qd == floor(qd)) v = (int8_t)qd;
    else atomicAnd(ok, 0);
  } else if (m[I] != 0) {
    atomicAnd(ok, 0);
  }
  dq[I] = v;
}

// max |x| and max |b| (as the bit patterns of non-negative doubles, which
// order like the values) into ds[S_MAXX], ds[S_MAXB], and max |x| over the
// cells outside the box U = [ui0, ui1] x [uj0, uj1] of every layer (1-based;
// tx, ty the array's row and plane extents) into ds[S_MAXO]; all start at 0
__global__ void k_maxabs2(const double* __restrict__ x, const double* __restrict__ b, long long n, int tx, int ty,
                          int ui0, int ui1, int uj0, int uj1, double* ds, const uint8_t* __restrict__ m) {
  dep_wait();
  unsigned long long mx = 0, mb = 0, mo = 0;
  const long long nrows = n / tx;  // rows of all layers
  for (long long row = blockIdx.x; row < nrows; row += gridDim.x) {
    const int j = (int)(row % ty) + 1;
    const bool row_u = j >= uj0 && j <= uj1;
    const double* xr = x + row * tx;
    const double* br = b + row * tx;
    for (int i0 = threadIdx.x; i0 < tx; i0 += blockDim.x) {
      const unsigned long long ux = (unsigned long long)__double_as_longlong(xr[i0]) & 0x7FFFFFFFFFFFFFFFULL;
      const unsigned long long ub = (unsigned long long)__double_as_longlong(br[i0]) & 0x7FFFFFFFFFFFFFFFULL;
      const bool in_u = m ? m[row * tx + i0] != 0 : (row_u && i0 + 1 >= ui0 && i0 + 1 <= ui1);
      mx = ux > mx ? ux : mx;
      mb = ub > mb ? ub : mb;
      mo = (!in_u && ux > mo) ? ux : mo;
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long ox = __shfl_down_sync(0xffffffffu, mx, o), ob = __shfl_down_sync(0xffffffffu, mb, o);
    const unsigned long long oo = __shfl_down_sync(0xffffffffu, mo, o);
    mx = ox > mx ? ox : mx;
    mb = ob > mb ? ob : mb;
    mo = oo > mo ? oo : mo;
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMax((unsigned long long*)(ds + S_MAXX), mx);
    atomicMax((unsigned long long*)(ds + S_MAXB), mb);
    if (mo) atomicMax((unsigned long long*)(ds + S_MAXO), mo);
  }
}

// x += e * iscale, with max |x| of the result into ds[S_MAXX] (reset by the
// fused pass's final reduction): a grid-stride pass of 4 blocks per SM,
// one atomic per block
__global__ void __launch_bounds__(kMxThreads) k_update_scaled_max(double* __restrict__ x, const float* __restrict__ e,
                                                                  const double* __restrict__ ds, long long n,
                                                                  double* dsw) {
  dep_wait();
  const double is = ds[S_ICUR];
  const int pe = pow2_exponent(is);  // iscale = 2^pe
  unsigned long long mx = 0;
  const long long st = (long long)gridDim.x * blockDim.x;
  for (long long I0 = (long long)blockIdx.x * blockDim.x + threadIdx.x; I0 < n; I0 += 4 * st) {
    double v[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {  // loads of 4 cells in flight
      const long long I = I0 + u * st;
      if (I < n) v[u] = __dadd_rn(x[I], f2d_pow2(e[I], pe, is));
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const long long I = I0 + u * st;
      if (I < n) {
        x[I] = v[u];
        const unsigned long long ub = (unsigned long long)__double_as_longlong(v[u]) & 0x7FFFFFFFFFFFFFFFULL;
        mx = ub > mx ? ub : mx;
      }
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long ox = __shfl_down_sync(0xffffffffu, mx, o);
    mx = ox > mx ? ox : mx;
  }
  __shared__ unsigned long long sh[kMxThreads / 32];
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = mx;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < kMxThreads / 32; ++w) mx = sh[w] > mx ? sh[w] : mx;
    if (mx) atomicMax((unsigned long long*)(dsw + S_MAXX), mx);
  }
}

// the same with 16-byte accesses (x and e 16-byte aligned): 4 cells a
// group, two groups of a thread in flight; the last n % 4 cells by block 0
//
// msk (optional): a group of 4 dry cells is skipped (e = +0 there, so x stays
// as it is up to the sign of a zero); the max |x| of the dry cells, which no
// update changes, is in S_MAXO, from which S_MAXX starts.
__global__ void __launch_bounds__(kMxThreads) k_update_scaled_max4(double* __restrict__ x, const float* __restrict__ e,
                                                                   const double* __restrict__ ds, long long n,
                                                                   double* dsw, const uint8_t* __restrict__ msk) {
  dep_wait();
  const double is = ds[S_ICUR];
  const int pe = pow2_exponent(is);  // iscale = 2^pe
  unsigned long long mx = 0;
  auto upd = [&](double xo, float ev) {
    const double v = __dadd_rn(xo, f2d_pow2(ev, pe, is));
    const unsigned long long ub = (unsigned long long)__double_as_longlong(v) & 0x7FFFFFFFFFFFFFFFULL;
    mx = ub > mx ? ub : mx;
    return v;
  };
  const long long ng = n >> 2;
  const long long st = (long long)gridDim.x * blockDim.x;
  const float4* e4 = reinterpret_cast<const float4*>(e);
  double2* x2 = reinterpret_cast<double2*>(x);
  for (long long g0 = (long long)blockIdx.x * blockDim.x + threadIdx.x; g0 < ng; g0 += 2 * st) {
    float4 ev[2];
    double2 xa[2], xb[2];
    bool act[2];
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      const long long g = g0 + u * st;
      act[u] = g < ng;
      if (act[u] && msk) {
        const uchar4 mm = reinterpret_cast<const uchar4*>(msk)[g];
        act[u] = (mm.x | mm.y | mm.z | mm.w) != 0;
      }
    }
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      const long long g = g0 + u * st;
      if (act[u]) {
        ev[u] = e4[g];
        xa[u] = x2[2 * g];
        xb[u] = x2[2 * g + 1];
      }
    }
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      const long long g = g0 + u * st;
      if (act[u]) {
        double2 ra, rb;
        ra.x = upd(xa[u].x, ev[u].x);
        ra.y = upd(xa[u].y, ev[u].y);
        rb.x = upd(xb[u].x, ev[u].z);
        rb.y = upd(xb[u].y, ev[u].w);
        x2[2 * g] = ra;
        x2[2 * g + 1] = rb;
      }
    }
  }
  if (blockIdx.x == 0 && threadIdx.x < (n & 3)) {
    const long long I = (ng << 2) + threadIdx.x;
    x[I] = upd(x[I], e[I]);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long ox = __shfl_down_sync(0xffffffffu, mx, o);
    mx = ox > mx ? ox : mx;
  }
  __shared__ unsigned long long sh[kMxThreads / 32];
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = mx;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < kMxThreads / 32; ++w) mx = sh[w] > mx ? sh[w] : mx;
    if (mx) atomicMax((unsigned long long*)(dsw + S_MAXX), mx);
  }
}

void launch_resid_int(int kind, const double* x, const double* b, const int8_t* dq, const Geom& g, const Box& bx,
                      long long lo, long long n, const double* ds, float* b32, float* r32, bool neumann,
                      double* partials, cudaStream_t s) {
#define CFMG_INT(K)                                                                                        \
  if (kind == K) {                                                                                         \
    if (neumann)                                                                                           \
      launch_dep(k_resid_int<K, true>, kMxParts, kMxThreads, 0, s, x, b, dq, g, bx, lo, n, ds, b32, r32, partials); \
    else                                                                                                   \
      launch_dep(k_resid_int<K, false>, kMxParts, kMxThreads, 0, s, x, b, dq, g, bx, lo, n, ds, b32, r32, partials); \
    return;                                                                                                \
  }
  CFMG_INT(OPK_RESID5)
  CFMG_INT(OPK_RESID9)
  CFMG_INT(OPK_RESID7)
#undef CFMG_INT
}

void launch_rhs32_shift(const uint8_t* m, const double* mean_scale, float* b32, float* r32, long long n,
                        cudaStream_t s, bool skip_dry) {
  const bool a16 = ((uintptr_t)m | (uintptr_t)b32 | (uintptr_t)r32) % 16 == 0;
  if (a16) {
    const long long nt = (n >> 4) + 1;  // groups of 16, and one thread for the rest
    if (skip_dry && !r32)
      launch_dep(k_rhs32_shift16<true>, (unsigned)((nt + 255) / 256), 256, 0, s, m, mean_scale, b32, r32, n);
    else
      launch_dep(k_rhs32_shift16<false>, (unsigned)((nt + 255) / 256), 256, 0, s, m, mean_scale, b32, r32, n);
  } else {
    launch_dep(k_rhs32_shift, (unsigned)((n + 255) / 256), 256, 0, s, m, mean_scale, b32, r32, n);
  }
}

void launch_make_dq(const double* diag, const uint8_t* m, double Q, int8_t* dq, long long n, int* ok,
                    cudaStream_t s) {
  launch_dep(k_make_dq, (unsigned)((n + 255) / 256), 256, 0, s, diag, m, Q, dq, n, ok);
}

void launch_maxabs2(const double* x, const double* b, long long n, int tx, int ty, int ui0, int ui1, int uj0, int uj1,
                    double* ds, cudaStream_t s, const uint8_t* m) {
  launch_dep(k_maxabs2, 1024, 256, 0, s, x, b, n, tx, ty, ui0, ui1, uj0, uj1, ds, m);
}

void launch_update_scaled_max(double* x, const float* e, double* ds, long long n, cudaStream_t s,
                              const uint8_t* msk) {
  static int nsm = 0;
  if (!nsm) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  }
  if (((uintptr_t)x | (uintptr_t)e) % 16 == 0 && (uintptr_t)msk % 4 == 0)
    launch_dep(k_update_scaled_max4, nsm * 4, kMxThreads, 0, s, x, e, ds, n, ds, msk);
  else
    launch_dep(k_update_scaled_max, nsm * 4, kMxThreads, 0, s, x, e, ds, n, ds);  // 4 blocks per SM: measured 4 % faster than 8
}

void launch_resid_fused(int kind, double* r, const double* x, const double* b, const double* d, const uint8_t* m,
                        const Geom& g, const Box& bx, long long lo, long long n, const double* scale, float* b32,
                        float* r32, bool neumann, double* partials, cudaStream_t s) {
#define CFMG_FUSED(K)                                                                                            \
  if (kind == K) {                                                                                               \
    if (neumann)                                                                                                 \
      launch_dep(k_resid_fused<K, true>, kMxParts, kMxThreads, 0, s, r, x, b, d, m, g, bx, lo, n, scale, b32, r32, partials); \
    else                                                                                                         \
      launch_dep(k_resid_fused<K, false>, kMxParts, kMxThreads, 0, s, r, x, b, d, m, g, bx, lo, n, scale, b32, r32, partials); \
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
  launch_dep(k_fused_final, 1, kMxParts, 0, s, partials, ds, normb, nwet, norm_kind);
}

void launch_rhs32_mean(const double* r, const uint8_t* m, const double* mean_scale, float* b32, float* r32,
                       long long n, cudaStream_t s) {
  launch_dep(k_rhs32_mean, (unsigned)((n + 255) / 256), 256, 0, s, r, m, mean_scale, b32, r32, n);
}

void launch_update_scaled(double* x, const float* e, const double* iscale, long long n, cudaStream_t s) {
  launch_dep(k_update_scaled, (unsigned)((n + 255) / 256), 256, 0, s, x, e, iscale, n);
}

}  // namespace cfmg
