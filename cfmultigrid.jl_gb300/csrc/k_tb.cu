// Temporally blocked FP32 Jacobi smoother for the mixed-precision cycles
// (2D 5-point and 9-point operators, closed topology).
//
// One smoothing call of the reference (nite pairs of sweeps,
// src/laplacian.jl:95-112, src/laplacian9.jl:2-47) reads and writes the
// whole level 2*nite times. Here a CTA loads a tile of x, b and
// omega*idiag once, runs all 2*nite sweeps on it in shared memory, each
// sweep valid on a region one cell narrower than the last, and writes the
// tile's core (a halo of H = 2*nite cells trimmed) to the level's other x
// buffer: the tiles overlap, so the update cannot be in place. HBM traffic
// drops from 16 B per cell and sweep to about 21 B per cell for the whole
// call. Three forms: the lean packed form (k_smooth_tb5, 128 x 48 tiles,
// the default, with an optional residual/restriction epilogue), the first
// packed form (k_smooth_tb3, 128 x 64) and the scalar form (k_smooth_tb,
// 128 x 72, also the batched solver's tile).
//
// Correctness rests on the mixed form's invariant: in the FP32 correction
// fields every cell outside the wet interior holds 0 and has
// omega*idiag = 0, so a sweep leaves it at 0. Updating every cell of the
// box U = [nh, nx+nh+1] x [nh, ny+nh+1] with the same formula is then
// bit-identical to the reference's per-sweep ranges (and to the
// single-sweep FP32 kernels), while cells outside U stay 0 in both
// buffers. The per-cell arithmetic is the same Ar<float> sequence.
#include "ops_dev.cuh"

namespace cfmg {

constexpr int kTbW = 128;      // tile width (threads.x)
constexpr int kTbTy = 8;       // threads.y
constexpr int kTbRows = 9;     // rows per thread
constexpr int kTbH = kTbTy * kTbRows;  // tile height 72

template <int ST>
__device__ __forceinline__ float tb_update(float c, float wv, float bv, float cff, float n, float s, float e,
                                           float wst, float ne, float nw, float se, float sw) {
  typedef Ar<float> A;
  if (ST == 5) {
    // sloop2d!: ((xW + xE) + xS) + xN with S = j-1, N = j+1
    const float s4 = A::add(A::add(A::add(wst, e), s), n);
    return A::sub(A::mul(cff, c), A::mul(wv, A::sub(bv, s4)));
  } else {
    // in-plane laplacian9: b - faces/2 - diagonals/4, diagonals in the
    // order (i-1,j-1), (i+1,j-1), (i-1,j+1), (i+1,j+1)
    const float f = A::add(A::add(A::add(wst, e), s), n);
    const float d = A::add(A::add(A::add(sw, se), nw), ne);
    float t = A::fmx(f, -0.5f, bv);
    t = A::fmx(d, -0.25f, t);
    return A::sub(A::mul(cff, c), A::mul(wv, t));
  }
}

// One tile: x is the current x, xo the other buffer (receives the
// smoothed field). U (1-based, inclusive) is the update box; (bx, by) the
// tile, bz the k-layer. smem holds 4 kTbH x kTbW floats.
template <int ST, int NITE>
__device__ __forceinline__ void tb_tile(const float* __restrict__ x, float* __restrict__ xo,
                                        const float* __restrict__ b, const float* __restrict__ w, float cff, int tx,
                                        int ty, int ui0, int ui1, int uj0, int uj1, int bx, int by, int bz,
                                        float* smem) {
  constexpr int H = 2 * NITE;
  constexpr int CW = kTbW - 2 * H, CH = kTbH - 2 * H;
  float* X = smem;               // [kTbH][kTbW]
  float* Y = smem + kTbH * kTbW;
  float* B = smem + 2 * kTbH * kTbW;
  float* W = smem + 3 * kTbH * kTbW;

  const int li = threadIdx.x;
  const int r0 = threadIdx.y * kTbRows;
  const int gi = ui0 + bx * CW - H + li;  // 1-based global column
  const int gj0 = uj0 + by * CH - H + r0;  // first global row of this thread
  const long long plane = (long long)tx * ty * bz;

  unsigned inU = 0;  // bit r: cell (gi, gj0+r) lies in U
  const bool col_in = gi >= 1 && gi <= tx;
  const bool col_u = gi >= ui0 && gi <= ui1;
#pragma unroll
  for (int r = 0; r < kTbRows; ++r) {
    const int gj = gj0 + r;
    const bool in = col_in && gj >= 1 && gj <= ty;
    const long long I = plane + (long long)(gi - 1) + (long long)tx * (gj - 1);
    X[(r0 + r) * kTbW + li] = in ? x[I] : 0.f;
    B[(r0 + r) * kTbW + li] = in ? b[I] : 0.f;
    W[(r0 + r) * kTbW + li] = in ? w[I] : 0.f;
    if (col_u && gj >= uj0 && gj <= uj1) inU |= 1u << r;
  }
  __syncthreads();

  // Warp-uniform fast path: threadIdx.y is constant across a warp, so a
  // warp whose rows are all valid for a sweep, in a tile whose loaded
  // region lies inside U, skips the per-row margin and per-cell U tests.
  const int ti0 = ui0 + bx * CW - H, tj0 = uj0 + by * CH - H;  // tile origin
  const bool tile_in_u = ti0 >= ui0 && ti0 + kTbW - 1 <= ui1 && tj0 >= uj0 && tj0 + kTbH - 1 <= uj1;
#pragma unroll 1
  for (int s = 0; s < 2 * NITE; ++s) {
    const float* src = (s & 1) ? Y : X;
    float* dst = (s & 1) ? X : Y;
    const int m = s + 1;  // valid margin after this sweep
    const bool col_ok = li >= m && li < kTbW - m;
    if (col_ok) {
      // sliding 3x3 window down the thread's column segment
      float wm, cm, em;  // row j-1 (west, centre, east)
      float w0, c0, e0;  // row j
      {
        const int rr = (r0 - 1 < 0) ? 0 : r0 - 1;
        wm = src[rr * kTbW + li - 1];
        cm = src[rr * kTbW + li];
        em = src[rr * kTbW + li + 1];
      }
      w0 = src[r0 * kTbW + li - 1];
      c0 = src[r0 * kTbW + li];
      e0 = src[r0 * kTbW + li + 1];
      if (tile_in_u && r0 >= m && r0 + kTbRows <= kTbH - m) {
#pragma unroll
        for (int r = 0; r < kTbRows; ++r) {
          const int lj = r0 + r;
          const float wp = src[(lj + 1) * kTbW + li - 1];
          const float cp = src[(lj + 1) * kTbW + li];
          const float ep = src[(lj + 1) * kTbW + li + 1];
          dst[lj * kTbW + li] = tb_update<ST>(c0, W[lj * kTbW + li], B[lj * kTbW + li], cff, cp, cm, e0, w0, ep, wp,
                                              em, wm);
          wm = w0; cm = c0; em = e0;
          w0 = wp; c0 = cp; e0 = ep;
        }
      } else {
#pragma unroll
        for (int r = 0; r < kTbRows; ++r) {
          const int lj = r0 + r;
          const int rn = (lj + 1 < kTbH) ? lj + 1 : lj;
          const float wp = src[rn * kTbW + li - 1];
          const float cp = src[rn * kTbW + li];
          const float ep = src[rn * kTbW + li + 1];
          if (lj >= m && lj < kTbH - m) {
            dst[lj * kTbW + li] = (inU >> r & 1u)
                                      ? tb_update<ST>(c0, W[lj * kTbW + li], B[lj * kTbW + li], cff, cp, cm, e0, w0,
                                                      ep, wp, em, wm)
                                      : c0;
          }
          wm = w0; cm = c0; em = e0;
          w0 = wp; c0 = cp; e0 = ep;
        }
      }
    }
    __syncthreads();
  }
  // 2*NITE sweeps: the result is in X; write the core cells of U
  if (li >= H && li < kTbW - H) {
#pragma unroll
    for (int r = 0; r < kTbRows; ++r) {
      const int lj = r0 + r;
      if (lj >= H && lj < kTbH - H && (inU >> r & 1u)) {
        const long long I = plane + (long long)(gi - 1) + (long long)tx * (gj0 + r - 1);
        xo[I] = X[lj * kTbW + li];
      }
    }
  }
}

// ---------------------------------------------------------------------
// Packed form: the same passes with two columns per thread and the FP32x2
// instructions of sm_100+ (add/mul/fma.rn.f32x2 round each lane exactly as
// the scalar _rn operations do, so the result is the same bit for bit). A 128 x 64 tile lives in shared memory as two planes per
// row, even columns then odd columns, so that every shared load of a warp
// reads 32 consecutive words. b and -omega*idiag of the thread's own 4 x 2
// cells stay in registers. Every sweep computes the whole tile (cells near
// the tile edge read clamped neighbours and hold values that no later sweep
// of the valid region reads); cells outside U keep their value.
// Packed operations with an explicit rounding modifier. A packed product
// feeding a packed sum is still contracted into one FMA by ptxas, so the
// one place where a product is summed (cff*c - w*t) adds in scalar.
union F2U {
  float2 f;
  unsigned long long u;
};
__device__ __forceinline__ float2 p_add(float2 a, float2 b) {
  F2U x, y, r;
  x.f = a;
  y.f = b;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r.u) : "l"(x.u), "l"(y.u));
  return r.f;
}
__device__ __forceinline__ float2 p_mul(float2 a, float2 b) {
  F2U x, y, r;
  x.f = a;
  y.f = b;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r.u) : "l"(x.u), "l"(y.u));
  return r.f;
}
__device__ __forceinline__ float2 p_fma(float2 a, float2 b, float2 c) {
  F2U x, y, z, r;
  x.f = a;
  y.f = b;
  z.f = c;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r.u) : "l"(x.u), "l"(y.u), "l"(z.u));
  return r.f;
}

constexpr int kT3W = 128, kT3H = 64;  // tile
constexpr int kT3Tx = 64, kT3Ty = 16, kT3Rows = 4;
constexpr int kT3Half = kT3W / 2;

template <int ST, int NITE>
__device__ __forceinline__ void tb3_tile(const float* __restrict__ x, float* __restrict__ xo,
                                         const float* __restrict__ b, const float* __restrict__ w, float cff, int tx,
                                         int ty, int ui0, int ui1, int uj0, int uj1, int bx, int by, int bz,
                                         float* smem) {
  constexpr int H = 2 * NITE;
  constexpr int CW = kT3W - 2 * H, CH = kT3H - 2 * H;
  float* P0 = smem;              // [kT3H][even | odd]
  float* P1 = smem + kT3H * kT3W;
  const int lx = threadIdx.x;
  const int r0 = threadIdx.y * kT3Rows;
  const int gi0 = ui0 + bx * CW - H + 2 * lx;  // 1-based global column of the even cell
  const int gj0 = uj0 + by * CH - H + r0;
  const long long plane = (long long)tx * ty * bz;
  float2 B[kT3Rows], NW[kT3Rows];
  unsigned inU = 0;  // bit 2r + e
#pragma unroll
  for (int r = 0; r < kT3Rows; ++r) {
    const int gj = gj0 + r;
    float v[2], bb[2], ww[2];
#pragma unroll
    for (int e = 0; e < 2; ++e) {
      const int gi = gi0 + e;
      const bool in = gi >= 1 && gi <= tx && gj >= 1 && gj <= ty;
      const long long I = plane + (long long)(gi - 1) + (long long)tx * (gj - 1);
      v[e] = in ? x[I] : 0.f;
      bb[e] = in ? b[I] : 0.f;
      ww[e] = in ? w[I] : 0.f;
      if (gi >= ui0 && gi <= ui1 && gj >= uj0 && gj <= uj1) inU |= 1u << (2 * r + e);
    }
    P0[(r0 + r) * kT3W + lx] = v[0];
    P0[(r0 + r) * kT3W + kT3Half + lx] = v[1];
    B[r] = make_float2(bb[0], bb[1]);
    NW[r] = make_float2(-ww[0], -ww[1]);
  }
  __syncthreads();
  const int ti0 = ui0 + bx * CW - H, tj0 = uj0 + by * CH - H;  // tile origin
  const bool tile_in_u = ti0 >= ui0 && ti0 + kT3W - 1 <= ui1 && tj0 >= uj0 && tj0 + kT3H - 1 <= uj1;
  const float2 cff2 = make_float2(cff, cff);
  const int lw = lx > 0 ? lx - 1 : 0, le = lx < kT3Half - 1 ? lx + 1 : kT3Half - 1;
#pragma unroll 1
  for (int s = 0; s < 2 * NITE; ++s) {
    const float* src = (s & 1) ? P1 : P0;
    float* dst = (s & 1) ? P0 : P1;
    // (west, even, odd, east) of a row; rows outside the tile are clamped
    auto ld = [&](int rr, float& wv, float& av, float& bv, float& ev) {
      rr = rr < 0 ? 0 : (rr >= kT3H ? kT3H - 1 : rr);
      const float* row = src + rr * kT3W;
      av = row[lx];
      bv = row[kT3Half + lx];
      wv = row[kT3Half + lw];
      ev = row[le];
    };
    float wm, am, bm, em, w0, a0, b0, e0;
    ld(r0 - 1, wm, am, bm, em);
    ld(r0, w0, a0, b0, e0);
#pragma unroll
    for (int r = 0; r < kT3Rows; ++r) {
      float wp, ap, bp, ep;
      ld(r0 + r + 1, wp, ap, bp, ep);
      // faces ((W + E) + S) + N, S = row j-1
      float2 f = p_add(make_float2(w0, a0), make_float2(b0, e0));
      f = p_add(f, make_float2(am, bm));
      f = p_add(f, make_float2(ap, bp));
      float2 t;
      if (ST == 5) {
        t = p_add(B[r], make_float2(-f.x, -f.y));  // b - s4
      } else {
        // diagonals in the order (i-1,j-1), (i+1,j-1), (i-1,j+1), (i+1,j+1)
        float2 d = p_add(make_float2(wm, am), make_float2(bm, em));
        d = p_add(d, make_float2(wp, ap));
        d = p_add(d, make_float2(bp, ep));
        t = p_fma(f, make_float2(-0.5f, -0.5f), B[r]);
        t = p_fma(d, make_float2(-0.25f, -0.25f), t);
      }
      // cff*c - w*t: the two products packed, their sum in scalar adds
      // (ptxas fuses a packed mul and a packed add into one FMA even with
      // an explicit rounding modifier; a GPU probe showed 1-4 ulp changes)
      const float2 m1 = p_mul(cff2, make_float2(a0, b0)), m2 = p_mul(NW[r], t);
      float2 o = make_float2(__fadd_rn(m1.x, m2.x), __fadd_rn(m1.y, m2.y));
      if (!tile_in_u) {
        if (!(inU >> (2 * r) & 1u)) o.x = a0;
        if (!(inU >> (2 * r + 1) & 1u)) o.y = b0;
      }
      dst[(r0 + r) * kT3W + lx] = o.x;
      dst[(r0 + r) * kT3W + kT3Half + lx] = o.y;
      wm = w0; am = a0; bm = b0; em = e0;
      w0 = wp; a0 = ap; b0 = bp; e0 = ep;
    }
    __syncthreads();
  }
  // 2*NITE sweeps: the result is in P0; write the core cells of U
#pragma unroll
  for (int r = 0; r < kT3Rows; ++r) {
    const int lj = r0 + r;
    if (lj < H || lj >= kT3H - H) continue;
#pragma unroll
    for (int e = 0; e < 2; ++e) {
      const int lc = 2 * lx + e;
      if (lc >= H && lc < kT3W - H && (inU >> (2 * r + e) & 1u)) {
        const long long I = plane + (long long)(gi0 + e - 1) + (long long)tx * (gj0 + r - 1);
        xo[I] = P0[lj * kT3W + e * kT3Half + lx];
      }
    }
  }
}

template <int ST, int NITE>
__global__ void __launch_bounds__(kT3Tx * kT3Ty, 1) k_smooth_tb3(const float* __restrict__ x, float* __restrict__ xo,
                                                                 const float* __restrict__ b,
                                                                 const float* __restrict__ w, float cff, int tx,
                                                                 int ty, int ui0, int ui1, int uj0, int uj1) {
  dep_wait();
  extern __shared__ float smem[];
  tb3_tile<ST, NITE>(x, xo, b, w, cff, tx, ty, ui0, ui1, uj0, uj1, (int)blockIdx.x, (int)blockIdx.y,
                     (int)blockIdx.z, smem);
}

// ---------------------------------------------------------------------
// Lean packed form: the tb3 layout (even and odd planes per row) with pad
// rows and pad columns, so that every shared load of a row is one base
// register plus an immediate and no index is clamped; several rows per
// thread; the sum (west + east) of each row formed once, where it starts
// the faces of the row as centre, ((W + E) + S) + N, and the diagonals of
// the row as south neighbour, ((SW + SE) + NW) + NE; and b - s4 formed as
// fma(s4, -1, b), whose product is exact. Tiles whose loaded region lies
// inside U with 8-byte aligned pairs (all but the boundary tiles) load and
// store through row pointers with 64-bit accesses and no per-cell tests.
constexpr int kT5W = 128, kT5Tx = 64;
constexpr int kT5Half = 66;              // one plane of a row: pad, 64 cells, pad
constexpr int kT5Row = 2 * kT5Half;      // even plane then odd plane
// one buffer of a TY x ROWS tile: pad row, TY*ROWS rows, pad row
template <int TY, int ROWS>
__host__ __device__ constexpr int t5_plane() { return (TY * ROWS + 2) * kT5Row; }

template <int ST, int ROWS, bool ALL_U>
__device__ __forceinline__ void tb5_sweep(const float* __restrict__ src, float* __restrict__ dst,
                                          const float2 (&B)[ROWS], const float2 (&WT)[ROWS], float2 cff2,
                                          unsigned inU) {
  // src, dst: padded row r0 (tile row r0 - 1) at this thread's column k;
  // even cell 2k at +1, odd cell 2k+1 at +kT5Half+1, the west neighbour of
  // the even cell (odd 2k-1) at +kT5Half, the east neighbour of the odd
  // cell (even 2k+2) at +2
  float wv = src[kT5Half], av = src[1], bv = src[kT5Half + 1], ev = src[2];
  float2 sm = p_add(make_float2(wv, av), make_float2(bv, ev)), Cm = make_float2(av, bv);
  src += kT5Row;
  wv = src[kT5Half]; av = src[1]; bv = src[kT5Half + 1]; ev = src[2];
  float2 s0 = p_add(make_float2(wv, av), make_float2(bv, ev)), C0 = make_float2(av, bv);
#pragma unroll
  for (int r = 0; r < ROWS; ++r) {
    src += kT5Row;
    wv = src[kT5Half]; av = src[1]; bv = src[kT5Half + 1]; ev = src[2];
    const float2 Cp = make_float2(av, bv), NWp = make_float2(wv, av), NEp = make_float2(bv, ev);
    // faces ((W + E) + S) + N, S = row j-1
    float2 f = p_add(s0, Cm);
    f = p_add(f, Cp);
    float2 t;
    if (ST == 5) {
      t = p_fma(f, make_float2(-1.f, -1.f), B[r]);  // b - s4
    } else {
      // diagonals in the order (i-1,j-1), (i+1,j-1), (i-1,j+1), (i+1,j+1)
      float2 d = p_add(sm, NWp);
      d = p_add(d, NEp);
      t = p_fma(f, make_float2(-0.5f, -0.5f), B[r]);
      t = p_fma(d, make_float2(-0.25f, -0.25f), t);
    }
    // cff*c - w*t: the two products packed, their difference in scalar
    const float2 m1 = p_mul(cff2, C0), m2 = p_mul(WT[r], t);
    float2 o = make_float2(__fsub_rn(m1.x, m2.x), __fsub_rn(m1.y, m2.y));
    if (!ALL_U) {
      if (!(inU >> (2 * r) & 1u)) o.x = C0.x;
      if (!(inU >> (2 * r + 1) & 1u)) o.y = C0.y;
    }
    dst += kT5Row;
    dst[1] = o.x;
    dst[kT5Half + 1] = o.y;
    sm = s0; Cm = C0;
    s0 = p_add(NWp, NEp);
    C0 = Cp;
  }
}

// Residual of the smoothed tile for the thread's cells (epilogue of a
// pre-smoothing pass): r = msk * ((d*x + b) - s4) for the 5-point operator,
// msk * fma(diags, -1/4, fma(s4, -1/2, d*x + b)) for the 9-point one, the
// arithmetic of the reference's residual kernels; 0 outside the residual box.
template <int ST, int ROWS>
__device__ __forceinline__ void tb5_resid(const float* __restrict__ src, float* __restrict__ dst,
                                          const float2 (&B)[ROWS], const float2* __restrict__ Ds,
                                          const ushort* __restrict__ Ms, unsigned inbox) {
  float wv = src[kT5Half], av = src[1], bv = src[kT5Half + 1], ev = src[2];
  float2 sm = p_add(make_float2(wv, av), make_float2(bv, ev)), Cm = make_float2(av, bv);
  src += kT5Row;
  wv = src[kT5Half]; av = src[1]; bv = src[kT5Half + 1]; ev = src[2];
  float2 s0 = p_add(make_float2(wv, av), make_float2(bv, ev)), C0 = make_float2(av, bv);
#pragma unroll
  for (int r = 0; r < ROWS; ++r) {
    src += kT5Row;
    wv = src[kT5Half]; av = src[1]; bv = src[kT5Half + 1]; ev = src[2];
    const float2 Cp = make_float2(av, bv), NWp = make_float2(wv, av), NEp = make_float2(bv, ev);
    float2 f = p_add(s0, Cm);
    f = p_add(f, Cp);
    const float2 dr = Ds[r * kT5Tx];
    float2 v = make_float2(__fadd_rn(__fmul_rn(dr.x, C0.x), B[r].x), __fadd_rn(__fmul_rn(dr.y, C0.y), B[r].y));
    if (ST == 5) {
      v = make_float2(__fsub_rn(v.x, f.x), __fsub_rn(v.y, f.y));
    } else {
      float2 dg = p_add(sm, NWp);
      dg = p_add(dg, NEp);
      v = p_fma(f, make_float2(-0.5f, -0.5f), v);
      v = p_fma(dg, make_float2(-0.25f, -0.25f), v);
    }
    const unsigned mr = Ms[r * kT5Tx];
    const uint8_t m0 = (uint8_t)(mr & 0xffu), m1 = (uint8_t)(mr >> 8);
    float rx = mask_mul(m0, v.x), ry = mask_mul(m1, v.y);
    rx = (inbox >> (2 * r) & 1u) ? rx : 0.f;
    ry = (inbox >> (2 * r + 1) & 1u) ? ry : 0.f;
    dst += kT5Row;
    dst[1] = rx;
    dst[kT5Half + 1] = ry;
    sm = s0; Cm = C0;
    s0 = p_add(NWp, NEp);
    C0 = Cp;
  }
}

// PER (x-periodic topology, 5-point): the tiles cover the interior columns
// [ui0, ui1] = [nh+1, nx+nh], and a tile column outside them reads its
// periodic image, so the sweeps see the periodic domain. With nh >= 2 that
// is what the reference's interior gets from its linear-range sweeps with a
// fill! after each pair; the caller fills the halo columns after the pass.
//
// UPD (the last post-smoothing pass of a mixed-precision cycle on level 1):
// the smoothed FP32 correction e is not stored; the pass applies the FP64
// solution update x += e * iscale to the core cells of U instead, with the
// arithmetic of k_update_scaled_max, and collects max |x| of the results
// into ds[S_MAXX]. Outside U e is +0, so those cells keep their value.
//
// One tile (bx, by) of layer bz per call: the standalone kernel takes its
// block index, the batched one the tiles of its work table.
template <int ST, int NITE, int TY, int ROWS, bool EPI, bool PER, bool UPD>
__device__ __forceinline__ void tb5_tile(const float* __restrict__ x, float* __restrict__ xo,
                                         const float* __restrict__ b, const float* __restrict__ w, float cff, int tx,
                                         int ty, int ui0, int ui1, int uj0, int uj1, TbEpi ep, int bx, int by,
                                         int bz, float* smem) {
  // with the epilogue the core is 2 cells narrower: r is needed one cell
  // beyond it, and x one cell beyond that
  constexpr int H = 2 * NITE + (EPI ? 2 : 0), TH = TY * ROWS;
  constexpr int CW = kT5W - 2 * H, CH = TH - 2 * H;
  float* P0 = smem;
  float* P1 = smem + t5_plane<TY, ROWS>();
  // epilogue only: diag and mask of the tile, one float2 / two bytes per thread and row
  float2* Dsm = reinterpret_cast<float2*>(smem + 2 * t5_plane<TY, ROWS>());
  ushort* Msm = reinterpret_cast<ushort*>(Dsm + TH * kT5Tx);
  const int lx = threadIdx.x;
  const int r0 = threadIdx.y * ROWS;  // first tile row of this thread
  const int ti0 = ui0 + bx * CW - H, tj0 = uj0 + by * CH - H;  // tile origin (1-based)
  const int gi0 = ti0 + 2 * lx;  // global column of the even cell
  // linear index of the thread's even cell in its first row (may lie
  // outside the array for boundary tiles: used only under the bounds tests)
  const long long I0 = (long long)tx * ty * bz + (long long)(gi0 - 1) + (long long)tx * (tj0 + r0 - 1);
  const bool cols_in = ti0 >= ui0 && ti0 + kT5W - 1 <= ui1, rows_in = tj0 >= uj0 && tj0 + TH - 1 <= uj1;
  const bool tile_in_u = rows_in && (PER || cols_in);  // periodic: every column is updated
  // the parity of I0 is the same for every thread of the tile
  const bool fast = rows_in && cols_in && ((I0 | tx) & 1) == 0;
  float2 B[ROWS], WT[ROWS];
  unsigned inU = ~0u;  // bit 2r + e: cell in U
  float* prow = P0 + (r0 + 1) * kT5Row + lx;  // padded row r0 + 1 = tile row r0
  if (fast) {
    const float2* xp = reinterpret_cast<const float2*>(x + I0);
    const float2* bp = reinterpret_cast<const float2*>(b + I0);
    const float2* wp = reinterpret_cast<const float2*>(w + I0);
    const int st = tx >> 1;
#pragma unroll
    for (int r = 0; r < ROWS; ++r) {
      const float2 v = __ldg(xp + r * st);
      B[r] = __ldg(bp + r * st);
      WT[r] = __ldg(wp + r * st);
      prow[r * kT5Row + 1] = v.x;
      prow[r * kT5Row + kT5Half + 1] = v.y;
      if constexpr (EPI) {
        Dsm[(r0 + r) * kT5Tx + lx] = __ldg(reinterpret_cast<const float2*>(ep.d + I0) + r * st);
        Msm[(r0 + r) * kT5Tx + lx] = __ldg(reinterpret_cast<const ushort*>(ep.m + I0) + r * st);
      }
    }
  } else {
    inU = 0;
#pragma unroll
    for (int r = 0; r < ROWS; ++r) {
      const int gj = tj0 + r0 + r;
      const bool row_in = gj >= 1 && gj <= ty, row_u = gj >= uj0 && gj <= uj1;
      float v[2], bb[2], ww[2];
#pragma unroll
      for (int e = 0; e < 2; ++e) {
        int gi = gi0 + e;
        long long I = I0 + (long long)r * tx + e;
        if (PER) {  // the periodic image among the interior columns
          const int nx = ui1 - ui0 + 1, gm = ui0 + (((gi - ui0) % nx) + nx) % nx;
          I += gm - gi;
          gi = gm;
        }
        const bool in = row_in && gi >= 1 && gi <= tx;
        v[e] = in ? x[I] : 0.f;
        bb[e] = in ? b[I] : 0.f;
        ww[e] = in ? w[I] : 0.f;
        if (row_u && (PER || (gi >= ui0 && gi <= ui1))) inU |= 1u << (2 * r + e);
      }
      prow[r * kT5Row + 1] = v[0];
      prow[r * kT5Row + kT5Half + 1] = v[1];
      B[r] = make_float2(bb[0], bb[1]);
      WT[r] = make_float2(ww[0], ww[1]);
      if constexpr (EPI) {
        float dd[2];
        unsigned mm[2];
#pragma unroll
        for (int e = 0; e < 2; ++e) {
          const int gi = gi0 + e;
          const bool in = row_in && gi >= 1 && gi <= tx;
          const long long I = I0 + (long long)r * tx + e;
          dd[e] = in ? ep.d[I] : 0.f;
          mm[e] = in ? ep.m[I] : 0u;
        }
        Dsm[(r0 + r) * kT5Tx + lx] = make_float2(dd[0], dd[1]);
        Msm[(r0 + r) * kT5Tx + lx] = (ushort)(mm[0] | (mm[1] << 8));
      }
    }
  }
  // zero the pads that are read: the pad rows, the even plane's east pad
  // and the odd plane's west pad (values read only by the tile's edge cells)
  if (threadIdx.y == 0) {
    for (int c = lx; c < kT5Row; c += kT5Tx) {
      P0[c] = P1[c] = 0.f;
      P0[(TH + 1) * kT5Row + c] = P1[(TH + 1) * kT5Row + c] = 0.f;
    }
  }
  if (lx < 2) {
    const int c = kT5Half - 1 + lx;
#pragma unroll
    for (int r = 0; r < ROWS; ++r) P0[(r0 + r + 1) * kT5Row + c] = P1[(r0 + r + 1) * kT5Row + c] = 0.f;
  }
  __syncthreads();
  const float2 cff2 = make_float2(cff, cff);
  const int base = r0 * kT5Row + lx;
#pragma unroll 1
  for (int s = 0; s < 2 * NITE; ++s) {
    const float* src = ((s & 1) ? P1 : P0) + base;
    float* dst = ((s & 1) ? P0 : P1) + base;
    if (tile_in_u)
      tb5_sweep<ST, ROWS, true>(src, dst, B, WT, cff2, inU);
    else
      tb5_sweep<ST, ROWS, false>(src, dst, B, WT, cff2, inU);
    __syncthreads();
  }
  if constexpr (EPI) {
    // residual of the smoothed x into P1 (free now), then its restriction.
    // coarse cell (ii, jj) takes fine cell (2(ii-nh-1)+nh+1, likewise j) as
    // its anchor; the thread owning an anchor in the core restricts it. Its
    // Rcoef values are requested first, so that they arrive during the
    // residual pass.
    const int nh = ep.nh;
    const int ea = (nh + 1 - ti0) & 1;  // anchor column within the thread's pair
    const int lc = 2 * lx + ea, gi = ti0 + lc;
    const int ii = ((gi - nh - 1) >> 1) + nh + 1;
    const bool col_a = lc >= H && lc < kT5W - H && ii >= ep.ci0 && ii <= ep.ci1;
    const int pr = (nh + 1 - tj0 - r0) & 1;  // anchor rows of the thread: r = pr, pr + 2, ...
    float rc[ROWS];
#pragma unroll
    for (int r = 0; r < ROWS; ++r) {
      rc[r] = 0.f;
      const int lj = r0 + r;
      const int jj = ((tj0 + lj - nh - 1) >> 1) + nh + 1;
      if (col_a && (r & 1) == pr && lj >= H && lj < TH - H && jj >= ep.cj0 && jj <= ep.cj1)
        rc[r] = __ldg(ep.rcoef + (long long)(ii - 1) + (long long)ep.ctx * (jj - 1));
    }
    unsigned inbox = 0;
#pragma unroll
    for (int r = 0; r < ROWS; ++r) {
      const int gj = tj0 + r0 + r;
      const bool row_in = gj >= ep.rj0 && gj <= ep.rj1;
#pragma unroll
      for (int e = 0; e < 2; ++e) {
        const int gie = gi0 + e;
        if (row_in && gie >= ep.ri0 && gie <= ep.ri1) inbox |= 1u << (2 * r + e);
      }
    }
    tb5_resid<ST, ROWS>(P0 + base, P1 + base, B, Dsm + r0 * kT5Tx + lx, Msm + r0 * kT5Tx + lx, inbox);
    __syncthreads();
    if (col_a) {
      auto R = [&](int lj, int c) { return P1[(lj + 1) * kT5Row + (c & 1) * kT5Half + (c >> 1) + 1]; };
#pragma unroll
      for (int r = 0; r < ROWS; ++r) {
        if ((r & 1) != pr) continue;
        const int lj = r0 + r;
        const int jj = ((tj0 + lj - nh - 1) >> 1) + nh + 1;
        if (lj < H || lj >= TH - H || jj < ep.cj0 || jj > ep.cj1) continue;
        float sr;
        if (ep.pkind == 2) {  // restriction_vertices!: 1-2-1 x 1-2-1, left fold
          sr = __fmaf_rn(R(lj - 1, lc), 2.f, R(lj - 1, lc - 1));
          sr = __fadd_rn(sr, R(lj - 1, lc + 1));
          sr = __fmaf_rn(R(lj, lc - 1), 2.f, sr);
          sr = __fmaf_rn(R(lj, lc), 4.f, sr);
          sr = __fmaf_rn(R(lj, lc + 1), 2.f, sr);
          sr = __fadd_rn(sr, R(lj + 1, lc - 1));
          sr = __fmaf_rn(R(lj + 1, lc), 2.f, sr);
          sr = __fadd_rn(sr, R(lj + 1, lc + 1));
        } else {  // 2 x 2 block of cell centres
          sr = __fadd_rn(__fadd_rn(__fadd_rn(R(lj, lc), R(lj, lc + 1)), R(lj + 1, lc)), R(lj + 1, lc + 1));
        }
        const long long C = (long long)(ii - 1) + (long long)ep.ctx * (jj - 1);
        ep.bc[C] = __fmul_rn(rc[r], sr);
        ep.xc[C] = 0.f;
      }
    }
  }
  // 2*NITE sweeps: the result is in P0; write the core cells of U
  if constexpr (UPD) {
    const double is = ep.ds[S_ICUR];
    const int pe = pow2_exponent(is);  // iscale = 2^pe
    unsigned long long mx = 0;
    auto upd = [&](double xv, float e) {
      const double v = __dadd_rn(xv, f2d_pow2(e, pe, is));
      const unsigned long long ub = (unsigned long long)__double_as_longlong(v) & 0x7FFFFFFFFFFFFFFFULL;
      mx = ub > mx ? ub : mx;
      return v;
    };
    if (fast) {
      if (2 * lx >= H && 2 * lx < kT5W - H) {
        double2* xp = reinterpret_cast<double2*>(ep.xd + I0);
        const int st = tx >> 1;
        double2 xv[ROWS];
#pragma unroll
        for (int r = 0; r < ROWS; ++r) {  // all loads in flight before the first use
          const int lj = r0 + r;
          if (lj >= H && lj < TH - H) xv[r] = xp[r * st];
        }
#pragma unroll
        for (int r = 0; r < ROWS; ++r) {
          const int lj = r0 + r;
          if (lj >= H && lj < TH - H)
            xp[r * st] = make_double2(upd(xv[r].x, prow[r * kT5Row + 1]), upd(xv[r].y, prow[r * kT5Row + kT5Half + 1]));
        }
      }
    } else {
#pragma unroll
      for (int r = 0; r < ROWS; ++r) {
        const int lj = r0 + r;
        if (lj < H || lj >= TH - H) continue;
#pragma unroll
        for (int e = 0; e < 2; ++e) {
          const int lc = 2 * lx + e;
          if (lc >= H && lc < kT5W - H && (inU >> (2 * r + e) & 1u) && (!PER || gi0 + e <= ui1)) {
            const long long I = I0 + (long long)r * tx + e;
            ep.xd[I] = upd(ep.xd[I], prow[r * kT5Row + e * kT5Half + 1]);
          }
        }
      }
    }
    // max over the CTA, one atomic (bit patterns of non-negative doubles order like the values)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long ox = __shfl_down_sync(0xffffffffu, mx, o);
      mx = ox > mx ? ox : mx;
    }
    __shared__ unsigned long long wmx[kT5Tx * TY / 32];
    const int tid = threadIdx.y * kT5Tx + threadIdx.x;
    if ((tid & 31) == 0) wmx[tid >> 5] = mx;
    __syncthreads();
    if (tid == 0) {
      unsigned long long m = 0;
#pragma unroll
      for (int w = 0; w < kT5Tx * TY / 32; ++w) m = wmx[w] > m ? wmx[w] : m;
      if (m) atomicMax(reinterpret_cast<unsigned long long*>(ep.ds + S_MAXX), m);
    }
    return;
  }
  if (fast) {
    // H is even: the pair's two cells are both core columns or neither
    if (2 * lx >= H && 2 * lx < kT5W - H) {
      float2* op = reinterpret_cast<float2*>(xo + I0);
      const int st = tx >> 1;
#pragma unroll
      for (int r = 0; r < ROWS; ++r) {
        const int lj = r0 + r;
        if (lj >= H && lj < TH - H) op[r * st] = make_float2(prow[r * kT5Row + 1], prow[r * kT5Row + kT5Half + 1]);
      }
    }
    return;
  }
#pragma unroll
  for (int r = 0; r < ROWS; ++r) {
    const int lj = r0 + r;
    if (lj < H || lj >= TH - H) continue;
#pragma unroll
    for (int e = 0; e < 2; ++e) {
      const int lc = 2 * lx + e;
      if (lc >= H && lc < kT5W - H && (inU >> (2 * r + e) & 1u) && (!PER || gi0 + e <= ui1))
        xo[I0 + (long long)r * tx + e] = prow[r * kT5Row + e * kT5Half + 1];
    }
  }
}

template <int ST, int NITE, int TY, int ROWS, int MINB, bool EPI, bool PER = false, bool UPD = false>
__global__ void __launch_bounds__(kT5Tx * TY, MINB) k_smooth_tb5(const float* __restrict__ x, float* __restrict__ xo,
                                                                 const float* __restrict__ b,
                                                                 const float* __restrict__ w, float cff, int tx,
                                                                 int ty, int ui0, int ui1, int uj0, int uj1,
                                                                 TbEpi ep) {
  dep_wait();
  extern __shared__ float smem[];
  tb5_tile<ST, NITE, TY, ROWS, EPI, PER, UPD>(x, xo, b, w, cff, tx, ty, ui0, ui1, uj0, uj1, ep, (int)blockIdx.x,
                                              (int)blockIdx.y, (int)blockIdx.z, smem);
}

template <int ST, int NITE>
__global__ void __launch_bounds__(kTbW * kTbTy, 1) k_smooth_tb(const float* __restrict__ x, float* __restrict__ xo,
                                                               const float* __restrict__ b,
                                                               const float* __restrict__ w, float cff, int tx,
                                                               int ty, int ui0, int ui1, int uj0, int uj1) {
  dep_wait();
  extern __shared__ float smem[];
  tb_tile<ST, NITE>(x, xo, b, w, cff, tx, ty, ui0, ui1, uj0, uj1, (int)blockIdx.x, (int)blockIdx.y, (int)blockIdx.z,
                    smem);
}

// Batched form: a grid-stride loop over windows of 1024 entries of a tile
// table (tab[t] = {OPK_TB Op, tile of the Op, instance}); the tiles of
// instances that are still active are compacted and run one after the
// other. The barrier at the end of each tile keeps the next tile's loads
// behind this tile's last shared-memory reads.
template <int ST, int NITE>
__global__ void __launch_bounds__(kTbW * kTbTy, 1) k_btb(const Op* __restrict__ ops, const int4* __restrict__ tab,
                                                         long long ntiles, int win, const int* __restrict__ active) {
  dep_wait();
  extern __shared__ float smem[];
  __shared__ int list[kTbW * kTbTy];
  __shared__ int wsum[kTbW * kTbTy / 32 + 1];
  const int tid = threadIdx.y * kTbW + threadIdx.x;
  const int nt = kTbW * kTbTy;
  for (long long base = (long long)blockIdx.x * win; base < ntiles; base += (long long)gridDim.x * win) {
    // ordered compaction of the window's active tiles
    const long long c = base + tid;
    bool ok = false;
    if (tid < win && c < ntiles) ok = active[tab[c].z] != 0;
    const unsigned bal = __ballot_sync(0xffffffffu, ok);
    const int lane = tid & 31, wid = tid >> 5;
    if (lane == 0) wsum[wid] = __popc(bal);
    __syncthreads();
    if (tid == 0) {
      int a = 0;
      for (int w = 0; w < nt / 32; ++w) {
        const int v = wsum[w];
        wsum[w] = a;
        a += v;
      }
      wsum[nt / 32] = a;
    }
    __syncthreads();
    if (ok) list[wsum[wid] + __popc(bal & ((1u << lane) - 1u))] = tid;
    __syncthreads();
    const int cnt = wsum[nt / 32];
    for (int q = 0; q < cnt; ++q) {
      const int4 en = tab[base + list[q]];
      const Op& op = ops[en.x];
      const long long per_layer = (long long)op.kf0 * op.kf1;
      const int bz = (int)(en.y / per_layer);
      const int rem = (int)(en.y - (long long)bz * per_layer);
      tb_tile<ST, NITE>((const float*)op.x, (float*)op.y, (const float*)op.b, (const float*)op.w, (float)op.cff,
                        op.g.tx, op.g.ty, op.box.i0, op.box.i1, op.box.j0, op.box.j1, rem % op.kf0, rem / op.kf0, bz,
                        smem);
      __syncthreads();
    }
    __syncthreads();  // list is rewritten by the next window
  }
}

// Batched form of the lean packed pass (8 x 6 rows a tile, as the
// standalone pass): the same windowed walk over a tile table as k_btb, each
// active tile run by tb5_tile; the barrier after a tile keeps the next
// tile's loads behind this tile's last shared-memory reads.
template <int ST, int NITE>
__global__ void __launch_bounds__(kT5Tx * 8, 2) k_btb5(const Op* __restrict__ ops, const int4* __restrict__ tab,
                                                       long long ntiles, int win, const int* __restrict__ active) {
  dep_wait();
  extern __shared__ float smem[];
  constexpr int nt = kT5Tx * 8;
  __shared__ int list[nt];
  __shared__ int wsum[nt / 32 + 1];
  const int tid = threadIdx.y * kT5Tx + threadIdx.x;
  for (long long base = (long long)blockIdx.x * win; base < ntiles; base += (long long)gridDim.x * win) {
    const long long c = base + tid;
    bool ok = false;
    if (tid < win && c < ntiles) ok = active[tab[c].z] != 0;
    const unsigned bal = __ballot_sync(0xffffffffu, ok);
    const int lane = tid & 31, wid = tid >> 5;
    if (lane == 0) wsum[wid] = __popc(bal);
    __syncthreads();
    if (tid == 0) {
      int a = 0;
      for (int w = 0; w < nt / 32; ++w) {
        const int v = wsum[w];
        wsum[w] = a;
        a += v;
      }
      wsum[nt / 32] = a;
    }
    __syncthreads();
    if (ok) list[wsum[wid] + __popc(bal & ((1u << lane) - 1u))] = tid;
    __syncthreads();
    const int cnt = wsum[nt / 32];
    for (int q = 0; q < cnt; ++q) {
      const int4 en = tab[base + list[q]];
      const Op& op = ops[en.x];
      const long long per_layer = (long long)op.kf0 * op.kf1;
      const int bz = (int)(en.y / per_layer);
      const int rem = (int)(en.y - (long long)bz * per_layer);
      tb5_tile<ST, NITE, 8, 6, false, false, false>((const float*)op.x, (float*)op.y, (const float*)op.b,
                                                    (const float*)op.w, (float)op.cff, op.g.tx, op.g.ty, op.box.i0,
                                                    op.box.i1, op.box.j0, op.box.j1, TbEpi{}, rem % op.kf0,
                                                    rem / op.kf0, bz, smem);
      __syncthreads();
    }
    __syncthreads();  // list is rewritten by the next window
  }
}

template <int ST, int NITE>
static void launch_tb3_n(const float* x, float* xo, const float* b, const float* w, float cff, int tx, int ty,
                         int nz, int ui0, int ui1, int uj0, int uj1, cudaStream_t s) {
  constexpr int H = 2 * NITE;
  constexpr int CW = kT3W - 2 * H, CH = kT3H - 2 * H;
  const size_t smem = 2 * (size_t)kT3H * kT3W * sizeof(float);
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_smooth_tb3<ST, NITE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    attr = true;
  }
  dim3 grid((unsigned)((ui1 - ui0 + CW) / CW), (unsigned)((uj1 - uj0 + CH) / CH), (unsigned)nz);
  launch_dep(k_smooth_tb3<ST, NITE>, grid, dim3(kT3Tx, kT3Ty, 1), smem, s, x, xo, b, w, cff, tx, ty, ui0, ui1, uj0, uj1);
}

template <int ST, int NITE, int TY, int ROWS, int MINB, bool EPI, bool PER = false, bool UPD = false>
static void launch_tb5_n(const float* x, float* xo, const float* b, const float* w, float cff, int tx, int ty,
                         int nz, int ui0, int ui1, int uj0, int uj1, const TbEpi& ep, cudaStream_t s) {
  constexpr int H = 2 * NITE + (EPI ? 2 : 0);
  constexpr int CW = kT5W - 2 * H, CH = TY * ROWS - 2 * H;
  const size_t smem = 2 * (size_t)t5_plane<TY, ROWS>() * sizeof(float) +
                      (EPI ? (size_t)TY * ROWS * kT5Tx * (sizeof(float2) + sizeof(ushort)) : 0);
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_smooth_tb5<ST, NITE, TY, ROWS, MINB, EPI, PER, UPD>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    attr = true;
  }
  dim3 grid((unsigned)((ui1 - ui0 + CW) / CW), (unsigned)((uj1 - uj0 + CH) / CH), (unsigned)nz);
  launch_dep(k_smooth_tb5<ST, NITE, TY, ROWS, MINB, EPI, PER, UPD>, grid, dim3(kT5Tx, TY, 1), smem, s, x, xo, b, w, cff, tx, ty, ui0, ui1, uj0, uj1, ep);
}

template <int ST, int NITE>
static void launch_tb_n(int version, const float* x, float* xo, const float* b, const float* w, float cff, int tx,
                        int ty, int nz, int ui0, int ui1, int uj0, int uj1, cudaStream_t s) {
  if (version >= 5) {
    // 8 x 6 rows per tile, 2 CTAs per SM (measured best at 4096^2 down to
    // the 262^2 coarsest level of 20 pairs, which runs as 99 tiles)
    launch_tb5_n<ST, NITE, 8, 6, 2, false>(x, xo, b, w, cff, tx, ty, nz, ui0, ui1, uj0, uj1, TbEpi{}, s);
    return;
  }
  if (version >= 3) {
    launch_tb3_n<ST, NITE>(x, xo, b, w, cff, tx, ty, nz, ui0, ui1, uj0, uj1, s);
    return;
  }
  constexpr int H = 2 * NITE;
  constexpr int CW = kTbW - 2 * H, CH = kTbH - 2 * H;
  const size_t smem = 4 * (size_t)kTbH * kTbW * sizeof(float);
  static bool attr = false;  // one attribute set per instantiation (single-threaded host use)
  if (!attr) {
    cudaFuncSetAttribute(k_smooth_tb<ST, NITE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    attr = true;
  }
  dim3 grid((unsigned)((ui1 - ui0 + CW) / CW), (unsigned)((uj1 - uj0 + CH) / CH), (unsigned)nz);
  launch_dep(k_smooth_tb<ST, NITE>, grid, dim3(kTbW, kTbTy, 1), smem, s, x, xo, b, w, cff, tx, ty, ui0, ui1, uj0, uj1);
}

// nite pairs of sweeps in one pass (nite in 1..kTbMaxPairs); returns false when the
// caller must fall back to single sweeps.
bool launch_smooth_tb(int version, int stencil, int nite, const float* x, float* xo, const float* b, const float* w,
                      float cff, int tx, int ty, int nz, int ui0, int ui1, int uj0, int uj1, cudaStream_t s) {
#define CFMG_TB(ST, N)                                                                       \
  if (stencil == ST && nite == N) {                                                          \
    launch_tb_n<ST, N>(version, x, xo, b, w, cff, tx, ty, nz, ui0, ui1, uj0, uj1, s);        \
    return true;                                                                             \
  }
  CFMG_TB(5, 1) CFMG_TB(5, 2) CFMG_TB(5, 3) CFMG_TB(5, 4) CFMG_TB(5, 5)
  CFMG_TB(5, 6) CFMG_TB(5, 7) CFMG_TB(5, 8) CFMG_TB(5, 9) CFMG_TB(5, 10)
  CFMG_TB(9, 1) CFMG_TB(9, 2) CFMG_TB(9, 3) CFMG_TB(9, 4) CFMG_TB(9, 5)
  CFMG_TB(9, 6) CFMG_TB(9, 7) CFMG_TB(9, 8) CFMG_TB(9, 9) CFMG_TB(9, 10)
#undef CFMG_TB
  return false;
}

bool launch_smooth_tb_periodic(int nite, const float* x, float* xo, const float* b, const float* w, float cff,
                               int tx, int ty, int nz, int ui0, int ui1, int uj0, int uj1, cudaStream_t s) {
#define CFMG_TBP(N)                                                                                    \
  if (nite == N) {                                                                                     \
    launch_tb5_n<5, N, 8, 6, 2, false, true>(x, xo, b, w, cff, tx, ty, nz, ui0, ui1, uj0, uj1, TbEpi{}, s); \
    return true;                                                                                       \
  }
  CFMG_TBP(1) CFMG_TBP(2) CFMG_TBP(3) CFMG_TBP(4) CFMG_TBP(5)
  CFMG_TBP(6) CFMG_TBP(7) CFMG_TBP(8) CFMG_TBP(9) CFMG_TBP(10)
#undef CFMG_TBP
  return false;
}

bool launch_smooth_tb_upd(int stencil, int nite, const float* x, const float* b, const float* w, float cff, int tx,
                          int ty, int nz, int ui0, int ui1, int uj0, int uj1, double* xd, double* ds, cudaStream_t s) {
  TbEpi ep{};
  ep.xd = xd;
  ep.ds = ds;
#define CFMG_TBU(ST, N)                                                                                       \
  if (stencil == ST && nite == N) {                                                                           \
    launch_tb5_n<ST, N, 8, 6, 2, false, false, true>(x, nullptr, b, w, cff, tx, ty, nz, ui0, ui1, uj0, uj1, ep, s); \
    return true;                                                                                              \
  }
  CFMG_TBU(5, 1) CFMG_TBU(5, 2) CFMG_TBU(5, 3)
  CFMG_TBU(9, 1) CFMG_TBU(9, 2) CFMG_TBU(9, 3)
#undef CFMG_TBU
  return false;
}

bool launch_smooth_tb_epi(int stencil, int nite, const float* x, float* xo, const float* b, const float* w, float cff,
                          int tx, int ty, int ui0, int ui1, int uj0, int uj1, const TbEpi& ep, cudaStream_t s) {
  // 8 x 6 rows as the plain passes (64-row tiles measured slower: 15.1 against 14.3 ms per config-2 solve)
#define CFMG_TBE(ST, N)                                                                              \
  if (stencil == ST && nite == N) {                                                                  \
    launch_tb5_n<ST, N, 8, 6, 2, true>(x, xo, b, w, cff, tx, ty, 1, ui0, ui1, uj0, uj1, ep, s);     \
    return true;                                                                                     \
  }
  CFMG_TBE(5, 1) CFMG_TBE(5, 2) CFMG_TBE(5, 3)
  CFMG_TBE(9, 1) CFMG_TBE(9, 2) CFMG_TBE(9, 3)
#undef CFMG_TBE
  return false;
}

// tile counts of one pass over the box U (the host builds OPK_TB Ops with
// these: kf0 x kf1 tiles per layer)
void tb_tiles(int nite, int ui0, int ui1, int uj0, int uj1, int* ntx, int* nty) {
  const int H = 2 * nite, CW = kTbW - 2 * H, CH = kTbH - 2 * H;
  *ntx = (ui1 - ui0 + CW) / CW;
  *nty = (uj1 - uj0 + CH) / CH;
}

// tile counts of one lean packed pass (8 x 6 rows) over the box U
void tb5_tiles(int nite, int ui0, int ui1, int uj0, int uj1, int* ntx, int* nty) {
  const int H = 2 * nite, CW = kT5W - 2 * H, CH = 8 * 6 - 2 * H;
  *ntx = (ui1 - ui0 + CW) / CW;
  *nty = (uj1 - uj0 + CH) / CH;
}

template <int ST, int NITE>
static void launch_btb5_n(const Op* ops, const int4* tab, long long ntiles, const int* active, cudaStream_t s) {
  const size_t smem = 2 * (size_t)t5_plane<8, 6>() * sizeof(float);
  static bool attr = false;
  static int nsm = 0;
  if (!attr) {
    cudaFuncSetAttribute(k_btb5<ST, NITE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    attr = true;
  }
  // two resident CTAs per SM, each taking windows of `win` tiles
  const long long g = 2LL * nsm;
  long long win = (ntiles + g - 1) / g;
  if (win > kT5Tx * 8) win = kT5Tx * 8;
  const long long windows = (ntiles + win - 1) / win;
  const long long grid = windows < g ? windows : g;
  launch_dep(k_btb5<ST, NITE>, (unsigned)grid, dim3(kT5Tx, 8, 1), smem, s, ops, tab, ntiles, (int)win, active);
}

bool launch_btb5(int stencil, int nite, const Op* ops, const int4* tab, long long ntiles, const int* active,
                 cudaStream_t s) {
  if (ntiles <= 0) return true;
#define CFMG_BTB5(ST, N)                                             \
  if (stencil == ST && nite == N) {                                  \
    launch_btb5_n<ST, N>(ops, tab, ntiles, active, s);               \
    return true;                                                     \
  }
  CFMG_BTB5(5, 1) CFMG_BTB5(5, 2) CFMG_BTB5(5, 3)
  CFMG_BTB5(9, 1) CFMG_BTB5(9, 2) CFMG_BTB5(9, 3)
#undef CFMG_BTB5
  return false;
}

template <int ST, int NITE>
static void launch_btb_n(const Op* ops, const int4* tab, long long ntiles, const int* active, cudaStream_t s) {
  const size_t smem = 4 * (size_t)kTbH * kTbW * sizeof(float);
  static bool attr = false;
  static int nsm = 0;
  if (!attr) {
    cudaFuncSetAttribute(k_btb<ST, NITE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    attr = true;
  }
  // one resident CTA per SM, each taking windows of `win` tiles
  long long win = (ntiles + nsm - 1) / nsm;
  if (win > kTbW * kTbTy) win = kTbW * kTbTy;
  const long long windows = (ntiles + win - 1) / win;
  const long long grid = windows < nsm ? windows : nsm;
  launch_dep(k_btb<ST, NITE>, (unsigned)grid, dim3(kTbW, kTbTy, 1), smem, s, ops, tab, ntiles, (int)win, active);
}

bool launch_btb(int stencil, int nite, const Op* ops, const int4* tab, long long ntiles, const int* active,
                cudaStream_t s) {
  if (ntiles <= 0) return true;
#define CFMG_BTB(ST, N)                                              \
  if (stencil == ST && nite == N) {                                  \
    launch_btb_n<ST, N>(ops, tab, ntiles, active, s);                \
    return true;                                                     \
  }
  CFMG_BTB(5, 1) CFMG_BTB(5, 2) CFMG_BTB(5, 3)
  CFMG_BTB(9, 1) CFMG_BTB(9, 2) CFMG_BTB(9, 3)
#undef CFMG_BTB
  return false;
}

}  // namespace cfmg
