// Per-cell arithmetic of the multigrid operators, shared by the standalone
// kernels (k_ops.cu) and the coarse-level program engine (k_coarse.cu), so
// that both paths round identically.
//
// Every sum and product goes through the _rn intrinsics so that nvcc
// cannot contract a multiply and an add into one FMA: the FP64
// instantiation rounds exactly where the Julia reference rounds. The only
// FMAs used are ones whose product is exact (a multiplication by 1/2, 1/4,
// 2, 4 or 8), which round once on the same exact value as the reference's
// two-step form.
#pragma once

#include "cfmg_internal.h"

namespace cfmg {

template <class T>
struct Ar;
template <>
struct Ar<double> {
  static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
  static __device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
  static __device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
  // a*w + c with w a power of two (exact product): one rounding, same value
  static __device__ __forceinline__ double fmx(double a, double w, double c) { return __fma_rn(a, w, c); }
};
template <>
struct Ar<float> {
  static __device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
  static __device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
  static __device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
  static __device__ __forceinline__ float fmx(float a, float w, float c) { return __fmaf_rn(a, w, c); }
};

// msk*v for a UInt8 mask, as the reference's promote-and-multiply: 1 -> v,
// 0 -> a zero carrying v's sign, other values -> (double)m*v.
template <class T>
__device__ __forceinline__ T mask_mul(uint8_t m, T v) {
  if (m == 1) return v;
  if (m == 0) return copysign(T(0), v);
  return Ar<T>::mul(T(m), v);
}

__device__ __forceinline__ long long lin(const Geom& g, int i, int j, int k) {
  return (long long)(i - 1) + g.n1 * ((long long)(j - 1) + (long long)g.ty * (k - 1));
}

__device__ __forceinline__ int c2f(int i, int nh) { return (i - nh - 1) * 2 + nh + 1; }  // src/gmg_types.jl:25
__device__ __forceinline__ int f2c(int i, int nh) { return (i - nh - 1) / 2 + nh + 1; }  // src/gmg_types.jl:26

// ------------------------------------------------------------- stencils
template <class T>
__device__ __forceinline__ T sum4(const T* x, long long I, long long n1) {
  typedef Ar<T> A;
  return A::add(A::add(A::add(x[I - 1], x[I + 1]), x[I - n1]), x[I + n1]);
}
template <class T>
__device__ __forceinline__ T diags4(const T* x, long long I, long long n1) {
  typedef Ar<T> A;
  return A::add(A::add(A::add(x[I - 1 - n1], x[I + 1 - n1]), x[I - 1 + n1]), x[I + 1 + n1]);
}
template <class T>
__device__ __forceinline__ T faces6(const T* x, long long I, long long n1, long long n2) {
  typedef Ar<T> A;
  return A::add(A::add(A::add(A::add(A::add(x[I - 1], x[I + 1]), x[I - n1]), x[I + n1]), x[I - n2]), x[I + n2]);
}
template <class T>
__device__ __forceinline__ T edges12(const T* x, long long I, long long n1, long long n2) {
  typedef Ar<T> A;
  T e = A::add(x[I - 1 - n1], x[I + 1 - n1]);
  e = A::add(e, x[I - 1 + n1]);
  e = A::add(e, x[I + 1 + n1]);
  e = A::add(e, x[I - 1 - n2]);
  e = A::add(e, x[I + 1 - n2]);
  e = A::add(e, x[I - 1 + n2]);
  e = A::add(e, x[I + 1 + n2]);
  e = A::add(e, x[I - n1 - n2]);
  e = A::add(e, x[I + n1 - n2]);
  e = A::add(e, x[I - n1 + n2]);
  e = A::add(e, x[I + n1 + n2]);
  return e;
}
template <class T>
__device__ __forceinline__ T vc_sum(const T* x, const T* cE, const T* cN, long long I, long long n1) {
  typedef Ar<T> A;
  T s = A::add(A::mul(cE[I - 1], x[I - 1]), A::mul(cE[I], x[I + 1]));
  s = A::add(s, A::mul(cN[I - n1], x[I - n1]));
  return A::add(s, A::mul(cN[I], x[I + n1]));
}

// ---------------------------------------------------------- sweeps at I
// v_* return the new value at I, d_* store it.
// sloop2d! (src/laplacian.jl:66-73): y = (1-w)x - (w*idiag)*(b - s4)
template <class T>
__device__ __forceinline__ T v_sweep5(const T* x, const T* b, const T* w, T cff, long long n1, long long I) {
  typedef Ar<T> A;
  return A::sub(A::mul(cff, x[I]), A::mul(w[I], A::sub(b[I], sum4(x, I, n1))));
}
// sloop3d_v1! (src/laplacian.jl:11-20)
template <class T>
__device__ __forceinline__ T v_sweep7(const T* x, const T* b, const T* w, T cff, long long n1, long long n2,
                                      long long I) {
  typedef Ar<T> A;
  return A::sub(A::mul(cff, x[I]), A::mul(w[I], A::sub(b[I], faces6(x, I, n1, n2))));
}
// in-plane laplacian9 (2D 9-point extension): b - faces/2 - diagonals/4
template <class T>
__device__ __forceinline__ T v_sweep9(const T* x, const T* b, const T* w, T cff, long long n1, long long I) {
  typedef Ar<T> A;
  T t = A::fmx(sum4(x, I, n1), T(-0.5), b[I]);
  t = A::fmx(diags4(x, I, n1), T(-0.25), t);
  return A::sub(A::mul(cff, x[I]), A::mul(w[I], t));
}
// smooth_laplacian9! body (src/laplacian9.jl:14-44)
template <class T>
__device__ __forceinline__ T v_sweep19(const T* x, const T* b, const T* w, T cff, long long n1, long long n2,
                                       long long I) {
  typedef Ar<T> A;
  T t = A::fmx(faces6(x, I, n1, n2), T(-0.5), b[I]);
  t = A::fmx(edges12(x, I, n1, n2), T(-0.25), t);
  return A::sub(A::mul(cff, x[I]), A::mul(w[I], t));
}
template <class T>
__device__ __forceinline__ T v_sweepvc(const T* x, const T* b, const T* w, const T* cE, const T* cN, T cff,
                                       long long n1, long long I) {
  typedef Ar<T> A;
  return A::sub(A::mul(cff, x[I]), A::mul(w[I], A::sub(b[I], vc_sum(x, cE, cN, I, n1))));
}
template <class T>
__device__ __forceinline__ void d_sweep5(const T* x, T* y, const T* b, const T* w, T cff, long long n1, long long I) {
  y[I] = v_sweep5(x, b, w, cff, n1, I);
}
template <class T>
__device__ __forceinline__ void d_sweep7(const T* x, T* y, const T* b, const T* w, T cff, long long n1, long long n2,
                                         long long I) {
  y[I] = v_sweep7(x, b, w, cff, n1, n2, I);
}
template <class T>
__device__ __forceinline__ void d_sweep9(const T* x, T* y, const T* b, const T* w, T cff, long long n1, long long I) {
  y[I] = v_sweep9(x, b, w, cff, n1, I);
}
template <class T>
__device__ __forceinline__ void d_sweep19(const T* x, T* y, const T* b, const T* w, T cff, long long n1, long long n2,
                                          long long I) {
  y[I] = v_sweep19(x, b, w, cff, n1, n2, I);
}
template <class T>
__device__ __forceinline__ void d_sweepvc(const T* x, T* y, const T* b, const T* w, const T* cE, const T* cN, T cff,
                                          long long n1, long long I) {
  y[I] = v_sweepvc(x, b, w, cE, cN, cff, n1, I);
}

// ------------------------------------------------------- residuals at I
// v_* return the residual value, d_* store it.
// rloop2d! (src/laplacian.jl:87-93): r = msk*((diag*x + b) - s4)
template <class T>
__device__ __forceinline__ T v_resid5(const T* x, const T* b, const T* d, const uint8_t* m, long long n1, long long I) {
  typedef Ar<T> A;
  return mask_mul(m[I], A::sub(A::add(A::mul(d[I], x[I]), b[I]), sum4(x, I, n1)));
}
// rloop3d! (src/laplacian.jl:43-51)
template <class T>
__device__ __forceinline__ T v_resid7(const T* x, const T* b, const T* d, const uint8_t* m, long long n1, long long n2,
                                      long long I) {
  typedef Ar<T> A;
  return mask_mul(m[I], A::sub(A::add(A::mul(d[I], x[I]), b[I]), faces6(x, I, n1, n2)));
}
template <class T>
__device__ __forceinline__ T v_resid9(const T* x, const T* b, const T* d, const uint8_t* m, long long n1, long long I) {
  typedef Ar<T> A;
  T v = A::add(A::mul(d[I], x[I]), b[I]);
  v = A::fmx(sum4(x, I, n1), T(-0.5), v);
  v = A::fmx(diags4(x, I, n1), T(-0.25), v);
  return mask_mul(m[I], v);
}
// residual_laplacian9! (src/laplacian9.jl:49-73)
template <class T>
__device__ __forceinline__ T v_resid19(const T* x, const T* b, const T* d, const uint8_t* m, long long n1,
                                       long long n2, long long I) {
  typedef Ar<T> A;
  T v = A::add(A::mul(d[I], x[I]), b[I]);
  v = A::fmx(faces6(x, I, n1, n2), T(-0.5), v);
  v = A::fmx(edges12(x, I, n1, n2), T(-0.25), v);
  return mask_mul(m[I], v);
}
template <class T>
__device__ __forceinline__ void d_resid5(T* r, const T* x, const T* b, const T* d, const uint8_t* m, long long n1,
                                         long long I) {
  r[I] = v_resid5(x, b, d, m, n1, I);
}
template <class T>
__device__ __forceinline__ void d_resid7(T* r, const T* x, const T* b, const T* d, const uint8_t* m, long long n1,
                                         long long n2, long long I) {
  r[I] = v_resid7(x, b, d, m, n1, n2, I);
}
template <class T>
__device__ __forceinline__ void d_resid9(T* r, const T* x, const T* b, const T* d, const uint8_t* m, long long n1,
                                         long long I) {
  r[I] = v_resid9(x, b, d, m, n1, I);
}
template <class T>
__device__ __forceinline__ void d_resid19(T* r, const T* x, const T* b, const T* d, const uint8_t* m, long long n1,
                                          long long n2, long long I) {
  r[I] = v_resid19(x, b, d, m, n1, n2, I);
}
template <class T>
__device__ __forceinline__ T v_residvc(const T* x, const T* b, const T* d, const T* cE, const T* cN, const uint8_t* m,
                                       long long n1, long long I) {
  typedef Ar<T> A;
  return mask_mul(m[I], A::sub(A::add(A::mul(d[I], x[I]), b[I]), vc_sum(x, cE, cN, I, n1)));
}
template <class T>
__device__ __forceinline__ void d_residvc(T* r, const T* x, const T* b, const T* d, const T* cE, const T* cN,
                                          const uint8_t* m, long long n1, long long I) {
  r[I] = v_residvc(x, b, d, cE, cN, m, n1, I);
}

// ---------------------------------------------------------- restriction
// Coarse interior cell (ii, jj, kk) of kind 0 centres 2D (rcloop2d!,
// src/RP_on_centers.jl:117-133), 1 centres 3D (rcloop3d!, :5-23),
// 2 vertices 2D (rvloop2d!, src/RP_on_vertices.jl:96-115), 3 vertices 3D
// (restriction_vertices!, :1-32).
template <class T, int KIND>
__device__ __forceinline__ T v_restrict(const T* x, const T* coef, const Geom& gf, const Geom& gc, int ii, int jj,
                                        int kk, long long& C) {
  typedef Ar<T> A;
  const int nh = gc.nh;
  const int i = c2f(ii, nh), j = c2f(jj, nh);
  const long long n1 = gf.n1, n2 = gf.n2;
  T s;
  if (KIND == 0) {
    long long F = lin(gf, i, j, kk);
    s = A::add(A::add(A::add(x[F], x[F + 1]), x[F + n1]), x[F + 1 + n1]);
  } else if (KIND == 1) {
    long long F = lin(gf, i, j, c2f(kk, nh));
    s = A::add(x[F], x[F + 1]);
    s = A::add(s, x[F + n1]);
    s = A::add(s, x[F + 1 + n1]);
    s = A::add(s, x[F + n2]);
    s = A::add(s, x[F + 1 + n2]);
    s = A::add(s, x[F + n1 + n2]);
    s = A::add(s, x[F + 1 + n1 + n2]);
  } else if (KIND == 2) {  // 1-2-1 x 1-2-1
    long long F = lin(gf, i, j, kk);
    s = A::fmx(x[F - n1], T(2), x[F - 1 - n1]);
    s = A::add(s, x[F + 1 - n1]);
    s = A::fmx(x[F - 1], T(2), s);
    s = A::fmx(x[F], T(4), s);
    s = A::fmx(x[F + 1], T(2), s);
    s = A::add(s, x[F - 1 + n1]);
    s = A::fmx(x[F + n1], T(2), s);
    s = A::add(s, x[F + 1 + n1]);
  } else {  // 27 points, weights 1-2-4-8, left fold in source order
    long long F = lin(gf, i, j, c2f(kk, nh));
    bool first = true;
    s = T(0);
#pragma unroll
    for (int dk = -1; dk <= 1; ++dk)
#pragma unroll
      for (int dj = -1; dj <= 1; ++dj)
#pragma unroll
        for (int di = -1; di <= 1; ++di) {
          const int w = (2 - (di < 0 ? -di : di)) * (2 - (dj < 0 ? -dj : dj)) * (2 - (dk < 0 ? -dk : dk));
          T v = x[F + di + dj * n1 + dk * n2];
          if (first) {
            s = (w == 1) ? v : A::mul(T(w), v);
            first = false;
          } else {
            s = (w == 1) ? A::add(s, v) : A::fmx(v, T(w), s);
          }
        }
  }
  C = lin(gc, ii, jj, kk);
  return A::mul(coef[C], s);
}
template <class T, int KIND>
__device__ __forceinline__ void d_restrict(const T* x, T* xc, const T* coef, const Geom& gf, const Geom& gc, int ii,
                                           int jj, int kk) {
  long long C;
  const T v = v_restrict<T, KIND>(x, coef, gf, gc, ii, jj, kk, C);
  xc[C] = v;
}

// --------------------------------------------------------- prolongation
// square (src/RP_on_centers.jl:1-3): 3*(x[i+di,j,k+dk]+x[i,j+dj,k+dk]) + x[i+di,j+dj,k+dk]
template <class T>
__device__ __forceinline__ T square3(const T* x, long long C, long long di, long long dj, long long dk) {
  typedef Ar<T> A;
  return A::add(A::mul(T(3), A::add(x[C + di + dk], x[C + dj + dk])), x[C + di + dj + dk]);
}

// Fine parent (p, q, qk): i = nh+1+2p, j = nh+1+2q, and k = kf0+qk (2D) or
// nh+1+2qk (3D). The parent updates its 4 (2D) or 8 (3D) children, which no
// other parent touches. Kinds as in d_restrict: pcloop2d!
// (src/RP_on_centers.jl:146-163), pcloop3d! (:84-104), pvloop2d!
// (src/RP_on_vertices.jl:117-137), prolongation_vertices! (:34-72).
// ASSIGN: the fine x is known to hold +0 at every updated cell, so it is
// not read: x = +0 + coef*v gives the same value and the same zero sign.
template <class T, int KIND, bool ASSIGN = false>
__device__ __forceinline__ void d_prolong(T* xf, const T* x, const T* coef, const Geom& gf, const Geom& gc, int p,
                                          int q, int qk, int kf0) {
  typedef Ar<T> A;
  const int nh = gf.nh;
  const int i = nh + 1 + 2 * p, j = nh + 1 + 2 * q;
  const int ic = f2c(i, nh), jc = f2c(j, nh);
  const long long c1 = gc.n1, c2 = gc.n2, f1 = gf.n1, f2 = gf.n2;
  if (KIND == 0) {
    const int k = kf0 + qk;
    const long long C = lin(gc, ic, jc, k), F = lin(gf, i, j, k);
    const T x9 = A::mul(x[C], T(9));
    // every load of the four children before the first store, so that they
    // are in flight together (the compiler cannot move a load of one child
    // above the store of another: the arrays might alias)
    T bb[4], cf[4], xo[4];
#pragma unroll
    for (int dj = 0; dj <= 1; ++dj)
#pragma unroll
      for (int di = 0; di <= 1; ++di) {
        const int c = 2 * dj + di;
        const long long Fi = F + di + dj * f1;
        bb[c] = square3(x, C, (long long)(2 * di - 1), (2 * dj - 1) * c1, 0LL);
        cf[c] = coef[Fi];
        xo[c] = ASSIGN ? T(0) : xf[Fi];
      }
#pragma unroll
    for (int dj = 0; dj <= 1; ++dj)
#pragma unroll
      for (int di = 0; di <= 1; ++di) {
        const int c = 2 * dj + di;
        xf[F + di + dj * f1] = A::add(xo[c], A::mul(cf[c], A::add(bb[c], x9)));
      }
  } else if (KIND == 1) {
    const int k = nh + 1 + 2 * qk;
    const int kc = f2c(k, nh);
    const long long C = lin(gc, ic, jc, kc), F = lin(gf, i, j, k);
    const T x28 = A::mul(x[C], T(28));
#pragma unroll
    for (int dj = 0; dj <= 1; ++dj)
#pragma unroll
      for (int di = 0; di <= 1; ++di) {
        const long long ddi = 2 * di - 1, ddj = (2 * dj - 1) * c1;
        T a = square3(x, C, ddi, ddj, -c2);
        T bb = A::mul(square3(x, C, ddi, ddj, 0LL), T(3));
        T c = square3(x, C, ddi, ddj, c2);
        long long F0 = F + di + dj * f1, F1 = F0 + f2;
        xf[F0] = A::add(ASSIGN ? T(0) : xf[F0], A::mul(coef[F0], A::add(A::add(bb, a), x28)));
        xf[F1] = A::add(ASSIGN ? T(0) : xf[F1], A::mul(coef[F1], A::add(A::add(bb, c), x28)));
      }
  } else if (KIND == 2) {
    const int k = kf0 + qk;
    const long long C = lin(gc, ic, jc, k), F = lin(gf, i, j, k);
    const T x00 = x[C], x10 = x[C + 1], x01 = x[C + c1], x11 = x[C + 1 + c1];
    const long long o[4] = {0, 1, f1, 1 + f1};
    T cf[4], xo[4];  // loads of the four children first, as in KIND 0
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      cf[c] = coef[F + o[c]];
      xo[c] = ASSIGN ? T(0) : xf[F + o[c]];
    }
    xf[F] = A::add(xo[0], A::mul(cf[0], x00));
    xf[F + 1] = A::add(xo[1], A::mul(cf[1], A::add(x00, x10)));
    xf[F + f1] = A::add(xo[2], A::mul(cf[2], A::add(x00, x01)));
    xf[F + 1 + f1] = A::add(xo[3], A::mul(cf[3], A::add(A::add(A::add(x00, x10), x01), x11)));
  } else {
    const int k = nh + 1 + 2 * qk;
    const int kc = f2c(k, nh);
    const long long C = lin(gc, ic, jc, kc), F = lin(gf, i, j, k);
    const T x000 = x[C], x100 = x[C + 1], x010 = x[C + c1], x001 = x[C + c2];
    const T x110 = x[C + 1 + c1], x101 = x[C + 1 + c2], x011 = x[C + c1 + c2], x111 = x[C + 1 + c1 + c2];
    auto upd = [&](long long Fi, T v) { xf[Fi] = A::add(ASSIGN ? T(0) : xf[Fi], A::mul(coef[Fi], v)); };
    upd(F, x000);
    upd(F + 1, A::add(x000, x100));
    upd(F + f1, A::add(x000, x010));
    upd(F + f2, A::add(x000, x001));
    upd(F + 1 + f1, A::add(A::add(A::add(x000, x100), x010), x110));
    upd(F + 1 + f2, A::add(A::add(A::add(x000, x100), x001), x101));
    upd(F + f1 + f2, A::add(A::add(A::add(x000, x001), x010), x011));
    T s = A::add(x000, x100);
    s = A::add(s, x001);
    s = A::add(s, x101);
    s = A::add(s, x010);
    s = A::add(s, x110);
    s = A::add(s, x011);
    s = A::add(s, x111);
    upd(F + 1 + f1 + f2, s);
  }
}

// ------------------------------------------------------- fixed point
// Integer form of the mixed loop's level-1 residual (k_mixed.cu, k_batch.cu).
// round(v * 2^k) for |v| 2^k < 2^59, ties away from zero; zero and
// subnormal v give 0. Branch-free: with M = m << 10 (m the 53-bit
// significand, v = m 2^(ex-1075)), round(m 2^sh) = ((M >> (t-1)) + 1) >> 1
// for t = 10 - sh: the range bound keeps sh <= 5, so t >= 5, and t is
// capped at 64, where the result is 0 as for any shift past the significand.
__device__ __forceinline__ long long to_fix(double v, int k) {
  const long long u = __double_as_longlong(v);
  const int ex = (int)(((unsigned long long)u >> 52) & 0x7ffULL);
  const unsigned long long M = (((unsigned long long)u & 0x000FFFFFFFFFFFFFULL) | 0x0010000000000000ULL) << 10;
  const int t = min(max(1085 - ex - k, 1), 64);
  const long long r = ex ? (long long)(((M >> (t - 1)) + 1ULL) >> 1) : 0LL;
  return u < 0 ? -r : r;
}
// k = 58 - E for max(|x|, |b|) < 2^E (device scalars S_MAXX, S_MAXB)
__device__ __forceinline__ int fix_exponent(const double* ds) {
  const double mx = fmax(ds[S_MAXX], ds[S_MAXB]);
  int e = 0;
  if (mx > 0 && isfinite(mx)) frexp(mx, &e);  // mx < 2^e
  return 58 - e;
}

// e * 2^p as a double, exactly, with integer operations on the bits of the
// float (the FP64 pipe then only adds: x + e*2^p rounds once, as
// fma((double)e, 2^p, x) does). Zeros keep their sign; subnormal, infinite
// and NaN e, and a result outside the normal range, take the FP64 path
// (s2p = 2^p as a double).
// the FP64 product for the rare e that the bit assembly does not cover; out
// of line, so that it stays a branch that only warps holding such an e take
// (inline, the compiler predicates it and every cell pays the FP64 pipe)
static __device__ __noinline__ double f2d_pow2_slow(float e, double s2p) { return __dmul_rn((double)e, s2p); }
__device__ __forceinline__ double f2d_pow2(float e, int p, double s2p) {
  // zero and normal e by integer operations on the bits, with no branch:
  // a divergent branch here had the compiler issue the caller's FP64 add on
  // both paths
  const unsigned u = __float_as_uint(e);
  const unsigned long long sgn = (unsigned long long)(u >> 31) << 63;
  const int ex = (int)((u >> 23) & 0xffu);
  const int dex = ex - 127 + 1023 + p;
  const bool zero = (u & 0x7fffffffu) == 0u;
  const bool normal = ex != 0 && ex != 255 && dex > 0 && dex < 2047;
  const unsigned long long bits =
      sgn | ((unsigned long long)(unsigned)dex << 52) | ((unsigned long long)(u & 0x7fffffu) << 29);
  double v = __longlong_as_double((long long)(zero ? sgn : bits));
  if (!zero && !normal) v = f2d_pow2_slow(e, s2p);
  return v;
}
// the exponent p of a power of two 2^p held in a double
__device__ __forceinline__ int pow2_exponent(double v) {
  return (int)(((unsigned long long)__double_as_longlong(v) >> 52) & 0x7ffULL) - 1023;
}

// ------------------------------------------------------------------ halo
// fill! for :xperio (src/halo.jl:6-9) on one (j,k) line. Each statement's
// right-hand columns are read before any is written, as Julia's sliced
// assignment does (this matters when nx < nh).
constexpr int kMaxNh = 8;
template <class T>
__device__ __forceinline__ void d_fill_line(T* row, int tx, int nh) {
  T tmp[kMaxNh];
#pragma unroll
  for (int i = 0; i < kMaxNh; ++i)
    if (i < nh) tmp[i] = row[tx - 2 * nh + i];
#pragma unroll
  for (int i = 0; i < kMaxNh; ++i)
    if (i < nh) row[i] = tmp[i];
#pragma unroll
  for (int i = 0; i < kMaxNh; ++i)
    if (i < nh) tmp[i] = row[nh + i];
#pragma unroll
  for (int i = 0; i < kMaxNh; ++i)
    if (i < nh) row[tx - nh + i] = tmp[i];
}

}  // namespace cfmg
