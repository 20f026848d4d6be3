// Per-level multigrid operators: Jacobi sweeps, residuals, restriction,
// prolongation, periodic halo fill and the masked norm.
//
// Instantiated for double (the FP64 drop-in) and float (the cycles of the
// mixed-precision form). Every sum and product goes through the _rn
// intrinsics so that nvcc cannot contract a multiply and an add into one
// FMA: the FP64 instantiation rounds exactly where the Julia reference
// rounds, and is bit-identical to it. The only FMAs used are ones whose
// product is exact (a multiplication by 1/2, 1/4, 2, 4 or 8), which round
// once on the same exact value as the reference's two-step form.
//
// These kernels are single-pass and keep the reference's own loop ranges,
// halo cells included; they are FP64-issue bound on GB300 (the FP64 pipe
// runs at 1/64 of the FP32 rate), so their memory traffic is not the limit.
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

constexpr int kThreads = 256;

inline unsigned nblocks(long long n, int per = kThreads) { return (unsigned)((n + per - 1) / per); }

// ----------------------------------------------------------------- sweeps
// sloop2d! (src/laplacian.jl:66-73): y = (1-w)x - (w*idiag)*(b - s4) over
// the linear range 1+n1 .. length-n1.
template <class T>
__global__ void __launch_bounds__(kThreads) k_sweep5_2d(const T* __restrict__ x, T* __restrict__ y,
                                                        const T* __restrict__ b, const T* __restrict__ w, T cff,
                                                        long long n1, long long lo, long long hi) {
  long long I = lo + (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (I >= hi) return;
  typedef Ar<T> A;
  T s = A::add(A::add(A::add(x[I - 1], x[I + 1]), x[I - n1]), x[I + n1]);
  y[I] = A::sub(A::mul(cff, x[I]), A::mul(w[I], A::sub(b[I], s)));
}

// sloop3d_v1! (src/laplacian.jl:11-20): 7-point, linear range 1+n2 .. length-n2.
template <class T>
__global__ void __launch_bounds__(kThreads) k_sweep7_3d(const T* __restrict__ x, T* __restrict__ y,
                                                        const T* __restrict__ b, const T* __restrict__ w, T cff,
                                                        long long n1, long long n2, long long lo, long long hi) {
  long long I = lo + (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (I >= hi) return;
  typedef Ar<T> A;
  T s = A::add(A::add(A::add(A::add(A::add(x[I - 1], x[I + 1]), x[I - n1]), x[I + n1]), x[I - n2]), x[I + n2]);
  y[I] = A::sub(A::mul(cff, x[I]), A::mul(w[I], A::sub(b[I], s)));
}

// Thread mapping of a box kernel: x over i, y over j, z over k.
struct BoxIdx {
  int i, j, k;
  bool ok;
};
__device__ __forceinline__ BoxIdx box_idx(const Box& bx) {
  BoxIdx r;
  r.i = bx.i0 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
  r.j = bx.j0 + (int)(blockIdx.y * blockDim.y + threadIdx.y);
  r.k = bx.k0 + (int)blockIdx.z;
  r.ok = r.i <= bx.i1 && r.j <= bx.j1 && r.k <= bx.k1;
  return r;
}
inline dim3 box_grid(const Box& bx, dim3 blk) {
  int ni = bx.i1 - bx.i0 + 1, nj = bx.j1 - bx.j0 + 1, nk = bx.k1 - bx.k0 + 1;
  return dim3((unsigned)((ni + blk.x - 1) / blk.x), (unsigned)((nj + blk.y - 1) / blk.y), (unsigned)nk);
}
inline bool box_empty(const Box& bx) { return bx.i1 < bx.i0 || bx.j1 < bx.j0 || bx.k1 < bx.k0; }
static const dim3 kBoxBlk(64, 4, 1);

// In-plane part of laplacian9 (2D 9-point extension): faces/2, diagonals/4.
template <class T>
__device__ __forceinline__ T faces4(const T* x, long long I, long long n1) {
  typedef Ar<T> A;
  return A::add(A::add(A::add(x[I - 1], x[I + 1]), x[I - n1]), x[I + n1]);
}
template <class T>
__device__ __forceinline__ T diags4(const T* x, long long I, long long n1) {
  typedef Ar<T> A;
  return A::add(A::add(A::add(x[I - 1 - n1], x[I + 1 - n1]), x[I - 1 + n1]), x[I + 1 + n1]);
}

template <class T>
__global__ void __launch_bounds__(kThreads) k_sweep9_2d(const T* __restrict__ x, T* __restrict__ y,
                                                        const T* __restrict__ b, const T* __restrict__ w, T cff,
                                                        Geom g, Box bx) {
  BoxIdx q = box_idx(bx);
  if (!q.ok) return;
  typedef Ar<T> A;
  long long I = lin(g, q.i, q.j, q.k);
  T t = A::fmx(faces4(x, I, g.n1), T(-0.5), b[I]);   // b - faces/2
  t = A::fmx(diags4(x, I, g.n1), T(-0.25), t);      // - diagonals/4
  y[I] = A::sub(A::mul(cff, x[I]), A::mul(w[I], t));
}

// 19-point stencil of smooth_laplacian9! (src/laplacian9.jl:14-44).
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
__global__ void __launch_bounds__(kThreads) k_sweep19_3d(const T* __restrict__ x, T* __restrict__ y,
                                                         const T* __restrict__ b, const T* __restrict__ w, T cff,
                                                         Geom g, Box bx) {
  BoxIdx q = box_idx(bx);
  if (!q.ok) return;
  typedef Ar<T> A;
  long long I = lin(g, q.i, q.j, q.k);
  T t = A::fmx(faces6(x, I, g.n1, g.n2), T(-0.5), b[I]);
  t = A::fmx(edges12(x, I, g.n1, g.n2), T(-0.25), t);
  y[I] = A::sub(A::mul(cff, x[I]), A::mul(w[I], t));
}

// Variable-coefficient 5-point sweep over sloop2d!'s linear range.
template <class T>
__device__ __forceinline__ T vc_sum(const T* x, const T* cE, const T* cN, long long I, long long n1) {
  typedef Ar<T> A;
  T s = A::add(A::mul(cE[I - 1], x[I - 1]), A::mul(cE[I], x[I + 1]));
  s = A::add(s, A::mul(cN[I - n1], x[I - n1]));
  return A::add(s, A::mul(cN[I], x[I + n1]));
}

template <class T>
__global__ void __launch_bounds__(kThreads) k_sweep_vc_2d(const T* __restrict__ x, T* __restrict__ y,
                                                          const T* __restrict__ b, const T* __restrict__ w,
                                                          const T* __restrict__ cE, const T* __restrict__ cN, T cff,
                                                          long long n1, long long lo, long long hi) {
  long long I = lo + (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (I >= hi) return;
  typedef Ar<T> A;
  T s = vc_sum(x, cE, cN, I, n1);
  y[I] = A::sub(A::mul(cff, x[I]), A::mul(w[I], A::sub(b[I], s)));
}

// -------------------------------------------------------------- residuals
// rloop2d! (src/laplacian.jl:87-93): r = msk*((diag*x + b) - s4).
template <class T>
__global__ void __launch_bounds__(kThreads) k_resid5_2d(T* __restrict__ r, const T* __restrict__ x,
                                                        const T* __restrict__ b, const T* __restrict__ d,
                                                        const uint8_t* __restrict__ m, long long n1, long long lo,
                                                        long long hi) {
  long long I = lo + (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (I >= hi) return;
  typedef Ar<T> A;
  T s = A::add(A::add(A::add(x[I - 1], x[I + 1]), x[I - n1]), x[I + n1]);
  r[I] = mask_mul(m[I], A::sub(A::add(A::mul(d[I], x[I]), b[I]), s));
}

// rloop3d! (src/laplacian.jl:43-51): interior box only.
template <class T>
__global__ void __launch_bounds__(kThreads) k_resid7_3d(T* __restrict__ r, const T* __restrict__ x,
                                                        const T* __restrict__ b, const T* __restrict__ d,
                                                        const uint8_t* __restrict__ m, Geom g, Box bx) {
  BoxIdx q = box_idx(bx);
  if (!q.ok) return;
  typedef Ar<T> A;
  long long I = lin(g, q.i, q.j, q.k);
  T s = faces6(x, I, g.n1, g.n2);
  r[I] = mask_mul(m[I], A::sub(A::add(A::mul(d[I], x[I]), b[I]), s));
}

// residual of the 2D 9-point extension, interior box.
template <class T>
__global__ void __launch_bounds__(kThreads) k_resid9_2d(T* __restrict__ r, const T* __restrict__ x,
                                                        const T* __restrict__ b, const T* __restrict__ d,
                                                        const uint8_t* __restrict__ m, Geom g, Box bx) {
  BoxIdx q = box_idx(bx);
  if (!q.ok) return;
  typedef Ar<T> A;
  long long I = lin(g, q.i, q.j, q.k);
  T v = A::add(A::mul(d[I], x[I]), b[I]);
  v = A::fmx(faces4(x, I, g.n1), T(-0.5), v);
  v = A::fmx(diags4(x, I, g.n1), T(-0.25), v);
  r[I] = mask_mul(m[I], v);
}

// residual_laplacian9! (src/laplacian9.jl:49-73), interior box.
template <class T>
__global__ void __launch_bounds__(kThreads) k_resid19_3d(T* __restrict__ r, const T* __restrict__ x,
                                                         const T* __restrict__ b, const T* __restrict__ d,
                                                         const uint8_t* __restrict__ m, Geom g, Box bx) {
  BoxIdx q = box_idx(bx);
  if (!q.ok) return;
  typedef Ar<T> A;
  long long I = lin(g, q.i, q.j, q.k);
  T v = A::add(A::mul(d[I], x[I]), b[I]);
  v = A::fmx(faces6(x, I, g.n1, g.n2), T(-0.5), v);
  v = A::fmx(edges12(x, I, g.n1, g.n2), T(-0.25), v);
  r[I] = mask_mul(m[I], v);
}

template <class T>
__global__ void __launch_bounds__(kThreads) k_resid_vc_2d(T* __restrict__ r, const T* __restrict__ x,
                                                          const T* __restrict__ b, const T* __restrict__ d,
                                                          const T* __restrict__ cE, const T* __restrict__ cN,
                                                          const uint8_t* __restrict__ m, long long n1, long long lo,
                                                          long long hi) {
  long long I = lo + (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (I >= hi) return;
  typedef Ar<T> A;
  T s = vc_sum(x, cE, cN, I, n1);
  r[I] = mask_mul(m[I], A::sub(A::add(A::mul(d[I], x[I]), b[I]), s));
}

// ------------------------------------------------------------ restriction
__device__ __forceinline__ int c2f(int i, int nh) { return (i - nh - 1) * 2 + nh + 1; }  // src/gmg_types.jl:25

// Thread per coarse interior cell (ii, jj, kk); the coarse b is written.
template <class T, int KIND>
__global__ void __launch_bounds__(kThreads) k_restrict(const T* __restrict__ x, T* __restrict__ xc,
                                                       const T* __restrict__ coef, Geom gf, Geom gc, Box cb) {
  BoxIdx q = box_idx(cb);
  if (!q.ok) return;
  typedef Ar<T> A;
  const int nh = gc.nh;
  const int i = c2f(q.i, nh), j = c2f(q.j, nh);
  const long long n1 = gf.n1, n2 = gf.n2;
  T s;
  if (KIND == 0) {  // rcloop2d! (src/RP_on_centers.jl:117-133)
    long long F = lin(gf, i, j, q.k);
    s = A::add(A::add(A::add(x[F], x[F + 1]), x[F + n1]), x[F + 1 + n1]);
  } else if (KIND == 1) {  // rcloop3d! (src/RP_on_centers.jl:5-23)
    long long F = lin(gf, i, j, c2f(q.k, nh));
    s = A::add(x[F], x[F + 1]);
    s = A::add(s, x[F + n1]);
    s = A::add(s, x[F + 1 + n1]);
    s = A::add(s, x[F + n2]);
    s = A::add(s, x[F + 1 + n2]);
    s = A::add(s, x[F + n1 + n2]);
    s = A::add(s, x[F + 1 + n1 + n2]);
  } else if (KIND == 2) {  // rvloop2d! (src/RP_on_vertices.jl:96-115): 1-2-1 x 1-2-1
    long long F = lin(gf, i, j, q.k);
    s = A::fmx(x[F - n1], T(2), x[F - 1 - n1]);
    s = A::add(s, x[F + 1 - n1]);
    s = A::fmx(x[F - 1], T(2), s);
    s = A::fmx(x[F], T(4), s);
    s = A::fmx(x[F + 1], T(2), s);
    s = A::add(s, x[F - 1 + n1]);
    s = A::fmx(x[F + n1], T(2), s);
    s = A::add(s, x[F + 1 + n1]);
  } else {  // restriction_vertices! (src/RP_on_vertices.jl:1-32): 27 points, 1-2-4-8
    long long F = lin(gf, i, j, c2f(q.k, nh));
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
  long long C = lin(gc, q.i, q.j, q.k);
  xc[C] = A::mul(coef[C], s);
}

// ----------------------------------------------------------- prolongation
__device__ __forceinline__ int f2c(int i, int nh) { return (i - nh - 1) / 2 + nh + 1; }  // src/gmg_types.jl:26

// square (src/RP_on_centers.jl:1-3): 3*(x[i+di,j,k+dk]+x[i,j+dj,k+dk]) + x[i+di,j+dj,k+dk]
template <class T>
__device__ __forceinline__ T square3(const T* x, long long C, long long di, long long dj, long long dk) {
  typedef Ar<T> A;
  return A::add(A::mul(T(3), A::add(x[C + di + dk], x[C + dj + dk])), x[C + di + dj + dk]);
}

// Thread per fine parent (i, j, k) = (nh+1+2p, nh+1+2q, ...); each parent
// updates its 4 (2D) or 8 (3D) children, which no other thread touches.
template <class T, int KIND>
__global__ void __launch_bounds__(kThreads) k_prolong(T* __restrict__ xf, const T* __restrict__ x,
                                                      const T* __restrict__ coef, Geom gf, Geom gc, int np_i,
                                                      int np_j, int kf0, int kf1, int np_k) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  const int qj = blockIdx.y * blockDim.y + threadIdx.y;
  const int qk = blockIdx.z;
  if (p >= np_i || qj >= np_j) return;
  typedef Ar<T> A;
  const int nh = gf.nh;
  const int i = nh + 1 + 2 * p, j = nh + 1 + 2 * qj;
  const int ic = f2c(i, nh), jc = f2c(j, nh);
  const long long c1 = gc.n1, c2 = gc.n2, f1 = gf.n1, f2 = gf.n2;
  if (KIND == 0) {  // pcloop2d! (src/RP_on_centers.jl:146-163)
    const int k = kf0 + qk;
    if (k > kf1) return;
    const long long C = lin(gc, ic, jc, k), F = lin(gf, i, j, k);
    const T x9 = A::mul(x[C], T(9));
#pragma unroll
    for (int dj = 0; dj <= 1; ++dj)
#pragma unroll
      for (int di = 0; di <= 1; ++di) {
        T bb = square3(x, C, (long long)(2 * di - 1), (2 * dj - 1) * c1, 0LL);
        long long Fi = F + di + dj * f1;
        xf[Fi] = A::add(xf[Fi], A::mul(coef[Fi], A::add(bb, x9)));
      }
  } else if (KIND == 1) {  // pcloop3d! (src/RP_on_centers.jl:84-104)
    if (qk >= np_k) return;
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
        xf[F0] = A::add(xf[F0], A::mul(coef[F0], A::add(A::add(bb, a), x28)));
        xf[F1] = A::add(xf[F1], A::mul(coef[F1], A::add(A::add(bb, c), x28)));
      }
  } else if (KIND == 2) {  // pvloop2d! (src/RP_on_vertices.jl:117-137)
    const int k = kf0 + qk;
    if (k > kf1) return;
    const long long C = lin(gc, ic, jc, k), F = lin(gf, i, j, k);
    const T x00 = x[C], x10 = x[C + 1], x01 = x[C + c1], x11 = x[C + 1 + c1];
    xf[F] = A::add(xf[F], A::mul(coef[F], x00));
    xf[F + 1] = A::add(xf[F + 1], A::mul(coef[F + 1], A::add(x00, x10)));
    xf[F + f1] = A::add(xf[F + f1], A::mul(coef[F + f1], A::add(x00, x01)));
    xf[F + 1 + f1] = A::add(xf[F + 1 + f1], A::mul(coef[F + 1 + f1], A::add(A::add(A::add(x00, x10), x01), x11)));
  } else {  // prolongation_vertices! (src/RP_on_vertices.jl:34-72)
    if (qk >= np_k) return;
    const int k = nh + 1 + 2 * qk;
    const int kc = f2c(k, nh);
    const long long C = lin(gc, ic, jc, kc), F = lin(gf, i, j, k);
    const T x000 = x[C], x100 = x[C + 1], x010 = x[C + c1], x001 = x[C + c2];
    const T x110 = x[C + 1 + c1], x101 = x[C + 1 + c2], x011 = x[C + c1 + c2], x111 = x[C + 1 + c1 + c2];
    auto upd = [&](long long Fi, T v) { xf[Fi] = A::add(xf[Fi], A::mul(coef[Fi], v)); };
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

// ------------------------------------------------------------------- halo
// fill! for :xperio (src/halo.jl:6-9). One thread per (j,k) line copies the
// nh columns through registers, so the copies of each statement read
// before they write, as Julia's sliced assignment does.
constexpr int kMaxNh = 8;
template <class T>
__global__ void __launch_bounds__(kThreads) k_fill_xperio(T* __restrict__ x, int tx, int nh, long long nlines) {
  long long L = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (L >= nlines) return;
  T* row = x + L * tx;
  T tmp[kMaxNh];
#pragma unroll
  for (int i = 0; i < kMaxNh; ++i)
    if (i < nh) tmp[i] = row[tx - 2 * nh + i];  // x[end+1-2nh : end-nh]
#pragma unroll
  for (int i = 0; i < kMaxNh; ++i)
    if (i < nh) row[i] = tmp[i];  // -> x[1:nh]
#pragma unroll
  for (int i = 0; i < kMaxNh; ++i)
    if (i < nh) tmp[i] = row[nh + i];  // x[nh+1 : 2nh]
#pragma unroll
  for (int i = 0; i < kMaxNh; ++i)
    if (i < nh) row[tx - nh + i] = tmp[i];  // -> x[end+1-nh : end]
}

// ------------------------------------------------------------------- norm
// Deterministic two-stage reduction: block b sums the elements b, b+P,
// b+2P, ... strided by the whole grid (fixed grid of kNormParts blocks),
// then one block adds the kNormParts partials in a fixed tree.
template <class T>
__global__ void __launch_bounds__(kThreads) k_norm_partial(const T* __restrict__ x, const uint8_t* __restrict__ m,
                                                           long long n, double* __restrict__ partials) {
  double s = 0.0;
  for (long long I = (long long)blockIdx.x * blockDim.x + threadIdx.x; I < n; I += (long long)gridDim.x * blockDim.x) {
    uint8_t mm = m[I];
    if (mm) {
      double v = (double)x[I];
      s = (mm == 1) ? __fma_rn(v, v, s) : __dadd_rn(s, __dmul_rn((double)mm, __dmul_rn(v, v)));
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s = __dadd_rn(s, __shfl_down_sync(0xffffffffu, s, o));
  __shared__ double ws[kThreads / 32];
  if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    s = threadIdx.x < kThreads / 32 ? ws[threadIdx.x] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s = __dadd_rn(s, __shfl_down_sync(0xffffffffu, s, o));
    if (threadIdx.x == 0) partials[blockIdx.x] = s;
  }
}

__global__ void __launch_bounds__(kNormParts) k_norm_final(const double* __restrict__ partials, double* out,
                                                           const double* normb, int norm_kind) {
  __shared__ double sh[kNormParts];
  sh[threadIdx.x] = partials[threadIdx.x];
  __syncthreads();
  for (int w = kNormParts / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) sh[threadIdx.x] = __dadd_rn(sh[threadIdx.x], sh[threadIdx.x + w]);
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    double sum = sh[0];
    if (norm_kind == CFMG_NORM_REF_SQUARED) {
      if (sum == 0.0) sum = 1.0;
      out[0] = sum;
      if (normb) out[1] = (*normb > 0.0) ? sum / *normb : 0.0;
    } else {
      out[0] = sum;
      if (normb) out[1] = (*normb > 0.0) ? sqrt(sum / *normb) : 0.0;
    }
  }
}

// --------------------------------------------------------------- launchers
template <class T>
void launch_sweep5_2d(const T* x, T* y, const T* b, const T* w, T cff, const Geom& g, cudaStream_t s) {
  long long lo = g.n1, hi = g.len - g.n1;
  if (hi <= lo) return;
  k_sweep5_2d<T><<<nblocks(hi - lo), kThreads, 0, s>>>(x, y, b, w, cff, g.n1, lo, hi);
}
template <class T>
void launch_sweep7_3d(const T* x, T* y, const T* b, const T* w, T cff, const Geom& g, cudaStream_t s) {
  long long lo = g.n2, hi = g.len - g.n2;
  if (hi <= lo) return;
  k_sweep7_3d<T><<<nblocks(hi - lo), kThreads, 0, s>>>(x, y, b, w, cff, g.n1, g.n2, lo, hi);
}
template <class T>
void launch_sweep9_2d(const T* x, T* y, const T* b, const T* w, T cff, const Geom& g, const Box& bx,
                      cudaStream_t s) {
  if (box_empty(bx)) return;
  k_sweep9_2d<T><<<box_grid(bx, kBoxBlk), kBoxBlk, 0, s>>>(x, y, b, w, cff, g, bx);
}
template <class T>
void launch_sweep19_3d(const T* x, T* y, const T* b, const T* w, T cff, const Geom& g, const Box& bx,
                       cudaStream_t s) {
  if (box_empty(bx)) return;
  k_sweep19_3d<T><<<box_grid(bx, kBoxBlk), kBoxBlk, 0, s>>>(x, y, b, w, cff, g, bx);
}
template <class T>
void launch_sweep_vc_2d(const T* x, T* y, const T* b, const T* w, const T* cE, const T* cN, T cff, const Geom& g,
                        cudaStream_t s) {
  long long lo = g.n1, hi = g.len - g.n1;
  if (hi <= lo) return;
  k_sweep_vc_2d<T><<<nblocks(hi - lo), kThreads, 0, s>>>(x, y, b, w, cE, cN, cff, g.n1, lo, hi);
}
template <class T>
void launch_resid5_2d(T* r, const T* x, const T* b, const T* d, const uint8_t* m, const Geom& g, cudaStream_t s) {
  long long lo = g.n1, hi = g.len - g.n1;
  if (hi <= lo) return;
  k_resid5_2d<T><<<nblocks(hi - lo), kThreads, 0, s>>>(r, x, b, d, m, g.n1, lo, hi);
}
template <class T>
void launch_resid7_3d(T* r, const T* x, const T* b, const T* d, const uint8_t* m, const Geom& g, const Box& bx,
                      cudaStream_t s) {
  if (box_empty(bx)) return;
  k_resid7_3d<T><<<box_grid(bx, kBoxBlk), kBoxBlk, 0, s>>>(r, x, b, d, m, g, bx);
}
template <class T>
void launch_resid9_2d(T* r, const T* x, const T* b, const T* d, const uint8_t* m, const Geom& g, const Box& bx,
                      cudaStream_t s) {
  if (box_empty(bx)) return;
  k_resid9_2d<T><<<box_grid(bx, kBoxBlk), kBoxBlk, 0, s>>>(r, x, b, d, m, g, bx);
}
template <class T>
void launch_resid19_3d(T* r, const T* x, const T* b, const T* d, const uint8_t* m, const Geom& g, const Box& bx,
                       cudaStream_t s) {
  if (box_empty(bx)) return;
  k_resid19_3d<T><<<box_grid(bx, kBoxBlk), kBoxBlk, 0, s>>>(r, x, b, d, m, g, bx);
}
template <class T>
void launch_resid_vc_2d(T* r, const T* x, const T* b, const T* d, const T* cE, const T* cN, const uint8_t* m,
                        const Geom& g, cudaStream_t s) {
  long long lo = g.n1, hi = g.len - g.n1;
  if (hi <= lo) return;
  k_resid_vc_2d<T><<<nblocks(hi - lo), kThreads, 0, s>>>(r, x, b, d, cE, cN, m, g.n1, lo, hi);
}
template <class T>
void launch_restrict(int kind, const T* xf, T* bc, const T* Rcoef, const Geom& gf, const Geom& gc, const Box& cb,
                     cudaStream_t s) {
  if (box_empty(cb)) return;
  dim3 grid = box_grid(cb, kBoxBlk);
  switch (kind) {
    case 0: k_restrict<T, 0><<<grid, kBoxBlk, 0, s>>>(xf, bc, Rcoef, gf, gc, cb); break;
    case 1: k_restrict<T, 1><<<grid, kBoxBlk, 0, s>>>(xf, bc, Rcoef, gf, gc, cb); break;
    case 2: k_restrict<T, 2><<<grid, kBoxBlk, 0, s>>>(xf, bc, Rcoef, gf, gc, cb); break;
    default: k_restrict<T, 3><<<grid, kBoxBlk, 0, s>>>(xf, bc, Rcoef, gf, gc, cb); break;
  }
}
template <class T>
void launch_prolong(int kind, T* xf, const T* xc, const T* Pcoef, const Geom& gf, const Geom& gc, int nxf, int nyf,
                    int nzf, int kf0, int kf1, cudaStream_t s) {
  // parents: i = nh+1 : 2 : nx+nh (likewise j, and k in 3D)
  const int np_i = (nxf + 1) / 2, np_j = (nyf + 1) / 2;
  const bool threed = (kind == 1 || kind == 3);
  const int np_k = threed ? (nzf + 1) / 2 : (kf1 - kf0 + 1);
  if (np_i <= 0 || np_j <= 0 || np_k <= 0) return;
  dim3 blk(64, 4, 1);
  dim3 grid((unsigned)((np_i + 63) / 64), (unsigned)((np_j + 3) / 4), (unsigned)np_k);
  switch (kind) {
    case 0: k_prolong<T, 0><<<grid, blk, 0, s>>>(xf, xc, Pcoef, gf, gc, np_i, np_j, kf0, kf1, np_k); break;
    case 1: k_prolong<T, 1><<<grid, blk, 0, s>>>(xf, xc, Pcoef, gf, gc, np_i, np_j, kf0, kf1, np_k); break;
    case 2: k_prolong<T, 2><<<grid, blk, 0, s>>>(xf, xc, Pcoef, gf, gc, np_i, np_j, kf0, kf1, np_k); break;
    default: k_prolong<T, 3><<<grid, blk, 0, s>>>(xf, xc, Pcoef, gf, gc, np_i, np_j, kf0, kf1, np_k); break;
  }
}
template <class T>
void launch_fill_xperio(T* x, const Geom& g, cudaStream_t s) {
  long long nlines = (long long)g.ty * g.tz;
  k_fill_xperio<T><<<nblocks(nlines), kThreads, 0, s>>>(x, g.tx, g.nh, nlines);
}
template <class T>
void launch_norm(const T* x, const uint8_t* m, size_t n, double* partials, double* out, const double* normb,
                 int norm_kind, cudaStream_t s) {
  k_norm_partial<T><<<kNormParts, kThreads, 0, s>>>(x, m, (long long)n, partials);
  k_norm_final<<<1, kNormParts, 0, s>>>(partials, out, normb, norm_kind);
}

#define CFMG_INST(T)                                                                                             \
  template void launch_sweep5_2d<T>(const T*, T*, const T*, const T*, T, const Geom&, cudaStream_t);            \
  template void launch_sweep7_3d<T>(const T*, T*, const T*, const T*, T, const Geom&, cudaStream_t);            \
  template void launch_sweep9_2d<T>(const T*, T*, const T*, const T*, T, const Geom&, const Box&, cudaStream_t); \
  template void launch_sweep19_3d<T>(const T*, T*, const T*, const T*, T, const Geom&, const Box&,              \
                                     cudaStream_t);                                                              \
  template void launch_sweep_vc_2d<T>(const T*, T*, const T*, const T*, const T*, const T*, T, const Geom&,      \
                                      cudaStream_t);                                                             \
  template void launch_resid5_2d<T>(T*, const T*, const T*, const T*, const uint8_t*, const Geom&, cudaStream_t); \
  template void launch_resid7_3d<T>(T*, const T*, const T*, const T*, const uint8_t*, const Geom&, const Box&,   \
                                    cudaStream_t);                                                               \
  template void launch_resid9_2d<T>(T*, const T*, const T*, const T*, const uint8_t*, const Geom&, const Box&,   \
                                    cudaStream_t);                                                               \
  template void launch_resid19_3d<T>(T*, const T*, const T*, const T*, const uint8_t*, const Geom&, const Box&,  \
                                     cudaStream_t);                                                              \
  template void launch_resid_vc_2d<T>(T*, const T*, const T*, const T*, const T*, const T*, const uint8_t*,      \
                                      const Geom&, cudaStream_t);                                                \
  template void launch_restrict<T>(int, const T*, T*, const T*, const Geom&, const Geom&, const Box&,            \
                                   cudaStream_t);                                                                \
  template void launch_prolong<T>(int, T*, const T*, const T*, const Geom&, const Geom&, int, int, int, int, int, \
                                  cudaStream_t);                                                                 \
  template void launch_fill_xperio<T>(T*, const Geom&, cudaStream_t);                                            \
  template void launch_norm<T>(const T*, const uint8_t*, size_t, double*, double*, const double*, int, cudaStream_t);

CFMG_INST(double)
CFMG_INST(float)
template void launch_fill_xperio<uint8_t>(uint8_t*, const Geom&, cudaStream_t);

}  // namespace cfmg
