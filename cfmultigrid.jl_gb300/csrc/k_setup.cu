// Element-wise kernels of the device-side operator setup
// (setup_operators!, src/gmg_setup.jl:264-366) and of the format
// conversions. The setup itself chains these with the restriction,
// prolongation and residual kernels, exactly as the reference drives its
// own operators through the function tables to derive the coefficients.
#include "cfmg_internal.h"

namespace cfmg {

constexpr int kT = 256;
inline unsigned nb(size_t n) { return (unsigned)((n + kT - 1) / kT); }

// Default mask value of cell (i,j,k) before fill! (get_default_msk!,
// src/gmg_setup.jl:289-308).
__device__ __forceinline__ uint8_t defmsk_raw(int i, int j, int k, int nx, int ny, int nz, int nh, bool vertices,
                                              bool threed) {
  if (vertices) {
    int k0 = threed ? nh + 1 : 1, k1 = threed ? nh + nz : nz;
    return (k >= k0 && k <= k1 && j >= nh + 2 && j <= ny + nh && i >= nh + 2 && i <= nx + nh) ? 1 : 0;
  }
  int k0 = threed ? nh + 1 : 1, k1 = threed ? nz + nh : nz;
  return (k >= k0 && k <= k1 && j >= nh + 1 && j <= ny + nh && i >= nh + 1 && i <= nx + nh) ? 1 : 0;
}

// mode SET: msk = default; MUL: msk *= default; SCALE_F64: f *= default*coef.
// With :xperio the halo columns take the value of their periodic partner
// (the fill! at the end of get_default_msk!).
__global__ void k_default_msk(int mode, uint8_t* msk, double* f, double coef, int nx, int ny, int nz, int nh,
                              int tx, int ty, long long len, bool vertices, bool threed, bool xperio) {
  dep_wait();
  long long I = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (I >= len) return;
  int i = (int)(I % tx) + 1;
  long long q = I / tx;
  int j = (int)(q % ty) + 1;
  int k = (int)(q / ty) + 1;
  int is = i;
  if (xperio) {
    if (i <= nh) is = i + nx;           // x[1:nh] = x[end+1-2nh:end-nh]
    else if (i > tx - nh) is = i - nx;  // x[end+1-nh:end] = x[nh+1:2nh]
  }
  uint8_t d = defmsk_raw(is, j, k, nx, ny, nz, nh, vertices, threed);
  if (mode == DEFMSK_SET) msk[I] = d;
  else if (mode == DEFMSK_MUL) msk[I] = (uint8_t)(msk[I] * d);
  else f[I] = __dmul_rn(f[I], __dmul_rn((double)d, coef));
}

void launch_default_msk(int mode, uint8_t* msk, double* f, double coef, const Level& l, bool vertices, bool threed,
                        bool xperio, cudaStream_t s) {
  launch_dep(k_default_msk, nb(l.len), kT, 0, s, mode, msk, f, coef, l.nx, l.ny, l.nz, l.nh, l.tx, l.ty, (long long)l.len, vertices, threed, xperio);
}

__global__ void k_fill_f64(double* a, double v, long long n) {
  dep_wait();
  long long I = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (I < n) a[I] = v;
}
void launch_fill_f64(double* a, double v, size_t n, cudaStream_t s) {
  launch_dep(k_fill_f64, nb(n), kT, 0, s, a, v, (long long)n);
}

__global__ void k_u8_to_f64(const uint8_t* m, double* out, long long n) {
  dep_wait();
  long long I = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (I < n) out[I] = (double)m[I];
}
void launch_u8_to_f64(const uint8_t* m, double* out, size_t n, cudaStream_t s) {
  launch_dep(k_u8_to_f64, nb(n), kT, 0, s, m, out, (long long)n);
}

// msk = b > threshold (compute_msk_dev, src/gmg_setup.jl:360-362)
__global__ void k_threshold(const double* b, uint8_t* msk, double thr, long long n) {
  dep_wait();
  long long I = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (I < n) msk[I] = (b[I] > thr) ? 1 : 0;
}
void launch_threshold(const double* b, uint8_t* msk, double thr, size_t n, cudaStream_t s) {
  launch_dep(k_threshold, nb(n), kT, 0, s, b, msk, thr, (long long)n);
}

// Rcoef = msk * f(b) (compute_Rcoef!, src/gmg_setup.jl:203-211)
__global__ void k_rcoef(const uint8_t* msk, const double* b, double* R, bool vertices, double coef, long long n) {
  dep_wait();
  long long I = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (I >= n) return;
  double bb = b[I];
  double fr = vertices ? ((bb > 0.0) ? coef : 0.0) : ((bb > 0.0) ? __ddiv_rn(4.0, bb) : 0.0);
  R[I] = __dmul_rn((double)msk[I], fr);
}
void launch_rcoef(const uint8_t* msk, const double* b, double* R, bool vertices, double coef, size_t n,
                  cudaStream_t s) {
  launch_dep(k_rcoef, nb(n), kT, 0, s, msk, b, R, vertices, coef, (long long)n);
}

// Pcoef = (x>0 ? 1/x : 0) * msk (compute_Pcoef!, src/gmg_setup.jl:232-236)
__global__ void k_pcoef(const uint8_t* msk, const double* x, double* P, long long n) {
  dep_wait();
  long long I = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (I >= n) return;
  double xv = x[I];
  P[I] = __dmul_rn((xv > 0) ? __ddiv_rn(1.0, xv) : 0.0, (double)msk[I]);
}
void launch_pcoef(const uint8_t* msk, const double* x, double* P, size_t n, cudaStream_t s) {
  launch_dep(k_pcoef, nb(n), kT, 0, s, msk, x, P, (long long)n);
}

// diag = -r*msk; idiag = diag>0 ? 1/diag : 0 (compute_diag!, src/gmg_setup.jl:258-261)
__global__ void k_diag(const uint8_t* msk, const double* r, double* diag, double* idiag, long long n) {
  dep_wait();
  long long I = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (I >= n) return;
  double d = __dmul_rn(-r[I], (double)msk[I]);
  diag[I] = d;
  idiag[I] = (d > 0.0) ? __ddiv_rn(1.0, d) : 0.0;
}
void launch_diag(const uint8_t* msk, const double* r, double* diag, double* idiag, size_t n, cudaStream_t s) {
  launch_dep(k_diag, nb(n), kT, 0, s, msk, r, diag, idiag, (long long)n);
}

// widiag = omega*idiag: the product the reference forms inside every sweep
// (src/laplacian.jl:69, `omega*idiag[I]`), computed once.
__global__ void k_widiag(const double* idiag, double* w, double omega, long long n) {
  dep_wait();
  long long I = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (I < n) w[I] = __dmul_rn(omega, idiag[I]);
}
void launch_widiag(const double* idiag, double* w, double omega, size_t n, cudaStream_t s) {
  launch_dep(k_widiag, nb(n), kT, 0, s, idiag, w, omega, (long long)n);
}

// Coarse kappa of the variable-coefficient operator: mean of kappa over the
// wet children (1 where none is wet); written on the coarse interior.
__global__ void k_restrict_kappa(const double* kf, const uint8_t* mf, double* kc, Geom gf, Geom gc, Box cb) {
  dep_wait();
  int ii = cb.i0 + (int)(blockIdx.x * blockDim.x + threadIdx.x);
  int jj = cb.j0 + (int)(blockIdx.y * blockDim.y + threadIdx.y);
  int kk = cb.k0 + (int)blockIdx.z;
  if (ii > cb.i1 || jj > cb.j1 || kk > cb.k1) return;
  int nh = gc.nh;
  int i = (ii - nh - 1) * 2 + nh + 1, j = (jj - nh - 1) * 2 + nh + 1;
  double s = 0.0, cnt = 0.0;
  for (int dj = 0; dj <= 1; ++dj)
    for (int di = 0; di <= 1; ++di) {
      long long F = (long long)(i + di - 1) + gf.n1 * ((long long)(j + dj - 1) + (long long)gf.ty * (kk - 1));
      if (mf[F]) {
        s = __dadd_rn(s, kf[F]);
        cnt = __dadd_rn(cnt, 1.0);
      }
    }
  long long C = (long long)(ii - 1) + gc.n1 * ((long long)(jj - 1) + (long long)gc.ty * (kk - 1));
  kc[C] = cnt > 0 ? __ddiv_rn(s, cnt) : 1.0;
}
void launch_restrict_kappa(const double* kf, const uint8_t* mf, double* kc, const Geom& gf, const Geom& gc,
                           const Box& cb, cudaStream_t s) {
  dim3 blk(64, 4, 1);
  dim3 grid((unsigned)((cb.i1 - cb.i0 + 64) / 64), (unsigned)((cb.j1 - cb.j0 + 4) / 4), (unsigned)(cb.k1 - cb.k0 + 1));
  launch_dep(k_restrict_kappa, grid, blk, 0, s, kf, mf, kc, gf, gc, cb);
}

// Face coefficients: cE[I] between I and I+1, cN[I] between I and I+n1,
// (kappa_I + kappa_J)/2 when both cells are wet, else 0.
__global__ void k_face_coef(const double* kap, const uint8_t* m, double* cE, double* cN, long long n1, long long n) {
  dep_wait();
  long long I = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (I >= n) return;
  double e = 0.0, nn = 0.0;
  if (I + 1 < n && m[I] && m[I + 1]) e = __dmul_rn(0.5, __dadd_rn(kap[I], kap[I + 1]));
  if (I + n1 < n && m[I] && m[I + n1]) nn = __dmul_rn(0.5, __dadd_rn(kap[I], kap[I + n1]));
  cE[I] = e;
  cN[I] = nn;
}
void launch_face_coef(const double* kappa, const uint8_t* msk, double* cE, double* cN, const Geom& g,
                      cudaStream_t s) {
  launch_dep(k_face_coef, nb((size_t)g.len), kT, 0, s, kappa, msk, cE, cN, g.n1, g.len);
}

__global__ void k_to_f32(const double* a, float* out, long long n) {
  dep_wait();
  long long I = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (I < n) out[I] = (float)a[I];
}
void launch_to_f32(const double* a, float* out, size_t n, cudaStream_t s) {
  launch_dep(k_to_f32, nb(n), kT, 0, s, a, out, (long long)n);
}

// The FP32 omega*idiag of every cell of the 5-, 7-, 9- and 19-point
// operators is a function of diag alone (k_diag, k_widiag), and diag is a
// multiple of 1/Q (Q = 1 for the 5- and 7-point operators, whose weights are
// 1; Q = 4 for the weights 1/2 and 1/4), so a one-byte code c = Q*diag and a
// table of 256 floats reproduce it: the table entries are computed with the
// same FP64 operations on the same exact diag = c/Q.
__global__ void k_wq_table(float* tab, double omega, double Q) {
  dep_wait();
  const int c = threadIdx.x;
  const double d = (double)c / Q;  // exact: c < 256 and Q a power of two
  const double id = (d > 0.0) ? __ddiv_rn(1.0, d) : 0.0;
  tab[c] = (float)__dmul_rn(omega, id);
}
void launch_wq_table(float* tab, double omega, double Q, cudaStream_t s) {
  launch_dep(k_wq_table, 1, 256, 0, s, tab, omega, Q);
}

__global__ void k_make_wq(const double* __restrict__ diag, const float* __restrict__ w32, const float* __restrict__ tab,
                          double Q, uint8_t* wq, long long n, int* ok) {
  dep_wait();
  const long long I = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (I >= n) return;
  const double d = diag[I];
  unsigned c = 0;
  if (d > 0.0) {
    const double qd = d * Q;
    if (qd >= 1.0 && qd <= 255.0 && qd == floor(qd)) c = (unsigned)qd;
    else atomicAnd(ok, 0);
  }
  if (__float_as_uint(tab[c]) != __float_as_uint(w32[I])) atomicAnd(ok, 0);
  wq[I] = (uint8_t)c;
}
void launch_make_wq(const double* diag, const float* w32, const float* tab, double Q, uint8_t* wq, long long n,
                    int* ok, cudaStream_t s) {
  launch_dep(k_make_wq, nb(n), kT, 0, s, diag, w32, tab, Q, wq, n, ok);
}

// qact[r * nq + t] = 1 when a cell of quad t (linear offsets 4t .. 4t+3 of a
// plane) is wet in one of the planes 1 + run*r .. of the 3D sweep range
// (0-based planes 1 .. tz-2); 0 when all of them are dry
__global__ void k_make_qact(const uint8_t* __restrict__ m, uint8_t* __restrict__ qact, long long n2, int tz, int run,
                            long long nq, int nruns) {
  dep_wait();
  const long long T = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (T >= nq * nruns) return;
  const int r = (int)(T / nq);
  const long long t = T - (long long)r * nq;
  const int k0 = 1 + r * run, k1 = min(k0 + run, tz - 1);
  unsigned any = 0;
  for (int k = k0; k < k1; ++k)
    for (int c = 0; c < 4; ++c) {
      const long long o = 4 * t + c;
      if (o < n2) any |= m[n2 * k + o];
    }
  qact[T] = any ? 1 : 0;
}
void launch_make_qact(const uint8_t* m, uint8_t* qact, long long n2, int tz, int run, cudaStream_t s) {
  const long long nq = (n2 + 3) / 4;
  const int nruns = (tz - 2 + run - 1) / run;
  if (nruns <= 0) return;
  launch_dep(k_make_qact, nb(nq * nruns), kT, 0, s, m, qact, n2, tz, run, nq, nruns);
}

}  // namespace cfmg
