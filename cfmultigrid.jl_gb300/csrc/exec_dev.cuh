// Per-item execution of an Op, shared by the coarse-level program engine
// (k_coarse.cu) and the batched solver (k_batch.cu): work items t, t+st, ...
// below e of the Op's index space, with the same per-cell device code as
// the standalone kernels.
#pragma once
#include "ops_dev.cuh"

namespace cfmg {

__device__ __forceinline__ void box3(const Box& b, long long t, int& i, int& j, int& k) {
  const long long ni = b.i1 - b.i0 + 1, nj = b.j1 - b.j0 + 1;
  i = b.i0 + (int)(t % ni);
  const long long q = t / ni;
  j = b.j0 + (int)(q % nj);
  k = b.k0 + (int)(q / nj);
}

// Items are taken U at a time per thread: all U values are computed before
// any is stored, so their loads are in flight together (U = 1 in the
// register-capped program engine). Outputs never alias the inputs of the same Op (Jacobi sweeps
// write the partner buffer, residuals r, restrictions the coarse b).
#define CFMG_ILP(...)                                                    \
  for (; t < e; t += U * st) {                                           \
    T v_[U];                                                             \
    long long i_[U];                                                     \
    _Pragma("unroll") for (int u = 0; u < U; ++u) {                     \
      const long long tt = t + u * st;                                   \
      i_[u] = -1;                                                        \
      if (tt < e) {                                                      \
        __VA_ARGS__                                                      \
      }                                                                  \
    }                                                                    \
    _Pragma("unroll") for (int u = 0; u < U; ++u) if (i_[u] >= 0) y[i_[u]] = v_[u]; \
  }

template <class T, int U>
__device__ void exec(const Op& op, long long t, long long st, long long e) {
  const T* x = (const T*)op.x;
  const T* b = (const T*)op.b;
  const T* w = (const T*)op.w;
  const T* d = (const T*)op.d;
  const T* cE = (const T*)op.cE;
  const T* cN = (const T*)op.cN;
  const T* coef = (const T*)op.coef;
  T* y = (T*)op.y;
  const T cff = (T)op.cff;
  const long long n1 = op.g.n1, n2 = op.g.n2;
  int i, j, k;
  switch (op.kind) {
    case OPK_SWEEP5:
      CFMG_ILP(i_[u] = op.lo + tt; v_[u] = v_sweep5(x, b, w, cff, n1, i_[u]);)
      break;
    case OPK_SWEEP7:
      CFMG_ILP(i_[u] = op.lo + tt; v_[u] = v_sweep7(x, b, w, cff, n1, n2, i_[u]);)
      break;
    case OPK_SWEEPVC:
      for (; t < e; t += st) d_sweepvc(x, y, b, w, cE, cN, cff, n1, op.lo + t);
      break;
    case OPK_SWEEP9:
      CFMG_ILP(box3(op.box, tt, i, j, k); i_[u] = lin(op.g, i, j, k); v_[u] = v_sweep9(x, b, w, cff, n1, i_[u]);)
      break;
    case OPK_SWEEP19:
      for (; t < e; t += st) {
        box3(op.box, t, i, j, k);
        d_sweep19(x, y, b, w, cff, n1, n2, lin(op.g, i, j, k));
      }
      break;
    case OPK_RESID5:
      CFMG_ILP(i_[u] = op.lo + tt; v_[u] = v_resid5(x, b, d, op.m, n1, i_[u]);)
      break;
    case OPK_RESIDVC:
      for (; t < e; t += st) d_residvc(y, x, b, d, cE, cN, op.m, n1, op.lo + t);
      break;
    case OPK_RESID7:
      CFMG_ILP(box3(op.box, tt, i, j, k); i_[u] = lin(op.g, i, j, k); v_[u] = v_resid7(x, b, d, op.m, n1, n2, i_[u]);)
      break;
    case OPK_RESID9:
      CFMG_ILP(box3(op.box, tt, i, j, k); i_[u] = lin(op.g, i, j, k); v_[u] = v_resid9(x, b, d, op.m, n1, i_[u]);)
      break;
    case OPK_RESID19:
      for (; t < e; t += st) {
        box3(op.box, t, i, j, k);
        d_resid19(y, x, b, d, op.m, n1, n2, lin(op.g, i, j, k));
      }
      break;
#define CFMG_RESTRICT_CASE(K)                                                              \
  case OPK_RESTRICT0 + K:                                                                  \
    CFMG_ILP(box3(op.box, tt, i, j, k); v_[u] = v_restrict<T, K>(x, coef, op.g, op.gc, i, j, k, i_[u]);) \
    break;
      CFMG_RESTRICT_CASE(0)
      CFMG_RESTRICT_CASE(1)
      CFMG_RESTRICT_CASE(2)
    case OPK_RESTRICT3:
      for (; t < e; t += st) {
        box3(op.box, t, i, j, k);
        d_restrict<T, 3>(x, y, coef, op.g, op.gc, i, j, k);
      }
      break;
#undef CFMG_RESTRICT_CASE
#define CFMG_PROLONG_CASE(K)                                                   \
  case OPK_PROLONG0 + K:                                                       \
    for (; t < e; t += st) {                                                   \
      const int p = (int)(t % op.np_i);                                        \
      const long long q = t / op.np_i;                                         \
      d_prolong<T, K>(y, x, coef, op.g, op.gc, p, (int)(q % op.np_j), (int)(q / op.np_j), op.kf0); \
    }                                                                          \
    break;
      CFMG_PROLONG_CASE(0)
      CFMG_PROLONG_CASE(1)
      CFMG_PROLONG_CASE(2)
      CFMG_PROLONG_CASE(3)
#undef CFMG_PROLONG_CASE
    case OPK_FILL:
      for (; t < e; t += st) d_fill_line(y + t * op.g.tx, op.g.tx, op.g.nh);
      break;
    case OPK_ZERO:
      for (; t < e; t += st) y[t] = T(0);
      break;
    case OPK_F32TO64:
      for (; t < e; t += st) ((double*)op.y)[t] = (double)((const float*)op.x)[t];
      break;
    case OPK_F64TO32:
      for (; t < e; t += st) ((float*)op.y)[t] = (float)((const double*)op.x)[t];
      break;
    default:
      break;
  }
}
#undef CFMG_ILP

}  // namespace cfmg
