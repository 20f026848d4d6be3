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

template <class T>
__device__ void exec(const Op& op, long long t, long long st, long long e) {
  const T* x = (const T*)op.x;
  const T* b = (const T*)op.b;
  const T* w = (const T*)op.w;
  const T* d = (const T*)op.d;
  T* y = (T*)op.y;
  const T cff = (T)op.cff;
  const long long n1 = op.g.n1, n2 = op.g.n2;
  int i, j, k;
  switch (op.kind) {
    case OPK_SWEEP5:
      for (; t < e; t += st) d_sweep5(x, y, b, w, cff, n1, op.lo + t);
      break;
    case OPK_SWEEP7:
      for (; t < e; t += st) d_sweep7(x, y, b, w, cff, n1, n2, op.lo + t);
      break;
    case OPK_SWEEPVC:
      for (; t < e; t += st) d_sweepvc(x, y, b, w, (const T*)op.cE, (const T*)op.cN, cff, n1, op.lo + t);
      break;
    case OPK_SWEEP9:
      for (; t < e; t += st) {
        box3(op.box, t, i, j, k);
        d_sweep9(x, y, b, w, cff, n1, lin(op.g, i, j, k));
      }
      break;
    case OPK_SWEEP19:
      for (; t < e; t += st) {
        box3(op.box, t, i, j, k);
        d_sweep19(x, y, b, w, cff, n1, n2, lin(op.g, i, j, k));
      }
      break;
    case OPK_RESID5:
      for (; t < e; t += st) d_resid5(y, x, b, d, op.m, n1, op.lo + t);
      break;
    case OPK_RESIDVC:
      for (; t < e; t += st) d_residvc(y, x, b, d, (const T*)op.cE, (const T*)op.cN, op.m, n1, op.lo + t);
      break;
    case OPK_RESID7:
      for (; t < e; t += st) {
        box3(op.box, t, i, j, k);
        d_resid7(y, x, b, d, op.m, n1, n2, lin(op.g, i, j, k));
      }
      break;
    case OPK_RESID9:
      for (; t < e; t += st) {
        box3(op.box, t, i, j, k);
        d_resid9(y, x, b, d, op.m, n1, lin(op.g, i, j, k));
      }
      break;
    case OPK_RESID19:
      for (; t < e; t += st) {
        box3(op.box, t, i, j, k);
        d_resid19(y, x, b, d, op.m, n1, n2, lin(op.g, i, j, k));
      }
      break;
#define CFMG_RESTRICT_CASE(K)                                                  \
  case OPK_RESTRICT0 + K:                                                      \
    for (; t < e; t += st) {                                                \
      box3(op.box, t, i, j, k);                                                \
      d_restrict<T, K>(x, y, (const T*)op.coef, op.g, op.gc, i, j, k);         \
    }                                                                          \
    break;
      CFMG_RESTRICT_CASE(0)
      CFMG_RESTRICT_CASE(1)
      CFMG_RESTRICT_CASE(2)
      CFMG_RESTRICT_CASE(3)
#define CFMG_PROLONG_CASE(K)                                                   \
  case OPK_PROLONG0 + K:                                                       \
    for (; t < e; t += st) {                                                \
      const int p = (int)(t % op.np_i);                                        \
      const long long q = t / op.np_i;                                         \
      d_prolong<T, K>(y, x, (const T*)op.coef, op.g, op.gc, p, (int)(q % op.np_j), (int)(q / op.np_j), op.kf0); \
    }                                                                          \
    break;
      CFMG_PROLONG_CASE(0)
      CFMG_PROLONG_CASE(1)
      CFMG_PROLONG_CASE(2)
      CFMG_PROLONG_CASE(3)
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

}  // namespace cfmg
