// Coarse-level program engine.
//
// On coarse levels a multigrid cycle is a long chain of tiny operators (the
// coarsest solve alone is 2*ndeepest sweeps on a few hundred cells), whose
// cost as separate launches is launch latency, not work. Here one
// cluster of kEngineCtas CTAs executes a whole program of Ops: every CTA
// takes a cluster-strided share of each Op's work items, then the cluster
// barrier (release/acquire at cluster scope) makes the Op's global-memory
// writes visible before the next Op reads them. The per-cell arithmetic is
// the same device code as the standalone kernels, so results are identical.
#include "ops_dev.cuh"

namespace cfmg {

__device__ __forceinline__ unsigned cluster_rank() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ void cluster_barrier() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

__device__ __forceinline__ void box3(const Box& b, long long t, int& i, int& j, int& k) {
  const long long ni = b.i1 - b.i0 + 1, nj = b.j1 - b.j0 + 1;
  i = b.i0 + (int)(t % ni);
  const long long q = t / ni;
  j = b.j0 + (int)(q % nj);
  k = b.k0 + (int)(q / nj);
}

template <class T>
__device__ void exec(const Op& op, long long t, long long st) {
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
      for (; t < op.n; t += st) d_sweep5(x, y, b, w, cff, n1, op.lo + t);
      break;
    case OPK_SWEEP7:
      for (; t < op.n; t += st) d_sweep7(x, y, b, w, cff, n1, n2, op.lo + t);
      break;
    case OPK_SWEEPVC:
      for (; t < op.n; t += st) d_sweepvc(x, y, b, w, (const T*)op.cE, (const T*)op.cN, cff, n1, op.lo + t);
      break;
    case OPK_SWEEP9:
      for (; t < op.n; t += st) {
        box3(op.box, t, i, j, k);
        d_sweep9(x, y, b, w, cff, n1, lin(op.g, i, j, k));
      }
      break;
    case OPK_SWEEP19:
      for (; t < op.n; t += st) {
        box3(op.box, t, i, j, k);
        d_sweep19(x, y, b, w, cff, n1, n2, lin(op.g, i, j, k));
      }
      break;
    case OPK_RESID5:
      for (; t < op.n; t += st) d_resid5(y, x, b, d, op.m, n1, op.lo + t);
      break;
    case OPK_RESIDVC:
      for (; t < op.n; t += st) d_residvc(y, x, b, d, (const T*)op.cE, (const T*)op.cN, op.m, n1, op.lo + t);
      break;
    case OPK_RESID7:
      for (; t < op.n; t += st) {
        box3(op.box, t, i, j, k);
        d_resid7(y, x, b, d, op.m, n1, n2, lin(op.g, i, j, k));
      }
      break;
    case OPK_RESID9:
      for (; t < op.n; t += st) {
        box3(op.box, t, i, j, k);
        d_resid9(y, x, b, d, op.m, n1, lin(op.g, i, j, k));
      }
      break;
    case OPK_RESID19:
      for (; t < op.n; t += st) {
        box3(op.box, t, i, j, k);
        d_resid19(y, x, b, d, op.m, n1, n2, lin(op.g, i, j, k));
      }
      break;
#define CFMG_RESTRICT_CASE(K)                                                  \
  case OPK_RESTRICT0 + K:                                                      \
    for (; t < op.n; t += st) {                                                \
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
    for (; t < op.n; t += st) {                                                \
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
      for (; t < op.n; t += st) d_fill_line(y + t * op.g.tx, op.g.tx, op.g.nh);
      break;
    case OPK_ZERO:
      for (; t < op.n; t += st) y[t] = T(0);
      break;
    default:
      break;
  }
}

__global__ void __launch_bounds__(kEngineThreads) k_program(const Op* __restrict__ prog, int nops) {
  __shared__ Op op;
  const long long t0 = (long long)cluster_rank() * blockDim.x + threadIdx.x;
  const long long st = (long long)kEngineCtas * blockDim.x;
  for (int o = 0; o < nops; ++o) {
    if (threadIdx.x < sizeof(Op) / sizeof(int)) ((int*)&op)[threadIdx.x] = ((const int*)&prog[o])[threadIdx.x];
    __syncthreads();
    if (op.kind == OPK_F32TO64) {
      for (long long t = t0; t < op.n; t += st) ((double*)op.y)[t] = (double)((const float*)op.x)[t];
    } else if (op.kind == OPK_F64TO32) {
      for (long long t = t0; t < op.n; t += st) ((float*)op.y)[t] = (float)((const double*)op.x)[t];
    } else if (op.prec == 0) {
      exec<double>(op, t0, st);
    } else {
      exec<float>(op, t0, st);
    }
    cluster_barrier();
  }
}

void launch_program(const Op* prog, int nops, cudaStream_t s) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(kEngineCtas, 1, 1);
  cfg.blockDim = dim3(kEngineThreads, 1, 1);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = kEngineCtas;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, k_program, prog, nops);
}

}  // namespace cfmg
