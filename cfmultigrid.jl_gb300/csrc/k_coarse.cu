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
#include "exec_dev.cuh"

namespace cfmg {

__device__ __forceinline__ unsigned cluster_rank() {
  unsigned r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ void cluster_barrier() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// Block-wide FP64 sum (fixed order: warp shuffles, then warp 0 over the
// per-warp sums); the result is valid in thread 0.
__device__ __forceinline__ double block_sum(double v, double* sh) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = __dadd_rn(v, __shfl_down_sync(0xffffffffu, v, o));
  const int wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  __syncthreads();
  if ((threadIdx.x & 31) == 0) sh[wid] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    v = (int)threadIdx.x < nw ? sh[threadIdx.x] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = __dadd_rn(v, __shfl_down_sync(0xffffffffu, v, o));
  }
  return v;
}

// Cluster-wide sum: every CTA's block sum goes to red[rank]; after a
// cluster barrier CTA 0's thread 0 adds them in rank order.
__device__ __forceinline__ double cluster_sum(double v, double* red, double* sh, bool& leader) {
  v = block_sum(v, sh);
  const unsigned rank = cluster_rank();
  if (threadIdx.x == 0) red[rank] = v;
  cluster_barrier();
  leader = (rank == 0 && threadIdx.x == 0);
  double t = 0.0;
  if (leader)
    for (int r = 0; r < kEngineCtas; ++r) t = __dadd_rn(t, red[r]);
  return t;
}

__device__ __forceinline__ unsigned long long globaltimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Runs one program; returns after its last Op. red: this cluster's
// kEngineCtas reduction slots.
__device__ void run_program(const Op* __restrict__ prog, int nops, long long t0, long long st, double* red,
                            Op& op, double* sh) {
  int o = 0;
  while (o < nops) {
    if (threadIdx.x < sizeof(Op) / sizeof(int)) ((int*)&op)[threadIdx.x] = ((const int*)&prog[o])[threadIdx.x];
    __syncthreads();
    int next = o + 1;
    bool leader = false;
    double* sc = op.sc;
    switch (op.kind) {
      case OPK_F32TO64:
        for (long long t = t0; t < op.n; t += st) ((double*)op.y)[t] = (double)((const float*)op.x)[t];
        break;
      case OPK_F64TO32:
        for (long long t = t0; t < op.n; t += st) ((float*)op.y)[t] = (float)((const double*)op.x)[t];
        break;
      case OPK_NORM64: {
        const double* x = (const double*)op.x;
        double v = 0.0;
        for (long long t = t0; t < op.n; t += st) {
          const uint8_t mm = op.m[t];
          if (mm) v = (mm == 1) ? __fma_rn(x[t], x[t], v) : __dadd_rn(v, __dmul_rn((double)mm, __dmul_rn(x[t], x[t])));
        }
        const double tot = cluster_sum(v, red, sh, leader);
        if (leader) sc[op.s0] = (op.s1 && tot == 0.0) ? 1.0 : tot;
        break;
      }
      case OPK_MEAN64: {
        const double* x = (const double*)op.x;
        double v = 0.0;
        for (long long t = t0; t < op.n; t += st)
          if (op.m[t]) v = __dadd_rn(v, x[t]);
        const double tot = cluster_sum(v, red, sh, leader);
        if (leader) sc[op.s0] = sc[op.s1] > 0 ? tot / sc[op.s1] : 0.0;
        break;
      }
      case OPK_RATIO:
        if (cluster_rank() == 0 && threadIdx.x == 0) {
          const double nb = sc[op.s2];
          const double q = nb > 0.0 ? sc[op.s1] / nb : 0.0;
          // a NaN or Inf |b| gives a NaN ratio (reported as non-finite), not 0
          sc[op.s0] = !isfinite(nb) ? __longlong_as_double(0x7ff8000000000000LL)
                                    : (op.norm_kind == CFMG_NORM_L2 ? sqrt(q) : q);
        }
        break;
      case OPK_SCALE:
        if (cluster_rank() == 0 && threadIdx.x == 0) {
          const double nwet = sc[op.s2] > 0 ? sc[op.s2] : 1.0;
          const double rms = sqrt(sc[op.s1] / nwet);
          const bool ok = rms > 0 && isfinite(rms);
          sc[op.s0] = ok ? 1.0 / rms : 1.0;
          sc[op.s0 + 1] = ok ? rms : 1.0;
        }
        break;
      case OPK_RHS32: {
        const double* r = (const double*)op.x;
        const double mean = sc[op.s1], scale = sc[op.s0];
        for (long long t = t0; t < op.n; t += st) {
          const float f = op.m[t] ? (float)((r[t] - mean) * scale) : 0.f;
          ((float*)op.y)[t] = f;
          ((float*)op.y2)[t] = f;
        }
        break;
      }
      case OPK_UPDATE: {
        const float* e = (const float*)op.x;
        double* x = (double*)op.y;
        const double is = sc[op.s0];
        for (long long t = t0; t < op.n; t += st) x[t] = __fma_rn((double)e[t], is, x[t]);
        break;
      }
      case OPK_BRANCH: {
        const double res = sc[op.s0], nite = sc[op.s1];
        const bool cont = res > op.tol && nite < (double)op.maxite;
        cluster_barrier();  // every thread has read before the count moves
        if (cont && cluster_rank() == 0 && threadIdx.x == 0) sc[op.s1] = nite + 1.0;
        next = cont ? o + 1 : op.s2;
        break;
      }
      case OPK_JUMP:
        next = op.s2;
        break;
      case OPK_STAMP:
        if (cluster_rank() == 0 && threadIdx.x == 0) sc[op.s0] = (double)globaltimer();
        break;
      case OPK_HIST:
        if (cluster_rank() == 0 && threadIdx.x == 0) sc[op.s0 + (int)sc[op.s1]] = sc[op.s2];
        break;
      case OPK_ZERO_IF:
        if (sc[op.s0] != 0.0)
          for (long long t = t0; t < op.n; t += st) ((double*)op.y)[t] = 0.0;
        break;
      default:
        if (op.prec == 0) exec<double, 1>(op, t0, st, op.n);
        else exec<float, 1>(op, t0, st, op.n);
        break;
    }
    cluster_barrier();
    o = next;
  }
}

__global__ void __launch_bounds__(kEngineThreads) k_program(const Op* __restrict__ prog, int nops, double* red) {
  dep_wait();
  __shared__ Op op;
  __shared__ double sh[32];
  const long long t0 = (long long)cluster_rank() * blockDim.x + threadIdx.x;
  const long long st = (long long)kEngineCtas * blockDim.x;
  run_program(prog, nops, t0, st, red, op, sh);
}

// Batched engine: every cluster takes instances off a shared queue
// (counter[0]; the caller orders the instances largest first) and runs
// each instance's whole program. counter[1 + cluster] carries the index
// from the cluster's leader to its other CTAs.
__global__ void __launch_bounds__(kEngineThreads) k_batch(const Op* const* __restrict__ progs,
                                                         const int* __restrict__ nops, int ninst, int* counter,
                                                         double* red) {
  __shared__ Op op;
  __shared__ double sh[32];
  const int cid = blockIdx.x / kEngineCtas;
  const long long t0 = (long long)cluster_rank() * blockDim.x + threadIdx.x;
  const long long st = (long long)kEngineCtas * blockDim.x;
  double* myred = red + (long long)cid * kEngineCtas;
  while (true) {
    if (cluster_rank() == 0 && threadIdx.x == 0) counter[1 + cid] = atomicAdd(&counter[0], 1);
    cluster_barrier();
    const int inst = *(volatile int*)&counter[1 + cid];
    cluster_barrier();  // all have read before the leader takes the next one
    if (inst >= ninst) break;
    run_program(progs[inst], nops[inst], t0, st, myred, op, sh);
  }
}

int engine_max_clusters() {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(kEngineCtas, 1, 1);
  cfg.blockDim = dim3(kEngineThreads, 1, 1);
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = kEngineCtas;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  int n = 0;
  if (cudaOccupancyMaxActiveClusters(&n, k_batch, &cfg) != cudaSuccess) {
    cudaGetLastError();
    return 1;
  }
  return n > 0 ? n : 1;
}

void launch_batch(const Op* const* progs, const int* nops, int ninst, int* counter, double* red, int nclusters,
                  cudaStream_t s) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(kEngineCtas * nclusters), 1, 1);
  cfg.blockDim = dim3(kEngineThreads, 1, 1);
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = kEngineCtas;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, k_batch, progs, nops, ninst, counter, red);
}

void launch_program(const Op* prog, int nops, double* red, cudaStream_t s) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(kEngineCtas, 1, 1);
  cfg.blockDim = dim3(kEngineThreads, 1, 1);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute attr[2];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = kEngineCtas;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  // a programmatic dependent of the kernel before it (k_program opens with dep_wait)
  attr[1].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[1].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = tl_dep_launch ? 2 : 1;
  cudaLaunchKernelEx(&cfg, k_program, prog, nops, red);
}

}  // namespace cfmg
