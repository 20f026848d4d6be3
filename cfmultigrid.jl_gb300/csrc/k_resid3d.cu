// Fixed-point level-1 residual of the 3D 7-point operator (rloop3d! over
// the interior box, src/laplacian.jl:44-64, in the integer form of the mixed
// loop's fused pass) with TMA-staged planes.
//
// The strip form (k_resid_int2d, k_mixed.cu) walks the rows of a plane and
// loads the x of the planes below and above each row separately: every x is
// read three times and converted three times, and its warps, waiting on
// those loads with few bytes in flight, ran at 2.3 TB/s. Here a block owns a
// 32 x 16 column tile of the interior box (two rows a thread; 32 x 8 with
// one row a thread as an option) and marches along k through a run of kt
// planes. One thread issues each plane's loads as TMA copies
// (cp.async.bulk.tensor) into a ring of shared-memory stages that complete
// on mbarriers: x with a one-cell halo in i and j (a 36 x 18 box of doubles
// starting on an even column), b (34 x 16 doubles) and dq (48 x 16 bytes
// from a copy whose rows are padded to a multiple of 16 bytes). The threads
// convert each x of a plane once (their own cells, and one halo cell for
// 100 of them) into a ring of three converted planes; the residual at plane
// k takes its four in-plane neighbours from converted plane k and its
// k -/+ 1 neighbours from the thread's registers. The loads of the next
// planes of the ring are in flight while a plane is computed, without
// registers held for them, and every x comes from DRAM about once.
//
// Per cell the arithmetic is the strip form's: the same exact integer R, the
// same FP32 right-hand side f = R * 2^-(k+q) * scale, sum f^2 in double-float
// per thread and the exact sum R in 128 bits. Only the order in which the
// per-thread sums are combined differs.
//
// Every wait on an mbarrier is bounded (one second of %globaltimer). A block
// whose wait runs out waits (bounded again) for its copies in flight, writes
// NaN into its partial sums, so that the solve loop stops on a non-finite
// residual, and 1 into ds[S_FAULT], which the solve reports.
#include <cuda.h>

#include <mutex>

#include "cfmg_internal.h"
#include "ops_dev.cuh"

namespace cfmg {
namespace {

// JT rows of the tile per thread: a 32 x 8*JT column tile, 256 threads.
// JT = 2 halves the barriers, mbarrier waits and TMA issues per cell and
// converts fewer halo cells (100 for 512 cells against 84 for 256).
template <int JT>
struct R3Cfg {
  static constexpr int TI = 32, TJ = 8 * JT;   // column tile
  static constexpr int Stages = JT == 1 ? 4 : 3;  // planes in the TMA ring
  static constexpr int XW = 36, XH = TJ + 2;   // x box (halo of one cell, even first column)
  static constexpr int BW = 34;                // b box (even first column)
  static constexpr int DW = 48;                // dq box (first column a multiple of 16)
  static constexpr int PW = 34, PH = TJ + 2;   // converted plane: tile + halo
  static constexpr int Halo = 2 * PW + 2 * TJ;
  static constexpr int XBytes = XW * XH * 8;
  static constexpr int BBytes = BW * TJ * 8;
  static constexpr int DBytes = DW * TJ;
  static constexpr int XSlot = (XBytes + 127) / 128 * 128;  // x box rounded up to 128 bytes
  static constexpr int StageBytes = XSlot + BBytes + DBytes;
  static constexpr int PBytes = PW * PH * 8;
  static constexpr int Smem = Stages * StageBytes + 3 * PBytes + Stages * 8;
  static_assert(TI * 8 == kMxThreads, "a thread per column of the tile, JT rows each");
  static_assert(Halo <= kMxThreads, "a halo cell per thread at most");
  static_assert(BBytes % 128 == 0 && DBytes % 128 == 0, "TMA destinations on 128-byte boundaries");
};

int dq_pitch_of(int tx) { return (tx + 15) & ~15; }

struct R3Space {
  int c0, r0, p0;    // 0-based column, row and plane of the box's first cell
  int ni, nj, nk;    // box extent
  int nti, ntj;      // column tiles in i and j
  int kt, nkc;       // planes per task, runs of planes along k
  long long n1, n2;  // strides of b32 and r32 (elements)
};

__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ unsigned long long globaltimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ bool mbar_try(unsigned bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.b32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}

// false when the phase has not completed within one second
__device__ __forceinline__ bool mbar_wait(unsigned bar, unsigned parity) {
  if (mbar_try(bar, parity)) return true;
  const unsigned long long t0 = globaltimer();
  while (!mbar_try(bar, parity))
    if (globaltimer() - t0 > 1000000000ULL) return false;
  return true;
}

__device__ __forceinline__ void tma3(unsigned dst, const CUtensorMap* map, int c, int r, int p, unsigned bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
      "[%5];"
      :
      : "r"(dst), "l"(reinterpret_cast<unsigned long long>(map)), "r"(c), "r"(r), "r"(p), "r"(bar)
      : "memory");
}

struct R3Task {
  int c0t, r0t, ka, np;  // first column and row of the tile, first plane, planes streamed (kt + 2 at most)
};
template <int JT>
__device__ __forceinline__ R3Task r3_task(const R3Space& sp, int T) {
  R3Task t;
  const int tI = T % sp.nti, rest = T / sp.nti;
  const int tJ = rest % sp.ntj, kc = rest / sp.ntj;
  t.c0t = sp.c0 + R3Cfg<JT>::TI * tI;
  t.r0t = sp.r0 + R3Cfg<JT>::TJ * tJ;
  t.ka = sp.p0 + kc * sp.kt;
  const int kb = min(t.ka + sp.kt, sp.p0 + sp.nk);
  t.np = kb - t.ka + 2;  // planes ka-1 .. kb
  return t;
}

// tcol (optional, JT = 2 tiles): 1 for each (tile, interior plane) with a wet
// cell. A task whose output planes are all dry is skipped: its cells' b32 is
// +0 already and their residuals add exact zeros to the sums. The block's
// tasks' flags are gathered in shared memory first (up to kR3MaxTasks per
// block; later ones count as wet), and the issue cursor and the consumers
// skip the same tasks.
constexpr int kR3MaxTasks = 64;
template <int JT, bool NEUMANN>
__global__ void __launch_bounds__(kMxThreads) k_resid_int3d(const __grid_constant__ CUtensorMap mx,
                                                            const __grid_constant__ CUtensorMap mb,
                                                            const __grid_constant__ CUtensorMap md, R3Space sp,
                                                            double* ds, float* __restrict__ b32,
                                                            float* __restrict__ r32, double* __restrict__ partials,
                                                            const uint8_t* __restrict__ tcol) {
  typedef R3Cfg<JT> G;
  extern __shared__ __align__(128) unsigned char smem[];
  long long* pring = reinterpret_cast<long long*>(smem + G::Stages * G::StageBytes);
  unsigned long long* bars = reinterpret_cast<unsigned long long*>(smem + G::Stages * G::StageBytes + 3 * G::PBytes);
  const int tid = threadIdx.x, ti = tid & 31, tj = tid >> 5;  // own cells: rows tj + 8u, u < JT
  if (tid == 0) {
    for (int s = 0; s < G::Stages; ++s)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bars + s)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<unsigned long long>(&mx)) : "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<unsigned long long>(&mb)) : "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<unsigned long long>(&md)) : "memory");
  }
  __syncthreads();
  dep_wait();  // x and b are the predecessor's output
  constexpr int q = 0;  // Q = 1 for the 7-point weights
  const int k = fix_exponent(ds);
  const double scale = ds[S_NEXT];
  const float fm = (float)ldexp(scale, -(k + q));  // power of two: R -> r * scale
  const int ntasks = sp.nti * sp.ntj * sp.nkc;
  // wet flags of the block's tasks (bit m: task blockIdx.x + m * gridDim.x),
  // the same in every thread
  unsigned long long wt = ~0ULL;
  if (tcol) {
    wt = 0;
    for (int m = 0; m < kR3MaxTasks; ++m) {
      const int T = blockIdx.x + m * gridDim.x;
      if (T >= ntasks) break;
      const R3Task t = r3_task<JT>(sp, T);
      const long long tile = (long long)((t.r0t - sp.r0) / R3Cfg<JT>::TJ) * sp.nti + (t.c0t - sp.c0) / R3Cfg<JT>::TI;
      int any = 0;
      for (int p = tid; p < t.np - 2; p += kMxThreads) any |= tcol[tile * sp.nk + (t.ka - sp.p0) + p];
      if (__syncthreads_or(any)) wt |= 1ULL << m;
    }
  }
  auto wet = [&](int T) {  // tasks beyond kR3MaxTasks count as wet
    const int m = (T - (int)blockIdx.x) / (int)gridDim.x;
    return m >= kR3MaxTasks || ((wt >> m) & 1ULL);
  };

  // issue cursor (thread 0): the block's sequence of (task, plane) in order
  int iT = blockIdx.x, iq = 0;
  while (iT < ntasks && !wet(iT)) iT += gridDim.x;
  unsigned long long in = 0;
  R3Task it = r3_task<JT>(sp, iT < ntasks ? iT : 0);
  auto issue_next = [&]() {
    if (iT >= ntasks) return;
    const int s = (int)(in % G::Stages);
    const unsigned bar = smem_u32(bars + s);
    unsigned char* st = smem + s * G::StageBytes;
    const bool full = iq >= 1 && iq <= it.np - 2;  // b and dq for planes ka .. kb-1 only
    const unsigned bytes = G::XBytes + (full ? G::BBytes + G::DBytes : 0);
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
    const int p = it.ka - 1 + iq;
    tma3(smem_u32(st), &mx, (it.c0t - 1) & ~1, it.r0t - 1, p, bar);
    if (full) {
      tma3(smem_u32(st + G::XSlot), &mb, it.c0t & ~1, it.r0t, p, bar);
      tma3(smem_u32(st + G::XSlot + G::BBytes), &md, it.c0t & ~15, it.r0t, p, bar);
    }
    ++in;
    if (++iq == it.np) {
      iT += gridDim.x;
      while (iT < ntasks && !wet(iT)) iT += gridDim.x;
      iq = 0;
      if (iT < ntasks) it = r3_task<JT>(sp, iT);
    }
  };
  if (tid == 0)
    for (int s = 0; s < G::Stages; ++s) issue_next();

  // this thread's halo cell (tid < Halo): its place in the converted plane
  int hp = -1, hx = 0;  // index in the converted plane, and in the x box without the column offset
  if (tid < G::Halo) {
    int hr, hc;
    if (tid < G::PW) {
      hr = 0;
      hc = tid;
    } else if (tid < 2 * G::PW) {
      hr = G::PH - 1;
      hc = tid - G::PW;
    } else {
      const int h = tid - 2 * G::PW;
      hr = 1 + (h >> 1);
      hc = (h & 1) ? G::PW - 1 : 0;
    }
    hp = hr * G::PW + hc;
    hx = hr * G::XW + hc;
  }
  float hi = 0.f, lo = 0.f;  // double-float sum of f^2
  __int128 s1 = 0;
  unsigned long long n = 0;  // planes consumed
  bool fault = false;
  for (int T = blockIdx.x; T < ntasks && !fault; T += gridDim.x) {
    if (!wet(T)) continue;
    const R3Task t = r3_task<JT>(sp, T);
    const int ox = (t.c0t - 1) - ((t.c0t - 1) & ~1), ob = t.c0t - (t.c0t & ~1), od = t.c0t - (t.c0t & ~15);
    const int col = t.c0t + ti;
    bool own[JT];
    long long Cm[JT], Cc[JT], Bp[JT];
    int dp[JT];
#pragma unroll
    for (int u = 0; u < JT; ++u) {
      own[u] = col < sp.c0 + sp.ni && t.r0t + tj + 8 * u < sp.r0 + sp.nj;
      Cm[u] = Cc[u] = Bp[u] = 0;
      dp[u] = -1;
    }
    for (int qq = 0; qq < t.np; ++qq, ++n) {
      const int s = (int)(n % G::Stages);
      const bool ok = mbar_wait(smem_u32(bars + s), (unsigned)((n / G::Stages) & 1));
      const unsigned char* st = smem + s * G::StageBytes;
      const double* xs = reinterpret_cast<const double*>(st);
      long long* P = pring + (qq % 3) * (G::PW * G::PH);
      long long Cn[JT], Bn[JT];
      int dn[JT];
#pragma unroll
      for (int u = 0; u < JT; ++u) {
        const int r = tj + 8 * u;
        Cn[u] = to_fix(xs[(r + 1) * G::XW + ti + 1 + ox], k);
        P[(r + 1) * G::PW + ti + 1] = Cn[u];
        Bn[u] = 0;
        dn[u] = -1;
        if (qq >= 1 && qq <= t.np - 2) {
          Bn[u] = to_fix(reinterpret_cast<const double*>(st + G::XSlot)[r * G::BW + ti + ob], k);
          dn[u] = (int)reinterpret_cast<const signed char*>(st + G::XSlot + G::BBytes)[r * G::DW + ti + od];
        }
      }
      if (hp >= 0) P[hp] = to_fix(xs[hx + ox], k);
      // the plane is converted and its stage free again; one thread refills it
      if (__syncthreads_or(!ok)) {
        fault = true;
        break;
      }
      if (tid == 0) {
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        issue_next();
      }
      if (qq >= 2) {  // plane m = ka + qq - 2 from converted plane m and own C(m-1), C(m), C(m+1)
        const long long* Pc = pring + ((qq - 1) % 3) * (G::PW * G::PH);
#pragma unroll
        for (int u = 0; u < JT; ++u) {
          const int row = t.r0t + tj + 8 * u;
          const int op = (tj + 8 * u + 1) * G::PW + ti + 1;
          long long R = (long long)dp[u] * Cc[u] + Bp[u] -
                        (Pc[op - 1] + Pc[op + 1] + Pc[op - G::PW] + Pc[op + G::PW] + Cm[u] + Cn[u]);
          R = (own[u] && dp[u] >= 0) ? R : 0LL;  // dry cells and cells outside the box
          const float f = __fmul_rn(__ll2float_rn(R), fm);
          if (own[u]) {
            const long long I = (long long)col + sp.n1 * row + sp.n2 * (t.ka + qq - 2);
            b32[I] = f;
            if (!NEUMANN && r32) r32[I] = f;
          }
          if (NEUMANN) s1 += (__int128)R;
          // p + e = f^2 exactly; (hi, lo) += p + e by TwoSum (explicit _rn operations)
          const float pp = __fmul_rn(f, f), e = __fmaf_rn(f, f, -pp);
          const float sn = __fadd_rn(hi, pp), bp = __fsub_rn(sn, hi);
          lo = __fadd_rn(lo, __fadd_rn(__fadd_rn(__fsub_rn(hi, __fsub_rn(sn, bp)), __fsub_rn(pp, bp)), e));
          hi = sn;
        }
      }
#pragma unroll
      for (int u = 0; u < JT; ++u) {
        Cm[u] = Cc[u];
        Cc[u] = Cn[u];
        Bp[u] = Bn[u];
        dp[u] = dn[u];
      }
    }
    __syncthreads();  // the converted-plane ring is reused by the next task
  }
  if (fault) {  // block-uniform (__syncthreads_or): drain the copies in flight, then report
    if (tid == 0) {
      for (unsigned long long m = n; m < in; ++m)
        if (!mbar_wait(smem_u32(bars + (m % G::Stages)), (unsigned)((m / G::Stages) & 1))) break;
      ds[S_FAULT] = 1.0;
      partials[blockIdx.x] = __longlong_as_double(0x7ff8000000000000LL);
      partials[kMxParts + blockIdx.x] = __longlong_as_double(0x7ff8000000000000LL);
      for (int i = gridDim.x + blockIdx.x; i < kMxParts; i += gridDim.x) partials[i] = partials[kMxParts + i] = 0.0;
    }
    return;
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
  if (ti == 0) {
    sh2[tj] = a2;
    sh1[tj] = a1;
  }
  __syncthreads();
  if (tid == 0) {
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

// tcol[(tJ * nti + tI) * nk + p] = 1 when tile (tI, tJ) of the JT = 2
// tiling holds a wet cell in interior plane p
__global__ void k_make_tcol(const uint8_t* __restrict__ m, uint8_t* __restrict__ tcol, R3Space sp) {
  const long long T = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long ntiles = (long long)sp.nti * sp.ntj;
  if (T >= ntiles * sp.nk) return;
  const long long tile = T / sp.nk;
  const int p = (int)(T - tile * sp.nk);
  const int tI = (int)(tile % sp.nti), tJ = (int)(tile / sp.nti);
  const int c0 = sp.c0 + R3Cfg<2>::TI * tI, r0 = sp.r0 + R3Cfg<2>::TJ * tJ;
  const int c1 = min(c0 + R3Cfg<2>::TI, sp.c0 + sp.ni), r1 = min(r0 + R3Cfg<2>::TJ, sp.r0 + sp.nj);
  unsigned any = 0;
  for (int r = r0; r < r1; ++r)
    for (int c = c0; c < c1; ++c) any |= m[(long long)c + sp.n1 * r + sp.n2 * (sp.p0 + p)];
  tcol[T] = any ? 1 : 0;
}

R3Space r3_space(const Geom& g, const Box& bx, int ti, int tj) {
  R3Space sp{};
  sp.c0 = bx.i0 - 1;
  sp.r0 = bx.j0 - 1;
  sp.p0 = bx.k0 - 1;
  sp.ni = bx.i1 - bx.i0 + 1;
  sp.nj = bx.j1 - bx.j0 + 1;
  sp.nk = bx.k1 - bx.k0 + 1;
  sp.nti = (sp.ni + ti - 1) / ti;
  sp.ntj = (sp.nj + tj - 1) / tj;
  sp.n1 = g.n1;
  sp.n2 = g.n2;
  return sp;
}

__global__ void k_pad_dq(const int8_t* __restrict__ dq, int8_t* __restrict__ dqp, int tx, int txp, long long rows) {
  const long long I = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (I >= rows * txp) return;
  const long long r = I / txp;
  const int c = (int)(I - r * txp);
  dqp[I] = c < tx ? dq[r * tx + c] : (int8_t)-128;
}

typedef CUresult (*PFN_encodeTiled)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                    const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                    CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
PFN_encodeTiled g_encode = nullptr;
std::once_flag g_encode_once;

PFN_encodeTiled encoder() {
  std::call_once(g_encode_once, [] {
    cudaDriverEntryPointQueryResult qr;
    void* f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &qr) ==
            cudaSuccess &&
        qr == cudaDriverEntryPointSuccess)
      g_encode = (PFN_encodeTiled)f;
    else
      cudaGetLastError();
  });
  return g_encode;
}

// a 3D tiled map of a tx x ty x tz array (row pitch `pitch` elements), box w x h x 1, zero fill outside
bool encode3(CUtensorMap* m, CUtensorMapDataType dt, int esize, const void* base, int tx, long long pitch, int ty,
             int tz, int w, int h) {
  PFN_encodeTiled enc = encoder();
  if (!enc) return false;
  const cuuint64_t dims[3] = {(cuuint64_t)tx, (cuuint64_t)ty, (cuuint64_t)tz};
  const cuuint64_t strides[2] = {(cuuint64_t)(pitch * esize), (cuuint64_t)(pitch * esize * ty)};
  const cuuint32_t box[3] = {(cuuint32_t)w, (cuuint32_t)h, 1};
  const cuuint32_t es[3] = {1, 1, 1};
  return enc(m, dt, 3, const_cast<void*>(base), dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
             CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int JT, bool NEUMANN>
int r3_grid() {
  static int blocks = 0;  // one wave: resident blocks per SM x SMs, at most kMxParts
  if (!blocks) {
    int dev = 0, nsm = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    cudaFuncSetAttribute(k_resid_int3d<JT, NEUMANN>, cudaFuncAttributeMaxDynamicSharedMemorySize, R3Cfg<JT>::Smem);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_resid_int3d<JT, NEUMANN>, kMxThreads, R3Cfg<JT>::Smem);
    blocks = nsm * (per > 0 ? per : 1);
    if (blocks > kMxParts || blocks <= 0) blocks = kMxParts;
  }
  return blocks;
}

template <int JT>
bool launch_r3(const double* x, const double* b, const int8_t* dqp, const Geom& g, const Box& bx, double* ds,
               float* b32, float* r32, bool neumann, double* partials, cudaStream_t s, const uint8_t* tcol) {
  typedef R3Cfg<JT> G;
  R3Space sp = r3_space(g, bx, G::TI, G::TJ);
  // the boxes start at column c0t-1 >= 0, row r0t-1 >= 0 and plane ka-1 >= 0
  if (sp.ni <= 0 || sp.nj <= 0 || sp.nk <= 0 || sp.c0 < 1 || sp.r0 < 1 || sp.p0 < 1) return false;
  CUtensorMap mx, mb, md;
  const int txp = dq_pitch_of(g.tx);
  if (!encode3(&mx, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 8, x, g.tx, g.tx, g.ty, g.tz, G::XW, G::XH) ||
      !encode3(&mb, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 8, b, g.tx, g.tx, g.ty, g.tz, G::BW, G::TJ) ||
      !encode3(&md, CU_TENSOR_MAP_DATA_TYPE_UINT8, 1, dqp, txp, txp, g.ty, g.tz, G::DW, G::TJ))
    return false;
  const int grid = neumann ? r3_grid<JT, true>() : r3_grid<JT, false>();
  // about 8 tasks per block: runs of kt planes (each streams kt + 2)
  const long long cols = (long long)sp.nti * sp.ntj;
  long long kt = (sp.nk * cols + 8LL * grid - 1) / (8LL * grid);
  kt = kt < 4 ? 4 : kt;
  sp.kt = (int)(kt > sp.nk ? sp.nk : kt);
  sp.nkc = (sp.nk + sp.kt - 1) / sp.kt;
  if (neumann)
    launch_dep(k_resid_int3d<JT, true>, grid, kMxThreads, G::Smem, s, mx, mb, md, sp, ds, b32, r32, partials, tcol);
  else
    launch_dep(k_resid_int3d<JT, false>, grid, kMxThreads, G::Smem, s, mx, mb, md, sp, ds, b32, r32, partials, tcol);
  return true;
}

}  // namespace

int dq_pitch(int tx) { return dq_pitch_of(tx); }

void launch_pad_dq(const int8_t* dq, int8_t* dqp, int tx, int txp, long long rows, cudaStream_t s) {
  const long long n = rows * txp;
  k_pad_dq<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(dq, dqp, tx, txp, rows);
}

bool launch_resid_int3d(const double* x, const double* b, const int8_t* dqp, const Geom& g, const Box& bx,
                        double* ds, float* b32, float* r32, bool neumann, double* partials, cudaStream_t s,
                        int rows_per_thread, const uint8_t* tcol) {
  // TMA: global addresses on 16 bytes, row and plane pitches multiples of 16 bytes
  if (!dqp || g.tx % 2 != 0 || ((uintptr_t)x | (uintptr_t)b | (uintptr_t)dqp) % 16 != 0) return false;
  // the skipped tasks' r32 would keep older values: skip only where r32 is not written
  if (rows_per_thread == 2) return launch_r3<2>(x, b, dqp, g, bx, ds, b32, r32, neumann, partials, s, r32 ? nullptr : tcol);
  return launch_r3<1>(x, b, dqp, g, bx, ds, b32, r32, neumann, partials, s, nullptr);
}

long long resid3d_tcol_size(const Geom& g, const Box& bx) {
  const R3Space sp = r3_space(g, bx, R3Cfg<2>::TI, R3Cfg<2>::TJ);
  return (long long)sp.nti * sp.ntj * sp.nk;
}

void launch_make_tcol(const uint8_t* m, uint8_t* tcol, const Geom& g, const Box& bx, cudaStream_t s) {
  const R3Space sp = r3_space(g, bx, R3Cfg<2>::TI, R3Cfg<2>::TJ);
  const long long n = (long long)sp.nti * sp.ntj * sp.nk;
  if (n <= 0) return;
  k_make_tcol<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(m, tcol, sp);
}

}  // namespace cfmg
