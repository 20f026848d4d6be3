// Temporally blocked FP32 smoother for the 3D 7-point operator of the
// mixed-precision cycles (closed topology): S = 2*nite Jacobi sweeps of
// smooth_laplacian! (src/laplacian.jl:24-41) in one streaming pass.
//
// A CTA owns a 64 x 32 (i, j) tile with an S-cell halo and marches along k
// through a chunk of planes. For every sweep level s = 1..S it keeps a ring
// of three planes in shared memory; b and omega*idiag keep a ring of S+1
// planes. Each step loads one new plane of x, b and omega*idiag, then
// computes level s at the plane s steps behind, level by level, so level S
// (the result) trails the loads by S planes. Level s is valid one cell
// further in from the tile edge than level s-1; the CTA writes the core of
// its tile for the planes of its k chunk. HBM traffic falls from 16 B per
// cell and sweep to about 16 B per cell for all S sweeps (plus the halo).
//
// As in the 2D blocked passes, correctness rests on the mixed form's
// invariant: in the FP32 correction fields every cell outside the wet
// interior holds 0 and has omega*idiag = 0, so updating every cell of the
// box U = [nh, n+nh+1]^3 with the same formula is bit-identical to the
// reference's linear sweep range, while cells outside U keep their value.
// The per-cell arithmetic is d_sweep7's Ar<float> sequence.
//
// L19: the 3D 19-point operator's smoothing call (smooth_laplacian9!,
// src/laplacian9.jl:2-47): one pair whatever nite is, the first sweep over
// the box E = icp x jcp x kcp (the interior and one cell around it), the
// second over the interior box U, in one pass (S = 2). Level 1 updates the
// cells of E, level 2 those of U; level 2 at a cell of U reads level 1 only
// inside E, so what level 1 holds elsewhere is never used. The result goes
// to the other x buffer, whose cells outside U hold +0 like the input's
// (the mixed form's invariant). The per-cell arithmetic is v_sweep19's:
// faces then edges, each a left fold, folded into b with the exact products
// by -1/2 and -1/4.
#include "ops_dev.cuh"

namespace cfmg {

constexpr int kT3dW = 64, kT3dH = 32;  // tile (i, j) with halo
constexpr int kT3dThreads = 1024;
constexpr int kT3dCells = kT3dW * kT3dH / kT3dThreads;  // cells per thread and plane (2)
constexpr int kT3dPlane = kT3dW * kT3dH;

template <int S, bool L19>
__global__ void __launch_bounds__(kT3dThreads, 1) k_smooth_tb3d(const float* __restrict__ x, float* __restrict__ xo,
                                                                const float* __restrict__ b,
                                                                const float* __restrict__ w, float cff, int tx, int ty,
                                                                int tz, int ui0, int ui1, int uj0, int uj1, int uk0,
                                                                int uk1, int kchunk, Box eb) {
  dep_wait();
  constexpr int H = S;
  constexpr int CW = kT3dW - 2 * H, CH = kT3dH - 2 * H;
  extern __shared__ float smem[];
  float* LV = smem;                            // levels 0..S-1, 3 planes each
  float* BR = smem + S * 3 * kT3dPlane;        // b ring, S+1 planes
  float* WR = BR + (S + 1) * kT3dPlane;        // omega*idiag ring, S+1 planes
  const int ti0 = ui0 + (int)blockIdx.x * CW - H;  // tile origin (1-based)
  const int tj0 = uj0 + (int)blockIdx.y * CH - H;
  const int ka = uk0 + (int)blockIdx.z * kchunk;  // output planes ka..kb
  const int kb = min(ka + kchunk - 1, uk1);
  const long long n1 = tx, n2 = (long long)tx * ty;
  auto lvl = [&](int s, int p) { return LV + (s * 3 + ((p % 3) + 3) % 3) * kT3dPlane; };
  auto ring = [&](float* R, int p) { return R + (((p % (S + 1)) + (S + 1)) % (S + 1)) * kT3dPlane; };
  // the thread's cells: c = threadIdx.x + e * kT3dThreads, (li, lj) = (c % W, c / W)
  // Plane p+1 is read from global memory into registers while the levels of
  // step p compute, and stored to shared memory at the start of step p+1.
  float rx[kT3dCells], rb[kT3dCells], rw[kT3dCells];
  auto fetch = [&](int p) {
#pragma unroll
    for (int e = 0; e < kT3dCells; ++e) {
      const int c = threadIdx.x + e * kT3dThreads;
      const int gi = ti0 + c % kT3dW, gj = tj0 + c / kT3dW;
      const bool in = gi >= 1 && gi <= tx && gj >= 1 && gj <= ty && p >= 1 && p <= tz;
      const long long I = (long long)(gi - 1) + n1 * (gj - 1) + n2 * (p - 1);
      rx[e] = in ? x[I] : 0.f;
      rb[e] = in ? b[I] : 0.f;
      rw[e] = in ? w[I] : 0.f;
    }
  };
  fetch(ka - S);
  for (int p = ka - S; p <= kb + S; ++p) {
    {
      float* X = lvl(0, p);
      float* Bp = ring(BR, p);
      float* Wp = ring(WR, p);
#pragma unroll
      for (int e = 0; e < kT3dCells; ++e) {
        const int c = threadIdx.x + e * kT3dThreads;
        X[c] = rx[e];
        Bp[c] = rb[e];
        Wp[c] = rw[e];
      }
    }
    if (p < kb + S) fetch(p + 1);
    __syncthreads();
    // level s at plane p - s, from level s-1 at planes p-s-1 .. p-s+1
#pragma unroll
    for (int s = 1; s <= S; ++s) {
      const int q = p - s;
      if (q >= ka - S + s && q <= kb + S - s) {
        const float* Xm = lvl(s - 1, q - 1);
        const float* X0 = lvl(s - 1, q);
        const float* Xp = lvl(s - 1, q + 1);
        const float* Bq = ring(BR, q);
        const float* Wq = ring(WR, q);
        float out[kT3dCells];
#pragma unroll
        for (int e = 0; e < kT3dCells; ++e) {
          const int c = threadIdx.x + e * kT3dThreads;
          const int li = c % kT3dW, lj = c / kT3dW;
          const int gi = ti0 + li, gj = tj0 + lj;
          const bool inU = (L19 && s == 1)
                               ? (gi >= eb.i0 && gi <= eb.i1 && gj >= eb.j0 && gj <= eb.j1 && q >= eb.k0 && q <= eb.k1)
                               : (gi >= ui0 && gi <= ui1 && gj >= uj0 && gj <= uj1 && q >= uk0 && q <= uk1);
          // neighbours, clamped to the tile (values outside the valid region are never used)
          const bool hw = li > 0, he = li < kT3dW - 1, hs = lj > 0, hn = lj < kT3dH - 1;
          const int cw = hw ? c - 1 : c, ce = he ? c + 1 : c;
          const int cs = hs ? c - kT3dW : c, cn = hn ? c + kT3dW : c;
          typedef Ar<float> A;
          float v;
          if (L19) {
            const int cws = (hw && hs) ? c - 1 - kT3dW : c, ces = (he && hs) ? c + 1 - kT3dW : c;
            const int cwn = (hw && hn) ? c - 1 + kT3dW : c, cen = (he && hn) ? c + 1 + kT3dW : c;
            const float f = A::add(A::add(A::add(A::add(A::add(X0[cw], X0[ce]), X0[cs]), X0[cn]), Xm[c]), Xp[c]);
            float e = A::add(X0[cws], X0[ces]);
            e = A::add(e, X0[cwn]);
            e = A::add(e, X0[cen]);
            e = A::add(e, Xm[cw]);
            e = A::add(e, Xm[ce]);
            e = A::add(e, Xp[cw]);
            e = A::add(e, Xp[ce]);
            e = A::add(e, Xm[cs]);
            e = A::add(e, Xm[cn]);
            e = A::add(e, Xp[cs]);
            e = A::add(e, Xp[cn]);
            float t = A::fmx(f, -0.5f, Bq[c]);
            t = A::fmx(e, -0.25f, t);
            v = A::sub(A::mul(cff, X0[c]), A::mul(Wq[c], t));
          } else {
            const float f = A::add(A::add(A::add(A::add(A::add(X0[cw], X0[ce]), X0[cs]), X0[cn]), Xm[c]), Xp[c]);
            v = A::sub(A::mul(cff, X0[c]), A::mul(Wq[c], A::sub(Bq[c], f)));
          }
          out[e] = inU ? v : X0[c];
        }
        if (s < S) {
          float* Y = lvl(s, q);
#pragma unroll
          for (int e = 0; e < kT3dCells; ++e) Y[threadIdx.x + e * kT3dThreads] = out[e];
        } else if (q >= ka && q <= kb) {
#pragma unroll
          for (int e = 0; e < kT3dCells; ++e) {
            const int c = threadIdx.x + e * kT3dThreads;
            const int li = c % kT3dW, lj = c / kT3dW;
            const int gi = ti0 + li, gj = tj0 + lj;
            if (li >= H && li < kT3dW - H && lj >= H && lj < kT3dH - H && gi >= ui0 && gi <= ui1 && gj >= uj0 &&
                gj <= uj1)
              xo[(long long)(gi - 1) + n1 * (gj - 1) + n2 * (q - 1)] = out[e];
          }
        }
      }
      __syncthreads();
    }
  }
}

template <int S, bool L19 = false>
static void launch_tb3d_s(const float* x, float* xo, const float* b, const float* w, float cff, int tx, int ty, int tz,
                          int ui0, int ui1, int uj0, int uj1, int uk0, int uk1, cudaStream_t st, Box eb = Box{}) {
  constexpr int CW = kT3dW - 2 * S, CH = kT3dH - 2 * S;
  const size_t smem = (size_t)(3 * S + 2 * (S + 1)) * kT3dPlane * sizeof(float);
  static bool attr = false;
  static int nsm = 0;
  if (!attr) {
    cudaFuncSetAttribute(k_smooth_tb3d<S, L19>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    attr = true;
  }
  const int ntx = (ui1 - ui0 + CW) / CW, nty = (uj1 - uj0 + CH) / CH;
  const int nk = uk1 - uk0 + 1;
  // k chunks: enough CTAs for about three waves of one CTA per SM
  int nchunk = (3 * nsm + ntx * nty - 1) / (ntx * nty);
  nchunk = nchunk < 1 ? 1 : (nchunk > nk ? nk : nchunk);
  const int kchunk = (nk + nchunk - 1) / nchunk;
  nchunk = (nk + kchunk - 1) / kchunk;
  dim3 grid((unsigned)ntx, (unsigned)nty, (unsigned)nchunk);
  launch_dep(k_smooth_tb3d<S, L19>, grid, kT3dThreads, smem, st, x, xo, b, w, cff, tx, ty, tz, ui0, ui1, uj0, uj1, uk0,
             uk1, kchunk, eb);
}

// the 19-point operator's pair (E, then the interior box U) in one pass, x -> xo
void launch_smooth_tb3d19(const float* x, float* xo, const float* b, const float* w, float cff, int tx, int ty, int tz,
                          const Box& interior, const Box& ext, cudaStream_t st) {
  launch_tb3d_s<2, true>(x, xo, b, w, cff, tx, ty, tz, interior.i0, interior.i1, interior.j0, interior.j1, interior.k0,
                         interior.k1, st, ext);
}

// nite pairs (1 or 2) of 7-point sweeps over the box U in one pass, x -> xo
bool launch_smooth_tb3d(int nite, const float* x, float* xo, const float* b, const float* w, float cff, int tx,
                        int ty, int tz, int ui0, int ui1, int uj0, int uj1, int uk0, int uk1, cudaStream_t st) {
  if (nite == 1) {
    launch_tb3d_s<2>(x, xo, b, w, cff, tx, ty, tz, ui0, ui1, uj0, uj1, uk0, uk1, st);
    return true;
  }
  if (nite == 2) {
    launch_tb3d_s<4>(x, xo, b, w, cff, tx, ty, tz, ui0, ui1, uj0, uj1, uk0, uk1, st);
    return true;
  }
  return false;
}

}  // namespace cfmg
