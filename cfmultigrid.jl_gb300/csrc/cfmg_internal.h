// Internal declarations shared by the libcfmg translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <utility>
#include <vector>

#include "../../include/cfmg.h"

namespace cfmg {

// ---- programmatic dependent launch
// Kernels of a cycle run back to back on one stream, each depending on the
// one before. Launched with the programmatic-serialization attribute, a
// kernel is scheduled as soon as its predecessor's blocks have all exited,
// before the predecessor's completion is processed, so the launch latency
// overlaps that completion. Every kernel launched this way opens with
// dep_wait(): griddepcontrol.wait returns once the predecessor has
// completed and its writes are visible, before the kernel touches global
// memory. Launched without the attribute it is a no-op, so a kernel that
// opens with dep_wait() is correct either way. (Letting each block trigger
// its dependents at its start, griddepcontrol.launch_dependents, measured
// slower: 14.4 against 13.5 ms per configuration-2 solve, with chains of
// waiting dependents holding SM slots.)
#ifdef __CUDACC__
__device__ __forceinline__ void dep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
#endif
// per host thread: whether launch_dep sets the attribute (the handle's
// CFMG_OPT_DEPENDENT_LAUNCH, applied by each of its launches)
extern thread_local bool tl_dep_launch;
template <typename... KArgs, typename... Args>
inline cudaError_t launch_dep(void (*k)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                              Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute a[1];
  a[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  a[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = a;
  cfg.numAttrs = tl_dep_launch ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, k, std::forward<Args>(args)...);
}

// One level of the hierarchy on the device. Reference layout: column-major
// tx*ty*tz arrays (src/gmg_types.jl:68-118), plus the derived arrays the
// kernels stream instead of recomputing:
//   widiag = omega*idiag (bit-identical to the reference's omega*idiag[I])
//   the FP32 copies used by the mixed-precision cycles.
struct Level {
  int nx, ny, nz, nh, tx, ty, tz;
  bool threed;
  size_t len;
  double *x, *y, *r, *b, *diag, *idiag, *widiag, *Rcoef, *Pcoef, *kappa;
  double *cE, *cN;  // face coefficients of the variable-coefficient operator
  uint8_t* msk;
  // mixed precision copies (used by CFMG_MIXED)
  float *x32, *y32, *r32, *b32, *widiag32, *diag32, *Rcoef32, *Pcoef32, *cE32, *cN32;
  // 3D 7-point mixed form: the FP32 omega*idiag as a one-byte code c = diag
  // (0: omega*idiag = 0) into the handle's table wtab (prepare_wq, cfmg_api.cu)
  uint8_t* wq;
  // the same levels, four-cell sweep: 1 for each (run of planes, quad of a
  // plane) holding a wet cell (launch_make_qact); dry quads are skipped
  uint8_t* qact;
  int xswap;  // 1: the FP32 x currently lives in y32 (after a temporally blocked smoothing)
  int ic0, ic1, jc0, jc1, kc0, kc1;  // interior box (1-based inclusive)
};

struct Box {  // 1-based inclusive index box
  int i0, i1, j0, j1, k0, k1;
};

// Geometry passed by value to kernels.
struct Geom {
  int tx, ty, tz, nh;
  long long len, n1, n2;  // n1 = tx, n2 = tx*ty
};

inline Geom geom(const Level& l) {
  Geom g;
  g.tx = l.tx; g.ty = l.ty; g.tz = l.tz; g.nh = l.nh;
  g.len = (long long)l.len;
  g.n1 = l.tx;
  g.n2 = (long long)l.tx * l.ty;
  return g;
}

// ---- per-level operators (k_ops.cu), templated on the field type T
// (double: bit-exact parity form; float: the mixed-precision cycles).
template <class T>
void launch_sweep5_2d(const T* x, T* y, const T* b, const T* widiag, T cff, const Geom& g, cudaStream_t s);
template <class T>
void launch_sweep7_3d(const T* x, T* y, const T* b, const T* widiag, T cff, const Geom& g, cudaStream_t s);
// the same FP32 7-point sweep with omega*idiag read as wtab[wq[I]]; x_zero:
// x holds +0 in every cell and is not read (four-cell form only, see
// sweep7_quad_ok)
void launch_sweep7_3d_q(const float* x, float* y, const float* b, const uint8_t* wq, const float* wtab, float cff,
                        const Geom& g, cudaStream_t s, bool x_zero = false, const uint8_t* qact = nullptr);
// quad activity flags of a 3D level for the four-cell sweep (runs of kQRunPlanes planes)
constexpr int kQRunPlanes = 4;
void launch_make_qact(const uint8_t* m, uint8_t* qact, long long n2, int tz, int run, cudaStream_t s);
bool sweep7_quad_ok(const Geom& g, const void* x, const void* y, const void* b, const void* wq);
// one smoothing call (npairs pairs) of a level held in one block's shared
// memory (k_ops.cu); stencil 5 (2D 5-point), 9 (2D 9-point), 7 (3D 7-point)
struct SmallSm {
  void* x;
  void* y;
  const void* b;
  const void* w;
  Geom g;
  int stencil, npairs;
  Box ext, in;
  double cff;
};
constexpr size_t kSmallSmemMax = 200 * 1024;  // 4 arrays of the level
// FP64 levels of at least this many cells run on a cluster of 8 CTAs (the
// FP64 pipe of one SM bounds the one-block form)
constexpr long long kSmallCluMinCells = 512;
template <class T>
void launch_small_smooth(const SmallSm& s, cudaStream_t st);
// FP32 3D 7-point cell-centred residual at the children of the coarse box cb
// restricted into the coarse b (k_ops.cu); dc: diag as one-byte codes
void launch_resid_restrict7c(const float* x, const float* b, const uint8_t* dc, const uint8_t* m, const float* rcoef,
                             float* bc, const Geom& gf, const Geom& gc, const Box& cb, cudaStream_t s,
                             bool skip_dry = false);
template <class T>
void launch_sweep9_2d(const T* x, T* y, const T* b, const T* widiag, T cff, const Geom& g, const Box& bx,
                      cudaStream_t s);
template <class T>
void launch_sweep19_3d(const T* x, T* y, const T* b, const T* widiag, T cff, const Geom& g, const Box& bx,
                       cudaStream_t s);
// variable coefficient: cE[I] / cN[I] are the face coefficients between I
// and I+1 / I+n1 (0 across a dry cell)
template <class T>
void launch_sweep_vc_2d(const T* x, T* y, const T* b, const T* widiag, const T* cE, const T* cN, T cff,
                        const Geom& g, cudaStream_t s);
template <class T>
void launch_resid5_2d(T* r, const T* x, const T* b, const T* diag, const uint8_t* msk, const Geom& g,
                      cudaStream_t s);
template <class T>
void launch_resid7_3d(T* r, const T* x, const T* b, const T* diag, const uint8_t* msk, const Geom& g,
                      const Box& bx, cudaStream_t s);
template <class T>
void launch_resid9_2d(T* r, const T* x, const T* b, const T* diag, const uint8_t* msk, const Geom& g,
                      const Box& bx, cudaStream_t s);
template <class T>
void launch_resid19_3d(T* r, const T* x, const T* b, const T* diag, const uint8_t* msk, const Geom& g,
                       const Box& bx, cudaStream_t s);
template <class T>
void launch_resid_vc_2d(T* r, const T* x, const T* b, const T* diag, const T* cE, const T* cN,
                        const uint8_t* msk, const Geom& g, cudaStream_t s);
// restriction: fine field -> coarse b over the coarse interior box;
// kind: 0 centres 2D, 1 centres 3D, 2 vertices 2D, 3 vertices 3D
template <class T>
void launch_restrict(int kind, const T* xf, T* bc, const T* Rcoef, const Geom& gf, const Geom& gc,
                     const Box& cbox, cudaStream_t s);
// prolongation: fine x += Pcoef * P(coarse x); same kinds; (nxf, nyf, nzf)
// are the fine level's nx, ny, nz and [kf0, kf1] its k-range of parents.
template <class T>
// fmsk != null (FP32 3D cell-centred only): parents whose eight children are all dry are skipped
void launch_prolong(int kind, T* xf, const T* xc, const T* Pcoef, const Geom& gf, const Geom& gc, int nxf, int nyf,
                    int nzf, int kf0, int kf1, bool assign, cudaStream_t s, const uint8_t* fmsk = nullptr);
template <class T>
void launch_fill_xperio(T* x, const Geom& g, cudaStream_t s);
// norm: deterministic sum of msk*x^2 (FP64 accumulation) over the whole
// array into out[0], with 0 -> 1 for the reference rule
// (src/operators_at_level.jl:21-23). When normb != nullptr, out[1] is the
// residual ratio: sum/normb (CFMG_NORM_REF_SQUARED) or sqrt(sum/normb) (L2).
template <class T>
void launch_norm(const T* x, const uint8_t* msk, size_t n, double* partials, double* out, const double* normb,
                 int norm_kind, cudaStream_t s);
constexpr int kNormParts = 1024;
// the handle's partial-sum scratch: two sums per block for the fused
// residual pass of the mixed loop (k_mixed.cu), one for the norms
constexpr int kPartials = 2 * kNormParts;
// the fused residual passes of the mixed loop (k_mixed.cu, k_resid3d.cu):
// threads per block, and at most kMxParts blocks with two partial sums each
constexpr int kMxThreads = 256;
constexpr int kMxParts = 1024;
static_assert(2 * kMxParts <= kPartials, "the fused pass writes 2*kMxParts partial sums");

// ---- operator descriptors and the coarse-level program engine (k_coarse.cu)
// One Op describes one launch-worth of work on one level: its kind, the
// arithmetic (prec 0 = double, 1 = float), its operands and its index space
// of n work items. Fine levels run an Op as a standalone kernel; consecutive
// Ops on coarse levels are gathered into a program that one cluster-launched
// kernel executes, with a cluster barrier between Ops.
enum OpKind : int {
  OPK_SWEEP5 = 0, OPK_SWEEP7, OPK_SWEEP9, OPK_SWEEP19, OPK_SWEEPVC,
  OPK_RESID5, OPK_RESID7, OPK_RESID9, OPK_RESID19, OPK_RESIDVC,
  OPK_RESTRICT0, OPK_RESTRICT1, OPK_RESTRICT2, OPK_RESTRICT3,
  OPK_PROLONG0, OPK_PROLONG1, OPK_PROLONG2, OPK_PROLONG3,
  OPK_FILL, OPK_ZERO, OPK_F32TO64, OPK_F64TO32,
  // solve-loop ops of whole-solve programs (the batched engine): they act
  // on the program's scalar block sc[] (see SolveSlot)
  OPK_NORM64,    // sc[s0] = sum msk*x^2 (0 -> 1 when s1 != 0)
  OPK_MEAN64,    // sc[s0] = (sum msk*x) / sc[s1]
  OPK_RATIO,     // sc[s0] = sc[s1]/sc[s2] (norm_kind REF) or sqrt of it (L2); 0 when sc[s2] <= 0
  OPK_SCALE,     // sc[s0] = 1/rms, sc[s0+1] = rms with rms = sqrt(sc[s1]/sc[s2])
  OPK_RHS32,     // y (b32) = y2 (r32) = msk ? (x - sc[s1]) * sc[s0] : 0
  OPK_UPDATE,    // y (x64) += (double) x (e32) * sc[s0]
  OPK_BRANCH,    // continue while sc[s0] > tol && sc[s1] < maxite (then sc[s1] += 1), else jump to s2
  OPK_JUMP,      // jump to s2
  OPK_STAMP,     // sc[s0] = %globaltimer (ns)
  OPK_HIST,      // sc[s0 + sc[s1]] = sc[s2]
  OPK_ZERO_IF,   // y[0..n) = 0 (double) when sc[s0] != 0
  // batched solver: one temporally blocked FP32 smoothing pass, x -> y over
  // the update box `box`; np_i = sweep pairs (1..3), np_j = stencil (5 or
  // 9), kf0 x kf1 tiles per layer, n = tiles in all layers
  OPK_TB,
};
struct Op {
  int kind, prec, lev, cls;  // cls: CFMG_K_* class for accounting
  long long n;               // work items
  long long lo;              // linear ops: first index
  Box box;                   // box ops: index box
  Geom g, gc;                // level (and coarse level for R/P)
  int np_i, np_j, kf0, kf1;  // prolongation parents
  double cff;
  const void *x, *b, *w, *d, *cE, *cN, *coef;
  void* y;  // the written field: sweep y, residual r, coarse b, fine x, filled/zeroed field
  const uint8_t* m;
  // solve-loop ops
  double* sc;
  void* y2;
  double tol;
  int s0, s1, s2, maxite, norm_kind;
  int inst;  // batched solver: the instance the Op belongs to
  int assign;  // standalone prolongation onto a fine x known to be +0: written, not read
  // standalone FP32 sweeps: omega*idiag read as wtab[wq[I]] instead of w[I] (same bits)
  const uint8_t* wq;
  const float* wtab;
  const uint8_t* qact;  // the level's quad activity flags (see Level), or null: every quad swept
  int form;  // OPK_TB: 5 the lean packed tiles (k_btb5), else the scalar tiles (k_btb)
};
// scalar block of a whole-solve program
enum SolveSlot { SS_NORMB = 0, SS_NR, SS_RES, SS_NITE, SS_NWET, SS_MEAN, SS_SCALE, SS_ISCALE, SS_T0, SS_T1,
                 SS_ZEROX, SS_HIST };
void launch_batch(const Op* const* progs, const int* nops, int ninst, int* counter, double* red, int nclusters,
                  cudaStream_t s);
int engine_max_clusters();
constexpr int kEngineCtas = 8;      // cluster size (portable)
constexpr int kEngineThreads = 1024;
void launch_op(const Op& op, cudaStream_t s);                   // one Op as a standalone kernel
void launch_program(const Op* prog, int nops, double* red, cudaStream_t s);  // a device-resident program

// 3D 7-point streaming blocked passes (k_tb3d.cu): nite (1 or 2) pairs over U
bool launch_smooth_tb3d(int nite, const float* x, float* xo, const float* b, const float* w, float cff, int tx,
                        int ty, int tz, int ui0, int ui1, int uj0, int uj1, int uk0, int uk1, cudaStream_t st);
// the 3D 19-point smoothing call (one pair: the box ext, then the interior) in one streaming pass, x -> xo
void launch_smooth_tb3d19(const float* x, float* xo, const float* b, const float* w, float cff, int tx, int ty, int tz,
                          const Box& interior, const Box& ext, cudaStream_t st);
// temporally blocked FP32 smoother (k_tb.cu): nite pairs of 5- or 9-point
// sweeps over the box U in one pass, x -> xo; false if nite is not
// 1..kTbMaxPairs. A pass of p pairs recomputes a halo of 2p cells around each
// tile: 3 pairs suit large levels, longer passes cut the launches of the
// many-pair coarsest solves.
constexpr int kTbMaxPairs = 10;
// version 5: lean packed FP32x2 passes (128 x 48 tiles); 3 (and 4): the first
// packed form; 1: one column per thread
bool launch_smooth_tb(int version, int stencil, int nite, const float* x, float* xo, const float* b, const float* w,
                      float cff, int tx, int ty, int nz, int ui0, int ui1, int uj0, int uj1, cudaStream_t s);
// the lean packed passes for the x-periodic topology, 5-point operator: the
// tiles cover the interior columns [ui0, ui1] and read the periodic images
// of the columns beside them; the caller fills the halo columns afterwards
bool launch_smooth_tb_periodic(int nite, const float* x, float* xo, const float* b, const float* w, float cff,
                               int tx, int ty, int nz, int ui0, int ui1, int uj0, int uj1, cudaStream_t s);
// The last pass of a V-cycle's pre-smoothing with the step that follows it
// in the same kernel (2D, single layer): the residual of the smoothed x,
// restricted to the coarse b, and the coarse x zeroed at the same cells.
// The residual box is the reference's for the operator (interior box for
// the 9-point, all cells of rows 2..ty-1 for the 5-point range); r outside
// it is 0, as in the level's r array.
struct TbEpi {
  const float* d;      // FP32 diag of the level
  const uint8_t* m;    // mask of the level
  const float* rcoef;  // FP32 Rcoef of the coarse level
  float* bc;           // coarse b
  float* xc;           // coarse x (current buffer)
  int ri0, ri1, rj0, rj1;  // residual box (1-based, inclusive)
  int nh;
  int ctx;             // coarse row stride
  int ci0, ci1, cj0, cj1;  // coarse interior box (1-based, inclusive)
  int pkind;           // restriction: 0 cell centres (2 x 2 sum), 2 vertices (1-2-1 x 1-2-1)
  double* xd;          // solution-update form: the level's FP64 x, updated in place
  double* ds;          // solution-update form: the handle's device scalars (S_ICUR, S_MAXX)
};
bool launch_smooth_tb_epi(int stencil, int nite, const float* x, float* xo, const float* b, const float* w, float cff,
                          int tx, int ty, int ui0, int ui1, int uj0, int uj1, const TbEpi& ep, cudaStream_t s);
// The last post-smoothing pass of a mixed-precision cycle on level 1 (2D,
// 1..3 pairs) with the FP64 solution update x += e * iscale in its output
// phase instead of storing e; max |x| of the updated cells goes to
// ds[S_MAXX]. False: no such form for these arguments.
bool launch_smooth_tb_upd(int stencil, int nite, const float* x, const float* b, const float* w, float cff, int tx,
                          int ty, int nz, int ui0, int ui1, int uj0, int uj1, double* xd, double* ds, cudaStream_t s);

// ---- batched solver (k_batch.cu): independent 2D instances advance in
// lockstep, one launch per step of the iteration for all of them. Every
// launch is a grid-stride loop over the chunks (kBChunk work items) of its
// Ops; a chunk of an instance that has converged is skipped.
constexpr int kBChunk = 1024;
constexpr int kBThreads = 256;
constexpr int kBStageChunk = 8192;  // items of one entry of a generic step's table (k_bstage)
// per-instance scalar block (double): see k_bfinal for their use
enum BSlot { BS_NORMB = 0, BS_RES, BS_NITE, BS_NWET, BS_NEXT, BS_CUR, BS_ICUR, BS_MEAN, BS_T0, BS_T1, BS_ZEROX,
             BS_MAXX, BS_MAXB, BS_SHIFT, BS_HIST };
// level-1 state of one instance for the FP64 steps of its solve loop
struct BInst {
  double *x, *b, *r, *d;
  const uint8_t* m;
  float *b32, *r32;
  const float* e32;  // the FP32 correction after the cycle
  double* sc;        // scalar block (BSlot)
  Geom g;
  Box box;
  long long lo, n;   // the residual's index space: linear lo + t (5-point) or the box (9-point)
  long long len;
  int kind, neumann, norm_kind, maxite;
  double tol;
  // integer form of the residual (when every instance has it): Q*diag, and
  // the index space as row strips (see k_resid_int2d)
  const int8_t* dq;
  long long row0;
  int c0, ncols, nrows, nstrips;
};
// Smoothing of a small level (the coarsest solve, or a coarse level's
// pre/post smoothing) of one instance by one block in shared memory: x, b,
// omega*idiag and y are staged, the npairs pairs of sweeps run with the
// operator's own ranges and per-cell arithmetic (prec 0: FP64, the FP32
// x and b converted as the coarsest solve does), and x goes back to x32.
struct BSmall {
  int inst, prec, stencil, npairs;  // stencil 5: linear range lo..lo+n; 9: ext then interior box
  Geom g;
  Box ext, in;
  long long lo, n;
  const float* b32;
  float* x32;
  const void* w;  // omega*idiag, FP64 or FP32 as prec
  const void* y;  // the level's partner buffer (cells outside the sweep ranges are read, never written)
  double cff;
};
constexpr int kBSmallBytes = 96 * 1024;  // shared memory of one block: 4 arrays
void launch_bsmall(const BSmall* s, int n, int smem, const int* active, cudaStream_t st);
// Coarse runs: one block per run {instance, first entry, end entry, 0}
// executes the instance's consecutive coarse-level steps in order, entries
// {0, Op} or {1, BSmall}; smem = the largest BSmall staging of the runs.
constexpr int kBRunThreads = 512;
void launch_brun(const Op* ops, const BSmall* sm, const int2* ent, const int4* runs, int nruns, int smem,
                 const int* active, cudaStream_t st);

// Work tables: one int4 per chunk (or tile) = {Op or instance, chunk of it,
// instance, 0}; a launch compacts the active entries of each window.
void launch_bstage(const Op* ops, const int4* tab, long long nchunks, const int* active, cudaStream_t s);
void tb_tiles(int nite, int ui0, int ui1, int uj0, int uj1, int* ntx, int* nty);
bool launch_btb(int stencil, int nite, const Op* ops, const int4* tab, long long ntiles, const int* active,
                cudaStream_t s);
// the same for the lean packed pass (OPK_TB Ops of form 5)
void tb5_tiles(int nite, int ui0, int ui1, int uj0, int uj1, int* ntx, int* nty);
bool launch_btb5(int stencil, int nite, const Op* ops, const int4* tab, long long ntiles, const int* active,
                 cudaStream_t s);
void launch_binit(const BInst* bi, int ninst, int zero_x, int* active, int* nactive, cudaStream_t s);
void launch_bres(int kind, bool neumann, const BInst* bi, const int4* tab, long long nchunks, const int* active,
                 double* partials, cudaStream_t s);
void launch_bfinal(const BInst* bi, const long long* cstart, int ninst, const double* partials, int* active,
                   int* nactive, cudaStream_t s);
// integer residual: warp tasks {instance, strip, row chunk, 0}, partials 2 per task
constexpr int kBIntRows = 32;
constexpr int kBIntCols = 30;  // output columns of a warp strip (lanes 1..30)
void launch_bres_int(int kind, bool neumann, const BInst* bi, const int4* ttab, long long ntasks, const int* active,
                     double* partials, cudaStream_t s);
void launch_brhs_shift(const BInst* bi, const int4* tab, long long nchunks, const int* active, cudaStream_t s);
void launch_brhs(const BInst* bi, const int4* tab, long long nchunks, const int* active, cudaStream_t s);
void launch_bupdate(const BInst* bi, const int4* tab, long long nchunks, const int* active, cudaStream_t s);
void launch_bcond(cudaGraphConditionalHandle hc, int* nactive, cudaStream_t s);

// device scalars of a handle (dscal[])
enum Scal { S_NORM = 0, S_RES = 1, S_NORMB = 2, S_NWET = 3, S_SCALE = 4, S_MEAN = 5, S_TMP0 = 6, S_ISCALE = 7,
            S_NEXT = 8, S_CUR = 9, S_ICUR = 10, S_MEAN2 = 11, S_MAXX = 12, S_MAXB = 13, S_NITE = 14,
            S_SHIFT = 15, S_MAXO = 16,
            // 1 after a bounded wait in a kernel ran out (k_resid3d.cu); the solve reports it
            S_FAULT = 17, S_COUNT = 18 };

// fused FP64 steps of the mixed loop (k_mixed.cu)
void launch_resid_fused(int kind, double* r, const double* x, const double* b, const double* d, const uint8_t* m,
                        const Geom& g, const Box& bx, long long lo, long long n, const double* scale, float* b32,
                        float* r32, bool neumann, double* partials, cudaStream_t s);
void launch_fused_final(const double* partials, double* ds, const double* normb, const double* nwet, int norm_kind,
                        cudaStream_t s);
void launch_rhs32_mean(const double* r, const uint8_t* m, const double* mean_scale, float* b32, float* r32,
                       long long n, cudaStream_t s);
void launch_update_scaled(double* x, const float* e, const double* iscale, long long n, cudaStream_t s);
// integer form of the fused pass (kinds 5-, 7- and 9-point)
void launch_resid_int(int kind, const double* x, const double* b, const int8_t* dq, const Geom& g, const Box& bx,
                      long long lo, long long n, const double* ds, float* b32, float* r32, bool neumann,
                      double* partials, cudaStream_t s);
// 2D single-layer form (each x converted once); false: use launch_resid_int.
// Its warps read x up to kResidIntReach elements before x[0] and after
// x[len-1] (lanes 0 and 31 beside a strip, the last strip past the row end)
// and never use those values: x must lie inside an allocation with at least
// that many elements on either side, as level 1's x does in a handle's arena
// (checked by cfmg_create).
constexpr int kResidIntReach = 32;
// sflag (optional): per-(plane, row, strip) wet flags (launch_make_sflag);
// strip tasks whose rows are all dry are skipped
bool launch_resid_int2d(int kind, const double* x, const double* b, const int8_t* dq, const Geom& g, const Box& bx,
                        const double* ds, float* b32, float* r32, bool neumann, double* partials, cudaStream_t s,
                        const uint8_t* sflag = nullptr);
long long resid_sflag_size(int kind, const Geom& g, const Box& bx);
void launch_make_sflag(int kind, const uint8_t* m, uint8_t* sflag, const Geom& g, const Box& bx, cudaStream_t s);
// 3D 7-point form with TMA-staged planes (k_resid3d.cu). dqp: dq with rows
// padded to txp = dq_pitch(tx) bytes (launch_pad_dq). false: not applicable
// (odd tx, misaligned arrays, no tensor-map encoder): use launch_resid_int2d.
int dq_pitch(int tx);
void launch_pad_dq(const int8_t* dq, int8_t* dqp, int tx, int txp, long long rows, cudaStream_t s);
// tcol (optional): per-(tile, plane) wet flags (launch_make_tcol); tasks whose
// planes are all dry are skipped (two rows a thread, and r32 not written, only)
bool launch_resid_int3d(const double* x, const double* b, const int8_t* dqp, const Geom& g, const Box& bx,
                        double* ds, float* b32, float* r32, bool neumann, double* partials, cudaStream_t s,
                        int rows_per_thread, const uint8_t* tcol = nullptr);
long long resid3d_tcol_size(const Geom& g, const Box& bx);
void launch_make_tcol(const uint8_t* m, uint8_t* tcol, const Geom& g, const Box& bx, cudaStream_t s);
// skip_dry: groups of 16 dry cells are neither read nor written (their b32 is +0 already)
void launch_rhs32_shift(const uint8_t* m, const double* mean_scale, float* b32, float* r32, long long n,
                        cudaStream_t s, bool skip_dry = false);
void launch_make_dq(const double* diag, const uint8_t* m, double Q, int8_t* dq, long long n, int* ok, cudaStream_t s);
// max |x|, max |b| and max |x| outside the box U of every layer (S_MAXX, S_MAXB, S_MAXO)
// m != null: "outside U" is instead every cell with m == 0 (the dry cells)
void launch_maxabs2(const double* x, const double* b, long long n, int tx, int ty, int ui0, int ui1, int uj0, int uj1,
                    double* ds, cudaStream_t s, const uint8_t* m = nullptr);
// msk != null: groups of 4 dry cells (e = +0 there) are skipped; their max |x| must be in S_MAXO
void launch_update_scaled_max(double* x, const float* e, double* ds, long long n, cudaStream_t s,
                              const uint8_t* msk = nullptr);

// message returned by cfmg_last_error(NULL) (cfmg_api.cu)
void set_global_error(const std::string& msg);

// ---- setup kernels (k_setup.cu)
enum DefMskMode { DEFMSK_SET = 0, DEFMSK_MUL = 1, DEFMSK_SCALE_F64 = 2 };
void launch_default_msk(int mode, uint8_t* msk, double* f, double coef, const Level& l, bool vertices, bool threed,
                        bool xperio, cudaStream_t s);
void launch_fill_f64(double* a, double v, size_t n, cudaStream_t s);
void launch_u8_to_f64(const uint8_t* m, double* out, size_t n, cudaStream_t s);
void launch_threshold(const double* b, uint8_t* msk, double thr, size_t n, cudaStream_t s);
void launch_rcoef(const uint8_t* msk, const double* b, double* Rcoef, bool vertices, double coef, size_t n,
                  cudaStream_t s);
void launch_pcoef(const uint8_t* msk, const double* x, double* Pcoef, size_t n, cudaStream_t s);
void launch_diag(const uint8_t* msk, const double* r, double* diag, double* idiag, size_t n, cudaStream_t s);
void launch_widiag(const double* idiag, double* widiag, double omega, size_t n, cudaStream_t s);
void launch_restrict_kappa(const double* kf, const uint8_t* mf, double* kc, const Geom& gf, const Geom& gc,
                           const Box& cbox, cudaStream_t s);
void launch_face_coef(const double* kappa, const uint8_t* msk, double* cE, double* cN, const Geom& g,
                      cudaStream_t s);
void launch_to_f32(const double* a, float* out, size_t n, cudaStream_t s);
// the omega*idiag code table: tab[c] = (float)(omega * (1 / (c / Q))) for c = 1..255, tab[0] = 0,
// with the FP64 operations of k_diag and k_widiag; then the codes of one level (ok cleared when
// a cell's diag is not c/Q or its FP32 omega*idiag differs from tab[c] in any bit)
void launch_wq_table(float* tab, double omega, double Q, cudaStream_t s);
void launch_make_wq(const double* diag, const float* w32, const float* tab, double Q, uint8_t* wq, long long n,
                    int* ok, cudaStream_t s);

}  // namespace cfmg
