// libcfmg host runtime: handle, level hierarchy, operator dispatch, cycles
// and the solve loop, behind the C ABI of include/cfmg.h.
//
// Structure mirrors the reference's Gmg object (src/gmg_types.jl:121-132):
// a handle owns the levels, and every operator is dispatched on
// (case, operator, location) exactly as allocate_mg binds the function
// tables (src/gmg_setup.jl:86-101,124-157). There is no CPU fallback:
// every operator is a CUDA kernel launch on the handle's stream.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <algorithm>
#include <mutex>
#include <unordered_map>

#include "cfmg_internal.h"

using namespace cfmg;

// ------------------------------------------------------------------ handle
struct cfmg_handle {
  cfmg_desc d;
  std::vector<Level> lv;  // lv[0] is level 1
  int device = 0;
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  void* arena = nullptr;
  size_t arena_bytes = 0;
  double* partials = nullptr;  // kPartials FP64 partial sums
  double* dscal = nullptr;     // device scalars, see enum Scal
  double* hscal = nullptr;     // pinned host mirror of dscal
  std::string err;
  bool mixed_dirty = true;     // FP32 coefficient copies need refreshing
  // captured graphs: one cycle + normresidual per cycle kind and precision
  cudaGraphExec_t graph[2][6] = {{nullptr}};
  long long graph_launches[2][6] = {{0}};
  // whole solve loops: a graph `while` node around one iteration
  cudaGraphExec_t sgraph[2][6] = {{nullptr}};
  double* dhist = nullptr;  // device residual history (maxite + 1)
  long long launches = 0;      // kernels launched (graph replays count every kernel node)
  bool capturing = false;
  // device-time profile of one kernel class on one level (cfmg_profile)
  int prof_cls = -1, prof_lev = 0, prof_prec = 0;
  std::vector<cudaEvent_t> ev_pool;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> ev_pending;
  long long prof_launches = 0;
  double prof_ms = 0.0;
  // coarse-level program engine
  bool engine_on = true;
  long long engine_cells = 20000;  // FP32 levels of at most this many cells run in the engine (FP64: 1/16)
  std::vector<cfmg::Op> pending;
  cfmg::Op* prog_pool = nullptr;   // device program store
  int pool_cap = 0, pool_used = 0;
  std::unordered_map<std::string, int> prog_cache;
  bool tb_on = true;  // temporally blocked FP32 smoothing on fine levels
  bool fuse_on = true;  // V-cycle descent: residual and restriction in the last pre-smoothing pass
  // mixed loop: the FP64 solution update in the cycle's last level-1
  // post-smoothing pass (upd_on); upd_req while a cycle runs that allows it,
  // upd_now for that pass, upd_done once it ran
  bool upd_on = true, upd_req = false, upd_now = false, upd_done = false;
  int tb_version = 5;  // 5: lean packed FP32x2 passes, 3: first packed form, 1: scalar passes
  int coarsest_fp64 = -1;  // mixed form: -1 FP64 when the coarsest level is small, 0 never, 1 always
  // adjoint scratch (level-1 FP64 arrays, allocated on the first cfmg_adjoint)
  double *adj_x = nullptr, *adj_b = nullptr, *adj_gk = nullptr;
  // integer form of the mixed loop's fused residual (k_mixed.cu): Q*diag of
  // level 1 as int8 (-128 on dry cells), usable when int_ok
  int8_t* dq = nullptr;
  bool int_ok = false;
  bool int_on = true;
  // 3D 7-point: dq with rows padded to 16 bytes for the TMA-staged pass
  // (k_resid3d.cu, CFMG_OPT_STAGED_RESIDUAL); r3_ran once that pass ran
  int8_t* dqp = nullptr;
  uint8_t* tcol = nullptr;   // wet flags of the staged pass's (tile, plane) pairs
  uint8_t* sflag = nullptr;  // wet flags of the strip pass's (plane, row, strip) triples
  bool r3_on = true, r3_ran = false;
  int r3_rows = 2;  // rows of its tile per thread (1 or 2)
  // mixed V-cycle, 3D 7-point: level 1's FP32 x is not zeroed before the
  // cycle; its first sweep reads it as +0 instead (x1_zero_ok)
  bool x1_zero = false;
  // CFMG_OPT_SKIP_DRY: 3D mixed passes skip groups of dry cells (their FP32
  // fields hold +0 and stay +0)
  bool dry_on = true;
  int small_min = 4;  // CFMG_OPT_SMALL_SMOOTH: fewest pairs of a call run in one block (0: never)
  bool host_loop = false;  // CFMG_OPT_HOST_LOOP
  // call order: the operators' coefficients exist once cfmg_setup_operators,
  // cfmg_bind_level or an upload of a coefficient field ran; cfmg_adjoint
  // needs a forward cfmg_solve before it
  bool coef_set = false, solved = false;
  bool dep_launch = true;  // CFMG_OPT_DEPENDENT_LAUNCH
  // FP32 omega*idiag as one-byte codes (CFMG_OPT_CODED_WIDIAG): wq_on the
  // option, wq_ok when every level's codes reproduce the floats (prepare_wq)
  bool wq_on = true, wq_ok = false;
  float* wtab = nullptr;  // 256 entries
  bool record = false;  // emit() records every Op (whole-solve programs) instead of running it
  bool record_tb = false;  // while recording: temporally blocked smoothing is recorded as OPK_TB Ops
};

constexpr int kProgPoolOps = 8192;  // device store of engine programs (~1.9 MB)

// Batched solves: independent instances (each a full handle on the batch's
// stream) whose whole mixed-precision solves run as programs of the
// batched engine, one launch for all of them.
struct cfmg_batch {
  cfmg_desc d;
  std::vector<cfmg_handle*> inst;
  cudaStream_t stream = nullptr;
  std::vector<int> order;  // queue order: largest instance first
  Op* progs = nullptr;     // all programs, concatenated (device)
  const Op** ptrs = nullptr;
  int* nops = nullptr;
  int* counter = nullptr;  // [0]: queue head, [1 + c]: cluster c's current instance
  double* red = nullptr;   // kEngineCtas reduction slots per cluster
  double* sc = nullptr;    // scalar blocks, nsc per instance
  double* nwet = nullptr;  // wet cells per instance
  int nsc = 0, nclusters = 0;
  bool built = false;
  cudaGraphExec_t graph[2] = {nullptr, nullptr};  // [zero_x]
  std::vector<double> hsc;
  std::string err;
  // lockstep form (closed topology, 5- and 9-point): see k_batch.cu
  bool lockstep = false;
  BInst* bi = nullptr;         // per-instance level-1 state (device)
  long long* l1start = nullptr;  // first level-1 chunk of each instance (device, ninst + 1)
  int4* l1tab = nullptr;       // level-1 chunk table {instance, chunk, instance, 0}
  long long l1chunks = 0;
  double* bpart = nullptr;     // 2 partial sums per level-1 chunk
  int* active = nullptr;       // per instance: still iterating
  int* nactive = nullptr;      // instances continuing after this iteration
  Op* sops = nullptr;          // the Ops of all cycle steps (device)
  int4* stab = nullptr;        // their chunk (or tile) tables {Op, chunk, instance, 0} (device)
  BSmall* ssm = nullptr;       // small-level smoothing descriptors (device)
  int2* rent = nullptr;        // coarse-run entries {0, Op} / {1, BSmall} (device)
  int4* runs = nullptr;        // coarse runs {instance, first entry, end entry, 0} (device)
  bool host_loop = false;      // CFMG_BOPT_HOST_LOOP
  bool coarse_runs = true;     // CFMG_BOPT_COARSE_RUNS
  bool interleave = true;      // CFMG_BOPT_INTERLEAVE
  bool int_all = false;        // every instance has the integer residual form
  int4* ttab = nullptr;        // its warp tasks {instance, strip, row chunk, 0}
  long long* tstart = nullptr; // first task of each instance (ninst + 1)
  long long ntasks = 0;
  int kind = 0;
  bool neumann = false;
  struct Step {
    int tb, stencil, nite;     // tb: OPK_TB Ops of one (stencil, nite), 1 scalar tiles, 4 lean packed
                               // tiles; 2: BSmall blocks; 3: coarse runs
    long long tab0;            // offset into stab (or ssm, or runs)
    long long nchunks;         // table entries (or BSmall blocks, or runs)
    int smem;                  // BSmall, coarse runs: shared memory bytes
  };
  std::vector<Step> steps;
};


namespace {

std::mutex g_err_mu;
std::string g_create_err;

}  // namespace

thread_local bool cfmg::tl_dep_launch = true;

void cfmg::set_global_error(const std::string& msg) {
  std::lock_guard<std::mutex> lk(g_err_mu);
  g_create_err = msg;
}

namespace {

int fail(cfmg_handle* h, int code, const std::string& msg) {
  if (h) h->err = msg;
  else {
    std::lock_guard<std::mutex> lk(g_err_mu);
    g_create_err = msg;
  }
  return code;
}

#define CUDA_OK(h, call)                                                                       \
  do {                                                                                         \
    cudaError_t _e = (call);                                                                   \
    if (_e != cudaSuccess)                                                                     \
      return fail((h), CFMG_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(_e));     \
  } while (0)

#define LAUNCH_OK(h)                                                                           \
  do {                                                                                         \
    cudaError_t _e = cudaGetLastError();                                                       \
    if (_e != cudaSuccess) return fail((h), CFMG_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(_e)); \
  } while (0)

#define TRY(expr)              \
  do {                         \
    int _rc = (expr);          \
    if (_rc != CFMG_OK) return _rc; \
  } while (0)

bool threed(const cfmg_handle* h) { return h->d.kase == CFMG_THREED; }
bool vertices(const cfmg_handle* h) { return h->d.location == CFMG_VERTICES; }
bool xperio(const cfmg_handle* h) { return h->d.topology == CFMG_XPERIO; }
int L(const cfmg_handle* h) { return (int)h->lv.size(); }

Box interior(const Level& l) { return Box{l.ic0, l.ic1, l.jc0, l.jc1, l.kc0, l.kc1}; }

int harvest(cfmg_handle* h) {
  for (auto& pr : h->ev_pending) {
    float ms = 0.f;
    CUDA_OK(h, cudaEventElapsedTime(&ms, pr.first, pr.second));
    h->prof_ms += ms;
    h->prof_launches += 1;
    h->ev_pool.push_back(pr.first);
    h->ev_pool.push_back(pr.second);
  }
  h->ev_pending.clear();
  return CFMG_OK;
}

int flush(cfmg_handle* h);

int sync(cfmg_handle* h) {
  TRY(flush(h));
  CUDA_OK(h, cudaStreamSynchronize(h->stream));
  return harvest(h);
}

// Kernel accounting and the optional per-class event profile. Every launch
// of the runtime goes through Launch: it counts the kernel and, when the
// profiled (class, level, precision) matches, brackets it with events.
struct Launch {
  cfmg_handle* h;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  Launch(cfmg_handle* hh, int cls, int lev, int prec, int nkernels = 1) : h(hh) {
    h->launches += nkernels;
    tl_dep_launch = h->dep_launch;
    if (h->prof_cls == cls && h->prof_lev == lev && h->prof_prec == prec && !h->capturing) {
      for (cudaEvent_t* e : {&e0, &e1}) {
        if (h->ev_pool.empty()) {
          cudaEvent_t ev;
          cudaEventCreate(&ev);
          h->ev_pool.push_back(ev);
        }
        *e = h->ev_pool.back();
        h->ev_pool.pop_back();
      }
      cudaEventRecord(e0, h->stream);
    }
  }
  ~Launch() {
    if (e0) {
      cudaEventRecord(e1, h->stream);
      h->ev_pending.emplace_back(e0, e1);
    }
  }
};

template <class T>
constexpr int prec_of() {
  return sizeof(T) == 8 ? CFMG_FP64 : CFMG_MIXED;
}

// Typed view of one level's arrays (FP64 drop-in or FP32 cycles).
template <class T>
struct View {
  T *x, *y, *r, *b;
  const T *diag, *widiag, *Rcoef, *Pcoef, *cE, *cN;
  const uint8_t* msk;
};
template <class T>
View<T> view(const Level& l);
template <>
View<double> view<double>(const Level& l) {
  return View<double>{l.x, l.y, l.r, l.b, l.diag, l.widiag, l.Rcoef, l.Pcoef, l.cE, l.cN, l.msk};
}
template <>
View<float> view<float>(const Level& l) {
  float* xs = l.xswap ? l.y32 : l.x32;  // the FP32 x and its partner buffer
  float* ys = l.xswap ? l.x32 : l.y32;
  return View<float>{xs, ys, l.r32, l.b32, l.diag32, l.widiag32, l.Rcoef32, l.Pcoef32, l.cE32, l.cN32, l.msk};
}

template <class T>
T* field_ptr(const Level& l, int f) {
  View<T> v = view<T>(l);
  switch (f) {
    case CFMG_X: return v.x;
    case CFMG_R: return v.r;
    case CFMG_B: return v.b;
    case CFMG_Y: return v.y;
    default: return nullptr;
  }
}

// ----------------------------------------------------------- op emission
// Every operator is an Op. emit() runs fine-level Ops as standalone kernels
// and gathers consecutive coarse-level Ops (level length <= engine_cells)
// into a pending program; flush() runs the pending program as one
// cluster-launched engine kernel. Programs are cached on the device by
// content, so a captured graph and later replays reuse the same copy.
Op mkop(int kind, int prec, int lev, int cls, const Level& l) {
  Op op;
  std::memset(&op, 0, sizeof(op));
  op.kind = kind;
  op.prec = prec;
  op.lev = lev;
  op.cls = cls;
  op.g = geom(l);
  return op;
}

long long box_count(const Box& b) {
  if (b.i1 < b.i0 || b.j1 < b.j0 || b.k1 < b.k0) return 0;
  return (long long)(b.i1 - b.i0 + 1) * (b.j1 - b.j0 + 1) * (b.k1 - b.k0 + 1);
}

int flush(cfmg_handle* h) {
  if (h->record || h->pending.empty()) return CFMG_OK;
  const int n = (int)h->pending.size();
  std::string key((const char*)h->pending.data(), (size_t)n * sizeof(Op));
  auto it = h->prog_cache.find(key);
  int off = -1;
  if (it != h->prog_cache.end()) {
    off = it->second;
  } else if (h->pool_used + n <= h->pool_cap) {
    // synchronous upload; allowed while the stream is being captured in
    // relaxed mode, and never overwrites a program a graph refers to
    CUDA_OK(h, cudaMemcpy(h->prog_pool + h->pool_used, h->pending.data(), (size_t)n * sizeof(Op),
                          cudaMemcpyHostToDevice));
    off = h->pool_used;
    h->pool_used += n;
    h->prog_cache.emplace(std::move(key), off);
  }
  if (off >= 0) {
    Launch k(h, CFMG_K_ENGINE, 0, h->pending[0].prec ? CFMG_MIXED : CFMG_FP64);
    launch_program(h->prog_pool + off, n, h->partials, h->stream);
  } else {  // pool full: run the Ops one by one
    for (const Op& op : h->pending) {
      Launch k(h, op.cls, op.lev, op.prec ? CFMG_MIXED : CFMG_FP64);
      launch_op(op, h->stream);
    }
  }
  h->pending.clear();
  LAUNCH_OK(h);
  return CFMG_OK;
}

// The engine's 8 SMs give about 1/19 of the GPU's FP64 rate, which suits
// only small FP64 levels; FP32 levels up to engine_cells cells go there.
long long engine_limit(const cfmg_handle* h, int prec) { return prec == 0 ? h->engine_cells / 16 : h->engine_cells; }

int emit(cfmg_handle* h, const Op& op) {
  if (op.n <= 0) return CFMG_OK;
  if (h->record) {
    h->pending.push_back(op);
    return CFMG_OK;
  }
  const Level& l = h->lv[op.lev - 1];
  if (h->engine_on && (long long)l.len <= engine_limit(h, op.prec)) {
    h->pending.push_back(op);
    return CFMG_OK;
  }
  TRY(flush(h));
  Launch k(h, op.cls, op.lev, op.prec ? CFMG_MIXED : CFMG_FP64);
  launch_op(op, h->stream);
  return CFMG_OK;
}

template <class T>
int fill_if(cfmg_handle* h, int lev, T* x) {
  if (!xperio(h)) return CFMG_OK;
  const Level& l = h->lv[lev - 1];
  Op op = mkop(OPK_FILL, prec_of<T>() == CFMG_FP64 ? 0 : 1, lev, CFMG_K_FILL, l);
  op.y = x;
  op.n = (long long)l.ty * l.tz;
  return emit(h, op);
}

template <class T>
constexpr int pc() {
  return sizeof(T) == 8 ? 0 : 1;
}

// ------------------------------------------------------- per-level operators
// x_zero (3D 7-point coded sweeps only, see x1_zero_ok): x holds +0 and is not read
template <class T>
int sweep(cfmg_handle* h, int lev, int kind, const T* x, T* y, const Box* bx, bool x_zero = false) {
  const Level& l = h->lv[lev - 1];
  View<T> v = view<T>(l);
  Op op = mkop(kind, pc<T>(), lev, CFMG_K_SWEEP, l);
  op.x = x; op.y = y; op.b = v.b; op.w = v.widiag; op.cE = v.cE; op.cN = v.cN;
  if (sizeof(T) == 4 && h->wq_on && h->wq_ok && !h->record) {  // standalone launches only; the engine reads w
    op.wq = l.wq;
    op.wtab = h->wtab;
    op.assign = x_zero ? 1 : 0;
    op.qact = h->dry_on ? l.qact : nullptr;
  }
  op.cff = 1.0 - h->d.omega;
  if (bx) {
    op.box = *bx;
    op.n = box_count(*bx);
  } else {
    const long long off = (kind == OPK_SWEEP7) ? op.g.n2 : op.g.n1;
    op.lo = off;
    op.n = op.g.len - 2 * off;
  }
  return emit(h, op);
}

// FP32 smoothing of a fine level in temporally blocked passes (closed
// topology, 2D 5- and 9-point): the result goes to the partner buffer.
template <class T>
bool tb_eligible(const cfmg_handle* h, int lev) {
  if (sizeof(T) != 4 || !h->tb_on || (h->record && !h->record_tb)) return false;
  // x-periodic: the lean packed passes of the 2D 5-point operator (standalone launches)
  if (xperio(h) && (h->record || h->tb_version != 5 || threed(h) || h->d.op != CFMG_LAPLACIAN)) return false;
  // 3D: 7-point streaming passes, opt-in (CFMG_OPT_TEMPORAL_BLOCKING = 4): at
  // 512 x 512 x 256 a 4-sweep pass measured 1.0-1.3 ms, no faster than
  // four single-sweep kernels at 66 % of HBM
  if (threed(h) && (h->d.op != CFMG_LAPLACIAN || h->record || h->tb_version != 4)) return false;
  if (h->d.op != CFMG_LAPLACIAN && h->d.op != CFMG_LAPLACIAN9) return false;
  const Level& l = h->lv[lev - 1];
  return !(h->engine_on && (long long)l.len <= engine_limit(h, CFMG_MIXED));
}

// 3D 19-point FP32 level of a closed topology, standalone: its smoothing
// call as one streaming pass (k_tb3d.cu, L19). The halo must hold the pass's
// first-sweep box (nh >= 2, as the reference's icp x jcp x kcp needs too).
bool tb3d19_ok(const cfmg_handle* h, int lev) {
  if (!h->tb_on || h->tb_version != 4 || h->record || xperio(h) || !threed(h) || h->d.op != CFMG_LAPLACIAN9)
    return false;
  const Level& l = h->lv[lev - 1];
  if (l.nh < 2) return false;
  return !(h->engine_on && (long long)l.len <= engine_limit(h, CFMG_MIXED));
}

// 3D 7-point: passes of up to 2 pairs (k_tb3d.cu), x -> partner buffer
int smooth_tb3d(cfmg_handle* h, int lev, int nite) {
  Level& l = h->lv[lev - 1];
  TRY(flush(h));
  for (int left = nite; left > 0;) {
    const int n = left > 2 ? 2 : left;
    View<float> v = view<float>(l);
    {
      Launch k(h, CFMG_K_SWEEP, lev, CFMG_MIXED);
      launch_smooth_tb3d(n, v.x, v.y, v.b, v.widiag, (float)(1.0 - h->d.omega), l.tx, l.ty, l.tz, l.nh,
                         l.nx + l.nh + 1, l.nh, l.ny + l.nh + 1, l.nh, l.nz + l.nh + 1, h->stream);
    }
    l.xswap ^= 1;
    left -= n;
  }
  LAUNCH_OK(h);
  return CFMG_OK;
}

int smooth_tb(cfmg_handle* h, int lev, int nite) {
  if (threed(h)) return smooth_tb3d(h, lev, nite);
  Level& l = h->lv[lev - 1];
  const int stencil = h->d.op == CFMG_LAPLACIAN9 ? 9 : 5;
  TRY(flush(h));
  if (xperio(h)) {  // periodic tiles over the interior columns, then fill! of the result
    const int per = nite > 3 ? kTbMaxPairs : 3;
    for (int left = nite; left > 0;) {
      const int n = left > per ? per : left;
      View<float> v = view<float>(l);
      {
        Launch k(h, CFMG_K_SWEEP, lev, CFMG_MIXED);
        launch_smooth_tb_periodic(n, v.x, v.y, v.b, v.widiag, (float)(1.0 - h->d.omega), l.tx, l.ty, l.tz,
                                  l.nh + 1, l.nx + l.nh, l.nh, l.ny + l.nh + 1, h->stream);
      }
      l.xswap ^= 1;
      left -= n;
      TRY(fill_if<float>(h, lev, view<float>(l).x));
    }
    LAUNCH_OK(h);
    return CFMG_OK;
  }
  // up to 3 pairs per pass (kTbMaxPairs for a long smoothing such as the
  // coarsest solve's; the batched solver's blocked kernel takes up to 3)
  const int per = (nite > 3 && !h->record) ? kTbMaxPairs : 3;
  for (int left = nite; left > 0;) {
    const int n = left > per ? per : left;
    View<float> v = view<float>(l);
    if (h->record) {  // the batched solver runs this pass (OPK_TB)
      Op op = mkop(OPK_TB, 1, lev, CFMG_K_SWEEP, l);
      op.x = v.x; op.y = v.y; op.b = v.b; op.w = v.widiag;
      op.cff = 1.0 - h->d.omega;
      op.box = Box{l.nh, l.nx + l.nh + 1, l.nh, l.ny + l.nh + 1, 1, l.tz};
      op.np_i = n;
      op.np_j = stencil;
      op.form = h->tb_version >= 5 ? 5 : 1;  // the tile form of the standalone passes
      if (op.form == 5) tb5_tiles(n, op.box.i0, op.box.i1, op.box.j0, op.box.j1, &op.kf0, &op.kf1);
      else tb_tiles(n, op.box.i0, op.box.i1, op.box.j0, op.box.j1, &op.kf0, &op.kf1);
      op.n = (long long)op.kf0 * op.kf1 * l.tz;
      h->pending.push_back(op);
      l.xswap ^= 1;
      left -= n;
      continue;
    }
    bool upd = false;
    {
      Launch k(h, CFMG_K_SWEEP, lev, CFMG_MIXED);
      // the cycle's last pass on level 1 may take the FP64 solution update
      if (h->upd_now && left == n && h->tb_version >= 5)
        upd = launch_smooth_tb_upd(stencil, n, v.x, v.b, v.widiag, (float)(1.0 - h->d.omega), l.tx, l.ty, l.tz, l.nh,
                                   l.nx + l.nh + 1, l.nh, l.ny + l.nh + 1, l.x, h->dscal, h->stream);
      if (!upd)
        launch_smooth_tb(h->tb_version, stencil, n, v.x, v.y, v.b, v.widiag, (float)(1.0 - h->d.omega), l.tx, l.ty,
                         l.tz, l.nh,
                         l.nx + l.nh + 1, l.nh, l.ny + l.nh + 1, h->stream);
    }
    if (upd) h->upd_done = true;  // the FP32 result was not stored: the buffers stay as they were
    else l.xswap ^= 1;
    left -= n;
  }
  LAUNCH_OK(h);
  return CFMG_OK;
}

// mg.smoother[lev] (src/gmg_setup.jl:124-139 selects among these)
// A long smoothing call (the coarsest solve) on a level whose four arrays fit
// one block's shared memory runs as one block (k_small_smooth) instead of
// 2*nite engine Ops: the pending Ops before it are flushed as their own
// program. Closed topology, the 5- and 2D 9-point and the 3D 7-point
// operators.
template <class T>
bool small_smooth_ok(const cfmg_handle* h, int lev, int nite) {
  if (h->record || xperio(h) || h->small_min <= 0 || nite < h->small_min) return false;
  if (!(h->d.op == CFMG_LAPLACIAN || (h->d.op == CFMG_LAPLACIAN9 && !threed(h)))) return false;
  if (sizeof(T) == 4 && lev == 1 && h->x1_zero) return false;  // that sweep must not read x
  const Level& l = h->lv[lev - 1];
  if (l.xswap) return false;
  const size_t lo = threed(h) ? (size_t)l.tx * l.ty : (size_t)l.tx;  // the linear ranges start here
  return 4 * l.len * sizeof(T) <= kSmallSmemMax && l.len > 2 * lo;
}

template <class T>
int small_smooth_run(cfmg_handle* h, int lev, int nite) {
  const Level& l = h->lv[lev - 1];
  const View<T> v = view<T>(l);
  TRY(flush(h));
  SmallSm s;
  std::memset(&s, 0, sizeof(s));
  s.x = const_cast<T*>(v.x);
  s.y = const_cast<T*>(v.y);
  s.b = v.b;
  s.w = v.widiag;
  s.g = geom(l);
  s.stencil = threed(h) ? 7 : (h->d.op == CFMG_LAPLACIAN9 ? 9 : 5);
  s.npairs = nite;
  s.ext = Box{l.nh, l.nx + l.nh + 1, l.nh, l.ny + l.nh + 1, 1, l.nz};
  s.in = interior(l);
  s.cff = 1.0 - h->d.omega;
  {
    Launch k(h, CFMG_K_SWEEP, lev, pc<T>() ? CFMG_MIXED : CFMG_FP64);
    launch_small_smooth<T>(s, h->stream);
  }
  LAUNCH_OK(h);
  return CFMG_OK;
}

template <class T>
int smooth_t(cfmg_handle* h, int lev, int nite) {
  if (tb_eligible<T>(h, lev)) return smooth_tb(h, lev, nite);
  if (small_smooth_ok<T>(h, lev, nite)) return small_smooth_run<T>(h, lev, nite);
  const Level& l = h->lv[lev - 1];
  View<T> v = view<T>(l);
  if (h->d.op == CFMG_LAPLACIAN9 && threed(h)) {
    // smooth_laplacian9! (src/laplacian9.jl:2-47): one pair whatever nite
    // is; sweep 1 over icp x jcp x kcp, sweep 2 over the interior; no fill!
    Box ext{l.nh, l.nx + l.nh + 1, l.nh, l.ny + l.nh + 1, l.nh, l.nz + l.nh + 1};
    Box in = interior(l);
    if (sizeof(T) == 4 && tb3d19_ok(h, lev)) {  // the pair in one streaming pass, into the other x buffer
      TRY(flush(h));
      {
        Launch k(h, CFMG_K_SWEEP, lev, CFMG_MIXED);
        const View<float> vf = view<float>(l);
        launch_smooth_tb3d19(vf.x, vf.y, vf.b, vf.widiag, (float)(1.0 - h->d.omega), l.tx, l.ty, l.tz, in, ext,
                             h->stream);
      }
      h->lv[lev - 1].xswap ^= 1;
      LAUNCH_OK(h);
      return CFMG_OK;
    }
    TRY(sweep<T>(h, lev, OPK_SWEEP19, v.x, v.y, &ext));
    return sweep<T>(h, lev, OPK_SWEEP19, v.y, v.x, &in);
  }
  for (int kt = 0; kt < nite; ++kt) {
    if (h->d.op == CFMG_LAPLACIAN9) {  // 2D 9-point extension
      Box ext{l.nh, l.nx + l.nh + 1, l.nh, l.ny + l.nh + 1, 1, l.nz};
      Box in = interior(l);
      TRY(sweep<T>(h, lev, OPK_SWEEP9, v.x, v.y, &ext));
      TRY(sweep<T>(h, lev, OPK_SWEEP9, v.y, v.x, &in));
    } else {
      // smooth_laplacian2d! (src/laplacian.jl:95-112), smooth_laplacian!
      // (src/laplacian.jl:24-41), variable coefficient
      const int k = h->d.op == CFMG_VARCOEF ? OPK_SWEEPVC : (threed(h) ? OPK_SWEEP7 : OPK_SWEEP5);
      // the mixed V-cycle's first level-1 sweep reads an x of +0 (x1_zero)
      const bool xz = sizeof(T) == 4 && lev == 1 && kt == 0 && h->x1_zero;
      h->x1_zero = h->x1_zero && !(sizeof(T) == 4 && lev == 1);
      TRY(sweep<T>(h, lev, k, v.x, v.y, nullptr, xz));
      TRY(sweep<T>(h, lev, k, v.y, v.x, nullptr));
    }
    TRY(fill_if<T>(h, lev, v.x));
  }
  return CFMG_OK;
}

// mg.residual[lev]
template <class T>
int residual_t(cfmg_handle* h, int lev) {
  const Level& l = h->lv[lev - 1];
  View<T> v = view<T>(l);
  Op op = mkop(OPK_RESID5, pc<T>(), lev, CFMG_K_RESIDUAL, l);
  op.x = v.x; op.y = v.r; op.b = v.b; op.d = v.diag; op.m = v.msk; op.cE = v.cE; op.cN = v.cN;
  Box in = interior(l);
  if (h->d.op == CFMG_LAPLACIAN9) {
    op.kind = threed(h) ? OPK_RESID19 : OPK_RESID9;  // interior box
    op.box = in;
    op.n = box_count(in);
  } else if (threed(h)) {
    op.kind = OPK_RESID7;  // rloop3d!: interior box
    op.box = in;
    op.n = box_count(in);
  } else {
    op.kind = h->d.op == CFMG_VARCOEF ? OPK_RESIDVC : OPK_RESID5;  // linear range 1+n1 .. len-n1
    op.lo = op.g.n1;
    op.n = op.g.len - 2 * op.g.n1;
  }
  TRY(emit(h, op));
  if (h->d.op == CFMG_LAPLACIAN9 && threed(h)) return CFMG_OK;  // residual_laplacian9!: no fill!
  return fill_if<T>(h, lev, v.r);
}

int rp_kind(const cfmg_handle* h) { return (vertices(h) ? 2 : 0) + (threed(h) ? 1 : 0); }

// mg.restriction[lev]: field of lev -> b of lev+1, then fill!
template <class T>
int restrict_t(cfmg_handle* h, int lev, int field) {
  const Level& f = h->lv[lev - 1];
  const Level& c = h->lv[lev];
  View<T> vc = view<T>(c);
  Op op = mkop(OPK_RESTRICT0 + rp_kind(h), pc<T>(), lev, CFMG_K_RESTRICT, f);
  op.gc = geom(c);
  op.x = field_ptr<T>(f, field);
  op.y = vc.b;
  op.coef = vc.Rcoef;
  op.box = interior(c);
  op.n = box_count(op.box);
  TRY(emit(h, op));
  return fill_if<T>(h, lev + 1, vc.b);
}

// mg.prolongation[lev]: x of lev += Pcoef * P(x of lev+1), then fill!
template <class T>
int zero_t(cfmg_handle* h, int lev, int field);

// onto_zero: the fine x is known to hold +0 (zeroed and not written since),
// so a standalone launch writes x = +0 + P x_coarse without reading it; the
// caller then skips zeroing it. A level of the program engine is zeroed here
// and prolonged as usual.
template <class T>
int prolong_t(cfmg_handle* h, int lev, bool onto_zero = false) {
  const Level& f = h->lv[lev - 1];
  const Level& c = h->lv[lev];
  View<T> vf = view<T>(f);
  View<T> vc = view<T>(c);
  const int kind = rp_kind(h);
  Op op = mkop(OPK_PROLONG0 + kind, pc<T>(), lev, CFMG_K_PROLONG, f);
  op.gc = geom(c);
  op.x = vc.x;
  op.y = vf.x;
  op.coef = vf.Pcoef;
  // parents i = nh+1 : 2 : nx+nh (likewise j, and k in 3D)
  op.np_i = (f.nx + 1) / 2;
  op.np_j = (f.ny + 1) / 2;
  int np_k;
  if (kind == 1 || kind == 3) {
    np_k = (f.nz + 1) / 2;
    op.kf0 = 0;
    op.kf1 = np_k - 1;
  } else {
    op.kf0 = f.kc0;
    op.kf1 = f.kc1;
    np_k = f.kc1 - f.kc0 + 1;
  }
  op.n = (long long)op.np_i * op.np_j * np_k;
  // FP32 cycles of a closed topology: parents whose children are all dry are skipped
  if (sizeof(T) == 4 && h->dry_on && !xperio(h)) op.m = f.msk;
  if (onto_zero) {
    if (!h->record && !(h->engine_on && (long long)f.len <= engine_limit(h, pc<T>()))) op.assign = 1;
    else TRY(zero_t<T>(h, lev, CFMG_X));
  }
  TRY(emit(h, op));
  return fill_if<T>(h, lev, vf.x);
}

template <class T>
int zero_t(cfmg_handle* h, int lev, int field) {
  const Level& l = h->lv[lev - 1];
  Op op = mkop(OPK_ZERO, pc<T>(), lev, CFMG_K_FILL, l);
  op.y = field_ptr<T>(l, field);
  op.n = (long long)l.len;
  return emit(h, op);
}

// Mixed form: the coarsest level is solved in FP64 (FP32 b -> FP64 b,
// ndeepest FP64 pairs, FP64 x -> FP32 x).
template <class T>
int coarsest_t(cfmg_handle* h, int nite);
template <>
int coarsest_t<double>(cfmg_handle* h, int nite) {
  return smooth_t<double>(h, L(h), nite);
}
bool coarsest_in_fp64(const cfmg_handle* h) {
  return L(h) > 1 && (h->coarsest_fp64 > 0 ||
                      (h->coarsest_fp64 < 0 && (long long)h->lv[L(h) - 1].len <= engine_limit(h, CFMG_FP64)));
}
template <>
int coarsest_t<float>(cfmg_handle* h, int nite) {
  if (L(h) == 1) return smooth_t<float>(h, 1, nite);
  const bool fp64 = coarsest_in_fp64(h);
  if (!fp64) return smooth_t<float>(h, L(h), nite);
  const int lev = L(h);
  const Level& c = h->lv[lev - 1];
  View<float> v = view<float>(c);
  Op op = mkop(OPK_F32TO64, 1, lev, CFMG_K_CONVERT, c);
  op.n = (long long)c.len;
  op.x = v.b; op.y = c.b;
  TRY(emit(h, op));
  op.x = v.x; op.y = c.x;
  TRY(emit(h, op));
  TRY(smooth_t<double>(h, lev, nite));
  op.kind = OPK_F64TO32;
  op.x = c.x; op.y = v.x;
  return emit(h, op);
}

// ------------------------------------------------------------------ cycles
// One descent step of a cycle at lev: pre-smoothing, residual, restriction
// of r to the coarse b, coarse x zeroed (src/gmg_cycles.jl:72-76). On FP32
// levels smoothed in lean packed passes (2D, closed topology), the last
// pass does the residual and the restriction in its epilogue.
bool fused_descent_ok(const cfmg_handle* h, int lev) {
  if (!h->fuse_on || h->record || h->tb_version != 5 || threed(h) || xperio(h) || lev >= L(h)) return false;
  if (h->d.op != CFMG_LAPLACIAN && h->d.op != CFMG_LAPLACIAN9) return false;
  return tb_eligible<float>(h, lev) && h->lv[lev - 1].tz == 1;
}

int smooth_tb_epi(cfmg_handle* h, int lev, int nite) {
  Level& l = h->lv[lev - 1];
  const Level& c = h->lv[lev];
  const int stencil = h->d.op == CFMG_LAPLACIAN9 ? 9 : 5;
  TRY(flush(h));
  for (int left = nite; left > 0;) {
    const int n = left > 3 ? 3 : left;
    View<float> v = view<float>(l);
    {
      Launch k(h, left > 3 ? CFMG_K_SWEEP : CFMG_K_DESCENT, lev, CFMG_MIXED);
      if (left > 3) {
        launch_smooth_tb(h->tb_version, stencil, n, v.x, v.y, v.b, v.widiag, (float)(1.0 - h->d.omega), l.tx, l.ty,
                         l.tz, l.nh, l.nx + l.nh + 1, l.nh, l.ny + l.nh + 1, h->stream);
      } else {
        const View<float> vc = view<float>(c);
        const Box in = interior(l), cin = interior(c);
        TbEpi ep;
        ep.d = v.diag; ep.m = l.msk; ep.rcoef = vc.Rcoef; ep.bc = vc.b; ep.xc = vc.x;
        ep.ri0 = in.i0; ep.ri1 = in.i1; ep.rj0 = in.j0; ep.rj1 = in.j1;
        ep.nh = c.nh; ep.ctx = c.tx;
        ep.ci0 = cin.i0; ep.ci1 = cin.i1; ep.cj0 = cin.j0; ep.cj1 = cin.j1;
        ep.pkind = vertices(h) ? 2 : 0;
        launch_smooth_tb_epi(stencil, n, v.x, v.y, v.b, v.widiag, (float)(1.0 - h->d.omega), l.tx, l.ty, l.nh,
                             l.nx + l.nh + 1, l.nh, l.ny + l.nh + 1, ep, h->stream);
      }
    }
    l.xswap ^= 1;
    left -= n;
  }
  LAUNCH_OK(h);
  return CFMG_OK;
}

// 3D 7-point cell-centred FP32 level (standalone, coded diag): the residual
// is formed at the children of the coarse interior cells and restricted in
// one pass (k_resid_restrict7c), which needs every such child inside the
// fine interior box
bool resid_restrict3d_ok(const cfmg_handle* h, int lev) {
  if (!h->fuse_on || h->record || !threed(h) || xperio(h) || lev >= L(h) || h->d.op != CFMG_LAPLACIAN ||
      vertices(h) || !h->wq_on || !h->wq_ok)
    return false;
  const Level& f = h->lv[lev - 1];
  if (h->engine_on && (long long)f.len <= engine_limit(h, CFMG_MIXED)) return false;
  const Box fi = interior(f), ci = interior(h->lv[lev]);
  auto c2f = [](int i, int nh) { return (i - nh - 1) * 2 + nh + 1; };
  return c2f(ci.i0, f.nh) >= fi.i0 && c2f(ci.i1, f.nh) + 1 <= fi.i1 && c2f(ci.j0, f.nh) >= fi.j0 &&
         c2f(ci.j1, f.nh) + 1 <= fi.j1 && c2f(ci.k0, f.nh) >= fi.k0 && c2f(ci.k1, f.nh) + 1 <= fi.k1;
}

int resid_restrict3d(cfmg_handle* h, int lev) {
  const Level& f = h->lv[lev - 1];
  const Level& c = h->lv[lev];
  const View<float> vf = view<float>(f), vc = view<float>(c);
  TRY(flush(h));
  {
    Launch k(h, CFMG_K_RESIDUAL, lev, CFMG_MIXED);
    launch_resid_restrict7c(vf.x, vf.b, f.wq, f.msk, vc.Rcoef, vc.b, geom(f), geom(c), interior(c), h->stream,
                            h->dry_on);
  }
  LAUNCH_OK(h);
  return CFMG_OK;
}

template <class T>
int descend_t(cfmg_handle* h, int lev, int nite) {
  if (sizeof(T) == 4 && fused_descent_ok(h, lev)) return smooth_tb_epi(h, lev, nite);
  if (sizeof(T) == 4 && resid_restrict3d_ok(h, lev)) {
    TRY(smooth_t<T>(h, lev, nite));
    TRY(resid_restrict3d(h, lev));
    return zero_t<T>(h, lev + 1, CFMG_X);
  }
  TRY(smooth_t<T>(h, lev, nite));
  TRY(residual_t<T>(h, lev));
  TRY(restrict_t<T>(h, lev, CFMG_R));
  return zero_t<T>(h, lev + 1, CFMG_X);
}

// vcycle! (src/gmg_cycles.jl:67-83)
template <class T>
int vcycle_t(cfmg_handle* h, int lev0) {
  const cfmg_desc& d = h->d;
  const int nl = L(h);
  for (int lev = lev0; lev <= nl - 1; ++lev) TRY(descend_t<T>(h, lev, d.npre));
  TRY(coarsest_t<T>(h, d.ndeepest));
  for (int lev = nl - 1; lev >= lev0; --lev) {
    TRY(prolong_t<T>(h, lev));
    // level 1's post-smoothing is the cycle's last step: with upd_req its
    // last pass may also apply the FP64 solution update
    h->upd_now = sizeof(T) == 4 && lev == 1 && h->upd_req;
    const int st = smooth_t<T>(h, lev, d.npost);
    h->upd_now = false;
    if (st != CFMG_OK) return st;
  }
  return CFMG_OK;
}

// fcycle! (src/gmg_cycles.jl:85-100). The descent zeroes x on levels
// 2..nl. In the FP32 correction cycle of a closed topology (every cell
// outside the wet interior +0 in both x buffers), nothing reads x on levels
// 2..nl-1 before the ascent's prolongation onto them, so those levels are
// not zeroed and that prolongation writes +0 + P x_coarse without reading
// (the same values). x1_zero: level 1's x holds +0 likewise (the caller's
// mixed iteration leaves it unzeroed).
template <class T>
int fcycle_t(cfmg_handle* h, bool x1_zero = false) {
  const int nl = L(h);
  const bool lazy = sizeof(T) == 4 && !xperio(h);
  for (int lev = 1; lev <= nl - 1; ++lev) {
    TRY(restrict_t<T>(h, lev, lev > 1 ? CFMG_B : CFMG_R));
    if (!lazy || lev + 1 == nl) TRY(zero_t<T>(h, lev + 1, CFMG_X));  // the coarsest solve reads it
  }
  TRY(coarsest_t<T>(h, h->d.ndeepest));
  for (int lev = nl - 1; lev >= 1; --lev) {
    TRY(prolong_t<T>(h, lev, lev >= 2 ? lazy : x1_zero));
    TRY(vcycle_t<T>(h, lev));
  }
  return CFMG_OK;
}

// x1_zero (F-cycle only): level 1's x is known to be +0, see fcycle_t
template <class T>
int cycle_body(cfmg_handle* h, int kind, bool x1_zero = false) {
  const cfmg_desc& d = h->d;
  switch (kind) {
    case CFMG_CYCLE_V:
    case CFMG_CYCLE_VREC:  // vcycle_recursive! is vcycle! when not verbose (src/gmg_cycles.jl:43-66)
      return vcycle_t<T>(h, 1);
    case CFMG_CYCLE_F:
      return fcycle_t<T>(h, x1_zero);
    case CFMG_CYCLE_ONELEV:  // onelevel! (src/gmg_cycles.jl:3-6)
      return smooth_t<T>(h, 1, d.ndeepest);
    case CFMG_CYCLE_TWOLEV:  // twolevels! (src/gmg_cycles.jl:8-23)
      if (L(h) < 2) return fail(h, CFMG_ERR_ARG, "twolev cycle needs at least 2 levels");
      TRY(descend_t<T>(h, 1, d.npre));
      TRY(smooth_t<T>(h, 2, d.ndeepest));
      TRY(prolong_t<T>(h, 1));
      return smooth_t<T>(h, 1, d.npost);
    case CFMG_CYCLE_NLEV:  // nlevels! (src/gmg_cycles.jl:25-41), quirks kept
      if (L(h) < 3) return fail(h, CFMG_ERR_ARG, "nlev cycle needs at least 3 levels");
      for (int lev = 1; lev <= 2; ++lev) TRY(descend_t<T>(h, lev, d.npre));
      return smooth_t<T>(h, L(h), d.ndeepest);
    default:
      return fail(h, CFMG_ERR_ARG, "unknown cycle kind");
  }
}

template <class T>
int cycle_t(cfmg_handle* h, int kind, bool x1_zero = false) {
  TRY(cycle_body<T>(h, kind, x1_zero));
  return flush(h);
}

// norm of one FP64 field into dscal[S_NORM] (and dscal[S_RES] when normb given)
int norm_dev(cfmg_handle* h, int lev, const double* x, const double* normb, int kind) {
  TRY(flush(h));
  const Level& l = h->lv[lev - 1];
  Launch k(h, CFMG_K_NORM, lev, CFMG_FP64, 2);
  launch_norm<double>(x, l.msk, l.len, h->partials, h->dscal + S_NORM, normb, kind, h->stream);
  LAUNCH_OK(h);
  return CFMG_OK;
}

// residual at level 1 followed by its norm ratio into dscal[S_RES]
int normresidual_dev(cfmg_handle* h, int kind) {
  TRY(residual_t<double>(h, 1));
  return norm_dev(h, 1, h->lv[0].r, h->dscal + S_NORMB, kind);
}

// The reference builds its coefficients inside get_gmg (src/gmg_setup.jl:
// 26-35), so none of its operators can run before them; here the handle
// and its coefficients are separate steps, and running an operator or a
// solve before the second is a call out of order.
int need_setup(cfmg_handle* h) {
  if (!h) return CFMG_ERR_ARG;
  if (!h->coef_set)
    return fail(h, CFMG_ERR_STATE,
                "operators not set up: call cfmg_setup_operators, cfmg_bind_level or upload the coefficients first");
  return CFMG_OK;
}

int check_lev(cfmg_handle* h, int lev, int lo_off = 0) {
  if (!h) return CFMG_ERR_ARG;
  if (lev < 1 || lev > L(h) - lo_off)
    return fail(h, CFMG_ERR_ARG, "level " + std::to_string(lev) + " out of range 1.." + std::to_string(L(h) - lo_off));
  return CFMG_OK;
}



// ------------------------------------------------------------------ setup
int setup_operators_body(cfmg_handle* h);
int setup_operators(cfmg_handle* h) {
  TRY(flush(h));
  const bool on = h->engine_on;
  h->engine_on = false;  // the setup interleaves element-wise kernels with the operators
  int rc = setup_operators_body(h);
  h->engine_on = on;
  return rc;
}
int setup_operators_body(cfmg_handle* h) {
  const int nl = L(h);
  const bool vert = vertices(h), t3 = threed(h), xp = xperio(h);
  cudaStream_t s = h->stream;
  // compute_msk_dev (src/gmg_setup.jl:322-366)
  for (int lev = 1; lev <= nl - 1; ++lev) {
    Level& f = h->lv[lev - 1];
    Level& c = h->lv[lev];
    const double threshold = vert ? 0.67 : 0.18;
    launch_fill_f64(c.Rcoef, 1.0, c.len, s);
    if (lev == 1) launch_u8_to_f64(f.msk, f.b, f.len, s);
    TRY(restrict_t<double>(h, lev, CFMG_B));
    const double coef = t3 ? (vert ? 1.0 / 64 : 1.0 / 8) : (vert ? 1.0 / 16 : 1.0 / 4);
    launch_default_msk(DEFMSK_SCALE_F64, nullptr, c.b, coef, c, vert, t3, xp, s);
    launch_threshold(c.b, c.msk, threshold, c.len, s);
    launch_default_msk(DEFMSK_MUL, f.msk, nullptr, 0.0, f, vert, t3, xp, s);
  }
  if (h->d.op == CFMG_VARCOEF) {
    for (int lev = 1; lev <= nl - 1; ++lev) {
      Level& f = h->lv[lev - 1];
      Level& c = h->lv[lev];
      launch_fill_f64(c.kappa, 1.0, c.len, s);
      launch_restrict_kappa(f.kappa, f.msk, c.kappa, geom(f), geom(c), interior(c), s);
      fill_if<double>(h, lev + 1, c.kappa);
    }
    for (int lev = 1; lev <= nl; ++lev) {
      Level& l = h->lv[lev - 1];
      launch_face_coef(l.kappa, l.msk, l.cE, l.cN, geom(l), s);
    }
  }
  for (int lev = 1; lev <= nl - 1; ++lev) {
    Level& f = h->lv[lev - 1];
    Level& c = h->lv[lev];
    // compute_Rcoef! (src/gmg_setup.jl:186-212)
    launch_u8_to_f64(c.msk, c.Rcoef, c.len, s);
    if (vert) launch_u8_to_f64(f.msk, f.b, f.len, s);
    else launch_fill_f64(f.b, 1.0, f.len, s);
    TRY(restrict_t<double>(h, lev, CFMG_B));
    launch_rcoef(c.msk, c.b, c.Rcoef, vert, t3 ? 1.0 / 16 : 1.0 / 4, c.len, s);
    // compute_Pcoef! (src/gmg_setup.jl:214-237)
    launch_u8_to_f64(f.msk, f.Pcoef, f.len, s);
    launch_fill_f64(f.x, 0.0, f.len, s);
    if (vert) launch_fill_f64(c.x, 1.0, c.len, s);
    else launch_u8_to_f64(c.msk, c.x, c.len, s);
    TRY(prolong_t<double>(h, lev));
    launch_pcoef(f.msk, f.x, f.Pcoef, f.len, s);
  }
  // compute_diag! (src/gmg_setup.jl:239-262)
  for (int lev = 1; lev <= nl; ++lev) {
    Level& l = h->lv[lev - 1];
    if (vert) launch_fill_f64(l.x, 1.0, l.len, s);
    else launch_u8_to_f64(l.msk, l.x, l.len, s);
    launch_fill_f64(l.b, 0.0, l.len, s);
    launch_fill_f64(l.diag, 0.0, l.len, s);
    TRY(residual_t<double>(h, lev));
    launch_diag(l.msk, l.r, l.diag, l.idiag, l.len, s);
    launch_widiag(l.idiag, l.widiag, h->d.omega, l.len, s);
  }
  LAUNCH_OK(h);
  h->mixed_dirty = true;
  return CFMG_OK;
}

// FP32 copies of the operator coefficients for the mixed-precision cycles.
bool fused_ok(const cfmg_handle* h);
int resid_kind(const cfmg_handle* h) {
  if (h->d.op == CFMG_LAPLACIAN9) return threed(h) ? OPK_RESID19 : OPK_RESID9;
  return threed(h) ? OPK_RESID7 : OPK_RESID5;
}

// Level-1 Q*diag for the integer form of the fused residual; int_ok when
// every wet cell's value is an integer in 0..127 and the mask is 0/1.
int prepare_int(cfmg_handle* h) {
  h->int_ok = false;
  const int kind = resid_kind(h);
  if (!fused_ok(h) || kind == OPK_RESID19) return CFMG_OK;
  const Level& l1 = h->lv[0];
  if (!h->dq) CUDA_OK(h, cudaMalloc((void**)&h->dq, l1.len));
  int* ok = (int*)h->partials;  // scratch
  const int one = 1;
  CUDA_OK(h, cudaMemcpyAsync(ok, &one, sizeof(int), cudaMemcpyHostToDevice, h->stream));
  launch_make_dq(l1.diag, l1.msk, kind == OPK_RESID9 ? 4.0 : 1.0, h->dq, (long long)l1.len, ok, h->stream);
  {
    const long long ns = resid_sflag_size(kind, geom(l1), interior(l1));
    if (ns > 0) {
      if (!h->sflag) CUDA_OK(h, cudaMalloc((void**)&h->sflag, (size_t)ns));
      launch_make_sflag(kind, l1.msk, h->sflag, geom(l1), interior(l1), h->stream);
    }
  }
  if (kind == OPK_RESID7) {
    const int txp = dq_pitch(l1.tx);
    if (!h->dqp) CUDA_OK(h, cudaMalloc((void**)&h->dqp, (size_t)txp * l1.ty * l1.tz));
    launch_pad_dq(h->dq, h->dqp, l1.tx, txp, (long long)l1.ty * l1.tz, h->stream);
    const long long nt = resid3d_tcol_size(geom(l1), interior(l1));
    if (nt > 0) {
      if (!h->tcol) CUDA_OK(h, cudaMalloc((void**)&h->tcol, (size_t)nt));
      launch_make_tcol(l1.msk, h->tcol, geom(l1), interior(l1), h->stream);
    }
  }
  int hok = 0;
  CUDA_OK(h, cudaMemcpyAsync(&hok, ok, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  CUDA_OK(h, cudaStreamSynchronize(h->stream));
  h->int_ok = hok != 0;
  return CFMG_OK;
}

// The FP32 omega*idiag of each level as one-byte codes into the handle's
// table, for the standalone FP32 7-point sweeps of 3D levels (bandwidth-
// bound: 13 instead of 16 bytes per cell, 249 -> 243 us per 512x512x256
// sweep). The 2D blocked passes keep the floats: they are issue-bound, and
// the table lookups made configuration 2 slower (14.0 against 13.6 ms).
// wq_ok only when every cell of every level reproduces its float exactly,
// so the coded and the streamed forms give the same bits.
int prepare_wq(cfmg_handle* h) {
  h->wq_ok = false;
  if (h->d.op != CFMG_LAPLACIAN && h->d.op != CFMG_LAPLACIAN9) return CFMG_OK;
  if (!h->wtab) return CFMG_OK;  // not a mixed-precision handle
  const double Q = h->d.op == CFMG_LAPLACIAN9 ? 4.0 : 1.0;
  int* ok = (int*)h->partials;  // scratch
  const int one = 1;
  CUDA_OK(h, cudaMemcpyAsync(ok, &one, sizeof(int), cudaMemcpyHostToDevice, h->stream));
  launch_wq_table(h->wtab, h->d.omega, Q, h->stream);
  for (Level& l : h->lv) {
    launch_make_wq(l.diag, l.widiag32, h->wtab, Q, l.wq, (long long)l.len, ok, h->stream);
    // four-cell 3D sweep: which (run of planes, quad) holds a wet cell
    if (l.threed && l.tz >= 3 && ((long long)l.tx * l.ty) % 4 == 0) {
      const long long nq = ((long long)l.tx * l.ty) / 4, nruns = (l.tz - 2 + kQRunPlanes - 1) / kQRunPlanes;
      if (!l.qact) CUDA_OK(h, cudaMalloc((void**)&l.qact, (size_t)(nq * nruns)));
      launch_make_qact(l.msk, l.qact, (long long)l.tx * l.ty, l.tz, kQRunPlanes, h->stream);
    }
  }
  int hok = 0;
  CUDA_OK(h, cudaMemcpyAsync(&hok, ok, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
  CUDA_OK(h, cudaStreamSynchronize(h->stream));
  LAUNCH_OK(h);
  h->wq_ok = hok != 0;
  return CFMG_OK;
}

int prepare_mixed(cfmg_handle* h) {
  if (!h->mixed_dirty) return CFMG_OK;
  for (Level& l : h->lv) {
    launch_to_f32(l.widiag, l.widiag32, l.len, h->stream);
    launch_to_f32(l.diag, l.diag32, l.len, h->stream);
    launch_to_f32(l.Rcoef, l.Rcoef32, l.len, h->stream);
    launch_to_f32(l.Pcoef, l.Pcoef32, l.len, h->stream);
    if (h->d.op == CFMG_VARCOEF) {
      launch_to_f32(l.cE, l.cE32, l.len, h->stream);
      launch_to_f32(l.cN, l.cN32, l.len, h->stream);
    }
  }
  TRY(prepare_wq(h));
  // number of wet cells of level 1 (for the residual scaling)
  const Level& l1 = h->lv[0];
  launch_fill_f64(l1.y, 1.0, l1.len, h->stream);
  launch_norm<double>(l1.y, l1.msk, l1.len, h->partials, h->dscal + S_TMP0, nullptr, CFMG_NORM_L2, h->stream);
  CUDA_OK(h, cudaMemcpyAsync(h->dscal + S_NWET, h->dscal + S_TMP0, sizeof(double), cudaMemcpyDeviceToDevice,
                             h->stream));
  CUDA_OK(h, cudaMemsetAsync(l1.y, 0, l1.len * sizeof(double), h->stream));
  LAUNCH_OK(h);
  TRY(prepare_int(h));
  h->mixed_dirty = false;
  return CFMG_OK;
}

// ------------------------------------------------------- mixed-precision
// Defect correction: r (FP64) -> scaled FP32 right-hand side of the
// correction equation on level 1, with the wet mean removed for the
// cell-centred (Neumann) operator.
__global__ void k_mean_partial(const double* r, const uint8_t* m, long long n, double* partials) {
  dep_wait();
  // Neumaier-compensated per-thread sums, fixed-order tree across the block
  double s = 0.0, c = 0.0;
  for (long long I = (long long)blockIdx.x * blockDim.x + threadIdx.x; I < n; I += (long long)gridDim.x * blockDim.x) {
    if (!m[I]) continue;
    double v = r[I];
    double t = __dadd_rn(s, v);
    c = __dadd_rn(c, (fabs(s) >= fabs(v)) ? __dadd_rn(__dsub_rn(s, t), v) : __dadd_rn(__dsub_rn(v, t), s));
    s = t;
  }
  s = __dadd_rn(s, c);
  __shared__ double sh[256];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int w = 128; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) partials[blockIdx.x] = sh[0];
}

__global__ void k_scale_from_norm(double* dscal, const double* partials, int nparts, bool remove_mean) {
  dep_wait();
  // dscal[S_NORM] = sum msk r^2 (raw or 1 if 0), dscal[S_NWET] = number of wet cells
  __shared__ double sh[kNormParts];
  double v = 0.0;
  if (remove_mean && (int)threadIdx.x < nparts) v = partials[threadIdx.x];
  sh[threadIdx.x] = v;
  __syncthreads();
  for (int w = kNormParts / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    double nwet = dscal[S_NWET] > 0 ? dscal[S_NWET] : 1.0;
    double rms = sqrt(dscal[S_NORM] / nwet);
    const bool ok = rms > 0 && isfinite(rms);
    dscal[S_SCALE] = ok ? 1.0 / rms : 1.0;
    dscal[S_ISCALE] = ok ? rms : 1.0;
    dscal[S_MEAN] = remove_mean ? sh[0] / nwet : 0.0;
  }
}

__global__ void k_rhs32(const double* r, const uint8_t* m, const double* dscal, float* b32, float* r32, long long n) {
  dep_wait();
  long long I = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (I >= n) return;
  double v = m[I] ? (r[I] - dscal[S_MEAN]) * dscal[S_SCALE] : 0.0;
  float f = (float)v;
  b32[I] = f;
  r32[I] = f;
}

// x += e / scale (the FP64 solution update)
__global__ void k_update(double* x, const float* e, const double* dscal, long long n) {
  dep_wait();
  long long I = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (I >= n) return;
  x[I] = __fma_rn((double)e[I], dscal[S_ISCALE], x[I]);
}

// ------------------------------------------------------------- adjoint
// wet-mean removal: x -= (sum msk x)/(sum msk) on wet cells, the sum in
// Neumaier-compensated FP64 (k_mean_partial above) with a fixed-order final
__global__ void k_mean_final(const double* partials, int nparts, double* dscal) {
  dep_wait();
  __shared__ double sh[kNormParts];
  sh[threadIdx.x] = (int)threadIdx.x < nparts ? partials[threadIdx.x] : 0.0;
  __syncthreads();
  for (int w = kNormParts / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) dscal[S_MEAN] = dscal[S_NWET] > 0 ? sh[0] / dscal[S_NWET] : 0.0;
}
__global__ void k_sub_mean(double* x, const uint8_t* m, const double* dscal, long long n) {
  dep_wait();
  long long I = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (I >= n) return;
  x[I] = m[I] ? x[I] - dscal[S_MEAN] : 0.0;
}

// dL/dkappa_k = sum over the faces of k with both cells wet of
// 1/2 (lam_k - lam_nb)(x_k - x_nb): the face coefficient (kappa_k+kappa_nb)/2
// enters A as c_f (x_nb - x_k) in both rows, so dL/dc_f = (lam_i-lam_j)(x_i-x_j).
__global__ void k_kappa_grad(const double* lam, const double* x, const uint8_t* m, double* gk, long long n1,
                             long long n) {
  dep_wait();
  long long I = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (I >= n) return;
  double s = 0.0;
  if (m[I]) {
    const long long nb[4] = {I - 1, I + 1, I - n1, I + n1};
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const long long J = nb[q];
      if (J >= 0 && J < n && m[J]) s += 0.5 * (lam[I] - lam[J]) * (x[I] - x[J]);
    }
  }
  gk[I] = s;
}

int count_wet(cfmg_handle* h) {
  const Level& l1 = h->lv[0];
  launch_fill_f64(l1.y, 1.0, l1.len, h->stream);
  launch_norm<double>(l1.y, l1.msk, l1.len, h->partials, h->dscal + S_TMP0, nullptr, CFMG_NORM_L2, h->stream);
  CUDA_OK(h, cudaMemcpyAsync(h->dscal + S_NWET, h->dscal + S_TMP0, sizeof(double), cudaMemcpyDeviceToDevice,
                             h->stream));
  CUDA_OK(h, cudaMemsetAsync(l1.y, 0, l1.len * sizeof(double), h->stream));
  LAUNCH_OK(h);
  return CFMG_OK;
}

int remove_wet_mean(cfmg_handle* h, double* x) {
  const Level& l1 = h->lv[0];
  const long long n = (long long)l1.len;
  launch_dep(k_mean_partial, kNormParts, 256, 0, h->stream, x, l1.msk, n, h->partials);
  launch_dep(k_mean_final, 1, kNormParts, 0, h->stream, h->partials, kNormParts, h->dscal);
  launch_dep(k_sub_mean, (unsigned)((n + 255) / 256), 256, 0, h->stream, x, l1.msk, h->dscal, n);
  h->launches += 3;
  LAUNCH_OK(h);
  return CFMG_OK;
}

// Fused path (closed topology): one pass gives the FP64 residual, its
// norm (and wet sum) and the scaled FP32 right-hand side of the next
// correction; a Neumann operator adds a mean-removing pass.
bool fused_ok(const cfmg_handle* h) { return !xperio(h) && h->d.op != CFMG_VARCOEF; }
bool int_path(const cfmg_handle* h) { return h->int_on && h->int_ok && fused_ok(h); }

int fused_residual(cfmg_handle* h) {
  TRY(flush(h));
  const Level& l1 = h->lv[0];
  Geom g = geom(l1);
  const bool neumann = !vertices(h);
  int kind;
  Box bx = interior(l1);
  long long lo = 0, n;
  if (h->d.op == CFMG_LAPLACIAN9) kind = threed(h) ? OPK_RESID19 : OPK_RESID9;
  else kind = threed(h) ? OPK_RESID7 : OPK_RESID5;
  if (kind == OPK_RESID5) {
    lo = g.n1;
    n = g.len - 2 * g.n1;
  } else {
    n = box_count(bx);
  }
  if (int_path(h)) {
    {
      // the F-cycle restricts level 1's r first: it must hold the right-hand side too
      Launch k(h, CFMG_K_RESIDUAL, 1, CFMG_FP64, 2);
      float* r32 = h->d.cycle == CFMG_CYCLE_F ? l1.r32 : nullptr;
      const bool r3 = kind == OPK_RESID7 && h->r3_on &&
                      launch_resid_int3d(l1.x, l1.b, h->dqp, g, bx, h->dscal, l1.b32, r32, neumann, h->partials,
                                         h->stream, h->r3_rows, h->dry_on ? h->tcol : nullptr);
      h->r3_ran |= r3;
      if (!r3 && !launch_resid_int2d(kind, l1.x, l1.b, h->dq, g, bx, h->dscal, l1.b32, r32, neumann, h->partials,
                                     h->stream, h->dry_on ? h->sflag : nullptr))
        launch_resid_int(kind, l1.x, l1.b, h->dq, g, bx, lo, n, h->dscal, l1.b32, r32, neumann, h->partials,
                         h->stream);
      launch_fused_final(h->partials, h->dscal, h->dscal + S_NORMB, neumann ? h->dscal + S_NWET : nullptr,
                         h->d.norm_kind, h->stream);
    }
    if (neumann) {
      Launch k(h, CFMG_K_CONVERT, 1, CFMG_MIXED);
      launch_rhs32_shift(l1.msk, h->dscal + S_MEAN2, l1.b32, h->d.cycle == CFMG_CYCLE_F ? l1.r32 : nullptr,
                         (long long)l1.len, h->stream, h->dry_on);
    }
    LAUNCH_OK(h);
    return CFMG_OK;
  }
  {
    Launch k(h, CFMG_K_RESIDUAL, 1, CFMG_FP64, 2);
    launch_resid_fused(kind, l1.r, l1.x, l1.b, l1.diag, l1.msk, g, bx, lo, n, h->dscal + S_NEXT, l1.b32, l1.r32,
                       neumann, h->partials, h->stream);
    launch_fused_final(h->partials, h->dscal, h->dscal + S_NORMB, neumann ? h->dscal + S_NWET : nullptr,
                       h->d.norm_kind, h->stream);
  }
  if (neumann) {
    Launch k(h, CFMG_K_CONVERT, 1, CFMG_MIXED);
    launch_rhs32_mean(l1.r, l1.msk, h->dscal + S_MEAN2, l1.b32, l1.r32, (long long)l1.len, h->stream);
  }
  LAUNCH_OK(h);
  return CFMG_OK;
}

__global__ void init_scale(double* ds) {
  dep_wait();
  const double nw = ds[S_NWET] > 0 ? ds[S_NWET] : 1.0;
  const double rms = sqrt(ds[S_NORMB] / nw);
  int e = 0;
  if (rms > 0 && isfinite(rms)) frexp(rms, &e);
  ds[S_NEXT] = ldexp(1.0, -e);
}

// The V-cycle's first read of level 1's FP32 x is its first pre-smoothing
// sweep: in the 3D 7-point coded four-cell form that sweep takes x as +0
// without reading it, so x is not zeroed. The cells the sweeps never write
// (planes 1 and tz) hold +0 from the arena's clearing, like every cell
// outside the wet interior of the mixed form's FP32 fields.
bool x1_zero_ok(const cfmg_handle* h, int kind) {
  if (kind != CFMG_CYCLE_V && kind != CFMG_CYCLE_VREC) return false;
  if (!threed(h) || h->d.op != CFMG_LAPLACIAN || xperio(h) || h->d.npre < 1 || h->record || !h->wq_on ||
      !h->wq_ok || tb_eligible<float>(h, 1) || L(h) < 2)
    return false;
  const Level& l = h->lv[0];
  if (h->engine_on && (long long)l.len <= engine_limit(h, CFMG_MIXED)) return false;
  const View<float> v = view<float>(l);
  return l.xswap == 0 && sweep7_quad_ok(geom(l), v.x, v.y, v.b, l.wq);
}

int mixed_iteration(cfmg_handle* h, int kind) {
  for (Level& l : h->lv) l.xswap = 0;  // every FP32 x is zeroed before use in the cycle
  // the F-cycle's first write of level 1's x is its last prolongation: the
  // x buffer (+0 outside the wet interior in both buffers) is assigned
  // there, not zeroed first
  const bool lazy = kind == CFMG_CYCLE_F && !xperio(h);
  h->x1_zero = !lazy && x1_zero_ok(h, kind);
  if (fused_ok(h)) {  // the right-hand side was made by the previous fused pass
    const Level& l1 = h->lv[0];
    if (!lazy && !h->x1_zero) TRY(zero_t<float>(h, 1, CFMG_X));
    // the update with max |x| can run in the cycle's last level-1 pass
    h->upd_req = h->upd_on && int_path(h);
    h->upd_done = false;
    const int st = cycle_t<float>(h, kind, lazy);
    h->upd_req = false;
    h->x1_zero = false;
    if (st != CFMG_OK) return st;
    if (!h->upd_done) {
      Launch k(h, CFMG_K_CONVERT, 1, CFMG_MIXED);
      // 3D: groups of dry cells are skipped (S_MAXO holds their max |x|, see cfmg_solve)
      if (int_path(h))
        launch_update_scaled_max(l1.x, view<float>(l1).x, h->dscal, (long long)l1.len, h->stream,
                                 threed(h) && h->dry_on ? l1.msk : nullptr);
      else launch_update_scaled(l1.x, view<float>(l1).x, h->dscal + S_ICUR, (long long)l1.len, h->stream);
    }
    LAUNCH_OK(h);
    return fused_residual(h);
  }
  const Level& l1 = h->lv[0];
  const long long n = (long long)l1.len;
  const unsigned nb = (unsigned)((n + 255) / 256);
  const bool remove_mean = !vertices(h);
  TRY(flush(h));
  {
    Launch k(h, CFMG_K_CONVERT, 1, CFMG_MIXED, remove_mean ? 3 : 2);
    if (remove_mean) launch_dep(k_mean_partial, kNormParts, 256, 0, h->stream, l1.r, l1.msk, n, h->partials);
    launch_dep(k_scale_from_norm, 1, kNormParts, 0, h->stream, h->dscal, h->partials, kNormParts, remove_mean);
    launch_dep(k_rhs32, nb, 256, 0, h->stream, l1.r, l1.msk, h->dscal, l1.b32, l1.r32, n);
  }
  if (!lazy && !h->x1_zero) TRY(zero_t<float>(h, 1, CFMG_X));
  LAUNCH_OK(h);
  const int st = cycle_t<float>(h, kind, lazy);
  h->x1_zero = false;
  TRY(st);
  {
    Launch k(h, CFMG_K_CONVERT, 1, CFMG_MIXED);
    launch_dep(k_update, nb, 256, 0, h->stream, l1.x, view<float>(l1).x, h->dscal, n);
  }
  LAUNCH_OK(h);
  return CFMG_OK;
}

// one solve iteration (cycle + normresidual + copy of the ratio to the host)
int iteration(cfmg_handle* h, int prec, int kind, int norm_kind) {
  if (prec == CFMG_MIXED) {
    TRY(mixed_iteration(h, kind));
    if (!fused_ok(h)) TRY(normresidual_dev(h, norm_kind));
  } else {
    TRY(cycle_t<double>(h, kind));
    TRY(normresidual_dev(h, norm_kind));
  }
  CUDA_OK(h, cudaMemcpyAsync(h->hscal, h->dscal, 2 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  return CFMG_OK;
}

int get_graph(cfmg_handle* h, int prec, int kind, int norm_kind, cudaGraphExec_t* out) {
  cudaGraphExec_t& ge = h->graph[prec][kind];
  if (!ge) {
    cudaGraph_t g = nullptr;
    CUDA_OK(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeRelaxed));
    const long long before = h->launches;
    h->capturing = true;
    int rc = iteration(h, prec, kind, norm_kind);
    h->capturing = false;
    h->graph_launches[prec][kind] = h->launches - before;
    h->launches = before;
    cudaError_t e = cudaStreamEndCapture(h->stream, &g);
    if (rc != CFMG_OK) {
      if (g) cudaGraphDestroy(g);
      return rc;
    }
    if (e != cudaSuccess) return fail(h, CFMG_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
    e = cudaGraphInstantiate(&ge, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
      ge = nullptr;
      return fail(h, CFMG_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(e));
    }
  }
  *out = ge;
  return CFMG_OK;
}

void drop_graphs(cfmg_handle* h) {
  for (auto* tab : {&h->graph, &h->sgraph})
    for (auto& row : *tab)
      for (auto& g : row)
        if (g) {
          cudaGraphExecDestroy(g);
          g = nullptr;
        }
}

// The solve! loop on the device (src/gmg_solver.jl:29-39): hist[nite] = res
// after every residual, and another iteration while res > tol and
// nite < maxite (the count moves before the iteration runs).
__global__ void k_loop_test(cudaGraphConditionalHandle hc, double* ds, double* hist, double tol, int maxite,
                            int first) {
  if (first) ds[S_NITE] = 0.0;
  const double res = ds[S_RES];
  const int nite = (int)ds[S_NITE];
  hist[nite] = res;
  // a NaN or Inf in b or in the residual ends the loop (reported as
  // CFMG_ERR_NONFINITE): an infinite |b| would otherwise give res = 0
  const bool more = isfinite(ds[S_NORMB]) && isfinite(res) && res > tol && nite < maxite;
  if (more) ds[S_NITE] = (double)(nite + 1);
  cudaGraphSetConditional(hc, more ? 1u : 0u);
}

int get_solve_graph(cfmg_handle* h, int prec, int kind, int norm_kind, cudaGraphExec_t* out) {
  cudaGraphExec_t& ge = h->sgraph[prec][kind];
  if (ge) {
    *out = ge;
    return CFMG_OK;
  }
  if (!h->dhist) CUDA_OK(h, cudaMalloc((void**)&h->dhist, sizeof(double) * (size_t)(h->d.maxite + 1)));
  cudaGraph_t g = nullptr;
  CUDA_OK(h, cudaGraphCreate(&g, 0));
  cudaGraphConditionalHandle hc;
  cudaError_t e = cudaGraphConditionalHandleCreate(&hc, g, 0, 0);
  auto bail = [&](const char* what) {
    cudaGraphDestroy(g);
    return fail(h, CFMG_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
  };
  if (e != cudaSuccess) return bail("conditional handle");
  // the test of the first residual, then while (test) { iteration; test }
  if ((e = cudaStreamBeginCaptureToGraph(h->stream, g, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed)) !=
      cudaSuccess)
    return bail("solve capture");
  k_loop_test<<<1, 1, 0, h->stream>>>(hc, h->dscal, h->dhist, h->d.tol, h->d.maxite, 1);
  if ((e = cudaStreamEndCapture(h->stream, &g)) != cudaSuccess) return bail("solve capture");
  cudaGraphNode_t first = nullptr;
  size_t nn = 1;
  if ((e = cudaGraphGetNodes(g, &first, &nn)) != cudaSuccess) return bail("solve graph");
  cudaGraphNodeParams cp = {};
  cp.type = cudaGraphNodeTypeConditional;
  cp.conditional.handle = hc;
  cp.conditional.type = cudaGraphCondTypeWhile;
  cp.conditional.size = 1;
  cudaGraphNode_t wnode;
  if ((e = cudaGraphAddNode(&wnode, g, &first, nullptr, 1, &cp)) != cudaSuccess) return bail("while node");
  cudaGraph_t body = cp.conditional.phGraph_out[0];
  if ((e = cudaStreamBeginCaptureToGraph(h->stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed)) !=
      cudaSuccess)
    return bail("solve capture");
  const long long before = h->launches;
  h->capturing = true;
  int rc = iteration(h, prec, kind, norm_kind);
  h->capturing = false;
  h->graph_launches[prec][kind] = h->launches - before;
  h->launches = before;
  if (rc == CFMG_OK) k_loop_test<<<1, 1, 0, h->stream>>>(hc, h->dscal, h->dhist, h->d.tol, h->d.maxite, 0);
  e = cudaStreamEndCapture(h->stream, &body);
  if (rc != CFMG_OK) {
    cudaGraphDestroy(g);
    return rc;
  }
  if (e != cudaSuccess) return bail("solve capture");
  e = cudaGraphInstantiate(&ge, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) {
    ge = nullptr;
    return fail(h, CFMG_ERR_CUDA, std::string("solve graph instantiate: ") + cudaGetErrorString(e));
  }
  *out = ge;
  return CFMG_OK;
}

// ------------------------------------------------ whole-solve programs
// Records the mixed-precision solve of one handle (the loop of cfmg_solve
// with mixed_iteration's steps) as a single engine program whose loop,
// norms and stopping test run on the device; sc is the program's scalar
// block (SolveSlot), nsc its length.
int record_solve_program(cfmg_handle* h, double* sc, std::vector<Op>& out) {
  const Level& l1 = h->lv[0];
  const long long n = (long long)l1.len;
  const int nk = h->d.norm_kind;
  const bool neumann = !vertices(h);
  h->record = true;
  h->pending.clear();
  auto sop = [&](int kind) {
    Op op = mkop(kind, 0, 1, CFMG_K_NORM, l1);
    op.sc = sc;
    op.n = n;
    op.norm_kind = nk;
    return op;
  };
  auto push = [&](const Op& op) { h->pending.push_back(op); };
  auto residual_norm = [&]() -> int {
    TRY(residual_t<double>(h, 1));
    Op o = sop(OPK_NORM64);
    o.x = l1.r; o.m = l1.msk; o.s0 = SS_NR; o.s1 = nk == CFMG_NORM_REF_SQUARED;
    push(o);
    o = sop(OPK_RATIO);
    o.s0 = SS_RES; o.s1 = SS_NR; o.s2 = SS_NORMB;
    push(o);
    o = sop(OPK_HIST);
    o.s0 = SS_HIST; o.s1 = SS_NITE; o.s2 = SS_RES;
    push(o);
    return CFMG_OK;
  };
  int rc = CFMG_OK;
  do {
    Op o = sop(OPK_STAMP);
    o.s0 = SS_T0;
    push(o);
    o = sop(OPK_ZERO_IF);  // solve from x = 0 when asked, else from the current x
    o.y = l1.x; o.s0 = SS_ZEROX;
    push(o);
    o = sop(OPK_NORM64);  // normb = norm(mg, 1, :b)
    o.x = l1.b; o.m = l1.msk; o.s0 = SS_NORMB; o.s1 = nk == CFMG_NORM_REF_SQUARED;
    push(o);
    if ((rc = residual_norm()) != CFMG_OK) break;
    const int branch = (int)h->pending.size();
    o = sop(OPK_BRANCH);
    o.s0 = SS_RES; o.s1 = SS_NITE; o.tol = h->d.tol; o.maxite = h->d.maxite;
    push(o);
    if (neumann) {
      o = sop(OPK_MEAN64);
      o.x = l1.r; o.m = l1.msk; o.s0 = SS_MEAN; o.s1 = SS_NWET;
      push(o);
    }
    o = sop(OPK_SCALE);
    o.s0 = SS_SCALE; o.s1 = SS_NR; o.s2 = SS_NWET;
    push(o);
    for (Level& l : h->lv) l.xswap = 0;
    o = sop(OPK_RHS32);
    o.x = l1.r; o.m = l1.msk; o.y = l1.b32; o.y2 = l1.r32; o.s0 = SS_SCALE; o.s1 = SS_MEAN;
    push(o);
    if ((rc = zero_t<float>(h, 1, CFMG_X)) != CFMG_OK) break;
    if ((rc = cycle_body<float>(h, h->d.cycle)) != CFMG_OK) break;
    o = sop(OPK_UPDATE);
    o.x = view<float>(l1).x; o.y = l1.x; o.s0 = SS_ISCALE;
    push(o);
    if ((rc = residual_norm()) != CFMG_OK) break;
    o = sop(OPK_JUMP);
    o.s2 = branch;
    push(o);
    h->pending[branch].s2 = (int)h->pending.size();  // the loop exits to the final stamp
    o = sop(OPK_STAMP);
    o.s0 = SS_T1;
    push(o);
  } while (false);
  h->record = false;
  out.swap(h->pending);
  h->pending.clear();
  return rc;
}

// ----------------------------------------------------------- allocation
std::vector<Level> create_levels(const cfmg_desc& d) {  // src/gmg_setup.jl:40-64
  std::vector<Level> out;
  int nx = d.nx, ny = d.ny, nz = d.nz;
  const bool t3 = d.kase == CFMG_THREED;
  const int maxlevs = d.nlevels > 0 ? d.nlevels : 29;
  auto mk = [&](int a, int b, int c) {
    Level l;
    std::memset(&l, 0, sizeof(l));
    l.nx = a; l.ny = b; l.nz = c; l.nh = d.nh;
    l.tx = a + 2 * d.nh;
    l.ty = b + 2 * d.nh;
    l.tz = t3 ? c + 2 * d.nh : c;
    l.threed = t3;
    l.len = (size_t)l.tx * l.ty * l.tz;
    l.ic0 = d.nh + 1; l.ic1 = a + d.nh;
    l.jc0 = d.nh + 1; l.jc1 = b + d.nh;
    l.kc0 = t3 ? d.nh + 1 : 1; l.kc1 = t3 ? c + d.nh : c;
    return l;
  };
  out.push_back(mk(nx, ny, nz));
  int lev = 1;
  while (((long long)nx * ny > 8) && (nx > 2) && (ny > 2) && (lev < maxlevs)) {
    nx /= 2;
    ny /= 2;
    if (t3) nz /= 2;
    out.push_back(mk(nx, ny, nz));
    lev += 1;
  }
  return out;
}

int validate(const cfmg_desc* d) {
  if (!d) return fail(nullptr, CFMG_ERR_ARG, "null descriptor");
  if (d->kase != CFMG_TWOD && d->kase != CFMG_THREED) return fail(nullptr, CFMG_ERR_ARG, "grid must be :twod or :threed");
  if (d->location != CFMG_CENTERS && d->location != CFMG_VERTICES)
    return fail(nullptr, CFMG_ERR_ARG, "location must be :centers or :vertices");
  if (d->op < CFMG_LAPLACIAN || d->op > CFMG_VARCOEF) return fail(nullptr, CFMG_ERR_ARG, "unknown operator");
  if (d->op == CFMG_VARCOEF && (d->kase != CFMG_TWOD || d->location != CFMG_CENTERS))
    return fail(nullptr, CFMG_ERR_UNSUPPORTED, "the variable-coefficient operator is 2D cell-centred only");
  if (d->topology != CFMG_CLOSED && d->topology != CFMG_XPERIO)
    return fail(nullptr, CFMG_ERR_ARG, "topology is not implemented");
  if (d->cycle < 0 || d->cycle > CFMG_CYCLE_VREC) return fail(nullptr, CFMG_ERR_ARG, "unknown cycle");
  if (d->nx < 1 || d->ny < 1 || d->nz < 1) return fail(nullptr, CFMG_ERR_ARG, "nx, ny, nz must be >= 1");
  if (d->nh < 2 || d->nh > 8) return fail(nullptr, CFMG_ERR_ARG, "nh must be in 2..8");
  if (d->npre < 0 || d->npost < 0 || d->ndeepest < 0 || d->maxite < 0 || d->nlevels < 0)
    return fail(nullptr, CFMG_ERR_ARG, "negative count");
  if (d->precision != CFMG_FP64 && d->precision != CFMG_MIXED) return fail(nullptr, CFMG_ERR_ARG, "unknown precision");
  if (d->norm_kind != CFMG_NORM_REF_SQUARED && d->norm_kind != CFMG_NORM_L2)
    return fail(nullptr, CFMG_ERR_ARG, "unknown norm kind");
  if (!(d->omega > 0.0 && d->omega < 2.0)) return fail(nullptr, CFMG_ERR_ARG, "omega must be in (0, 2)");
  long long cells = (long long)(d->nx + 2 * d->nh) * (d->ny + 2 * d->nh) *
                    (d->kase == CFMG_THREED ? d->nz + 2 * d->nh : d->nz);
  if (cells > (1LL << 40)) return fail(nullptr, CFMG_ERR_ARG, "grid too large");
  return CFMG_OK;
}

}  // namespace

// ===================================================================== ABI
extern "C" {

int cfmg_desc_default(cfmg_desc* d) {
  if (!d) return CFMG_ERR_ARG;
  std::memset(d, 0, sizeof(*d));
  d->kase = CFMG_THREED;
  d->location = CFMG_CENTERS;
  d->op = CFMG_LAPLACIAN;
  d->topology = CFMG_CLOSED;
  d->cycle = CFMG_CYCLE_V;
  d->nx = d->ny = d->nz = 64;
  d->nh = 3;
  d->nlevels = 0;
  d->npre = d->npost = 1;
  d->ndeepest = 20;
  d->maxite = 15;
  d->omega = 0.9;
  d->tol = 1e-10;
  d->precision = CFMG_FP64;
  d->norm_kind = CFMG_NORM_REF_SQUARED;
  return CFMG_OK;
}

}  // extern "C"

// A handle. `shared` (batch instances) puts it on a caller's stream without
// a program store of its own.
static int create_handle(const cfmg_desc* d, cudaStream_t shared, cfmg_handle** out) {
  if (!out) return fail(nullptr, CFMG_ERR_ARG, "null output pointer");
  *out = nullptr;
  TRY(validate(d));
  const int pool_ops = shared ? 0 : kProgPoolOps;
  cfmg_handle* h = new cfmg_handle();
  h->d = *d;
  h->lv = create_levels(*d);
  if (cudaGetDevice(&h->device) != cudaSuccess) {
    delete h;
    return fail(nullptr, CFMG_ERR_CUDA, "no CUDA device");
  }
  // arena: all level arrays, 256-byte aligned
  const bool mixed = d->precision == CFMG_MIXED;
  const bool vc = d->op == CFMG_VARCOEF;
  // coded omega*idiag: the 3D 7-point operator's standalone FP32 sweeps
  const bool coded = mixed && d->kase == CFMG_THREED && d->op == CFMG_LAPLACIAN;
  auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
  size_t total = al(kPartials * sizeof(double)) + al(S_COUNT * sizeof(double)) + al((size_t)pool_ops * sizeof(Op));
  for (const Level& l : h->lv) {
    size_t n = l.len;
    total += 8 * al(n * 8) + al(n);           // x y r b diag idiag widiag Rcoef Pcoef + msk (Pcoef counted below)
    total += al(n * 8);                       // Pcoef
    total += (vc ? 3 : 0) * al(n * 8);        // kappa cE cN
    total += (mixed ? 8 : 0) * al(n * 4);     // x32 y32 r32 b32 widiag32 diag32 Rcoef32 Pcoef32
    total += (mixed && vc ? 2 : 0) * al(n * 4);
    total += coded ? al(n) : 0;               // wq
  }
  total += coded ? al(256 * sizeof(float)) : 0;  // wtab
  if (cudaMalloc(&h->arena, total) != cudaSuccess) {
    cudaGetLastError();
    delete h;
    return fail(nullptr, CFMG_ERR_ALLOC, "device allocation of " + std::to_string(total) + " bytes failed");
  }
  h->arena_bytes = total;
  char* p = (char*)h->arena;
  auto take = [&](size_t b) {
    void* q = p;
    p += al(b);
    return q;
  };
  h->partials = (double*)take(kPartials * sizeof(double));
  h->prog_pool = (Op*)take((size_t)pool_ops * sizeof(Op));
  h->pool_cap = pool_ops;
  h->dscal = (double*)take(S_COUNT * sizeof(double));
  for (Level& l : h->lv) {
    size_t n = l.len;
    l.x = (double*)take(n * 8); l.y = (double*)take(n * 8); l.r = (double*)take(n * 8); l.b = (double*)take(n * 8);
    l.diag = (double*)take(n * 8); l.idiag = (double*)take(n * 8); l.widiag = (double*)take(n * 8);
    l.Rcoef = (double*)take(n * 8); l.Pcoef = (double*)take(n * 8);
    l.msk = (uint8_t*)take(n);
    if (vc) { l.kappa = (double*)take(n * 8); l.cE = (double*)take(n * 8); l.cN = (double*)take(n * 8); }
    if (mixed) {
      l.x32 = (float*)take(n * 4); l.y32 = (float*)take(n * 4); l.r32 = (float*)take(n * 4); l.b32 = (float*)take(n * 4);
      l.widiag32 = (float*)take(n * 4); l.diag32 = (float*)take(n * 4);
      l.Rcoef32 = (float*)take(n * 4); l.Pcoef32 = (float*)take(n * 4);
      if (vc) { l.cE32 = (float*)take(n * 4); l.cN32 = (float*)take(n * 4); }
    }
    if (coded) l.wq = (uint8_t*)take(n);
  }
  if (coded) h->wtab = (float*)take(256 * sizeof(float));
  // the fixed-point residual pass reads kResidIntReach elements beside level
  // 1's x (values it never uses): the arena holds the device scalars in front
  // of it and level 1's y behind it
  static_assert(S_COUNT * sizeof(double) <= 256, "the device scalars fill one 256-byte slot");
  {
    const char* base = (const char*)h->arena;
    const char* x0 = (const char*)h->lv[0].x;
    const char* x1 = (const char*)(h->lv[0].x + h->lv[0].len);
    if (x0 - base < kResidIntReach * (long)sizeof(double) ||
        base + total - x1 < kResidIntReach * (long)sizeof(double)) {
      cfmg_destroy(h);
      return fail(nullptr, CFMG_ERR_STATE, "arena layout leaves no room beside level 1's x");
    }
  }
  if ((!shared && cudaStreamCreateWithFlags(&h->own_stream, cudaStreamNonBlocking) != cudaSuccess) ||
      cudaHostAlloc((void**)&h->hscal, S_COUNT * sizeof(double), cudaHostAllocDefault) != cudaSuccess) {
    cudaGetLastError();
    cfmg_destroy(h);
    return fail(nullptr, CFMG_ERR_ALLOC, "stream or pinned allocation failed");
  }
  h->stream = shared ? shared : h->own_stream;
  if (cudaMemsetAsync(h->arena, 0, total, h->stream) != cudaSuccess) {
    cfmg_destroy(h);
    return fail(nullptr, CFMG_ERR_CUDA, "arena clear failed");
  }
  if (vc)
    for (Level& l : h->lv) launch_fill_f64(l.kappa, 1.0, l.len, h->stream);
  if (cudaStreamSynchronize(h->stream) != cudaSuccess || cudaGetLastError() != cudaSuccess) {
    cfmg_destroy(h);
    return fail(nullptr, CFMG_ERR_CUDA, "initialisation kernels failed (is this an sm_103 GPU?)");
  }
  *out = h;
  return CFMG_OK;
}

extern "C" {

int cfmg_create(const cfmg_desc* d, cfmg_handle** out) { return create_handle(d, nullptr, out); }

int cfmg_destroy(cfmg_handle* h) {
  if (!h) return CFMG_OK;
  if (h->stream) cudaStreamSynchronize(h->stream);
  drop_graphs(h);
  harvest(h);
  for (cudaEvent_t e : h->ev_pool) cudaEventDestroy(e);
  for (double* p : {h->adj_x, h->adj_b, h->adj_gk})
    if (p) cudaFree(p);
  if (h->dq) cudaFree(h->dq);
  if (h->dqp) cudaFree(h->dqp);
  if (h->tcol) cudaFree(h->tcol);
  if (h->sflag) cudaFree(h->sflag);
  for (Level& l : h->lv)
    if (l.qact) cudaFree(l.qact);
  if (h->dhist) cudaFree(h->dhist);
  if (h->arena) cudaFree(h->arena);
  if (h->hscal) cudaFreeHost(h->hscal);
  if (h->own_stream) cudaStreamDestroy(h->own_stream);
  delete h;
  return CFMG_OK;
}

const char* cfmg_last_error(const cfmg_handle* h) {
  if (h) return h->err.c_str();
  std::lock_guard<std::mutex> lk(g_err_mu);
  return g_create_err.c_str();
}

int cfmg_nlevels(const cfmg_handle* h, int* n) {
  if (!h || !n) return CFMG_ERR_ARG;
  *n = L(h);
  return CFMG_OK;
}

int cfmg_level_dims(const cfmg_handle* h, int lev, int* dims) {
  if (!h || !dims || lev < 1 || lev > L(h)) return CFMG_ERR_ARG;
  const Level& l = h->lv[lev - 1];
  dims[0] = l.nx; dims[1] = l.ny; dims[2] = l.nz; dims[3] = l.nh; dims[4] = l.tx; dims[5] = l.ty; dims[6] = l.tz;
  return CFMG_OK;
}

int cfmg_set_stream(cfmg_handle* h, void* stream) {
  if (!h) return CFMG_ERR_ARG;
  CUDA_OK(h, cudaStreamSynchronize(h->stream));
  h->stream = stream ? (cudaStream_t)stream : h->own_stream;
  return CFMG_OK;
}

int cfmg_synchronize(cfmg_handle* h) {
  if (!h) return CFMG_ERR_ARG;
  return sync(h);
}

static void* field_any(const Level& l, int f, size_t* elt) {
  *elt = 8;
  switch (f) {
    case CFMG_X: return l.x;
    case CFMG_R: return l.r;
    case CFMG_B: return l.b;
    case CFMG_Y: return l.y;
    case CFMG_DIAG: return l.diag;
    case CFMG_IDIAG: return l.idiag;
    case CFMG_RCOEF: return l.Rcoef;
    case CFMG_PCOEF: return l.Pcoef;
    case CFMG_KAPPA: return l.kappa;
    case CFMG_MSK: *elt = 1; return l.msk;
    default: return nullptr;
  }
}

int cfmg_field_ptr(cfmg_handle* h, int lev, int field, void** dptr) {
  TRY(check_lev(h, lev));
  size_t elt;
  void* p = field_any(h->lv[lev - 1], field, &elt);
  if (!p || !dptr) return fail(h, CFMG_ERR_ARG, "unknown field (kappa exists only for the varcoef operator)");
  *dptr = p;
  return CFMG_OK;
}

static int refresh_derived(cfmg_handle* h, int lev, int field) {
  Level& l = h->lv[lev - 1];
  if (field == CFMG_IDIAG) launch_widiag(l.idiag, l.widiag, h->d.omega, l.len, h->stream);
  if (h->d.op == CFMG_VARCOEF && (field == CFMG_KAPPA || field == CFMG_MSK))
    launch_face_coef(l.kappa, l.msk, l.cE, l.cN, geom(l), h->stream);
  if (field >= CFMG_DIAG) h->mixed_dirty = true;
  LAUNCH_OK(h);
  return CFMG_OK;
}

int cfmg_upload(cfmg_handle* h, int lev, int field, const void* src) {
  TRY(check_lev(h, lev));
  size_t elt;
  Level& l = h->lv[lev - 1];
  void* p = field_any(l, field, &elt);
  if (!p || !src) return fail(h, CFMG_ERR_ARG, "unknown field or null source");
  CUDA_OK(h, cudaMemcpyAsync(p, src, l.len * elt, cudaMemcpyDefault, h->stream));
  TRY(refresh_derived(h, lev, field));
  if (field >= CFMG_DIAG && field != CFMG_MSK && field != CFMG_KAPPA) h->coef_set = true;
  h->solved = false;
  return sync(h);
}

int cfmg_download(cfmg_handle* h, int lev, int field, void* dst) {
  TRY(check_lev(h, lev));
  size_t elt;
  Level& l = h->lv[lev - 1];
  void* p = field_any(l, field, &elt);
  if (!p || !dst) return fail(h, CFMG_ERR_ARG, "unknown field or null destination");
  CUDA_OK(h, cudaMemcpyAsync(dst, p, l.len * elt, cudaMemcpyDefault, h->stream));
  return sync(h);
}

int cfmg_bind_level(cfmg_handle* h, int lev, const double* diag, const double* idiag, const double* Rcoef,
                    const double* Pcoef, const uint8_t* msk) {
  TRY(check_lev(h, lev));
  Level& l = h->lv[lev - 1];
  cudaStream_t s = h->stream;
  if (diag) CUDA_OK(h, cudaMemcpyAsync(l.diag, diag, l.len * 8, cudaMemcpyDefault, s));
  if (idiag) CUDA_OK(h, cudaMemcpyAsync(l.idiag, idiag, l.len * 8, cudaMemcpyDefault, s));
  if (Rcoef) CUDA_OK(h, cudaMemcpyAsync(l.Rcoef, Rcoef, l.len * 8, cudaMemcpyDefault, s));
  if (Pcoef) CUDA_OK(h, cudaMemcpyAsync(l.Pcoef, Pcoef, l.len * 8, cudaMemcpyDefault, s));
  if (msk) CUDA_OK(h, cudaMemcpyAsync(l.msk, msk, l.len, cudaMemcpyDefault, s));
  TRY(refresh_derived(h, lev, CFMG_IDIAG));
  if (msk) TRY(refresh_derived(h, lev, CFMG_MSK));
  h->mixed_dirty = true;
  h->coef_set = true;
  h->solved = false;
  return sync(h);
}

int cfmg_set_default_msk(cfmg_handle* h) {
  if (!h) return CFMG_ERR_ARG;
  Level& l = h->lv[0];
  launch_default_msk(DEFMSK_SET, l.msk, nullptr, 0.0, l, vertices(h), threed(h), xperio(h), h->stream);
  LAUNCH_OK(h);
  return sync(h);
}

int cfmg_setup_operators(cfmg_handle* h) {
  if (!h) return CFMG_ERR_ARG;
  TRY(setup_operators(h));
  TRY(sync(h));
  h->coef_set = true;
  h->solved = false;
  return CFMG_OK;
}

int cfmg_smooth(cfmg_handle* h, int lev, int nite) {
  TRY(check_lev(h, lev));
  TRY(need_setup(h));
  if (nite < 0) return fail(h, CFMG_ERR_ARG, "nite must be >= 0");
  TRY(smooth_t<double>(h, lev, nite));
  return flush(h);
}

int cfmg_residual(cfmg_handle* h, int lev) {
  TRY(check_lev(h, lev));
  TRY(need_setup(h));
  TRY(residual_t<double>(h, lev));
  return flush(h);
}

int cfmg_restrict(cfmg_handle* h, int lev, int field) {
  TRY(check_lev(h, lev, 1));
  TRY(need_setup(h));
  if (field != CFMG_X && field != CFMG_R && field != CFMG_B && field != CFMG_Y)
    return fail(h, CFMG_ERR_ARG, "restriction field must be x, r, b or y");
  TRY(restrict_t<double>(h, lev, field));
  return flush(h);
}

int cfmg_prolong(cfmg_handle* h, int lev) {
  TRY(check_lev(h, lev, 1));
  TRY(need_setup(h));
  TRY(prolong_t<double>(h, lev));
  return flush(h);
}

int cfmg_zero(cfmg_handle* h, int lev, int field) {
  TRY(check_lev(h, lev));
  TRY(flush(h));
  size_t elt;
  Level& l = h->lv[lev - 1];
  void* p = field_any(l, field, &elt);
  if (!p) return fail(h, CFMG_ERR_ARG, "unknown field");
  CUDA_OK(h, cudaMemsetAsync(p, 0, l.len * elt, h->stream));
  if (field >= CFMG_DIAG) TRY(refresh_derived(h, lev, field));
  return CFMG_OK;
}

int cfmg_fill(cfmg_handle* h, int lev, int field) {
  TRY(check_lev(h, lev));
  size_t elt;
  Level& l = h->lv[lev - 1];
  void* p = field_any(l, field, &elt);
  if (!p) return fail(h, CFMG_ERR_ARG, "unknown field");
  if (!xperio(h)) return CFMG_OK;
  TRY(flush(h));
  if (elt == 1) launch_fill_xperio<uint8_t>((uint8_t*)p, geom(l), h->stream);
  else launch_fill_xperio<double>((double*)p, geom(l), h->stream);
  LAUNCH_OK(h);
  return CFMG_OK;
}

int cfmg_norm(cfmg_handle* h, int lev, int field, double* out) {
  TRY(check_lev(h, lev));
  size_t elt;
  Level& l = h->lv[lev - 1];
  void* p = field_any(l, field, &elt);
  if (!p || elt != 8 || !out) return fail(h, CFMG_ERR_ARG, "norm needs an FP64 field and an output");
  TRY(norm_dev(h, lev, (const double*)p, nullptr, CFMG_NORM_REF_SQUARED));
  CUDA_OK(h, cudaMemcpyAsync(h->hscal, h->dscal, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  TRY(sync(h));
  *out = h->hscal[0];
  return CFMG_OK;
}

int cfmg_normresidual(cfmg_handle* h, double normb, double* out) {
  if (!h || !out) return CFMG_ERR_ARG;
  TRY(need_setup(h));
  if (!(normb > 0.0)) {
    *out = 0.0;
    return CFMG_OK;
  }
  TRY(residual_t<double>(h, 1));
  double nr;
  TRY(cfmg_norm(h, 1, CFMG_R, &nr));
  *out = nr / normb;
  return CFMG_OK;
}

int cfmg_cycle(cfmg_handle* h, int kind) {
  if (!h) return CFMG_ERR_ARG;
  TRY(need_setup(h));
  return cycle_t<double>(h, kind);
}

// A NaN or Inf in b, or a residual that is not finite, ends the solve and
// makes it return CFMG_ERR_NONFINITE, with res and nite filled in.
// A bounded wait of the staged 3D residual pass (k_resid3d.cu) ran out: the
// pass set S_FAULT and NaN partial sums, which stopped the loop.
int fault_check(cfmg_handle* h) {
  if (!h->r3_ran) return CFMG_OK;
  double f = 0.0;
  CUDA_OK(h, cudaMemcpyAsync(&f, h->dscal + S_FAULT, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  TRY(sync(h));
  if (f == 0.0) return CFMG_OK;
  CUDA_OK(h, cudaMemsetAsync(h->dscal + S_FAULT, 0, sizeof(double), h->stream));
  return fail(h, CFMG_ERR_CUDA, "a wait for a TMA copy in the staged 3D residual pass ran out (1 s)");
}

int nonfinite_check(cfmg_handle* h, double normb, double res) {
  TRY(fault_check(h));
  if (std::isfinite(normb) && std::isfinite(res)) return CFMG_OK;
  return fail(h, CFMG_ERR_NONFINITE,
              std::string("non-finite ") + (std::isfinite(normb) ? "residual norm" : "norm of b") +
                  " (NaN or Inf in b, x or the coefficients)");
}

int cfmg_solve(cfmg_handle* h, double* res_out, int* nite_out, double* history) {
  if (!h || !res_out || !nite_out) return CFMG_ERR_ARG;
  TRY(need_setup(h));
  const cfmg_desc& d = h->d;
  int prec = d.precision;
  if (prec == CFMG_MIXED && L(h) == 1) prec = CFMG_FP64;  // no coarse level to correct with
  if (prec == CFMG_MIXED && d.cycle != CFMG_CYCLE_V && d.cycle != CFMG_CYCLE_F && d.cycle != CFMG_CYCLE_VREC)
    return fail(h, CFMG_ERR_UNSUPPORTED, "the mixed-precision form runs V and F cycles");
  if (prec == CFMG_MIXED) TRY(prepare_mixed(h));
  // normb = norm(mg, 1, :b) (src/gmg_solver.jl:22)
  const Level& l1 = h->lv[0];
  TRY(flush(h));
  {
    Launch k(h, CFMG_K_NORM, 1, CFMG_FP64, 2);
    launch_norm<double>(l1.b, l1.msk, l1.len, h->partials, h->dscal + S_NORMB, nullptr, d.norm_kind, h->stream);
  }
  LAUNCH_OK(h);
  if (prec == CFMG_MIXED && fused_ok(h)) {
    launch_dep(init_scale, 1, 1, 0, h->stream, h->dscal);  // the first right-hand side is scaled from |b|
    if (int_path(h)) {
      // fixed-point range of the first pass: max |x|, max |b|; and max |x|
      // outside the update box U, which no update changes: each iteration's
      // max |x| starts from it (the update in a smoothing pass sees U only)
      CUDA_OK(h, cudaMemsetAsync(h->dscal + S_MAXX, 0, 2 * sizeof(double), h->stream));
      CUDA_OK(h, cudaMemsetAsync(h->dscal + S_MAXO, 0, sizeof(double), h->stream));
      // 3D with dry cells skipped by the update: S_MAXO is the max |x| of the dry cells
      launch_maxabs2(l1.x, l1.b, (long long)l1.len, l1.tx, l1.ty, l1.nh, l1.nx + l1.nh + 1, l1.nh, l1.ny + l1.nh + 1,
                     h->dscal, h->stream, threed(h) && h->dry_on ? l1.msk : nullptr);
      h->launches += 1;
    }
    TRY(fused_residual(h));
  } else {
    TRY(normresidual_dev(h, d.norm_kind));
  }
  if (h->prof_cls < 0 && !h->host_loop) {
    // the whole loop as one graph launch; the history comes back at the end
    cudaGraphExec_t sg = nullptr;
    TRY(get_solve_graph(h, prec, d.cycle, d.norm_kind, &sg));
    CUDA_OK(h, cudaGraphLaunch(sg, h->stream));
    CUDA_OK(h, cudaMemcpyAsync(h->hscal, h->dscal, S_COUNT * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    TRY(sync(h));
    const int nite = (int)h->hscal[S_NITE];
    h->launches += 2 + (long long)nite * (h->graph_launches[prec][d.cycle] + 1);
    if (history)
      CUDA_OK(h, cudaMemcpy(history, h->dhist, sizeof(double) * (size_t)(nite + 1), cudaMemcpyDeviceToHost));
    *res_out = h->hscal[S_RES];
    *nite_out = nite;
    h->solved = true;
    return nonfinite_check(h, h->hscal[S_NORMB], h->hscal[S_RES]);
  }
  CUDA_OK(h, cudaMemcpyAsync(h->hscal, h->dscal, S_COUNT * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  TRY(sync(h));
  double res = h->hscal[S_RES];
  const double normb = h->hscal[S_NORMB];
  if (history) history[0] = res;
  int nite = 0;
  cudaGraphExec_t ge = nullptr;
  while (std::isfinite(normb) && std::isfinite(res) && (res > d.tol) && (nite < d.maxite)) {  // src/gmg_solver.jl:29-39
    nite += 1;
    if (h->prof_cls >= 0) {
      TRY(iteration(h, prec, d.cycle, d.norm_kind));  // eager, so launches can be bracketed
    } else {
      if (!ge) TRY(get_graph(h, prec, d.cycle, d.norm_kind, &ge));
      CUDA_OK(h, cudaGraphLaunch(ge, h->stream));
      h->launches += h->graph_launches[prec][d.cycle];
    }
    TRY(sync(h));
    res = h->hscal[S_RES];
    if (history) history[nite] = res;
  }
  *res_out = res;
  *nite_out = nite;
  h->solved = true;
  return nonfinite_check(h, normb, res);
}

int cfmg_solve_tol(cfmg_handle* h, double tol, int maxite, int norm_kind, double* res_out, int* nite_out,
                   double* history) {
  if (!h || !res_out || !nite_out) return CFMG_ERR_ARG;
  if (maxite < 0) return fail(h, CFMG_ERR_ARG, "maxite must be >= 0");
  if (norm_kind != CFMG_NORM_REF_SQUARED && norm_kind != CFMG_NORM_L2) return fail(h, CFMG_ERR_ARG, "unknown norm kind");
  if (!(tol >= 0.0)) return fail(h, CFMG_ERR_ARG, "tol must be >= 0");
  if (tol != h->d.tol || maxite != h->d.maxite || norm_kind != h->d.norm_kind) {
    // the captured graphs hold the stopping rule, the norm kind and the
    // history's length: rebuild them for the new values
    TRY(sync(h));
    drop_graphs(h);
    if (maxite > h->d.maxite && h->dhist) {
      cudaFree(h->dhist);
      h->dhist = nullptr;
    }
    h->d.tol = tol;
    h->d.maxite = maxite;
    h->d.norm_kind = norm_kind;
  }
  return cfmg_solve(h, res_out, nite_out, history);
}

int cfmg_adjoint_solve(cfmg_handle* h, const double* cot, double* grad_b, double* grad_kappa) {
  double res = 0.0;
  int nite = 0;
  return cfmg_adjoint(h, cot, grad_b, grad_kappa, &res, &nite);
}

int cfmg_adjoint(cfmg_handle* h, const double* g, double* grad_b, double* grad_kappa, double* res, int* nite) {
  if (!h || !g || !grad_b || !res || !nite) return CFMG_ERR_ARG;
  TRY(need_setup(h));
  if (!h->solved) return fail(h, CFMG_ERR_STATE, "cfmg_adjoint needs a forward cfmg_solve on this handle first");
  if (grad_kappa && h->d.op != CFMG_VARCOEF)
    return fail(h, CFMG_ERR_ARG, "grad_kappa needs the variable-coefficient operator");
  TRY(sync(h));
  Level& l1 = h->lv[0];
  const size_t bytes = l1.len * sizeof(double);
  for (double** p : {&h->adj_x, &h->adj_b, &h->adj_gk})
    if (!*p && cudaMalloc((void**)p, bytes) != cudaSuccess) {
      cudaGetLastError();
      return fail(h, CFMG_ERR_ALLOC, "adjoint scratch allocation failed");
    }
  cudaStream_t s = h->stream;
  const bool neumann = !vertices(h);
  // keep the forward state
  CUDA_OK(h, cudaMemcpyAsync(h->adj_x, l1.x, bytes, cudaMemcpyDeviceToDevice, s));
  CUDA_OK(h, cudaMemcpyAsync(h->adj_b, l1.b, bytes, cudaMemcpyDeviceToDevice, s));
  // A lam = P g (A symmetric), from lam = 0, with the forward's cycle and rule
  CUDA_OK(h, cudaMemcpyAsync(l1.b, g, bytes, cudaMemcpyDefault, s));
  if (neumann) {
    TRY(count_wet(h));
    TRY(remove_wet_mean(h, l1.b));
  }
  CUDA_OK(h, cudaMemsetAsync(l1.x, 0, bytes, s));
  TRY(cfmg_solve(h, res, nite, nullptr));
  if (neumann) {
    TRY(count_wet(h));
    TRY(remove_wet_mean(h, l1.x));
  }
  CUDA_OK(h, cudaMemcpyAsync(grad_b, l1.x, bytes, cudaMemcpyDefault, s));
  if (grad_kappa) {
    const long long n = (long long)l1.len;
    launch_dep(k_kappa_grad, (unsigned)((n + 255) / 256), 256, 0, s, l1.x, h->adj_x, l1.msk, h->adj_gk, l1.tx, n);
    h->launches += 1;
    LAUNCH_OK(h);
    CUDA_OK(h, cudaMemcpyAsync(grad_kappa, h->adj_gk, bytes, cudaMemcpyDefault, s));
  }
  // restore the forward solution and right-hand side
  CUDA_OK(h, cudaMemcpyAsync(l1.x, h->adj_x, bytes, cudaMemcpyDeviceToDevice, s));
  CUDA_OK(h, cudaMemcpyAsync(l1.b, h->adj_b, bytes, cudaMemcpyDeviceToDevice, s));
  return sync(h);
}

}  // extern "C"

namespace {

int bfail(cfmg_batch* b, int code, const std::string& msg) {
  if (b) b->err = msg;
  return code;
}

#define BCUDA(b, call)                                                                          \
  do {                                                                                          \
    cudaError_t _e = (call);                                                                    \
    if (_e != cudaSuccess) return bfail((b), CFMG_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(_e)); \
  } while (0)

__global__ void k_batch_init(double* sc, const double* nwet, int ninst, int nsc, double zero_x) {
  dep_wait();
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ninst * nsc) return;
  const int k = i % nsc;
  sc[i] = (k == SS_NWET) ? nwet[i / nsc] : (k == SS_ZEROX ? zero_x : 0.0);
}

int batch_build(cfmg_batch* b) {
  const int ninst = (int)b->inst.size();
  b->nsc = SS_HIST + b->d.maxite + 2;
  // per-instance FP32 coefficients and wet counts
  BCUDA(b, cudaMalloc((void**)&b->sc, sizeof(double) * (size_t)ninst * b->nsc));
  BCUDA(b, cudaMalloc((void**)&b->nwet, sizeof(double) * (size_t)ninst));
  for (int i = 0; i < ninst; ++i) {
    cfmg_handle* h = b->inst[i];
    int rc = prepare_mixed(h);
    if (rc == CFMG_OK) rc = count_wet(h);
    if (rc != CFMG_OK) return bfail(b, rc, "instance " + std::to_string(i) + ": " + h->err);
    BCUDA(b, cudaMemcpyAsync(b->nwet + i, h->dscal + S_NWET, sizeof(double), cudaMemcpyDeviceToDevice, b->stream));
  }
  // programs, in queue order (largest first)
  b->order.resize(ninst);
  for (int i = 0; i < ninst; ++i) b->order[i] = i;
  std::stable_sort(b->order.begin(), b->order.end(),
                   [&](int a, int c) { return b->inst[a]->lv[0].len > b->inst[c]->lv[0].len; });
  std::vector<Op> all;
  std::vector<size_t> off(ninst);
  std::vector<int> cnt(ninst);
  for (int q = 0; q < ninst; ++q) {
    const int i = b->order[q];
    std::vector<Op> prog;
    int rc = record_solve_program(b->inst[i], b->sc + (size_t)i * b->nsc, prog);
    if (rc != CFMG_OK) return bfail(b, rc, "instance " + std::to_string(i) + ": " + b->inst[i]->err);
    off[q] = all.size();
    cnt[q] = (int)prog.size();
    all.insert(all.end(), prog.begin(), prog.end());
  }
  BCUDA(b, cudaMalloc((void**)&b->progs, sizeof(Op) * all.size()));
  BCUDA(b, cudaMemcpy(b->progs, all.data(), sizeof(Op) * all.size(), cudaMemcpyHostToDevice));
  std::vector<const Op*> ptrs(ninst);
  for (int q = 0; q < ninst; ++q) ptrs[q] = b->progs + off[q];
  BCUDA(b, cudaMalloc((void**)&b->ptrs, sizeof(Op*) * (size_t)ninst));
  BCUDA(b, cudaMemcpy(b->ptrs, ptrs.data(), sizeof(Op*) * (size_t)ninst, cudaMemcpyHostToDevice));
  BCUDA(b, cudaMalloc((void**)&b->nops, sizeof(int) * (size_t)ninst));
  BCUDA(b, cudaMemcpy(b->nops, cnt.data(), sizeof(int) * (size_t)ninst, cudaMemcpyHostToDevice));
  b->nclusters = engine_max_clusters();
  if (b->nclusters > ninst) b->nclusters = ninst;
  BCUDA(b, cudaMalloc((void**)&b->counter, sizeof(int) * (size_t)(1 + b->nclusters)));
  BCUDA(b, cudaMalloc((void**)&b->red, sizeof(double) * (size_t)b->nclusters * kEngineCtas));
  // one graph per start mode: scalar init, queue reset, the batched engine
  const int tot = ninst * b->nsc;
  for (int z = 0; z < 2; ++z) {
    cudaGraph_t g = nullptr;
    BCUDA(b, cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeRelaxed));
    launch_dep(k_batch_init, (tot + 255) / 256, 256, 0, b->stream, b->sc, b->nwet, ninst, b->nsc, (double)z);
    cudaMemsetAsync(b->counter, 0, sizeof(int) * (size_t)(1 + b->nclusters), b->stream);
    launch_batch(b->ptrs, b->nops, ninst, b->counter, b->red, b->nclusters, b->stream);
    cudaError_t e = cudaStreamEndCapture(b->stream, &g);
    if (e != cudaSuccess) return bfail(b, CFMG_ERR_CUDA, std::string("batch capture: ") + cudaGetErrorString(e));
    e = cudaGraphInstantiate(&b->graph[z], g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return bfail(b, CFMG_ERR_CUDA, std::string("batch instantiate: ") + cudaGetErrorString(e));
  }
  b->hsc.resize((size_t)tot);
  b->built = true;
  return CFMG_OK;
}

// ---------------------------------------------------- lockstep batches
// One FP32 cycle of every instance as a sequence of steps aligned at the
// coarsest level: depth d is level nlev - d + 1 of an instance, which takes
// part in a step when nlev >= need.
enum VOp { V_SMOOTH, V_RESID, V_RESTRICT, V_ZERO, V_PROLONG, V_COARSEST };
struct VStep {
  int op, depth, need, arg;
};

// vcycle! from depth `top` (src/gmg_cycles.jl:67-83); `fblock`: a V-cycle
// inside the F-cycle, taken only by instances with at least `top` levels
void vsteps_v(std::vector<VStep>& s, const cfmg_desc& d, int top, bool fblock) {
  for (int dp = top; dp >= 2; --dp) {
    const int need = fblock ? top : dp;
    s.push_back({V_SMOOTH, dp, need, d.npre});
    s.push_back({V_RESID, dp, need, 0});
    s.push_back({V_RESTRICT, dp, need, CFMG_R});
    s.push_back({V_ZERO, dp - 1, need, 0});
  }
  s.push_back({V_COARSEST, 1, fblock ? top : 1, d.ndeepest});
  for (int dp = 2; dp <= top; ++dp) {
    const int need = fblock ? top : dp;
    s.push_back({V_PROLONG, dp, need, 0});
    s.push_back({V_SMOOTH, dp, need, d.npost});
  }
}

// fcycle! (src/gmg_cycles.jl:85-100): arg of a restriction at depth dp is
// resolved per instance (:r on level 1, :b below)
void vsteps_f(std::vector<VStep>& s, const cfmg_desc& d, int D) {
  for (int dp = D; dp >= 2; --dp) {
    s.push_back({V_RESTRICT, dp, dp, -1});
    s.push_back({V_ZERO, dp - 1, dp, 0});
  }
  s.push_back({V_COARSEST, 1, 1, d.ndeepest});
  for (int e = 2; e <= D; ++e) {
    s.push_back({V_PROLONG, e, e, 0});
    vsteps_v(s, d, e, true);
  }
}

// A smoothing (or the coarsest solve) of a level small enough for one
// block's shared memory, 2D 5- or 9-point: one BSmall block instead of a
// launch per sweep. Same sweeps, ranges and arithmetic as smooth_t.
bool small_smooth(cfmg_handle* h, const VStep& v, BSmall& out) {
  if (v.op != V_SMOOTH && v.op != V_COARSEST) return false;
  if (threed(h) || (h->d.op != CFMG_LAPLACIAN && h->d.op != CFMG_LAPLACIAN9)) return false;
  const int lev = L(h) - v.depth + 1;
  const Level& l = h->lv[lev - 1];
  const bool fp64 = v.op == V_COARSEST && coarsest_in_fp64(h);
  if (4 * (long long)l.len * (fp64 ? 8 : 4) > kBSmallBytes) return false;
  if (!fp64 && tb_eligible<float>(h, lev)) return false;
  if (l.xswap) return false;  // the FP32 x must be in x32
  std::memset(&out, 0, sizeof(out));
  out.prec = fp64 ? 0 : 1;
  out.stencil = h->d.op == CFMG_LAPLACIAN9 ? 9 : 5;
  out.npairs = v.arg;
  out.g = geom(l);
  out.ext = Box{l.nh, l.nx + l.nh + 1, l.nh, l.ny + l.nh + 1, 1, l.nz};
  out.in = interior(l);
  out.lo = out.g.n1;
  out.n = out.g.len - 2 * out.g.n1;
  out.b32 = l.b32;
  out.x32 = l.x32;
  out.w = fp64 ? (const void*)l.widiag : (const void*)l.widiag32;
  out.y = fp64 ? (const void*)l.y : (const void*)l.y32;
  out.cff = 1.0 - h->d.omega;
  return true;
}

int record_vstep(cfmg_handle* h, const VStep& v, std::vector<Op>& out) {
  const int nl = L(h);
  const int lev = nl - v.depth + 1;
  h->record = true;
  h->pending.clear();
  int rc = CFMG_OK;
  switch (v.op) {
    case V_SMOOTH: rc = smooth_t<float>(h, lev, v.arg); break;
    case V_RESID: rc = residual_t<float>(h, lev); break;
    case V_RESTRICT: rc = restrict_t<float>(h, lev, v.arg >= 0 ? v.arg : (lev > 1 ? CFMG_B : CFMG_R)); break;
    case V_ZERO: rc = zero_t<float>(h, lev, CFMG_X); break;
    case V_PROLONG: rc = prolong_t<float>(h, lev); break;
    case V_COARSEST: rc = coarsest_t<float>(h, v.arg); break;
  }
  h->record = false;
  out.swap(h->pending);
  h->pending.clear();
  return rc;
}

// One lockstep iteration of every active instance (see k_batch.cu).
int lockstep_body(cfmg_batch* b) {
  const int ninst = (int)b->inst.size();
  if (b->int_all) {
    launch_bres_int(b->kind, b->neumann, b->bi, b->ttab, b->ntasks, b->active, b->bpart, b->stream);
    launch_bfinal(b->bi, b->tstart, ninst, b->bpart, b->active, b->nactive, b->stream);
    if (b->neumann) launch_brhs_shift(b->bi, b->l1tab, b->l1chunks, b->active, b->stream);
  } else {
    launch_bres(b->kind, b->neumann, b->bi, b->l1tab, b->l1chunks, b->active, b->bpart, b->stream);
    launch_bfinal(b->bi, b->l1start, ninst, b->bpart, b->active, b->nactive, b->stream);
    if (b->neumann) launch_brhs(b->bi, b->l1tab, b->l1chunks, b->active, b->stream);
  }
  for (const cfmg_batch::Step& st : b->steps) {
    if (st.tb == 3) {
      launch_brun(b->sops, b->ssm, b->rent, b->runs + st.tab0, (int)st.nchunks, st.smem, b->active, b->stream);
    } else if (st.tb == 2) {
      launch_bsmall(b->ssm + st.tab0, (int)st.nchunks, st.smem, b->active, b->stream);
    } else if (st.tb == 4) {
      if (!launch_btb5(st.stencil, st.nite, b->sops, b->stab + st.tab0, st.nchunks, b->active, b->stream))
        return bfail(b, CFMG_ERR_UNSUPPORTED, "blocked pass shape");
    } else if (st.tb) {
      if (!launch_btb(st.stencil, st.nite, b->sops, b->stab + st.tab0, st.nchunks, b->active, b->stream))
        return bfail(b, CFMG_ERR_UNSUPPORTED, "blocked pass shape");
    } else {
      launch_bstage(b->sops, b->stab + st.tab0, st.nchunks, b->active, b->stream);
    }
  }
  launch_bupdate(b->bi, b->l1tab, b->l1chunks, b->active, b->stream);
  return CFMG_OK;
}

int lockstep_build(cfmg_batch* b) {
  const int ninst = (int)b->inst.size();
  const cfmg_desc& d = b->d;
  b->nsc = BS_HIST + d.maxite + 2;
  BCUDA(b, cudaMalloc((void**)&b->sc, sizeof(double) * (size_t)ninst * b->nsc));
  BCUDA(b, cudaMemsetAsync(b->sc, 0, sizeof(double) * (size_t)ninst * b->nsc, b->stream));
  int D = 0;
  for (int i = 0; i < ninst; ++i) {
    cfmg_handle* h = b->inst[i];
    int rc = prepare_mixed(h);
    if (rc != CFMG_OK) return bfail(b, rc, "instance " + std::to_string(i) + ": " + h->err);
    BCUDA(b, cudaMemcpyAsync(b->sc + (size_t)i * b->nsc + BS_NWET, h->dscal + S_NWET, sizeof(double),
                             cudaMemcpyDeviceToDevice, b->stream));
    D = std::max(D, L(h));
  }
  // the cycle's steps; an instance whose blocked passes would not leave every
  // FP32 x in its own buffer after one cycle is recorded without them
  std::vector<VStep> vs;
  vs.push_back({V_ZERO, 0, 1, 0});  // level 1 (resolved below): x = 0 before the cycle
  if (d.cycle == CFMG_CYCLE_F) vsteps_f(vs, d, D);
  else vsteps_v(vs, d, D, false);
  std::vector<std::vector<std::vector<Op>>> rec(ninst);  // [inst][step] -> Ops
  std::vector<std::vector<BSmall>> smalls(vs.size());     // [step] -> small-level smoothing blocks
  // [inst][step]: the instance takes part in the step / the step is on one
  // of its coarse levels (at most its engine threshold), which run as
  // coarse runs when CFMG_BOPT_COARSE_RUNS is on
  std::vector<std::vector<char>> part(ninst), coarse(ninst);
  for (int i = 0; i < ninst; ++i) {
    cfmg_handle* h = b->inst[i];
    for (int pass = 0; pass < 2; ++pass) {
      h->record_tb = pass == 0;
      for (Level& l : h->lv) l.xswap = 0;
      rec[i].assign(vs.size(), {});
      part[i].assign(vs.size(), 0);
      coarse[i].assign(vs.size(), 0);
      for (auto& sm : smalls)
        sm.erase(std::remove_if(sm.begin(), sm.end(), [&](const BSmall& q) { return q.inst == i; }), sm.end());
      for (size_t k = 0; k < vs.size(); ++k) {
        VStep v = vs[k];
        if (L(h) < v.need) continue;
        if (k == 0) v.depth = L(h);
        if (L(h) == 1 && v.op != V_ZERO && v.op != V_COARSEST) continue;
        part[i][k] = 1;
        const Level& lv = h->lv[L(h) - v.depth];  // the step's level (the finer one of a transfer)
        coarse[i][k] = b->coarse_runs && h->engine_on && (long long)lv.len <= engine_limit(h, CFMG_MIXED);
        BSmall sm;
        if (L(h) > 1 && small_smooth(h, v, sm)) {
          sm.inst = i;
          smalls[k].push_back(sm);
          continue;
        }
        int rc = record_vstep(h, v, rec[i][k]);
        if (rc != CFMG_OK) return bfail(b, rc, "instance " + std::to_string(i) + ": " + h->err);
        for (Op& op : rec[i][k]) {
          op.inst = i;
          if (op.kind == OPK_TB) coarse[i][k] = 0;  // blocked passes keep their own kernel
        }
      }
      bool home = true;
      for (const Level& l : h->lv) home = home && l.xswap == 0;
      if (home) break;
      if (pass == 1) return bfail(b, CFMG_ERR_UNSUPPORTED, "batched cycle leaves an FP32 field swapped");
    }
    h->record_tb = false;
  }
  // launches: per step, the k-th Op of every instance; OPK_TB Ops of one
  // (stencil, pairs) go to the blocked kernel, the rest to the generic one
  std::vector<Op> all;
  std::vector<int4> tab;
  auto add_step = [&](std::vector<Op>& ops, int tb, int stencil, int nite) {
    if (ops.empty()) return;
    cfmg_batch::Step st;
    st.tb = tb; st.stencil = stencil; st.nite = nite; st.smem = 0;
    st.tab0 = (long long)tab.size();
    std::vector<long long> nc(ops.size());
    long long mx = 0;
    const int o0 = (int)all.size();
    for (size_t j = 0; j < ops.size(); ++j) {
      all.push_back(ops[j]);
      nc[j] = tb ? ops[j].n : (ops[j].n + kBStageChunk - 1) / kBStageChunk;
      mx = std::max(mx, nc[j]);
    }
    if (b->interleave) {  // chunk c of every Op, then chunk c + 1, ...
      for (long long c = 0; c < mx; ++c)
        for (size_t j = 0; j < ops.size(); ++j)
          if (c < nc[j]) tab.push_back(make_int4(o0 + (int)j, (int)c, ops[j].inst, 0));
    } else {
      for (size_t j = 0; j < ops.size(); ++j)
        for (long long c = 0; c < nc[j]; ++c) tab.push_back(make_int4(o0 + (int)j, (int)c, ops[j].inst, 0));
    }
    st.nchunks = (long long)tab.size() - st.tab0;
    b->steps.push_back(st);
  };
  std::vector<BSmall> all_small;
  // coarse runs: an instance's consecutive coarse steps collect in pend[i]
  // and all collected runs go out as one launch (one block per run) before
  // the first step that some instance with a run takes on a larger level.
  // Instances are independent, so only each instance's own order matters.
  std::vector<int2> rent;
  std::vector<int4> runs;
  std::vector<std::vector<int2>> pend(ninst);
  std::vector<int> pend_smem(ninst, 0);
  auto small_bytes = [](const BSmall& q) { return (int)(4 * q.g.len * (q.prec == 0 ? 8 : 4)); };
  auto flush_runs = [&]() {
    cfmg_batch::Step st;
    st.tb = 3; st.stencil = 0; st.nite = 0; st.smem = 0;
    st.tab0 = (long long)runs.size();
    for (int i = 0; i < ninst; ++i) {
      if (pend[i].empty()) continue;
      runs.push_back(make_int4(i, (int)rent.size(), (int)(rent.size() + pend[i].size()), 0));
      rent.insert(rent.end(), pend[i].begin(), pend[i].end());
      st.smem = std::max(st.smem, pend_smem[i]);
      pend[i].clear();
      pend_smem[i] = 0;
    }
    st.nchunks = (long long)runs.size() - st.tab0;
    if (st.nchunks > 0) b->steps.push_back(st);
  };
  for (size_t k = 0; k < vs.size(); ++k) {
    bool cut = false;
    for (int i = 0; i < ninst && !cut; ++i) cut = part[i][k] && !coarse[i][k] && !pend[i].empty();
    if (cut) flush_runs();
    std::vector<BSmall> fine_small;
    for (const BSmall& q : smalls[k]) {
      if (!coarse[q.inst][k]) {
        fine_small.push_back(q);
        continue;
      }
      pend[q.inst].push_back(make_int2(1, (int)all_small.size()));
      pend_smem[q.inst] = std::max(pend_smem[q.inst], small_bytes(q));
      all_small.push_back(q);
    }
    for (int i = 0; i < ninst; ++i) {
      if (!coarse[i][k]) continue;
      for (const Op& op : rec[i][k]) {
        pend[i].push_back(make_int2(0, (int)all.size()));
        all.push_back(op);
      }
    }
    if (!fine_small.empty()) {  // independent of the other instances' Ops of this step
      cfmg_batch::Step st;
      st.tb = 2; st.stencil = 0; st.nite = 0;
      st.tab0 = (long long)all_small.size();
      st.nchunks = (long long)fine_small.size();
      st.smem = 0;
      for (const BSmall& q : fine_small) st.smem = std::max(st.smem, small_bytes(q));
      all_small.insert(all_small.end(), fine_small.begin(), fine_small.end());
      b->steps.push_back(st);
    }
    size_t depth = 0;
    for (int i = 0; i < ninst; ++i)
      if (!coarse[i][k]) depth = std::max(depth, rec[i][k].size());
    for (size_t q = 0; q < depth; ++q) {
      std::vector<Op> gen;
      std::vector<std::vector<Op>> tbs(16);  // [lean packed form?][stencil 9?][pairs]
      for (int i = 0; i < ninst; ++i) {
        if (coarse[i][k] || q >= rec[i][k].size()) continue;
        const Op& op = rec[i][k][q];
        if (op.kind == OPK_TB) tbs[(op.form == 5 ? 8 : 0) + (op.np_j == 9 ? 4 : 0) + op.np_i].push_back(op);
        else gen.push_back(op);
      }
      for (int t = 0; t < 16; ++t) add_step(tbs[t], t >= 8 ? 4 : 1, (t & 4) ? 9 : 5, t & 3);
      add_step(gen, 0, 0, 0);
    }
  }
  flush_runs();  // the cycle's last coarse steps
  // level-1 state and chunks
  std::vector<BInst> hb(ninst);
  std::vector<long long> l1(ninst + 1, 0);
  for (int i = 0; i < ninst; ++i) {
    cfmg_handle* h = b->inst[i];
    const Level& l = h->lv[0];
    BInst& B = hb[i];
    std::memset(&B, 0, sizeof(B));
    B.x = l.x; B.b = l.b; B.r = l.r; B.d = l.diag; B.m = l.msk;
    B.b32 = l.b32; B.r32 = l.r32; B.e32 = view<float>(l).x;
    B.sc = b->sc + (size_t)i * b->nsc;
    B.g = geom(l);
    B.box = interior(l);
    B.kind = h->d.op == CFMG_LAPLACIAN9 ? OPK_RESID9 : OPK_RESID5;
    if (B.kind == OPK_RESID5) {
      B.lo = B.g.n1;
      B.n = B.g.len - 2 * B.g.n1;
    } else {
      B.n = box_count(B.box);
    }
    B.len = (long long)l.len;
    B.dq = h->dq;
    if (B.kind == OPK_RESID5) {  // linear range: rows 2..ty-1, every column
      B.row0 = B.g.n1;
      B.c0 = 0;
      B.ncols = l.tx;
      B.nrows = l.ty - 2;
    } else {
      B.row0 = (long long)(B.box.j0 - 1) * B.g.n1;
      B.c0 = B.box.i0 - 1;
      B.ncols = B.box.i1 - B.box.i0 + 1;
      B.nrows = B.box.j1 - B.box.j0 + 1;
    }
    B.nstrips = (B.ncols + kBIntCols - 1) / kBIntCols;
    B.neumann = !vertices(h);
    B.norm_kind = h->d.norm_kind;
    B.maxite = h->d.maxite;
    B.tol = h->d.tol;
    l1[i + 1] = l1[i] + (B.len + kBChunk - 1) / kBChunk;
  }
  b->l1chunks = l1[ninst];
  // integer residual tasks (single-layer levels whose instances all have it)
  b->int_all = true;
  for (int i = 0; i < ninst; ++i) {
    const cfmg_handle* h = b->inst[i];
    b->int_all = b->int_all && int_path(h) && h->lv[0].tz == 1 && hb[i].nrows > 0 && hb[i].ncols > 0;
  }
  std::vector<int4> tt;
  std::vector<long long> ts(ninst + 1, 0);
  if (b->int_all) {
    for (int i = 0; i < ninst; ++i) {
      ts[i] = (long long)tt.size();
      const int nch = (hb[i].nrows + kBIntRows - 1) / kBIntRows;
      for (int ch = 0; ch < nch; ++ch)
        for (int st = 0; st < hb[i].nstrips; ++st) tt.push_back(make_int4(i, st, ch, 0));
    }
    ts[ninst] = (long long)tt.size();
    b->ntasks = ts[ninst];
    BCUDA(b, cudaMalloc((void**)&b->ttab, sizeof(int4) * tt.size()));
    BCUDA(b, cudaMemcpy(b->ttab, tt.data(), sizeof(int4) * tt.size(), cudaMemcpyHostToDevice));
    BCUDA(b, cudaMalloc((void**)&b->tstart, sizeof(long long) * ts.size()));
    BCUDA(b, cudaMemcpy(b->tstart, ts.data(), sizeof(long long) * ts.size(), cudaMemcpyHostToDevice));
  }
  // {instance, chunk, instance, partial slot}; interleaved like the steps' tables
  std::vector<int4> l1t;
  l1t.reserve((size_t)b->l1chunks);
  if (b->interleave) {
    long long mx = 0;
    for (int i = 0; i < ninst; ++i) mx = std::max(mx, l1[i + 1] - l1[i]);
    for (long long c = 0; c < mx; ++c)
      for (int i = 0; i < ninst; ++i)
        if (c < l1[i + 1] - l1[i]) l1t.push_back(make_int4(i, (int)c, i, (int)(l1[i] + c)));
  } else {
    for (int i = 0; i < ninst; ++i)
      for (long long c = l1[i]; c < l1[i + 1]; ++c) l1t.push_back(make_int4(i, (int)(c - l1[i]), i, (int)c));
  }
  BCUDA(b, cudaMalloc((void**)&b->l1tab, sizeof(int4) * l1t.size()));
  BCUDA(b, cudaMemcpy(b->l1tab, l1t.data(), sizeof(int4) * l1t.size(), cudaMemcpyHostToDevice));
  BCUDA(b, cudaMalloc((void**)&b->bi, sizeof(BInst) * ninst));
  BCUDA(b, cudaMemcpy(b->bi, hb.data(), sizeof(BInst) * ninst, cudaMemcpyHostToDevice));
  BCUDA(b, cudaMalloc((void**)&b->l1start, sizeof(long long) * (ninst + 1)));
  BCUDA(b, cudaMemcpy(b->l1start, l1.data(), sizeof(long long) * (ninst + 1), cudaMemcpyHostToDevice));
  BCUDA(b, cudaMalloc((void**)&b->bpart, sizeof(double) * 2 * (size_t)std::max(b->l1chunks, b->ntasks)));
  BCUDA(b, cudaMalloc((void**)&b->active, sizeof(int) * ninst));
  BCUDA(b, cudaMalloc((void**)&b->nactive, sizeof(int)));
  BCUDA(b, cudaMemset(b->active, 0, sizeof(int) * ninst));
  BCUDA(b, cudaMemset(b->nactive, 0, sizeof(int)));
  if (!all_small.empty()) {
    BCUDA(b, cudaMalloc((void**)&b->ssm, sizeof(BSmall) * all_small.size()));
    BCUDA(b, cudaMemcpy(b->ssm, all_small.data(), sizeof(BSmall) * all_small.size(), cudaMemcpyHostToDevice));
  }
  if (!runs.empty()) {
    BCUDA(b, cudaMalloc((void**)&b->rent, sizeof(int2) * rent.size()));
    BCUDA(b, cudaMemcpy(b->rent, rent.data(), sizeof(int2) * rent.size(), cudaMemcpyHostToDevice));
    BCUDA(b, cudaMalloc((void**)&b->runs, sizeof(int4) * runs.size()));
    BCUDA(b, cudaMemcpy(b->runs, runs.data(), sizeof(int4) * runs.size(), cudaMemcpyHostToDevice));
  }
  if (!all.empty()) {
    BCUDA(b, cudaMalloc((void**)&b->sops, sizeof(Op) * all.size()));
    BCUDA(b, cudaMemcpy(b->sops, all.data(), sizeof(Op) * all.size(), cudaMemcpyHostToDevice));
  }
  if (!tab.empty()) {  // every step may be a coarse run (instances of a few levels)
    BCUDA(b, cudaMalloc((void**)&b->stab, sizeof(int4) * tab.size()));
    BCUDA(b, cudaMemcpy(b->stab, tab.data(), sizeof(int4) * tab.size(), cudaMemcpyHostToDevice));
  }
  b->kind = hb[0].kind;
  b->neumann = hb[0].neumann != 0;
  for (int i = 1; i < ninst; ++i)
    if (hb[i].kind != b->kind || (hb[i].neumann != 0) != b->neumann)
      return bfail(b, CFMG_ERR_ARG, "batched instances must share the operator and location");
  // the graph: init, then while (any instance iterates) { iteration }
  for (int z = 0; z < 2; ++z) {
    cudaGraph_t g = nullptr;
    BCUDA(b, cudaGraphCreate(&g, 0));
    BCUDA(b, cudaStreamBeginCaptureToGraph(b->stream, g, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
    launch_binit(b->bi, ninst, z, b->active, b->nactive, b->stream);
    cudaError_t e = cudaStreamEndCapture(b->stream, &g);
    if (e != cudaSuccess) return bfail(b, CFMG_ERR_CUDA, std::string("batch capture: ") + cudaGetErrorString(e));
    cudaGraphNode_t init = nullptr;
    size_t nn = 1;
    BCUDA(b, cudaGraphGetNodes(g, &init, &nn));
    cudaGraphConditionalHandle hc;
    BCUDA(b, cudaGraphConditionalHandleCreate(&hc, g, 1, cudaGraphCondAssignDefault));
    cudaGraphNodeParams cp = {};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = hc;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t cnode;
    BCUDA(b, cudaGraphAddNode(&cnode, g, &init, nullptr, 1, &cp));
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    BCUDA(b, cudaStreamBeginCaptureToGraph(b->stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
    const int rb = lockstep_body(b);
    if (rb != CFMG_OK) {
      cudaStreamEndCapture(b->stream, &body);
      cudaGraphDestroy(g);
      return rb;
    }
    launch_bcond(hc, b->nactive, b->stream);
    e = cudaStreamEndCapture(b->stream, &body);
    if (e != cudaSuccess) return bfail(b, CFMG_ERR_CUDA, std::string("batch capture: ") + cudaGetErrorString(e));
    e = cudaGraphInstantiate(&b->graph[z], g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return bfail(b, CFMG_ERR_CUDA, std::string("batch instantiate: ") + cudaGetErrorString(e));
  }
  b->hsc.resize((size_t)ninst * b->nsc);
  b->built = true;
  return CFMG_OK;
}

}  // namespace

extern "C" {

int cfmg_batch_create(const cfmg_desc* d, int ninst, const int* nx, const int* ny, const int* nlevels,
                      cfmg_batch** out) {
  if (!out || !d || !nx || !ny || ninst < 1) return fail(nullptr, CFMG_ERR_ARG, "batch: bad arguments");
  *out = nullptr;
  if (d->precision != CFMG_MIXED) return fail(nullptr, CFMG_ERR_UNSUPPORTED, "batched solves use the mixed form");
  if (d->topology != CFMG_CLOSED || d->kase != CFMG_TWOD)
    return fail(nullptr, CFMG_ERR_UNSUPPORTED, "batched solves are 2D closed-topology");
  cfmg_batch* b = new cfmg_batch();
  b->d = *d;
  if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete b;
    return fail(nullptr, CFMG_ERR_CUDA, "batch stream creation failed");
  }
  for (int i = 0; i < ninst; ++i) {
    cfmg_desc di = *d;
    di.nx = nx[i];
    di.ny = ny[i];
    if (nlevels) di.nlevels = nlevels[i];
    cfmg_handle* h = nullptr;
    int rc = create_handle(&di, b->stream, &h);
    if (rc != CFMG_OK) {
      cfmg_batch_destroy(b);
      return fail(nullptr, rc, "batch instance " + std::to_string(i) + ": " + cfmg_last_error(nullptr));
    }
    b->inst.push_back(h);
  }
  b->lockstep = fused_ok(b->inst[0]);
  for (cfmg_handle* h : b->inst) h->tb_on = b->lockstep;  // the engine form runs no blocked passes
  *out = b;
  return CFMG_OK;
}

int cfmg_batch_destroy(cfmg_batch* b) {
  if (!b) return CFMG_OK;
  if (b->stream) cudaStreamSynchronize(b->stream);
  for (cudaGraphExec_t g : b->graph)
    if (g) cudaGraphExecDestroy(g);
  for (cfmg_handle* h : b->inst) cfmg_destroy(h);
  for (void* p : {(void*)b->progs, (void*)b->ptrs, (void*)b->nops, (void*)b->counter, (void*)b->red, (void*)b->sc,
                  (void*)b->nwet, (void*)b->bi, (void*)b->l1start, (void*)b->l1tab, (void*)b->bpart,
                  (void*)b->active, (void*)b->nactive, (void*)b->sops, (void*)b->stab, (void*)b->ssm,
                  (void*)b->ttab, (void*)b->tstart, (void*)b->rent, (void*)b->runs})
    if (p) cudaFree(p);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
  return CFMG_OK;
}

int cfmg_batch_instance(cfmg_batch* b, int i, cfmg_handle** h) {
  if (!b || !h || i < 0 || i >= (int)b->inst.size()) return CFMG_ERR_ARG;
  *h = b->inst[i];
  return CFMG_OK;
}

const char* cfmg_batch_last_error(const cfmg_batch* b) { return b ? b->err.c_str() : ""; }

int cfmg_batch_set_option(cfmg_batch* b, int option, long long value) {
  if (!b) return CFMG_ERR_ARG;
  if (option == CFMG_BOPT_HOST_LOOP) {
    b->host_loop = value != 0;
    return CFMG_OK;
  }
  if (option == CFMG_BOPT_COARSE_RUNS) {
    if (b->coarse_runs != (value != 0)) b->built = false;  // the iteration's launches change
    b->coarse_runs = value != 0;
    return CFMG_OK;
  }
  if (option == CFMG_BOPT_INTERLEAVE) {
    if (b->interleave != (value != 0)) b->built = false;  // the work tables change
    b->interleave = value != 0;
    return CFMG_OK;
  }
  return bfail(b, CFMG_ERR_ARG, "unknown batch option");
}

int cfmg_batch_solve(cfmg_batch* b, int zero_x, double* res, int* nite, double* t_done_ms) {
  if (!b) return CFMG_ERR_ARG;
  for (size_t i = 0; i < b->inst.size(); ++i)
    if (!b->inst[i]->coef_set)
      return bfail(b, CFMG_ERR_STATE, "instance " + std::to_string(i) + ": operators not set up (run "
                                      "cfmg_setup_operators or cfmg_bind_level on it first)");
  for (cfmg_handle* h : b->inst)
    if (h->mixed_dirty) b->built = false;  // coefficients changed since the programs were made
  if (!b->built) {
    for (cudaGraphExec_t& g : b->graph)
      if (g) {
        cudaGraphExecDestroy(g);
        g = nullptr;
      }
    for (void** p : {(void**)&b->progs, (void**)&b->ptrs, (void**)&b->nops, (void**)&b->counter, (void**)&b->red,
                     (void**)&b->sc, (void**)&b->nwet, (void**)&b->bi, (void**)&b->l1start, (void**)&b->l1tab,
                     (void**)&b->bpart, (void**)&b->active, (void**)&b->nactive, (void**)&b->sops,
                     (void**)&b->stab, (void**)&b->ssm, (void**)&b->ttab, (void**)&b->tstart, (void**)&b->rent,
                     (void**)&b->runs})
      if (*p) {
        cudaFree(*p);
        *p = nullptr;
      }
    b->steps.clear();
    TRY(b->lockstep ? lockstep_build(b) : batch_build(b));
  }
  const int ninst = (int)b->inst.size();
  if (b->lockstep && b->host_loop) {
    launch_binit(b->bi, ninst, zero_x ? 1 : 0, b->active, b->nactive, b->stream);
    for (;;) {
      TRY(lockstep_body(b));
      int na = 0;
      BCUDA(b, cudaMemcpyAsync(&na, b->nactive, sizeof(int), cudaMemcpyDeviceToHost, b->stream));
      BCUDA(b, cudaMemsetAsync(b->nactive, 0, sizeof(int), b->stream));
      BCUDA(b, cudaStreamSynchronize(b->stream));
      if (na == 0) break;
    }
  } else {
    BCUDA(b, cudaGraphLaunch(b->graph[zero_x ? 1 : 0], b->stream));
  }
  BCUDA(b, cudaMemcpyAsync(b->hsc.data(), b->sc, sizeof(double) * b->hsc.size(), cudaMemcpyDeviceToHost, b->stream));
  BCUDA(b, cudaStreamSynchronize(b->stream));
  const int kt0 = b->lockstep ? (int)BS_T0 : (int)SS_T0, kt1 = b->lockstep ? (int)BS_T1 : (int)SS_T1;
  const int kres = b->lockstep ? (int)BS_RES : (int)SS_RES, knite = b->lockstep ? (int)BS_NITE : (int)SS_NITE;
  double t0 = 1e300;
  for (int i = 0; i < ninst; ++i) t0 = std::min(t0, b->hsc[(size_t)i * b->nsc + kt0]);
  int bad = -1;
  for (int i = 0; i < ninst; ++i) {
    const double* c = &b->hsc[(size_t)i * b->nsc];
    if (res) res[i] = c[kres];
    if (nite) nite[i] = (int)c[knite];
    if (t_done_ms) t_done_ms[i] = (c[kt1] - t0) * 1e-6;
    if (bad < 0 && !std::isfinite(c[kres])) bad = i;
  }
  for (cfmg_handle* h : b->inst) h->solved = true;
  if (bad >= 0)
    return bfail(b, CFMG_ERR_NONFINITE, "instance " + std::to_string(bad) +
                                            ": non-finite residual norm (NaN or Inf in b, x or the coefficients)");
  return CFMG_OK;
}

int cfmg_launch_count(const cfmg_handle* h, long long* n) {
  if (!h || !n) return CFMG_ERR_ARG;
  *n = h->launches;
  return CFMG_OK;
}

int cfmg_set_option(cfmg_handle* h, int option, long long value) {
  if (!h) return CFMG_ERR_ARG;
  TRY(sync(h));
  if (option == CFMG_OPT_COARSEST_FP64) {
    if (value < -1 || value > 1) return fail(h, CFMG_ERR_ARG, "coarsest_fp64 must be -1, 0 or 1");
    h->coarsest_fp64 = (int)value;
    drop_graphs(h);
    return CFMG_OK;
  }
  if (option == CFMG_OPT_TEMPORAL_BLOCKING) {
    if (value < 0 || value > 5 || value == 2)
      return fail(h, CFMG_ERR_ARG, "temporal_blocking must be 0, 1, 3, 4 or 5");
    h->tb_on = value != 0;
    if (value) h->tb_version = (int)value;
    drop_graphs(h);
    return CFMG_OK;
  }
  if (option == CFMG_OPT_INT_RESIDUAL) {
    h->int_on = value != 0;
    drop_graphs(h);
    return CFMG_OK;
  }
  if (option == CFMG_OPT_HOST_LOOP) {
    h->host_loop = value != 0;
    return CFMG_OK;
  }
  if (option == CFMG_OPT_FUSED_DESCENT) {
    h->fuse_on = value != 0;
    drop_graphs(h);
    return CFMG_OK;
  }
  if (option == CFMG_OPT_FUSED_UPDATE) {
    h->upd_on = value != 0;
    drop_graphs(h);
    return CFMG_OK;
  }
  if (option == CFMG_OPT_SMALL_SMOOTH) {
    if (value < 0) return fail(h, CFMG_ERR_ARG, "small_smooth must be >= 0");
    h->small_min = (int)value;
    drop_graphs(h);
    return CFMG_OK;
  }
  if (option == CFMG_OPT_SKIP_DRY) {
    h->dry_on = value != 0;
    drop_graphs(h);
    return CFMG_OK;
  }
  if (option == CFMG_OPT_STAGED_RESIDUAL) {
    h->r3_on = value != 0;
    h->r3_rows = value == 1 ? 1 : 2;
    drop_graphs(h);
    return CFMG_OK;
  }
  if (option == CFMG_OPT_CODED_WIDIAG) {
    h->wq_on = value != 0;
    drop_graphs(h);
    return CFMG_OK;
  }
  if (option == CFMG_OPT_DEPENDENT_LAUNCH) {
    h->dep_launch = value != 0;
    drop_graphs(h);  // captured graphs embed the launch attributes
    return CFMG_OK;
  }
  if (option == CFMG_OPT_ENGINE_CELLS) {
    if (value < 0) return fail(h, CFMG_ERR_ARG, "engine_cells must be >= 0");
    h->engine_cells = value;
    h->engine_on = value > 0;
    drop_graphs(h);  // captured graphs embed the old split
    return CFMG_OK;
  }
  return fail(h, CFMG_ERR_ARG, "unknown option");
}

int cfmg_profile(cfmg_handle* h, int cls, int lev, int precision) {
  if (!h) return CFMG_ERR_ARG;
  TRY(sync(h));
  h->prof_cls = cls;
  h->prof_lev = lev;
  h->prof_prec = precision;
  h->prof_launches = 0;
  h->prof_ms = 0.0;
  return CFMG_OK;
}

int cfmg_profile_read(cfmg_handle* h, long long* launches, double* total_ms) {
  if (!h || !launches || !total_ms) return CFMG_ERR_ARG;
  TRY(sync(h));
  *launches = h->prof_launches;
  *total_ms = h->prof_ms;
  return CFMG_OK;
}

}  // extern "C"
