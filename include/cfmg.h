/*
 * libcfmg: GB300-native (sm_103a) geometric multigrid for CFMultigrid.jl.
 *
 * A C ABI: plain pointers, sizes and ints, no CUDA or torch types. Every
 * function returns an int status (CFMG_OK = 0); cfmg_last_error() gives
 * the message of the last failure. A handle is not thread-safe; calls on
 * one handle are issued in order on the handle's CUDA stream. Distinct
 * handles are independent.
 *
 * The reference (ClimFlows/CFMultigrid.jl) is pure Julia. Its hot path is
 * called through four per-level function tables
 *   mg.smoother[lev](mg, lev, nite), mg.residual[lev](mg, lev),
 *   mg.restriction[lev](mg, lev, field), mg.prolongation[lev](mg, lev)
 * (src/gmg_types.jl:128-131, bound in src/gmg_setup.jl:86-101), plus
 * solve!, norm, set_to_zero! and fill!. Each entry point below names the
 * Julia function it replaces; a Julia host binds them with ccall, one
 * closure per table entry, and a solve! method that calls cfmg_solve.
 *
 * Arrays crossing the ABI use the reference layout: one column-major
 * (i fastest) array of tx*ty*tz entries per level and field, with
 * tx = nx+2nh, ty = ny+2nh, tz = nz (2D) or nz+2nh (3D)
 * (src/gmg_types.jl:68-118). FP64 fields are double, the mask is uint8_t.
 * Pointers passed to upload/download/bind may be host or device memory.
 */
#ifndef CFMG_H
#define CFMG_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define CFMG_API __attribute__((visibility("default")))
#else
#define CFMG_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define CFMG_OK 0
#define CFMG_ERR_ARG 1         /* invalid argument (the reference's AssertionError) */
#define CFMG_ERR_CUDA 2        /* a CUDA call failed */
#define CFMG_ERR_ALLOC 3       /* device or pinned allocation failed */
#define CFMG_ERR_STATE 4       /* call out of order (e.g. solve before setup) */
#define CFMG_ERR_NONFINITE 5   /* NaN/Inf met in a residual norm */
#define CFMG_ERR_UNSUPPORTED 6 /* combination not implemented */

/* Param symbols (src/gmg_types.jl:41-59) */
#define CFMG_TWOD 0
#define CFMG_THREED 1
#define CFMG_CENTERS 0
#define CFMG_VERTICES 1
#define CFMG_LAPLACIAN 0  /* 5-point (2D) / 7-point (3D) */
#define CFMG_LAPLACIAN9 1 /* 19-point (3D, src/laplacian9.jl) / in-plane 9-point (2D) */
#define CFMG_VARCOEF 2    /* 2D cell-centred div(kappa grad x), face kappa = mean of the two cells */
#define CFMG_CLOSED 0
#define CFMG_XPERIO 1
/* cycles of solve!'s table (src/gmg_solver.jl:11-16) */
#define CFMG_CYCLE_V 0
#define CFMG_CYCLE_F 1
#define CFMG_CYCLE_ONELEV 2
#define CFMG_CYCLE_TWOLEV 3
#define CFMG_CYCLE_NLEV 4
#define CFMG_CYCLE_VREC 5
/* arithmetic of solve */
#define CFMG_FP64 0  /* plain FP64 drop-in, bit-identical pointwise to the reference */
#define CFMG_MIXED 1 /* FP32 cycles inside FP64 defect correction */
/* stopping rule */
#define CFMG_NORM_REF_SQUARED 0 /* the reference's sum(msk r^2)/sum(msk b^2) <= tol */
#define CFMG_NORM_L2 1          /* ||r||_2/||b||_2 <= tol */

/* field ids (src/gmg_types.jl:86-118) */
#define CFMG_X 0
#define CFMG_R 1
#define CFMG_B 2
#define CFMG_Y 3
#define CFMG_DIAG 4
#define CFMG_IDIAG 5
#define CFMG_RCOEF 6
#define CFMG_PCOEF 7
#define CFMG_KAPPA 8
#define CFMG_MSK 9

/* kernel classes for cfmg_profile */
#define CFMG_K_SWEEP 0    /* one Jacobi sweep (or a fused block of sweeps) */
#define CFMG_K_RESIDUAL 1
#define CFMG_K_RESTRICT 2
#define CFMG_K_PROLONG 3
#define CFMG_K_NORM 4
#define CFMG_K_FILL 5
#define CFMG_K_CONVERT 6  /* FP64 <-> FP32 transfers of the mixed form */
#define CFMG_K_ENGINE 7   /* one launch of the coarse-level program engine */
#define CFMG_K_DESCENT 8  /* a smoothing pass that also forms and restricts the residual (fused descent step) */

/* options for cfmg_set_option */
#define CFMG_OPT_ENGINE_CELLS 0 /* FP32 levels of at most this many cells (tx*ty*tz), FP64
                                   levels of at most 1/16 of it, run in the coarse-level
                                   engine; 0 turns the engine off (default 20000) */
#define CFMG_OPT_COARSEST_FP64 2 /* mixed form, coarsest-level smoothing in FP64: -1 (default) when the
                                    coarsest level holds at most 1/16 of CFMG_OPT_ENGINE_CELLS cells,
                                    0 never (FP32), 1 always */
#define CFMG_OPT_TEMPORAL_BLOCKING 1 /* FP32 smoothing of fine 2D levels runs all sweeps of a call in
                                        shared-memory passes: 5 (default) two columns per thread in packed
                                        FP32x2 arithmetic with padded tiles and vector loads, 3 the first
                                        packed form, 1 one column per thread; 4 as 3, plus streaming passes
                                        for 3D 7-point levels and the 3D 19-point pair in one pass; 0: one
                                        kernel per sweep. All give the same bits. */
#define CFMG_OPT_INT_RESIDUAL 3 /* mixed form, closed topology, 5-, 7- and 2D 9-point operators: 1
                                   (default) computes the level-1 residual exactly in 64-bit fixed point
                                   on the integer pipes; 0 in FP64 arithmetic */
#define CFMG_OPT_HOST_LOOP 4 /* cfmg_solve: 0 (default) runs the whole loop as one graph launch (a
                                `while` node); 1 launches one graph per iteration from the host, which
                                profilers that do not descend into conditional nodes can see */
#define CFMG_OPT_FUSED_DESCENT 5 /* mixed form, 2D closed topology, lean packed passes: 1 (default)
                                    the last pre-smoothing pass of a cycle's descent step also forms
                                    the residual, restricts it to the coarse b and zeroes the coarse x;
                                    0 separate kernels. Both give the same bits. */
#define CFMG_OPT_FUSED_UPDATE 6 /* mixed form, 2D closed topology, integer residual, lean packed passes:
                                   1 (default) the cycle's last level-1 post-smoothing pass also applies
                                   the FP64 solution update x += e * iscale (and collects max |x|)
                                   instead of storing the FP32 correction; 0 a separate kernel. Both give
                                   the same bits. */
#define CFMG_OPT_DEPENDENT_LAUNCH 7 /* 1 (default): the kernels of a cycle are launched as programmatic
                                       dependents of the kernel before them, so that a launch overlaps the
                                       completion of the previous kernel (each kernel waits for its
                                       predecessor's results before it reads or writes); 0 plain stream
                                       order. Both give the same bits. */
#define CFMG_OPT_CODED_WIDIAG 8 /* mixed form, 3D 7-point operator: 1 (default) the standalone FP32 sweeps
                                   read omega*idiag as a one-byte code diag into a 256-entry table (when
                                   every cell's code reproduces its float exactly) instead of a 4-byte
                                   float per cell; 0 the floats. Both give the same bits. */
#define CFMG_OPT_SMALL_SMOOTH 11 /* closed topology, 5-, 2D 9- and 3D 7-point operators: a smoothing
                                     call of at least this many pairs (default 4: the coarsest solve) on
                                     a level whose x, y, b and omega*idiag fit 200 KB runs as one block in
                                     shared memory; 0 never (separate sweeps). The same bits. */
#define CFMG_OPT_SKIP_DRY 10 /* mixed form, closed topology: 1 (default) passes skip groups of cells
                               that are all dry (their FP32 fields hold +0 and stay +0): the FP32
                               prolongation's parents, the strip residual's tasks; for the 3D 7-point
                               operator also the four-cell sweeps' quads, the staged residual's tile
                               runs, the residual-restriction's coarse cells, the level-1 solution
                               update (the dry cells' max |x| taken once per solve) and the wet-mean
                               shift; 0 every cell. Both give the same values (a zero in a dry cell can
                               keep its sign where the full pass would flip it). */
#define CFMG_OPT_STAGED_RESIDUAL 9 /* mixed form, 3D 7-point operator, integer residual: 2 (default) the
                                      level-1 residual pass stages each plane of a 32 x 16 column tile in
                                      shared memory by TMA and converts every x once (even tx only), two
                                      tile rows a thread; 1 the same with 32 x 8 tiles, one row a thread;
                                      0 the row-strip pass. The same residual and right-hand side; the
                                      norm's partial sums are added in another order. */

typedef struct cfmg_desc {
  int kase;     /* CFMG_TWOD / CFMG_THREED            (Param.case) */
  int location; /* CFMG_CENTERS / CFMG_VERTICES       (Param.location) */
  int op;       /* CFMG_LAPLACIAN / _LAPLACIAN9 / _VARCOEF (Param.operator) */
  int topology; /* CFMG_CLOSED / CFMG_XPERIO          (Param.topology) */
  int cycle;    /* CFMG_CYCLE_*                       (Param.cycle) */
  int nx, ny, nz, nh;
  int nlevels;  /* 0: the reference's hierarchy (src/gmg_setup.jl:40-64); else a cap */
  int npre, npost, ndeepest, maxite;
  double omega, tol;
  int precision; /* CFMG_FP64 / CFMG_MIXED */
  int norm_kind; /* CFMG_NORM_REF_SQUARED / CFMG_NORM_L2 */
} cfmg_desc;

typedef struct cfmg_handle cfmg_handle;

/* Fill `d` with the defaults of Param() (src/gmg_types.jl:41-59). */
CFMG_API int cfmg_desc_default(cfmg_desc* d);

/* get_gmg's allocation part (src/gmg_setup.jl:26-35, create_levels :40-64,
 * allocate_mg :77-104): builds the level hierarchy and allocates every
 * level's fields on the current CUDA device, all zero. The default mask and
 * operator setup are separate calls (cfmg_set_default_msk,
 * cfmg_setup_operators) or come from the caller (cfmg_bind_level). */
CFMG_API int cfmg_create(const cfmg_desc* d, cfmg_handle** out);
CFMG_API int cfmg_destroy(cfmg_handle* h);
/* Message of the last failure on `h` (or of the last failed cfmg_create when h is NULL). */
CFMG_API const char* cfmg_last_error(const cfmg_handle* h);

CFMG_API int cfmg_nlevels(const cfmg_handle* h, int* n);
/* dims = {nx, ny, nz, nh, tx, ty, tz} of level lev (1-based). */
CFMG_API int cfmg_level_dims(const cfmg_handle* h, int lev, int* dims);
/* Issue all work of `h` on `stream` (a cudaStream_t, NULL = the handle's own stream). */
CFMG_API int cfmg_set_stream(cfmg_handle* h, void* stream);
CFMG_API int cfmg_synchronize(cfmg_handle* h);

/* Copy a whole field of one level in or out (replaces reading/writing
 * mg.data[lev].x/b/... and mg.oper[lev].* in Julia). */
CFMG_API int cfmg_upload(cfmg_handle* h, int lev, int field, const void* src);
CFMG_API int cfmg_download(cfmg_handle* h, int lev, int field, void* dst);
/* Device address of a field (for zero-copy interop). */
CFMG_API int cfmg_field_ptr(cfmg_handle* h, int lev, int field, void** dptr);

/* Bind operator coefficients computed by the caller's own setup
 * (setup_operators!, src/gmg_setup.jl:264-287). Any pointer may be NULL to
 * keep the current array. */
CFMG_API int cfmg_bind_level(cfmg_handle* h, int lev, const double* diag, const double* idiag, const double* Rcoef,
                    const double* Pcoef, const uint8_t* msk);
/* set_default_msk! (src/gmg_setup.jl:106-122) on the device. */
CFMG_API int cfmg_set_default_msk(cfmg_handle* h);
/* setup_operators! (src/gmg_setup.jl:264-287) on the device: coarse masks
 * (compute_msk_dev), Rcoef, Pcoef, diag/idiag, from the level-1 mask. */
CFMG_API int cfmg_setup_operators(cfmg_handle* h);

/* Per-level operators: the function tables' entries. */
CFMG_API int cfmg_smooth(cfmg_handle* h, int lev, int nite);        /* mg.smoother[lev]    (src/laplacian.jl:24-41,95-112; src/laplacian9.jl:2-47) */
CFMG_API int cfmg_residual(cfmg_handle* h, int lev);                /* mg.residual[lev]    (src/laplacian.jl:53-64,114-128; src/laplacian9.jl:49-73) */
CFMG_API int cfmg_restrict(cfmg_handle* h, int lev, int field);     /* mg.restriction[lev] (src/RP_on_centers.jl:73-82,135-144; src/RP_on_vertices.jl:1-32,140-150) */
CFMG_API int cfmg_prolong(cfmg_handle* h, int lev);                 /* mg.prolongation[lev](src/RP_on_centers.jl:106-114,165-175; src/RP_on_vertices.jl:34-72,152-162) */
CFMG_API int cfmg_zero(cfmg_handle* h, int lev, int field);         /* set_to_zero!        (src/operators_at_level.jl:7-10) */
CFMG_API int cfmg_fill(cfmg_handle* h, int lev, int field);         /* fill!               (src/halo.jl:1-15) */
CFMG_API int cfmg_norm(cfmg_handle* h, int lev, int field, double* out); /* norm       (src/operators_at_level.jl:12-27) */
CFMG_API int cfmg_normresidual(cfmg_handle* h, double normb, double* out); /* normresidual! (src/operators_at_level.jl:29-36) */

/* One cycle of solve!'s table (src/gmg_cycles.jl): kind = CFMG_CYCLE_*. */
CFMG_API int cfmg_cycle(cfmg_handle* h, int kind);

/* solve!(mg) (src/gmg_solver.jl:9-42) on the fields already on the device
 * (b and the x warm start of level 1), with desc.tol, desc.maxite,
 * desc.norm_kind and desc.precision. `history` (may be NULL) receives
 * nite+1 entries (room for maxite+1): the residual after 0..nite cycles.
 * The loop, its stopping test and the history run on the device in one
 * graph launch (CFMG_OPT_HOST_LOOP = 1: one launch per iteration). */
CFMG_API int cfmg_solve(cfmg_handle* h, double* res, int* nite, double* history);
/* solve! with the stopping rule given per call, as a caller that keeps
 * Param.tol / Param.maxite on its side binds it: tol, maxite and norm_kind
 * replace the descriptor's (the captured graphs are rebuilt when they
 * change), then as cfmg_solve. Returns (res, nite) like solve!
 * (src/gmg_solver.jl:9-42); exhausting maxite is not an error. Errors:
 * CFMG_ERR_STATE before setup, CFMG_ERR_NONFINITE when b or the residual
 * norm is NaN/Inf (res and nite are still written). */
CFMG_API int cfmg_solve_tol(cfmg_handle* h, double tol, int maxite, int norm_kind, double* res, int* nite,
                            double* history);

/* Adjoint solve: the backward pass of solve! (no counterpart in the
 * reference; a Julia host exposes it as the pullback of a ChainRulesCore
 * rrule for solve!). After a forward cfmg_solve, with the cotangent
 * g = dL/dx of level 1 (reference layout, host or device pointer), solves
 * A lam = g with the same cycle, arithmetic and stopping rule (A is
 * symmetric) and writes dL/db = lam to grad_b and, for CFMG_VARCOEF,
 * dL/dkappa to grad_kappa (may be NULL): the sum over the cell's faces to
 * wet neighbours of (lam_k - lam_nb)(x_k - x_nb)/2. For the cell-centred
 * (Neumann) operator g and lam are projected to zero wet mean. The forward
 * x and b are restored. res/nite report the adjoint solve. The first call
 * allocates three level-1 FP64 scratch arrays. */
CFMG_API int cfmg_adjoint(cfmg_handle* h, const double* g, double* grad_b, double* grad_kappa, double* res,
                          int* nite);
/* The same backward pass without the adjoint solve's (res, nite): the
 * pullback's signature, cot = dL/dx in, dL/db and dL/dkappa out. */
CFMG_API int cfmg_adjoint_solve(cfmg_handle* h, const double* cot, double* grad_b, double* grad_kappa);

/* Batched solves (no counterpart in the reference, which solves one
 * problem at a time). ninst independent 2D closed-topology problems share
 * `d` (precision must be CFMG_MIXED) except for their sizes nx[i] x ny[i]
 * and level counts nlevels[i] (NULL: d->nlevels). Each instance is a full
 * handle (cfmg_batch_instance): upload its mask, run cfmg_setup_operators,
 * upload b, and read x back through the usual entry points.
 * cfmg_batch_solve runs every instance's whole mixed-precision solve in one
 * graph launch, from x = 0 when zero_x is non-zero and else from each
 * instance's current x (as solve! does). For the 5- and 9-point operators
 * the instances advance in lockstep: each kernel of an iteration covers all
 * instances that have not yet converged, and a graph `while` node repeats
 * the iteration until none is left (the variable-coefficient operator runs
 * each instance's whole solve as a program of the cluster engine instead).
 * Each instance stops at its own tolerance. res, nite and t_done_ms (time
 * from the batch start to that instance's convergence) receive ninst
 * entries each; any may be NULL.
 * cfmg_batch_set_option(b, CFMG_BOPT_HOST_LOOP, 1): the host repeats the
 * lockstep iteration instead of the `while` node (the same kernels; for
 * profilers that do not descend into conditional graph nodes). */
#define CFMG_BOPT_HOST_LOOP 0
/* cfmg_batch_set_option(b, CFMG_BOPT_COARSE_RUNS, 0/1): with 1 (default) the
 * steps of an iteration on an instance's coarse levels (those its engine
 * threshold, CFMG_OPT_ENGINE_CELLS, would put in the program engine) run as
 * one block per instance, a run of consecutive steps per launch, instead of
 * one launch per step; 0 launches every step for all instances. Same
 * values either way. */
#define CFMG_BOPT_COARSE_RUNS 1
/* cfmg_batch_set_option(b, CFMG_BOPT_INTERLEAVE, 0/1): with 1 (default) the
 * work tables of the lockstep launches list chunk (or tile) c of every
 * instance before chunk c + 1 of any, so that the chunks of one instance
 * fall to different blocks and the few instances still iterating late in a
 * batch are spread over the whole GPU; 0 lists each instance's chunks
 * together. Same values either way. */
#define CFMG_BOPT_INTERLEAVE 2
typedef struct cfmg_batch cfmg_batch;
CFMG_API int cfmg_batch_create(const cfmg_desc* d, int ninst, const int* nx, const int* ny, const int* nlevels,
                               cfmg_batch** out);
CFMG_API int cfmg_batch_destroy(cfmg_batch* b);
CFMG_API int cfmg_batch_instance(cfmg_batch* b, int i, cfmg_handle** h);
CFMG_API int cfmg_batch_solve(cfmg_batch* b, int zero_x, double* res, int* nite, double* t_done_ms);
CFMG_API const char* cfmg_batch_last_error(const cfmg_batch* b);
CFMG_API int cfmg_batch_set_option(cfmg_batch* b, int option, long long value);

/* Instrumentation (no counterpart in the reference, which has none).
 * cfmg_launch_count: kernels this handle has launched so far; a replay of a
 * captured solve iteration counts every kernel node in it.
 * cfmg_profile: from now on, bracket every launch of kernel class `cls`
 * (CFMG_K_*) on level `lev` in arithmetic `precision` with CUDA events on
 * the handle's stream (cls < 0 turns it off). While it is on, cfmg_solve
 * launches eagerly instead of replaying its graph. cfmg_profile_read
 * returns the number of bracketed launches and their summed device time. */
CFMG_API int cfmg_launch_count(const cfmg_handle* h, long long* n);
/* Tuning knobs (CFMG_OPT_*); no counterpart in the reference. */
CFMG_API int cfmg_set_option(cfmg_handle* h, int option, long long value);
CFMG_API int cfmg_profile(cfmg_handle* h, int cls, int lev, int precision);
CFMG_API int cfmg_profile_read(cfmg_handle* h, long long* launches, double* total_ms);

/* Masked norm without allocation. No counterpart in the reference.
 * For callers that cannot allocate device memory where they need the
 * reduction: an application whose device pool belongs to another allocator
 * (a Julia CuArray or PyTorch caching pool), or a deployment with a fixed
 * device-memory budget. Computes sum(msk[i]*x[i]^2) over n elements of
 * caller-owned device arrays (0 -> 1, as the reference's norm,
 * src/operators_at_level.jl:12-27) into out[0], a device or mapped host
 * address, asynchronously on `stream` (a cudaStream_t; NULL = legacy).
 * Its scratch is a static device array of 4096 doubles (32 KB) held on every
 * GPU that loads the library; n is limited to CFMG_NOALLOC_MAX_ELEMS and
 * larger n is rejected with CFMG_ERR_ARG. The first call on a device looks
 * up that array's device address; make it before any stream capture. The
 * address is kept per device and CUDA context: a device reset drops it, and
 * the next call looks it up again (so it, too, belongs before a capture).
 * Calls that overlap on the GPU race on the shared scratch. No cudaMalloc,
 * cudaFree or allocating library routine is called. Errors:
 * cfmg_last_error(NULL). */
#define CFMG_NOALLOC_MAX_ELEMS 268435456LL
CFMG_API int cfmg_norm_noalloc(const double* x, const uint8_t* msk, long long n, double* out, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* CFMG_H */
