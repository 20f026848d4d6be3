/*
 * CPU oracle for CFMultigrid.jl's geometric-multigrid path.
 *
 * TEST INFRASTRUCTURE ONLY. This library is the CPU restatement that the
 * CUDA product path (libcfmg) is compared against. Only the test suite, the
 * smoke check and the CPU-baseline leg of the benchmark load it. No
 * product code path calls it.
 *
 * It restates the Julia reference (ClimFlows/CFMultigrid.jl, src/) in
 * plain C++17, single-threaded, FP64, compiled with -ffp-contract=off so
 * that every sum and product is rounded exactly where the Julia source
 * rounds it. The mapping to the reference is given per function in
 * cfmg_oracle.cpp (file:line of the Julia source).
 *
 * Parity pins: the reference's own known-answer tests
 * (test/tests.jl, test/test_RP.jl, test/test_3d.jl, test/test_topology.jl)
 * are replayed against this oracle by tests/test_oracle_pins.py.
 */
#ifndef CFMG_ORACLE_H
#define CFMG_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Mirrors the fields of `Param` (src/gmg_types.jl:41-59) plus the level cap
 * `nlevels` (0 = the reference's natural hierarchy, src/gmg_setup.jl:40-64). */
typedef struct {
  int nx, ny, nz, nh;
  int npre, npost, ndeepest, maxite;
  double tol, omega;
  int location;  /* 0 = :centers, 1 = :vertices */
  int kase;      /* 0 = :twod, 1 = :threed */
  int op;        /* 0 = :laplacian, 1 = :laplacian9, 2 = variable-coefficient 5-point */
  int cycle;     /* 0 = :v, 1 = :f, 2 = :onelev, 3 = :twolev, 4 = :nlev, 5 = :vrec */
  int topology;  /* 0 = :closed, 1 = :xperio */
  int nlevels;   /* 0 = natural hierarchy, else a cap on the number of levels */
} orc_param;

typedef struct orc_gmg orc_gmg;

/* get_gmg(param) (src/gmg_setup.jl:26-35). Returns NULL on an invalid parameter set. */
orc_gmg* orc_get_gmg(const orc_param* p);
/* Same hierarchy and allocation, but without the default mask / setup / zeroing. */
orc_gmg* orc_allocate(const orc_param* p);
void orc_free(orc_gmg* g);

int orc_nlevels(const orc_gmg* g);
/* dims = {nx, ny, nz, nh, tx, ty, tz} of level `lev` (1-based). */
void orc_level_dims(const orc_gmg* g, int lev, int* dims);
/* Field pointers: 0=x 1=r 2=b 3=y 4=diag 5=idiag 6=Rcoef 7=Pcoef 8=kappa(cell coef). */
double* orc_field(orc_gmg* g, int lev, int field);
uint8_t* orc_msk(orc_gmg* g, int lev);

void orc_set_default_msk(orc_gmg* g);
void orc_setup_operators(orc_gmg* g);

void orc_smooth(orc_gmg* g, int lev, int nite);
void orc_residual(orc_gmg* g, int lev);
void orc_restrict(orc_gmg* g, int lev, int field);
void orc_prolong(orc_gmg* g, int lev);
void orc_zero(orc_gmg* g, int lev, int field);
void orc_fill(orc_gmg* g, int lev, int field);  /* field 9 = msk */
double orc_norm(orc_gmg* g, int lev, int field);
double orc_normresidual(orc_gmg* g, double normb);

void orc_cycle(orc_gmg* g, int kind);
/* solve!(mg) (src/gmg_solver.jl:9-42). history[0..nite] receives the
 * residual after 0..nite cycles when non-NULL (length maxite+1). */
void orc_solve(orc_gmg* g, double* res, int* nite, double* history);

#ifdef __cplusplus
}
#endif
#endif
