// CPU oracle for CFMultigrid.jl's geometric-multigrid path.
//
// TEST INFRASTRUCTURE ONLY: the CPU restatement that the CUDA product path
// is compared against. It is loaded by tests/, by __graft_entry__.smoke() and by
// the CPU-baseline leg of bench.py, never by the product.
//
// A plain, single-threaded FP64 restatement of the Julia reference
// (ClimFlows/CFMultigrid.jl). Every loop keeps the reference's index ranges
// and every expression keeps Julia's association: `a+b+c+d` is the left fold
// ((a+b)+c)+d and `w*id*(t)` is (w*id)*t. The file is compiled with
// -ffp-contract=off so no multiply-add is fused behind our back.
//
// Array layout follows src/gmg_types.jl:86-118: one column-major
// (i fastest) array of tx*ty*tz entries per field and level, 1-based
// indices in the comments and in `at()`.

#include "cfmg_oracle.h"

#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

namespace {

// Grid (src/gmg_types.jl:68-84).
struct Grid {
  int nx, ny, nz, nh, tx, ty, tz;
  bool threed;
  size_t len() const { return (size_t)tx * ty * tz; }
  size_t at(int i, int j, int k) const {
    return (size_t)(i - 1) + (size_t)tx * ((size_t)(j - 1) + (size_t)ty * (size_t)(k - 1));
  }
  // index ranges (src/gmg_types.jl:4-23), inclusive [lo, hi]
  int ic0() const { return nh + 1; }
  int ic1() const { return nx + nh; }
  int jc0() const { return nh + 1; }
  int jc1() const { return ny + nh; }
  int kc0() const { return threed ? nh + 1 : 1; }
  int kc1() const { return threed ? nz + nh : nz; }
};

Grid make_grid(int nx, int ny, int nz, int nh, bool threed) {
  Grid g;
  g.nx = nx; g.ny = ny; g.nz = nz; g.nh = nh;
  g.tx = nx + 2 * nh;
  g.ty = ny + 2 * nh;
  g.tz = threed ? nz + 2 * nh : nz;
  g.threed = threed;
  return g;
}

// c2fidx / f2cidx (src/gmg_types.jl:25-26)
inline int c2f(int i, int nh) { return (i - nh - 1) * 2 + nh + 1; }
inline int f2c(int i, int nh) {
  // Julia div truncates toward zero; arguments here are always >= 0.
  return (i - nh - 1) / 2 + nh + 1;
}

typedef std::vector<double> A;
typedef std::vector<uint8_t> M;

// Data + Operators (src/gmg_types.jl:86-118); kappa is the per-cell
// coefficient of the variable-coefficient extension (op == 2).
struct Level {
  Grid g;
  A x, r, b, y, diag, idiag, Rcoef, Pcoef, kappa;
  M msk;
};

}  // namespace

struct orc_gmg {
  orc_param p;
  std::vector<Level> lv;  // lv[0] is level 1
  Level& L(int lev) { return lv[lev - 1]; }
  int nlevels() const { return (int)lv.size(); }
  bool vertices() const { return p.location == 1; }
  bool threed() const { return p.kase == 1; }
};

namespace {

A& field(orc_gmg* g, int lev, int f) {
  Level& l = g->L(lev);
  switch (f) {
    case 0: return l.x;
    case 1: return l.r;
    case 2: return l.b;
    case 3: return l.y;
    case 4: return l.diag;
    case 5: return l.idiag;
    case 6: return l.Rcoef;
    case 7: return l.Pcoef;
    default: return l.kappa;
  }
}

// ---------------------------------------------------------------- halo.jl
// fill! (src/halo.jl:1-15): no-op when closed, periodic copy of nh x-layers
// when :xperio.
template <class T>
void fill_halo(orc_gmg* g, int lev, std::vector<T>& x) {
  if (g->p.topology == 0) return;
  const Grid& gr = g->L(lev).g;
  int nh = gr.nh, tx = gr.tx;
  // Julia evaluates each right-hand slice before assigning it, which
  // matters when nx < nh (source and destination columns overlap).
  std::vector<T> tmp(nh);
  for (int k = 1; k <= gr.tz; ++k)
    for (int j = 1; j <= gr.ty; ++j) {
      // x[1:nh,:,:] = x[end+1-2nh:end-nh,:,:]
      for (int i = 1; i <= nh; ++i) tmp[i - 1] = x[gr.at(tx - 2 * nh + i, j, k)];
      for (int i = 1; i <= nh; ++i) x[gr.at(i, j, k)] = tmp[i - 1];
      // x[end+1-nh:end,:,:] = x[nh+1:2nh,:,:]
      for (int i = 1; i <= nh; ++i) tmp[i - 1] = x[gr.at(nh + i, j, k)];
      for (int i = 1; i <= nh; ++i) x[gr.at(tx - nh + i, j, k)] = tmp[i - 1];
    }
}

// ----------------------------------------------------------- laplacian.jl
// sloop2d! (src/laplacian.jl:66-73): linear range 1+n1 .. length-n1.
void sloop2d(const A& x, A& y, const A& b, const A& idiag, const Grid& g, double omega) {
  const size_t n1 = g.tx, len = g.len();
  #pragma omp parallel for schedule(static)
  for (size_t I = n1; I < len - n1; ++I) {  // 0-based I for 1-based 1+n1..len-n1
    double s = ((x[I - 1] + x[I + 1]) + x[I - n1]) + x[I + n1];
    y[I] = (1.0 - omega) * x[I] - (omega * idiag[I]) * (b[I] - s);
  }
}

// rloop2d! (src/laplacian.jl:87-93)
void rloop2d(A& r, const A& x, const A& b, const A& diag, const M& msk, const Grid& g) {
  const size_t n1 = g.tx, len = g.len();
  #pragma omp parallel for schedule(static)
  for (size_t I = n1; I < len - n1; ++I) {
    double s = ((x[I - 1] + x[I + 1]) + x[I - n1]) + x[I + n1];
    r[I] = (double)msk[I] * (((diag[I] * x[I]) + b[I]) - s);
  }
}

// smooth_laplacian2d! (src/laplacian.jl:95-112)
void smooth_laplacian2d(orc_gmg* g, int lev, int nite) {
  Level& l = g->L(lev);
  for (int kt = 0; kt < nite; ++kt) {
    sloop2d(l.x, l.y, l.b, l.idiag, l.g, g->p.omega);
    sloop2d(l.y, l.x, l.b, l.idiag, l.g, g->p.omega);
    fill_halo(g, lev, l.x);
  }
}

// residual_laplacian2d! (src/laplacian.jl:114-128)
void residual_laplacian2d(orc_gmg* g, int lev) {
  Level& l = g->L(lev);
  rloop2d(l.r, l.x, l.b, l.diag, l.msk, l.g);
  fill_halo(g, lev, l.r);
}

// sloop3d_v1! (src/laplacian.jl:11-20): linear range 1+n2 .. length-n2.
void sloop3d(const A& x, A& y, const A& b, const A& idiag, const Grid& g, double omega) {
  const size_t n1 = g.tx, n2 = (size_t)g.tx * g.ty, len = g.len();
  #pragma omp parallel for schedule(static)
  for (size_t I = n2; I < len - n2; ++I) {
    double s = ((((x[I - 1] + x[I + 1]) + x[I - n1]) + x[I + n1]) + x[I - n2]) + x[I + n2];
    y[I] = (1.0 - omega) * x[I] - (omega * idiag[I]) * (b[I] - s);
  }
}

// smooth_laplacian! (src/laplacian.jl:24-41)
void smooth_laplacian3d(orc_gmg* g, int lev, int nite) {
  Level& l = g->L(lev);
  for (int kt = 0; kt < nite; ++kt) {
    sloop3d(l.x, l.y, l.b, l.idiag, l.g, g->p.omega);
    sloop3d(l.y, l.x, l.b, l.idiag, l.g, g->p.omega);
    fill_halo(g, lev, l.x);
  }
}

// rloop3d! + residual_laplacian! (src/laplacian.jl:43-64): interior only.
void residual_laplacian3d(orc_gmg* g, int lev) {
  Level& l = g->L(lev);
  const Grid& gr = l.g;
  const size_t n1 = gr.tx, n2 = (size_t)gr.tx * gr.ty;
  #pragma omp parallel for collapse(2) schedule(static)
  for (int k = gr.kc0(); k <= gr.kc1(); ++k)
    for (int j = gr.jc0(); j <= gr.jc1(); ++j)
      for (int i = gr.ic0(); i <= gr.ic1(); ++i) {
        size_t I = gr.at(i, j, k);
        const A& x = l.x;
        double s = ((((x[I - 1] + x[I + 1]) + x[I - n1]) + x[I + n1]) + x[I - n2]) + x[I + n2];
        l.r[I] = (double)l.msk[I] * (((l.diag[I] * x[I]) + l.b[I]) - s);
      }
  fill_halo(g, lev, l.r);
}

// ---------------------------------------------------------- laplacian9.jl
// 19-point stencil (src/laplacian9.jl:14-44): faces/2 and edges/4.
inline double faces19(const A& x, size_t I, size_t n1, size_t n2) {
  return ((((x[I - 1] + x[I + 1]) + x[I - n1]) + x[I + n1]) + x[I - n2]) + x[I + n2];
}
inline double edges19(const A& x, size_t I, size_t n1, size_t n2) {
  double e = x[I - 1 - n1] + x[I + 1 - n1];
  e = e + x[I - 1 + n1];
  e = e + x[I + 1 + n1];
  e = e + x[I - 1 - n2];
  e = e + x[I + 1 - n2];
  e = e + x[I - 1 + n2];
  e = e + x[I + 1 + n2];
  e = e + x[I - n1 - n2];
  e = e + x[I + n1 - n2];
  e = e + x[I - n1 + n2];
  e = e + x[I + n1 + n2];
  return e;
}

// smooth_laplacian9! (src/laplacian9.jl:2-47): ONE pair whatever nite is,
// first sweep over icp x jcp x kcp, second over the interior, no fill!.
void smooth_laplacian9_3d(orc_gmg* g, int lev, int /*nite*/) {
  Level& l = g->L(lev);
  const Grid& gr = l.g;
  const size_t n1 = gr.tx, n2 = (size_t)gr.tx * gr.ty;
  const double omega = g->p.omega, cff = 1.0 - omega;
  #pragma omp parallel for collapse(2) schedule(static)
  for (int k = gr.nh; k <= gr.nz + gr.nh + 1; ++k)
    for (int j = gr.nh; j <= gr.ny + gr.nh + 1; ++j)
      for (int i = gr.nh; i <= gr.nx + gr.nh + 1; ++i) {
        size_t I = gr.at(i, j, k);
        l.y[I] = cff * l.x[I] - (omega * l.idiag[I]) *
                                    ((l.b[I] - faces19(l.x, I, n1, n2) / 2) - edges19(l.x, I, n1, n2) / 4);
      }
  #pragma omp parallel for collapse(2) schedule(static)
  for (int k = gr.kc0(); k <= gr.kc1(); ++k)
    for (int j = gr.jc0(); j <= gr.jc1(); ++j)
      for (int i = gr.ic0(); i <= gr.ic1(); ++i) {
        size_t I = gr.at(i, j, k);
        l.x[I] = cff * l.y[I] - (omega * l.idiag[I]) *
                                    ((l.b[I] - faces19(l.y, I, n1, n2) / 2) - edges19(l.y, I, n1, n2) / 4);
      }
}

// residual_laplacian9! (src/laplacian9.jl:49-73): interior, no fill!.
void residual_laplacian9_3d(orc_gmg* g, int lev) {
  Level& l = g->L(lev);
  const Grid& gr = l.g;
  const size_t n1 = gr.tx, n2 = (size_t)gr.tx * gr.ty;
  #pragma omp parallel for collapse(2) schedule(static)
  for (int k = gr.kc0(); k <= gr.kc1(); ++k)
    for (int j = gr.jc0(); j <= gr.jc1(); ++j)
      for (int i = gr.ic0(); i <= gr.ic1(); ++i) {
        size_t I = gr.at(i, j, k);
        l.r[I] = (double)l.msk[I] *
                 ((((l.diag[I] * l.x[I]) + l.b[I]) - faces19(l.x, I, n1, n2) / 2) - edges19(l.x, I, n1, n2) / 4);
      }
}

// 2D 9-point extension of laplacian9: the in-plane terms of the 19-point
// stencil (4 faces / 2, 4 diagonals / 4). No Julia counterpart exists (the
// reference only wires :laplacian9 for :threed, src/gmg_setup.jl:124-138).
// Same sweep ranges as smooth_laplacian9!, but it honours nite and calls
// fill! after each pair and after the residual, as the 5-point 2D form does.
inline double faces9(const A& x, size_t I, size_t n1) {
  return ((x[I - 1] + x[I + 1]) + x[I - n1]) + x[I + n1];
}
inline double diags9(const A& x, size_t I, size_t n1) {
  return ((x[I - 1 - n1] + x[I + 1 - n1]) + x[I - 1 + n1]) + x[I + 1 + n1];
}

void smooth_laplacian9_2d(orc_gmg* g, int lev, int nite) {
  Level& l = g->L(lev);
  const Grid& gr = l.g;
  const size_t n1 = gr.tx;
  const double omega = g->p.omega, cff = 1.0 - omega;
  for (int kt = 0; kt < nite; ++kt) {
    #pragma omp parallel for collapse(2) schedule(static)
    for (int k = 1; k <= gr.nz; ++k)
      for (int j = gr.nh; j <= gr.ny + gr.nh + 1; ++j)
        for (int i = gr.nh; i <= gr.nx + gr.nh + 1; ++i) {
          size_t I = gr.at(i, j, k);
          l.y[I] = cff * l.x[I] - (omega * l.idiag[I]) * ((l.b[I] - faces9(l.x, I, n1) / 2) - diags9(l.x, I, n1) / 4);
        }
    #pragma omp parallel for collapse(2) schedule(static)
    for (int k = 1; k <= gr.nz; ++k)
      for (int j = gr.jc0(); j <= gr.jc1(); ++j)
        for (int i = gr.ic0(); i <= gr.ic1(); ++i) {
          size_t I = gr.at(i, j, k);
          l.x[I] = cff * l.y[I] - (omega * l.idiag[I]) * ((l.b[I] - faces9(l.y, I, n1) / 2) - diags9(l.y, I, n1) / 4);
        }
    fill_halo(g, lev, l.x);
  }
}

void residual_laplacian9_2d(orc_gmg* g, int lev) {
  Level& l = g->L(lev);
  const Grid& gr = l.g;
  const size_t n1 = gr.tx;
  #pragma omp parallel for collapse(2) schedule(static)
  for (int k = 1; k <= gr.nz; ++k)
    for (int j = gr.jc0(); j <= gr.jc1(); ++j)
      for (int i = gr.ic0(); i <= gr.ic1(); ++i) {
        size_t I = gr.at(i, j, k);
        l.r[I] = (double)l.msk[I] * ((((l.diag[I] * l.x[I]) + l.b[I]) - faces9(l.x, I, n1) / 2) - diags9(l.x, I, n1) / 4);
      }
  fill_halo(g, lev, l.r);
}

// Variable-coefficient 5-point operator (extension, no Julia counterpart):
// A x = sum_f c_f x_nb - diag x with face coefficient
// c_f = (kappa_i + kappa_nb)/2 when both cells are wet, else 0. With
// kappa == 1 it reproduces :laplacian bit for bit on wet cells, because
// 1*x is exact and dry x stays 0. Same sweep range as sloop2d!.
inline double face_coef(const A& kap, const M& msk, size_t I, size_t J) {
  return (msk[I] && msk[J]) ? 0.5 * (kap[I] + kap[J]) : 0.0;
}
inline double vc_sum(const A& x, const A& kap, const M& msk, size_t I, size_t n1) {
  double s = face_coef(kap, msk, I, I - 1) * x[I - 1] + face_coef(kap, msk, I, I + 1) * x[I + 1];
  s = s + face_coef(kap, msk, I, I - n1) * x[I - n1];
  s = s + face_coef(kap, msk, I, I + n1) * x[I + n1];
  return s;
}

void smooth_varcoef2d(orc_gmg* g, int lev, int nite) {
  Level& l = g->L(lev);
  const size_t n1 = l.g.tx, len = l.g.len();
  const double omega = g->p.omega;
  for (int kt = 0; kt < nite; ++kt) {
    for (int pass = 0; pass < 2; ++pass) {
      const A& x = pass == 0 ? l.x : l.y;
      A& y = pass == 0 ? l.y : l.x;
#pragma omp parallel for schedule(static)
      for (size_t I = n1; I < len - n1; ++I) {
        double s = vc_sum(x, l.kappa, l.msk, I, n1);
        y[I] = (1.0 - omega) * x[I] - (omega * l.idiag[I]) * (l.b[I] - s);
      }
    }
    fill_halo(g, lev, l.x);
  }
}

void residual_varcoef2d(orc_gmg* g, int lev) {
  Level& l = g->L(lev);
  const size_t n1 = l.g.tx, len = l.g.len();
#pragma omp parallel for schedule(static)
  for (size_t I = n1; I < len - n1; ++I) {
    double s = vc_sum(l.x, l.kappa, l.msk, I, n1);
    l.r[I] = (double)l.msk[I] * (((l.diag[I] * l.x[I]) + l.b[I]) - s);
  }
  fill_halo(g, lev, l.r);
}

// --------------------------------------------------------- RP_on_centers.jl
// square (src/RP_on_centers.jl:1-3)
inline double square(const A& x, const Grid& g, int i, int j, int k, int di, int dj, int dk) {
  return 3 * (x[g.at(i + di, j, k + dk)] + x[g.at(i, j + dj, k + dk)]) + x[g.at(i + di, j + dj, k + dk)];
}

// rcloop2d! + restriction_centers2d! (src/RP_on_centers.jl:117-144)
void restriction_centers2d(orc_gmg* g, int lev, int f) {
  const Grid& gc = g->L(lev + 1).g;
  const Grid& gf = g->L(lev).g;
  const A& x = field(g, lev, f);
  A& xc = g->L(lev + 1).b;
  const A& coef = g->L(lev + 1).Rcoef;
  int nh = gc.nh;
  for (int kk = gc.kc0(); kk <= gc.kc1(); ++kk) {
    int k = kk;
    #pragma omp parallel for schedule(static)
    for (int jj = gc.jc0(); jj <= gc.jc1(); ++jj) {
      int j = c2f(jj, nh);
      for (int ii = gc.ic0(); ii <= gc.ic1(); ++ii) {
        int i = c2f(ii, nh);
        xc[gc.at(ii, jj, kk)] = coef[gc.at(ii, jj, kk)] *
                                (((x[gf.at(i, j, k)] + x[gf.at(i + 1, j, k)]) + x[gf.at(i, j + 1, k)]) +
                                 x[gf.at(i + 1, j + 1, k)]);
      }
    }
  }
  fill_halo(g, lev + 1, xc);
}

// pcloop2d! + prolongation_centers2d! (src/RP_on_centers.jl:146-175)
void prolongation_centers2d(orc_gmg* g, int lev) {
  const Grid& gf = g->L(lev).g;
  const Grid& gc = g->L(lev + 1).g;
  const A& coef = g->L(lev).Pcoef;
  A& xf = g->L(lev).x;
  const A& x = g->L(lev + 1).x;
  int nh = gf.nh;
  for (int k = gf.kc0(); k <= gf.kc1(); ++k) {
    int kc = k;
    #pragma omp parallel for schedule(static)
    for (int j = nh + 1; j <= gf.ny + nh; j += 2) {
      int jc = f2c(j, nh);
      for (int i = nh + 1; i <= gf.nx + nh; i += 2) {
        int ic = f2c(i, nh);
        double x9 = x[gc.at(ic, jc, kc)] * 9;
        for (int dj = 0; dj <= 1; ++dj)
          for (int di = 0; di <= 1; ++di) {
            double bb = square(x, gc, ic, jc, kc, 2 * di - 1, 2 * dj - 1, 0);
            size_t F = gf.at(i + di, j + dj, k);
            xf[F] = xf[F] + coef[F] * (bb + x9);
          }
      }
    }
  }
  fill_halo(g, lev, xf);
}

// rcloop3d! + restriction_centers! (src/RP_on_centers.jl:5-23,73-82)
void restriction_centers3d(orc_gmg* g, int lev, int f) {
  const Grid& gc = g->L(lev + 1).g;
  const Grid& gf = g->L(lev).g;
  const A& x = field(g, lev, f);
  A& xc = g->L(lev + 1).b;
  const A& coef = g->L(lev + 1).Rcoef;
  int nh = gc.nh;
  for (int kk = gc.kc0(); kk <= gc.kc1(); ++kk) {
    int k = c2f(kk, nh);
    #pragma omp parallel for schedule(static)
    for (int jj = gc.jc0(); jj <= gc.jc1(); ++jj) {
      int j = c2f(jj, nh);
      for (int ii = gc.ic0(); ii <= gc.ic1(); ++ii) {
        int i = c2f(ii, nh);
        double s = x[gf.at(i, j, k)] + x[gf.at(i + 1, j, k)];
        s = s + x[gf.at(i, j + 1, k)];
        s = s + x[gf.at(i + 1, j + 1, k)];
        s = s + x[gf.at(i, j, k + 1)];
        s = s + x[gf.at(i + 1, j, k + 1)];
        s = s + x[gf.at(i, j + 1, k + 1)];
        s = s + x[gf.at(i + 1, j + 1, k + 1)];
        xc[gc.at(ii, jj, kk)] = coef[gc.at(ii, jj, kk)] * s;
      }
    }
  }
  fill_halo(g, lev + 1, xc);
}

// pcloop3d! + prolongation_centers! (src/RP_on_centers.jl:84-114). The
// z-face neighbour is absent and the centre weighs 28 (raw weights sum to 56).
void prolongation_centers3d(orc_gmg* g, int lev) {
  const Grid& gf = g->L(lev).g;
  const Grid& gc = g->L(lev + 1).g;
  const A& coef = g->L(lev).Pcoef;
  A& xf = g->L(lev).x;
  const A& x = g->L(lev + 1).x;
  int nh = gf.nh;
  for (int k = nh + 1; k <= gf.nz + nh; k += 2) {
    int kc = f2c(k, nh);
    #pragma omp parallel for schedule(static)
    for (int j = nh + 1; j <= gf.ny + nh; j += 2) {
      int jc = f2c(j, nh);
      for (int i = nh + 1; i <= gf.nx + nh; i += 2) {
        int ic = f2c(i, nh);
        double x28 = x[gc.at(ic, jc, kc)] * 28;
        for (int dj = 0; dj <= 1; ++dj)
          for (int di = 0; di <= 1; ++di) {
            double a = square(x, gc, ic, jc, kc, 2 * di - 1, 2 * dj - 1, -1);
            double bb = square(x, gc, ic, jc, kc, 2 * di - 1, 2 * dj - 1, 0) * 3;
            double c = square(x, gc, ic, jc, kc, 2 * di - 1, 2 * dj - 1, +1);
            size_t F0 = gf.at(i + di, j + dj, k);
            size_t F1 = gf.at(i + di, j + dj, k + 1);
            xf[F0] = xf[F0] + coef[F0] * ((bb + a) + x28);
            xf[F1] = xf[F1] + coef[F1] * ((bb + c) + x28);
          }
      }
    }
  }
  fill_halo(g, lev, xf);
}

// -------------------------------------------------------- RP_on_vertices.jl
// restriction_vertices! (src/RP_on_vertices.jl:1-32): 27-point full weighting.
void restriction_vertices3d(orc_gmg* g, int lev, int f) {
  const Grid& gc = g->L(lev + 1).g;
  const Grid& gf = g->L(lev).g;
  const A& x = field(g, lev, f);
  A& xc = g->L(lev + 1).b;
  const A& coef = g->L(lev + 1).Rcoef;
  int nh = gc.nh;
  for (int kk = gc.kc0(); kk <= gc.kc1(); ++kk) {
    int k = c2f(kk, nh);
    #pragma omp parallel for schedule(static)
    for (int jj = gc.jc0(); jj <= gc.jc1(); ++jj) {
      int j = c2f(jj, nh);
      for (int ii = gc.ic0(); ii <= gc.ic1(); ++ii) {
        int i = c2f(ii, nh);
        // left fold in source order: dk = -1, 0, +1; dj = -1, 0, +1; di = -1, 0, +1
        double s = 0.0;
        bool first = true;
        for (int dk = -1; dk <= 1; ++dk)
          for (int dj = -1; dj <= 1; ++dj)
            for (int di = -1; di <= 1; ++di) {
              int w = (2 - std::abs(di)) * (2 - std::abs(dj)) * (2 - std::abs(dk));  // 1,2,4,8
              double v = x[gf.at(i + di, j + dj, k + dk)];
              double t = (w == 1) ? v : (double)w * v;
              if (first) { s = t; first = false; } else s = s + t;
            }
        xc[gc.at(ii, jj, kk)] = coef[gc.at(ii, jj, kk)] * s;
      }
    }
  }
  fill_halo(g, lev + 1, xc);
}

// prolongation_vertices! (src/RP_on_vertices.jl:34-72): trilinear injection.
void prolongation_vertices3d(orc_gmg* g, int lev) {
  const Grid& gf = g->L(lev).g;
  const Grid& gc = g->L(lev + 1).g;
  const A& coef = g->L(lev).Pcoef;
  A& xf = g->L(lev).x;
  const A& x = g->L(lev + 1).x;
  int nh = gf.nh;
  for (int k = nh + 1; k <= gf.nz + nh; k += 2) {
    int kc = f2c(k, nh);
    #pragma omp parallel for schedule(static)
    for (int j = nh + 1; j <= gf.ny + nh; j += 2) {
      int jc = f2c(j, nh);
      for (int i = nh + 1; i <= gf.nx + nh; i += 2) {
        int ic = f2c(i, nh);
        auto X = [&](int a, int b, int c) { return x[gc.at(ic + a, jc + b, kc + c)]; };
        auto add = [&](int a, int b, int c, double v) {
          size_t F = gf.at(i + a, j + b, k + c);
          xf[F] = xf[F] + coef[F] * v;
        };
        add(0, 0, 0, X(0, 0, 0));
        add(1, 0, 0, X(0, 0, 0) + X(1, 0, 0));
        add(0, 1, 0, X(0, 0, 0) + X(0, 1, 0));
        add(0, 0, 1, X(0, 0, 0) + X(0, 0, 1));
        add(1, 1, 0, ((X(0, 0, 0) + X(1, 0, 0)) + X(0, 1, 0)) + X(1, 1, 0));
        add(1, 0, 1, ((X(0, 0, 0) + X(1, 0, 0)) + X(0, 0, 1)) + X(1, 0, 1));
        add(0, 1, 1, ((X(0, 0, 0) + X(0, 0, 1)) + X(0, 1, 0)) + X(0, 1, 1));
        double s = X(0, 0, 0) + X(1, 0, 0);
        s = s + X(0, 0, 1);
        s = s + X(1, 0, 1);
        s = s + X(0, 1, 0);
        s = s + X(1, 1, 0);
        s = s + X(0, 1, 1);
        s = s + X(1, 1, 1);
        add(1, 1, 1, s);
      }
    }
  }
  fill_halo(g, lev, xf);
}

// rvloop2d! + restriction_vertices2d! (src/RP_on_vertices.jl:96-115,140-150)
void restriction_vertices2d(orc_gmg* g, int lev, int f) {
  const Grid& gc = g->L(lev + 1).g;
  const Grid& gf = g->L(lev).g;
  const A& x = field(g, lev, f);
  A& xc = g->L(lev + 1).b;
  const A& coef = g->L(lev + 1).Rcoef;
  int nh = gc.nh;
  for (int kk = gc.kc0(); kk <= gc.kc1(); ++kk) {
    int k = kk;
    #pragma omp parallel for schedule(static)
    for (int j = nh + 1; j <= 2 * gc.ny + nh; j += 2) {
      int jc = f2c(j, nh);
      for (int i = nh + 1; i <= 2 * gc.nx + nh; i += 2) {
        int ic = f2c(i, nh);
        auto X = [&](int a, int b) { return x[gf.at(i + a, j + b, k)]; };
        double s = X(-1, -1) + 2 * X(0, -1);
        s = s + X(1, -1);
        s = s + 2 * X(-1, 0);
        s = s + 4 * X(0, 0);
        s = s + 2 * X(1, 0);
        s = s + X(-1, 1);
        s = s + 2 * X(0, 1);
        s = s + X(1, 1);
        xc[gc.at(ic, jc, kk)] = coef[gc.at(ic, jc, kk)] * s;
      }
    }
  }
  fill_halo(g, lev + 1, xc);
}

// pvloop2d! + prolongation_vertices2d! (src/RP_on_vertices.jl:117-137,152-162)
void prolongation_vertices2d(orc_gmg* g, int lev) {
  const Grid& gf = g->L(lev).g;
  const Grid& gc = g->L(lev + 1).g;
  const A& coef = g->L(lev).Pcoef;
  A& xf = g->L(lev).x;
  const A& x = g->L(lev + 1).x;
  int nh = gf.nh;
  for (int k = gf.kc0(); k <= gf.kc1(); ++k) {
    int kc = k;
    #pragma omp parallel for schedule(static)
    for (int j = nh + 1; j <= gf.ny + nh; j += 2) {
      int jc = f2c(j, nh);
      for (int i = nh + 1; i <= gf.nx + nh; i += 2) {
        int ic = f2c(i, nh);
        auto X = [&](int a, int b) { return x[gc.at(ic + a, jc + b, kc)]; };
        auto add = [&](int a, int b, double v) {
          size_t F = gf.at(i + a, j + b, k);
          xf[F] = xf[F] + coef[F] * v;
        };
        add(0, 0, X(0, 0));
        add(1, 0, X(0, 0) + X(1, 0));
        add(0, 1, X(0, 0) + X(0, 1));
        add(1, 1, ((X(0, 0) + X(1, 0)) + X(0, 1)) + X(1, 1));
      }
    }
  }
  fill_halo(g, lev, xf);
}

// ------------------------------------------------- operator tables (allocate_mg)
// get_smoother_and_residual / get_restriction_and_prolongation
// (src/gmg_setup.jl:124-157), plus the 2D 9-point and variable-coefficient
// extensions.
void smoother(orc_gmg* g, int lev, int nite) {
  if (g->threed()) {
    if (g->p.op == 1) smooth_laplacian9_3d(g, lev, nite);
    else smooth_laplacian3d(g, lev, nite);
  } else {
    if (g->p.op == 1) smooth_laplacian9_2d(g, lev, nite);
    else if (g->p.op == 2) smooth_varcoef2d(g, lev, nite);
    else smooth_laplacian2d(g, lev, nite);
  }
}

void residual(orc_gmg* g, int lev) {
  if (g->threed()) {
    if (g->p.op == 1) residual_laplacian9_3d(g, lev);
    else residual_laplacian3d(g, lev);
  } else {
    if (g->p.op == 1) residual_laplacian9_2d(g, lev);
    else if (g->p.op == 2) residual_varcoef2d(g, lev);
    else residual_laplacian2d(g, lev);
  }
}

void restriction(orc_gmg* g, int lev, int f) {
  if (g->threed()) {
    if (g->vertices()) restriction_vertices3d(g, lev, f);
    else restriction_centers3d(g, lev, f);
  } else {
    if (g->vertices()) restriction_vertices2d(g, lev, f);
    else restriction_centers2d(g, lev, f);
  }
}

void prolongation(orc_gmg* g, int lev) {
  if (g->threed()) {
    if (g->vertices()) prolongation_vertices3d(g, lev);
    else prolongation_centers3d(g, lev);
  } else {
    if (g->vertices()) prolongation_vertices2d(g, lev);
    else prolongation_centers2d(g, lev);
  }
}

// ----------------------------------------------------------- setup (gmg_setup.jl)
// get_default_msk! (src/gmg_setup.jl:289-308)
M default_msk(orc_gmg* g, int lev) {
  const Grid& gr = g->L(lev).g;
  M msk(gr.len(), 0);
  int nh = gr.nh;
  if (g->vertices()) {
    int k0 = g->threed() ? nh + 1 : 1, k1 = g->threed() ? nh + gr.nz : gr.nz;
    for (int k = k0; k <= k1; ++k)
      for (int j = nh + 2; j <= gr.ny + nh; ++j)
        for (int i = nh + 2; i <= gr.nx + nh; ++i) msk[gr.at(i, j, k)] = 1;
  } else {
    #pragma omp parallel for collapse(2) schedule(static)
    for (int k = gr.kc0(); k <= gr.kc1(); ++k)
      for (int j = gr.jc0(); j <= gr.jc1(); ++j)
        for (int i = gr.ic0(); i <= gr.ic1(); ++i) msk[gr.at(i, j, k)] = 1;
  }
  fill_halo(g, lev, msk);
  return msk;
}

// apply_default_msk! (src/gmg_setup.jl:310-319)
void apply_default_msk(orc_gmg* g, int lev) {
  M d = default_msk(g, lev);
  M& msk = g->L(lev).msk;
  for (size_t I = 0; I < msk.size(); ++I) msk[I] = (uint8_t)(msk[I] * d[I]);
}

// compute_msk_dev (src/gmg_setup.jl:322-366)
void compute_msk_dev(orc_gmg* g) {
  const bool vertices = g->vertices();
  for (int lev = 1; lev <= g->nlevels() - 1; ++lev) {
    Level& c = g->L(lev + 1);
    const double threshold = vertices ? 0.67 : 0.18;
    M msk0 = c.msk;
    std::fill(c.msk.begin(), c.msk.end(), 1);
    std::fill(c.Rcoef.begin(), c.Rcoef.end(), 1.0);
    if (lev == 1) {
      Level& f = g->L(1);
      for (size_t I = 0; I < f.b.size(); ++I) f.b[I] = (double)f.msk[I];
    }
    restriction(g, lev, 2);
    c.msk = msk0;
    M mdef = default_msk(g, lev + 1);
    double coef;
    if (g->threed()) coef = vertices ? 1.0 / 64 : 1.0 / 8;
    else coef = vertices ? 1.0 / 16 : 1.0 / 4;
    for (size_t I = 0; I < c.b.size(); ++I) c.b[I] = c.b[I] * ((double)mdef[I] * coef);
    for (size_t I = 0; I < c.b.size(); ++I) c.msk[I] = (c.b[I] > threshold) ? 1 : 0;
    apply_default_msk(g, lev);
  }
}

// compute_Rcoef! (src/gmg_setup.jl:186-212)
void compute_Rcoef(orc_gmg* g, int lev) {
  const bool vertices = g->vertices();
  Level& c = g->L(lev + 1);
  Level& f = g->L(lev);
  for (size_t I = 0; I < c.Rcoef.size(); ++I) c.Rcoef[I] = (double)c.msk[I];
  for (size_t I = 0; I < f.b.size(); ++I) f.b[I] = vertices ? (double)f.msk[I] : 1.0;
  restriction(g, lev, 2);
  const double coef = g->threed() ? 1.0 / 16 : 1.0 / 4;
  for (size_t I = 0; I < c.Rcoef.size(); ++I) {
    double bb = c.b[I];
    double fr = vertices ? ((bb > 0.0) ? coef : 0.0) : ((bb > 0.0) ? (4 / bb) : 0.0);
    c.Rcoef[I] = (double)c.msk[I] * fr;
  }
}

// compute_Pcoef! (src/gmg_setup.jl:214-237)
void compute_Pcoef(orc_gmg* g, int lev) {
  const bool vertices = g->vertices();
  Level& f = g->L(lev);
  Level& c = g->L(lev + 1);
  for (size_t I = 0; I < f.Pcoef.size(); ++I) f.Pcoef[I] = (double)f.msk[I];
  std::fill(f.x.begin(), f.x.end(), 0.0);
  for (size_t I = 0; I < c.x.size(); ++I) c.x[I] = vertices ? 1.0 : (double)c.msk[I];
  prolongation(g, lev);
  for (size_t I = 0; I < f.Pcoef.size(); ++I) {
    double xv = f.x[I];
    f.Pcoef[I] = ((xv > 0) ? 1 / xv : 0.0) * (double)f.msk[I];
  }
}

// compute_diag! (src/gmg_setup.jl:239-262)
void compute_diag(orc_gmg* g, int lev) {
  const bool vertices = g->vertices();
  Level& l = g->L(lev);
  for (size_t I = 0; I < l.x.size(); ++I) l.x[I] = vertices ? 1.0 : (double)l.msk[I];
  std::fill(l.b.begin(), l.b.end(), 0.0);
  std::fill(l.diag.begin(), l.diag.end(), 0.0);
  residual(g, lev);
  for (size_t I = 0; I < l.diag.size(); ++I) l.diag[I] = (-l.r[I]) * (double)l.msk[I];
  for (size_t I = 0; I < l.idiag.size(); ++I) l.idiag[I] = (l.diag[I] > 0.0) ? 1.0 / l.diag[I] : 0.0;
}

// Coarse kappa for the variable-coefficient extension: mean of kappa over
// the wet children (1 where no child is wet).
void restrict_kappa(orc_gmg* g, int lev) {
  const Grid& gc = g->L(lev + 1).g;
  const Grid& gf = g->L(lev).g;
  const A& kf = g->L(lev).kappa;
  const M& mf = g->L(lev).msk;
  A& kc = g->L(lev + 1).kappa;
  int nh = gc.nh;
  std::fill(kc.begin(), kc.end(), 1.0);
  for (int kk = gc.kc0(); kk <= gc.kc1(); ++kk)
    #pragma omp parallel for schedule(static)
    for (int jj = gc.jc0(); jj <= gc.jc1(); ++jj)
      for (int ii = gc.ic0(); ii <= gc.ic1(); ++ii) {
        int i = c2f(ii, nh), j = c2f(jj, nh);
        double s = 0.0, n = 0.0;
        for (int dj = 0; dj <= 1; ++dj)
          for (int di = 0; di <= 1; ++di) {
            size_t F = gf.at(i + di, j + dj, kk);
            if (mf[F]) { s = s + kf[F]; n = n + 1.0; }
          }
        kc[gc.at(ii, jj, kk)] = n > 0 ? s / n : 1.0;
      }
  fill_halo(g, lev + 1, kc);
}

// setup_operators! (src/gmg_setup.jl:264-287)
void setup_operators(orc_gmg* g) {
  compute_msk_dev(g);
  if (g->p.op == 2)
    for (int lev = 1; lev <= g->nlevels() - 1; ++lev) restrict_kappa(g, lev);
  for (int lev = 1; lev <= g->nlevels() - 1; ++lev) {
    compute_Rcoef(g, lev);
    compute_Pcoef(g, lev);
  }
  for (int lev = 1; lev <= g->nlevels(); ++lev) compute_diag(g, lev);
}

// --------------------------------------------------- operators_at_level.jl
void set_to_zero(orc_gmg* g, int lev, int f) {
  A& x = field(g, lev, f);
  std::fill(x.begin(), x.end(), 0.0);
}

// norm (src/operators_at_level.jl:12-27): sequential sum of msk*x^2 over
// the whole array, 0 replaced by 1.
double norm(orc_gmg* g, int lev, int f) {
  const A& x = field(g, lev, f);
  const M& msk = g->L(lev).msk;
  double sum = 0.0;
  for (size_t I = 0; I < x.size(); ++I) sum += (double)msk[I] * (x[I] * x[I]);
  if (sum == 0.0) sum = 1.0;
  return sum;
}

// normresidual! (src/operators_at_level.jl:29-36)
double normresidual(orc_gmg* g, double normb) {
  if (normb > 0.0) {
    residual(g, 1);
    return norm(g, 1, 1) / normb;
  }
  return 0.0;
}

// ---------------------------------------------------------- gmg_cycles.jl
void vcycle(orc_gmg* g, int lev0) {  // src/gmg_cycles.jl:67-83
  const orc_param& p = g->p;
  int L = g->nlevels();
  for (int lev = lev0; lev <= L - 1; ++lev) {
    smoother(g, lev, p.npre);
    residual(g, lev);
    restriction(g, lev, 1);
    set_to_zero(g, lev + 1, 0);
  }
  smoother(g, L, p.ndeepest);
  for (int lev = L - 1; lev >= lev0; --lev) {
    prolongation(g, lev);
    smoother(g, lev, p.npost);
  }
}

void fcycle(orc_gmg* g) {  // src/gmg_cycles.jl:85-100
  int L = g->nlevels();
  for (int lev = 1; lev <= L - 1; ++lev) {
    restriction(g, lev, lev > 1 ? 2 : 1);
    set_to_zero(g, lev + 1, 0);
  }
  smoother(g, L, g->p.ndeepest);
  for (int lev = L - 1; lev >= 1; --lev) {
    prolongation(g, lev);
    vcycle(g, lev);
  }
}

void onelevel(orc_gmg* g) { smoother(g, 1, g->p.ndeepest); }  // src/gmg_cycles.jl:3-6

void twolevels(orc_gmg* g) {  // src/gmg_cycles.jl:8-23
  smoother(g, 1, g->p.npre);
  residual(g, 1);
  restriction(g, 1, 1);
  set_to_zero(g, 2, 0);
  smoother(g, 2, g->p.ndeepest);
  prolongation(g, 1);
  smoother(g, 1, g->p.npost);
}

// nlevels! (src/gmg_cycles.jl:25-41), reproduced with its quirks: the
// coarse smoothing hits level mg.nlevels and the ascending loop is empty.
void nlevels_cycle(orc_gmg* g, int nlev) {
  for (int lev = 1; lev <= nlev - 1; ++lev) {
    smoother(g, lev, g->p.npre);
    residual(g, lev);
    restriction(g, lev, 1);
    set_to_zero(g, lev + 1, 0);
  }
  smoother(g, g->nlevels(), g->p.ndeepest);
}

void cycle(orc_gmg* g, int kind) {
  switch (kind) {
    case 1: fcycle(g); break;
    case 2: onelevel(g); break;
    case 3: twolevels(g); break;
    case 4: nlevels_cycle(g, 3); break;
    default: vcycle(g, 1); break;  // :v and :vrec (same arithmetic when not verbose)
  }
}

// create_levels (src/gmg_setup.jl:40-64) with an optional cap.
std::vector<Grid> create_levels(const orc_param& p) {
  int nx = p.nx, ny = p.ny, nz = p.nz;
  bool threed = p.kase == 1;
  const int maxlevs = p.nlevels > 0 ? p.nlevels : 29;
  std::vector<Grid> out;
  out.push_back(make_grid(nx, ny, nz, p.nh, threed));
  int lev = 1;
  while (true) {
    if (!((nx * ny > 8) && (nx > 2) && (ny > 2))) break;
    if (!(lev < maxlevs)) break;
    nx /= 2;
    ny /= 2;
    if (threed) nz /= 2;
    out.push_back(make_grid(nx, ny, nz, p.nh, threed));
    lev += 1;
  }
  return out;
}

}  // namespace

extern "C" {

orc_gmg* orc_allocate(const orc_param* p) {
  if (!p || p->nx < 1 || p->ny < 1 || p->nz < 1 || p->nh < 1) return nullptr;
  if (p->op == 2 && (p->kase != 0 || p->location != 0)) return nullptr;
  orc_gmg* g = new orc_gmg();
  g->p = *p;
  for (const Grid& gr : create_levels(*p)) {
    Level l;
    l.g = gr;
    size_t n = gr.len();
    l.x.assign(n, 0.0); l.r.assign(n, 0.0); l.b.assign(n, 0.0); l.y.assign(n, 0.0);
    l.diag.assign(n, 0.0); l.idiag.assign(n, 0.0); l.Rcoef.assign(n, 0.0); l.Pcoef.assign(n, 0.0);
    l.kappa.assign(n, 1.0);
    l.msk.assign(n, 0);
    g->lv.push_back(std::move(l));
  }
  return g;
}

void orc_set_default_msk(orc_gmg* g) {  // set_default_msk! (src/gmg_setup.jl:106-122)
  g->L(1).msk = default_msk(g, 1);
}

orc_gmg* orc_get_gmg(const orc_param* p) {  // get_gmg (src/gmg_setup.jl:26-35)
  orc_gmg* g = orc_allocate(p);
  if (!g) return nullptr;
  orc_set_default_msk(g);
  setup_operators(g);
  for (int lev = 1; lev <= g->nlevels(); ++lev)
    for (int f : {2, 0, 3, 1}) set_to_zero(g, lev, f);
  return g;
}

void orc_free(orc_gmg* g) { delete g; }
int orc_nlevels(const orc_gmg* g) { return g->nlevels(); }

void orc_level_dims(const orc_gmg* g, int lev, int* d) {
  const Grid& gr = g->lv[lev - 1].g;
  d[0] = gr.nx; d[1] = gr.ny; d[2] = gr.nz; d[3] = gr.nh; d[4] = gr.tx; d[5] = gr.ty; d[6] = gr.tz;
}

double* orc_field(orc_gmg* g, int lev, int f) { return field(g, lev, f).data(); }
uint8_t* orc_msk(orc_gmg* g, int lev) { return g->L(lev).msk.data(); }

void orc_setup_operators(orc_gmg* g) { setup_operators(g); }
void orc_smooth(orc_gmg* g, int lev, int nite) { smoother(g, lev, nite); }
void orc_residual(orc_gmg* g, int lev) { residual(g, lev); }
void orc_restrict(orc_gmg* g, int lev, int f) { restriction(g, lev, f); }
void orc_prolong(orc_gmg* g, int lev) { prolongation(g, lev); }
void orc_zero(orc_gmg* g, int lev, int f) { set_to_zero(g, lev, f); }
void orc_fill(orc_gmg* g, int lev, int f) {
  if (f == 9) fill_halo(g, lev, g->L(lev).msk);
  else fill_halo(g, lev, field(g, lev, f));
}
double orc_norm(orc_gmg* g, int lev, int f) { return norm(g, lev, f); }
double orc_normresidual(orc_gmg* g, double normb) { return normresidual(g, normb); }
void orc_cycle(orc_gmg* g, int kind) { cycle(g, kind); }

// solve! (src/gmg_solver.jl:9-42)
void orc_solve(orc_gmg* g, double* res_out, int* nite_out, double* history) {
  double normb = norm(g, 1, 2);
  double res = normresidual(g, normb);
  int nite = 0;
  if (history) history[0] = res;
  while ((res > g->p.tol) && (nite < g->p.maxite)) {
    nite += 1;
    cycle(g, g->p.cycle);
    res = normresidual(g, normb);
    if (history) history[nite] = res;
  }
  *res_out = res;
  *nite_out = nite;
}

}  // extern "C"
