/*
 * TEST INFRASTRUCTURE — NOT PART OF THE PRODUCT.
 *
 * CPU restatement ("oracle") of GALES-multi-fluid's fluid_mc assembly hot path,
 * used only by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg
 * as the checker.  It is never linked into, or called by, the CUDA library.
 *
 * PARITY UNPINNED for the assembly itself: the reference's element integral and
 * mixtures cannot be compiled here (they need Boost uBLAS, OpenMPI and Trilinos, which
 * are absent) and it ships no tests, golden vectors or fixtures.  The chemicals' EOS
 * this file mixes (custom_chemical, ideal_gas) is pinned against the reference's own
 * chemicals.hpp, compiled from its checkout (ref_classes.cpp,
 * tests/test_reference_pins.py).  This file restates the reference's arithmetic line by line,
 * keeping the reference's expression forms and summation orders so that, built
 * with -ffp-contract=off, it reproduces the reference's FP64 results up to
 * libm's pow and Boost uBLAS's internal loop orders.  Each function cites the
 * reference file:line it follows (paths relative to the reference project).
 *
 * Third-party arithmetic restated from its published algorithm:
 *   - Boost uBLAS 1.70 lu_factorize / lu_substitute (partial pivoting on the
 *     first max |.| of the column, reciprocal column scaling, unit-lower then
 *     upper triangular solves against the permuted identity), called by
 *     GALES::inverse (src/fem/base/algorithm.hpp:399-416).
 *   - Epetra FECrsGraph/FECrsMatrix (Trilinos 12.17): on one rank the graph of
 *     element dof blocks has sorted unique global columns per row and
 *     SumIntoGlobalValues adds into existing entries.
 *
 * The dimension-generic 3D form is an extension of fluid_2d.hpp (the
 * reference ships only the 2D integral); it reduces to the 2D code exactly.
 */
#include "../include/gales_asm.h"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

// magma mixtures replacing the chemicals (magma_oracle.cpp, gor_set_magma)
bool gor_magma_active();
int gor_magma_point(double p, double T, const double* Y, double sr, double* f, double (*comp)[3]);

namespace {

constexpr int MD = GALES_MAX_ND;
constexpr double TOL = DBL_EPSILON;  // fluid_2d.hpp:93, quad.hpp:370

/* ------------------------------------------------------------------------- */
/* Element tables: element.hpp:63-176 (2D), 360-477 (3D); quad.hpp:148-188,
 * 470-515 (weights).                                                          */
struct ElemType {
  int dim = 0, nen = 0, nq = 0, nsides = 0, nsn = 0, nqs = 0;
  double gp[8][3] = {};
  int side[6][4] = {};
  double sgp[6][4][3] = {};
  double W_in = 0, W_bd = 0;
};

bool make_elem_type(int dim, int nen, ElemType& et) {
  et = ElemType();
  et.dim = dim;
  et.nen = nen;
  if (dim == 2 && nen == 4) {
    const double gm = -1.0 / sqrt(3.0), gpl = 1.0 / sqrt(3.0);
    const double g[4][2] = {{gm, gm}, {gpl, gm}, {gpl, gpl}, {gm, gpl}};
    et.nq = 4;
    for (int i = 0; i < 4; ++i) { et.gp[i][0] = g[i][0]; et.gp[i][1] = g[i][1]; }
    et.nsides = 4; et.nsn = 2; et.nqs = 2;
    const int sd[4][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}};
    const double s[4][2][2] = {{{gm, -1.0}, {gpl, -1.0}}, {{1.0, gm}, {1.0, gpl}},
                               {{gpl, 1.0}, {gm, 1.0}}, {{-1.0, gpl}, {-1.0, gm}}};
    for (int i = 0; i < 4; ++i)
      for (int j = 0; j < 2; ++j) {
        et.side[i][j] = sd[i][j];
        et.sgp[i][j][0] = s[i][j][0];
        et.sgp[i][j][1] = s[i][j][1];
      }
    et.W_in = 1.0; et.W_bd = 1.0;
    return true;
  }
  if (dim == 2 && nen == 3) {
    et.nq = 3;
    const double g[3][2] = {{1.0 / 6.0, 1.0 / 6.0}, {4.0 / 6.0, 1.0 / 6.0}, {1.0 / 6.0, 4.0 / 6.0}};
    for (int i = 0; i < 3; ++i) { et.gp[i][0] = g[i][0]; et.gp[i][1] = g[i][1]; }
    et.nsides = 3; et.nsn = 2; et.nqs = 2;
    const int sd[3][2] = {{1, 2}, {2, 0}, {0, 1}};
    const double gm = 0.5 * (1.0 - 1.0 / sqrt(3.0)), gpl = 0.5 * (1.0 + 1.0 / sqrt(3.0));
    const double s[3][2][2] = {{{gpl, 1.0 - gpl}, {gm, 1.0 - gm}}, {{0.0, gpl}, {0.0, gm}},
                               {{gm, 0.0}, {gpl, 0.0}}};
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 2; ++j) {
        et.side[i][j] = sd[i][j];
        et.sgp[i][j][0] = s[i][j][0];
        et.sgp[i][j][1] = s[i][j][1];
      }
    et.W_in = 1.0 / 6.0; et.W_bd = 1.0 / 2.0;
    return true;
  }
  if (dim == 3 && nen == 8) {
    const double m = -1.0 / sqrt(3.0), p = 1.0 / sqrt(3.0);
    const double g[8][3] = {{m, m, m}, {p, m, m}, {p, p, m}, {m, p, m},
                            {m, m, p}, {p, m, p}, {p, p, p}, {m, p, p}};
    et.nq = 8;
    for (int i = 0; i < 8; ++i)
      for (int d = 0; d < 3; ++d) et.gp[i][d] = g[i][d];
    et.nsides = 6; et.nsn = 4; et.nqs = 4;
    const int sd[6][4] = {{4, 5, 6, 7}, {0, 3, 2, 1}, {0, 4, 7, 3},
                          {1, 2, 6, 5}, {2, 3, 7, 6}, {1, 5, 4, 0}};
    const double s[6][4][3] = {
        {{m, m, 1.0}, {p, m, 1.0}, {p, p, 1.0}, {m, p, 1.0}},
        {{m, m, -1.0}, {m, p, -1.0}, {p, p, -1.0}, {p, m, -1.0}},
        {{-1.0, m, m}, {-1.0, m, p}, {-1.0, p, p}, {-1.0, p, m}},
        {{1.0, m, m}, {1.0, p, m}, {1.0, p, p}, {1.0, m, p}},
        {{p, 1.0, m}, {m, 1.0, m}, {m, 1.0, p}, {p, 1.0, p}},
        {{p, -1.0, m}, {p, -1.0, p}, {m, -1.0, p}, {m, -1.0, m}}};
    for (int i = 0; i < 6; ++i)
      for (int j = 0; j < 4; ++j) {
        et.side[i][j] = sd[i][j];
        for (int d = 0; d < 3; ++d) et.sgp[i][j][d] = s[i][j][d];
      }
    et.W_in = 1.0; et.W_bd = 1.0;
    return true;
  }
  if (dim == 3 && nen == 4) {
    const double a = 0.1381966011250105, b = 0.5854101966249685;
    const double g[4][3] = {{a, a, a}, {b, a, a}, {a, b, a}, {a, a, b}};
    et.nq = 4;
    for (int i = 0; i < 4; ++i)
      for (int d = 0; d < 3; ++d) et.gp[i][d] = g[i][d];
    et.nsides = 4; et.nsn = 3; et.nqs = 3;
    const int sd[4][3] = {{1, 2, 3}, {0, 3, 2}, {0, 1, 3}, {0, 2, 1}};
    const double o = 1.0 / 6.0, f = 4.0 / 6.0;
    const double s[4][3][3] = {{{f, o, o}, {o, f, o}, {o, o, f}},
                               {{0.0, o, o}, {0.0, o, f}, {0.0, f, o}},
                               {{o, 0.0, o}, {f, 0.0, o}, {o, 0.0, f}},
                               {{o, o, 0.0}, {o, f, 0.0}, {f, o, 0.0}}};
    for (int i = 0; i < 4; ++i)
      for (int j = 0; j < 3; ++j) {
        et.side[i][j] = sd[i][j];
        for (int d = 0; d < 3; ++d) et.sgp[i][j][d] = s[i][j][d];
      }
    et.W_in = 1.0 / 24.0; et.W_bd = 1.0 / 6.0;
    return true;
  }
  return false;
}

/* ------------------------------------------------------------------------- */
/* quad: shape functions, mapping, metrics.  quad.hpp:148-383 (2D), 470-739 (3D). */
struct Quad {
  double sh[8] = {};
  double dl[3][8] = {};  // dsh/dxi, dsh/deta, dsh/dzeta
  double ds[3][8] = {};  // dsh/dx, dsh/dy, dsh/dz
  double J = 0, W_in = 0, W_bd = 0;
  double G[3][3] = {};
  double g[3] = {};
  double JN[3] = {};
  double xi = 0, eta = 0, zeta = 0;
  bool neg_jac = false;
  double JxW() const { return J * W_in; }               // quad.hpp:940
  double JNxW(int i) const { return JN[i] * W_bd; }     // quad.hpp:945
};

void sh_local(const ElemType& et, const double* pt, Quad& q) {
  const int nen = et.nen;
  if (et.dim == 2) {
    const double xi = pt[0], eta = pt[1];
    q.xi = xi; q.eta = eta;
    if (nen == 4) {  // quad.hpp:153-167
      q.sh[0] = 0.25 * (1.0 - xi) * (1.0 - eta);
      q.sh[1] = 0.25 * (1.0 + xi) * (1.0 - eta);
      q.sh[2] = 0.25 * (1.0 + xi) * (1.0 + eta);
      q.sh[3] = 0.25 * (1.0 - xi) * (1.0 + eta);
      q.dl[0][0] = -0.25 * (1. - eta); q.dl[1][0] = -0.25 * (1. - xi);
      q.dl[0][1] = 0.25 * (1. - eta);  q.dl[1][1] = -0.25 * (1. + xi);
      q.dl[0][2] = 0.25 * (1. + eta);  q.dl[1][2] = 0.25 * (1. + xi);
      q.dl[0][3] = -0.25 * (1. + eta); q.dl[1][3] = 0.25 * (1. - xi);
      q.W_in = 1.0; q.W_bd = 1.0;
    } else {  // quad.hpp:168-187
      q.sh[0] = 1.0 - xi - eta; q.sh[1] = xi; q.sh[2] = eta;
      q.dl[0][0] = -1.0; q.dl[1][0] = -1.0;
      q.dl[0][1] = 1.0;  q.dl[1][1] = 0.0;
      q.dl[0][2] = 0.0;  q.dl[1][2] = 1.0;
      q.W_in = 1.0 / 6.0; q.W_bd = 1.0 / 2.0;
    }
  } else {
    const double xi = pt[0], eta = pt[1], zeta = pt[2];
    q.xi = xi; q.eta = eta; q.zeta = zeta;
    if (nen == 8) {  // quad.hpp:476-499
      const double sx[8] = {-1, 1, 1, -1, -1, 1, 1, -1};
      const double sy[8] = {-1, -1, 1, 1, -1, -1, 1, 1};
      const double sz[8] = {-1, -1, -1, -1, 1, 1, 1, 1};
      for (int i = 0; i < 8; ++i) {
        const double ax = sx[i] < 0 ? (1.0 - xi) : (1.0 + xi);
        const double ay = sy[i] < 0 ? (1.0 - eta) : (1.0 + eta);
        const double az = sz[i] < 0 ? (1.0 - zeta) : (1.0 + zeta);
        q.sh[i] = 0.125 * ax * ay * az;
        q.dl[0][i] = (sx[i] < 0 ? -0.125 : 0.125) * ay * az;
        q.dl[1][i] = (sy[i] < 0 ? -0.125 : 0.125) * ax * az;
        q.dl[2][i] = (sz[i] < 0 ? -0.125 : 0.125) * ax * ay;
      }
      q.W_in = 1.0; q.W_bd = 1.0;
    } else {  // quad.hpp:500-514
      q.sh[0] = 1.0 - xi - eta - zeta; q.sh[1] = xi; q.sh[2] = eta; q.sh[3] = zeta;
      const double d[3][4] = {{-1.0, 1.0, 0.0, 0.0}, {-1.0, 0.0, 1.0, 0.0}, {-1.0, 0.0, 0.0, 1.0}};
      for (int k = 0; k < 3; ++k)
        for (int i = 0; i < 4; ++i) q.dl[k][i] = d[k][i];
      q.W_in = 1.0 / 24.0; q.W_bd = 1.0 / 6.0;
    }
  }
}

/* quad.hpp:196-231 (2D calc), 305-345 (metrics), 523-571 (3D calc), 666-691 */
void calc(const ElemType& et, const double X[8][3], Quad& q, bool interior) {
  const int nen = et.nen;
  if (et.dim == 2) {
    double dx_dxi = 0.0, dx_deta = 0.0, dy_dxi = 0.0, dy_deta = 0.0;
    for (int i = 0; i < nen; ++i) {
      dx_dxi += q.dl[0][i] * X[i][0];
      dx_deta += q.dl[1][i] * X[i][0];
      dy_dxi += q.dl[0][i] * X[i][1];
      dy_deta += q.dl[1][i] * X[i][1];
    }
    q.J = dx_dxi * dy_deta - dy_dxi * dx_deta;
    if (q.J <= 0.0) q.neg_jac = true;
    const double dxi_dx = (1 / q.J) * (dy_deta);
    const double deta_dx = (1 / q.J) * (-dy_dxi);
    const double dxi_dy = (1 / q.J) * (-dx_deta);
    const double deta_dy = (1 / q.J) * (dx_dxi);
    for (int i = 0; i < nen; ++i) {
      q.ds[0][i] = q.dl[0][i] * dxi_dx + q.dl[1][i] * deta_dx;
      q.ds[1][i] = q.dl[0][i] * dxi_dy + q.dl[1][i] * deta_dy;
    }
    if (interior) {
      q.g[0] = dxi_dx + deta_dx;
      q.g[1] = dxi_dy + deta_dy;
      q.G[0][0] = dxi_dx * dxi_dx + deta_dx * deta_dx;
      q.G[1][1] = dxi_dy * dxi_dy + deta_dy * deta_dy;
      q.G[0][1] = dxi_dx * dxi_dy + deta_dx * deta_dy;
      q.G[1][0] = q.G[0][1];
    } else {  // quad.hpp:245-292
      if (nen == 4) {
        if (q.eta == 1.0) { q.JN[0] = -dy_dxi; q.JN[1] = dx_dxi; }
        else if (q.eta == -1.0) { q.JN[0] = dy_dxi; q.JN[1] = -dx_dxi; }
        else if (q.xi == 1.0) { q.JN[0] = dy_deta; q.JN[1] = -dx_deta; }
        else if (q.xi == -1.0) { q.JN[0] = -dy_deta; q.JN[1] = dx_deta; }
      } else {
        if (q.xi == 0.0) { q.JN[0] = -dy_deta; q.JN[1] = dx_deta; }
        else if (q.eta == 0.0) { q.JN[0] = dy_dxi; q.JN[1] = -dx_dxi; }
        else { q.JN[0] = dy_deta - dy_dxi; q.JN[1] = dx_dxi - dx_deta; }
      }
    }
  } else {
    double dx_dxi = 0.0, dx_deta = 0.0, dx_dzeta = 0.0;
    double dy_dxi = 0.0, dy_deta = 0.0, dy_dzeta = 0.0;
    double dz_dxi = 0.0, dz_deta = 0.0, dz_dzeta = 0.0;
    for (int i = 0; i < nen; ++i) {
      dx_dxi += q.dl[0][i] * X[i][0];
      dx_deta += q.dl[1][i] * X[i][0];
      dx_dzeta += q.dl[2][i] * X[i][0];
      dy_dxi += q.dl[0][i] * X[i][1];
      dy_deta += q.dl[1][i] * X[i][1];
      dy_dzeta += q.dl[2][i] * X[i][1];
      dz_dxi += q.dl[0][i] * X[i][2];
      dz_deta += q.dl[1][i] * X[i][2];
      dz_dzeta += q.dl[2][i] * X[i][2];
    }
    q.J = dx_dxi * (dy_deta * dz_dzeta - dz_deta * dy_dzeta) -
          dy_dxi * (dx_deta * dz_dzeta - dz_deta * dx_dzeta) +
          dz_dxi * (dx_deta * dy_dzeta - dy_deta * dx_dzeta);
    if (q.J <= 0.0) q.neg_jac = true;
    const double iJ = 1 / q.J;
    const double dxi_dx = iJ * (dy_deta * dz_dzeta - dz_deta * dy_dzeta);
    const double deta_dx = iJ * (-dy_dxi * dz_dzeta + dz_dxi * dy_dzeta);
    const double dzeta_dx = iJ * (dy_dxi * dz_deta - dz_dxi * dy_deta);
    const double dxi_dy = iJ * (-dx_deta * dz_dzeta + dz_deta * dx_dzeta);
    const double deta_dy = iJ * (dx_dxi * dz_dzeta - dz_dxi * dx_dzeta);
    const double dzeta_dy = iJ * (-dx_dxi * dz_deta + dz_dxi * dx_deta);
    const double dxi_dz = iJ * (dx_deta * dy_dzeta - dy_deta * dx_dzeta);
    const double deta_dz = iJ * (-dx_dxi * dy_dzeta + dy_dxi * dx_dzeta);
    const double dzeta_dz = iJ * (dx_dxi * dy_deta - dy_dxi * dx_deta);
    for (int i = 0; i < nen; ++i) {
      q.ds[0][i] = q.dl[0][i] * dxi_dx + q.dl[1][i] * deta_dx + q.dl[2][i] * dzeta_dx;
      q.ds[1][i] = q.dl[0][i] * dxi_dy + q.dl[1][i] * deta_dy + q.dl[2][i] * dzeta_dy;
      q.ds[2][i] = q.dl[0][i] * dxi_dz + q.dl[1][i] * deta_dz + q.dl[2][i] * dzeta_dz;
    }
    if (interior) {
      q.g[0] = dxi_dx + deta_dx + dzeta_dx;
      q.g[1] = dxi_dy + deta_dy + dzeta_dy;
      q.g[2] = dxi_dz + deta_dz + dzeta_dz;
      q.G[0][0] = dxi_dx * dxi_dx + deta_dx * deta_dx + dzeta_dx * dzeta_dx;
      q.G[1][1] = dxi_dy * dxi_dy + deta_dy * deta_dy + dzeta_dy * dzeta_dy;
      q.G[2][2] = dxi_dz * dxi_dz + deta_dz * deta_dz + dzeta_dz * dzeta_dz;
      q.G[0][1] = dxi_dx * dxi_dy + deta_dx * deta_dy + dzeta_dx * dzeta_dy;
      q.G[1][2] = dxi_dy * dxi_dz + deta_dy * deta_dz + dzeta_dy * dzeta_dz;
      q.G[0][2] = dxi_dz * dxi_dx + deta_dz * deta_dx + dzeta_dz * dzeta_dx;
      q.G[1][0] = q.G[0][1];
      q.G[2][1] = q.G[1][2];
      q.G[2][0] = q.G[0][2];
    } else {  // quad.hpp:582-654
      const double xi = q.xi, eta = q.eta, zeta = q.zeta;
      double* JN = q.JN;
      if (nen == 8) {
        if (zeta == 1.0) {
          JN[0] = dy_dxi * dz_deta - dz_dxi * dy_deta;
          JN[1] = dz_dxi * dx_deta - dx_dxi * dz_deta;
          JN[2] = dx_dxi * dy_deta - dy_dxi * dx_deta;
        } else if (zeta == -1.0) {
          JN[0] = -dy_dxi * dz_deta + dz_dxi * dy_deta;
          JN[1] = -dz_dxi * dx_deta + dx_dxi * dz_deta;
          JN[2] = -dx_dxi * dy_deta + dy_dxi * dx_deta;
        } else if (eta == 1.0) {
          JN[0] = dy_dzeta * dz_dxi - dy_dxi * dz_dzeta;
          JN[1] = dz_dzeta * dx_dxi - dz_dxi * dx_dzeta;
          JN[2] = dx_dzeta * dy_dxi - dx_dxi * dy_dzeta;
        } else if (eta == -1.0) {
          JN[0] = -dy_dzeta * dz_dxi + dy_dxi * dz_dzeta;
          JN[1] = -dz_dzeta * dx_dxi + dz_dxi * dx_dzeta;
          JN[2] = -dx_dzeta * dy_dxi + dx_dxi * dy_dzeta;
        } else if (xi == 1.0) {
          JN[0] = dy_deta * dz_dzeta - dy_dzeta * dz_deta;
          JN[1] = dz_deta * dx_dzeta - dz_dzeta * dx_deta;
          JN[2] = dx_deta * dy_dzeta - dx_dzeta * dy_deta;
        } else if (xi == -1.0) {
          JN[0] = -dy_deta * dz_dzeta + dy_dzeta * dz_deta;
          JN[1] = -dz_deta * dx_dzeta + dz_dzeta * dx_deta;
          JN[2] = -dx_deta * dy_dzeta + dx_dzeta * dy_deta;
        }
      } else {
        if (xi == 0.0) {
          JN[0] = dz_deta * dy_dzeta - dy_deta * dz_dzeta;
          JN[1] = dx_deta * dz_dzeta - dz_deta * dx_dzeta;
          JN[2] = dy_deta * dx_dzeta - dx_deta * dy_dzeta;
        } else if (eta == 0.0) {
          JN[0] = dz_dzeta * dy_dxi - dy_dzeta * dz_dxi;
          JN[1] = dz_dxi * dx_dzeta - dx_dxi * dz_dzeta;
          JN[2] = dy_dzeta * dx_dxi - dx_dzeta * dy_dxi;
        } else if (zeta == 0.0) {
          JN[0] = dz_dxi * dy_deta - dy_dxi * dz_deta;
          JN[1] = dx_dxi * dz_deta - dx_deta * dz_dxi;
          JN[2] = dy_dxi * dx_deta - dx_dxi * dy_deta;
        } else {
          JN[0] = (dz_dzeta - dz_dxi) * (dy_deta - dy_dxi) - (dy_dzeta - dy_dxi) * (dz_deta - dz_dxi);
          JN[1] = (dx_dzeta - dx_dxi) * (dz_deta - dz_dxi) - (dx_deta - dx_dxi) * (dz_dzeta - dz_dxi);
          JN[2] = (dx_deta - dx_dxi) * (dy_dzeta - dy_dxi) - (dx_dzeta - dx_dxi) * (dy_deta - dy_dxi);
        }
      }
    }
  }
}

void make_quad(const ElemType& et, const double X[8][3], const double* pt, bool interior, Quad& q) {
  q = Quad();
  sh_local(et, pt, q);
  calc(et, X, q, interior);
}

/* compute_h: quad.hpp:356-383 (2D), 701-739 (3D).  del_v(i,j) = d v_i / d x_j. */
double compute_h(const Quad& q, int dim, const double* v, const double del_v[3][3]) {
  double nrm_v = 0.0;
  for (int i = 0; i < dim; ++i) nrm_v += v[i] * v[i];
  nrm_v = sqrt(nrm_v);
  double s0[3] = {0, 0, 0}, s1[3] = {0, 0, 0}, s2[3] = {0, 0, 0}, alpha[3] = {0, 0, 0};
  for (int i = 0; i < dim; ++i) s0[i] = v[i] / nrm_v;
  auto quadform = [&](const double* s) {
    double Gs[3] = {0, 0, 0};
    for (int i = 0; i < dim; ++i) {
      double t = 0.0;
      for (int j = 0; j < dim; ++j) t += q.G[i][j] * s[j];
      Gs[i] = t;
    }
    double r = 0.0;
    for (int i = 0; i < dim; ++i) r += s[i] * Gs[i];
    return r;
  };
  alpha[0] = quadform(s0);
  double acc[3] = {0, 0, 0};
  for (int i = 0; i < dim; ++i) {
    double t = 0.0;
    for (int j = 0; j < dim; ++j) t += del_v[i][j] * v[j];
    acc[i] = t;
  }
  double ip = 0.0;
  for (int i = 0; i < dim; ++i) ip += acc[i] * s0[i];
  for (int i = 0; i < dim; ++i) s1[i] = acc[i] - ip * s0[i];
  double nrm_s1 = 0.0;
  for (int i = 0; i < dim; ++i) nrm_s1 += s1[i] * s1[i];
  nrm_s1 = sqrt(nrm_s1);
  if (nrm_s1 > TOL)
    for (int i = 0; i < dim; ++i) s1[i] /= nrm_s1;
  alpha[1] = quadform(s1);
  if (dim == 3) {
    s2[0] = s0[1] * s1[2] - s0[2] * s1[1];
    s2[1] = s1[0] * s0[2] - s1[2] * s0[0];
    s2[2] = s0[0] * s1[1] - s0[1] * s1[0];
    double nrm_s2 = 0.0;
    for (int i = 0; i < 3; ++i) nrm_s2 += s2[i] * s2[i];
    nrm_s2 = sqrt(nrm_s2);
    if (nrm_s2 > TOL)
      for (int i = 0; i < 3; ++i) s2[i] /= nrm_s2;
    alpha[2] = quadform(s2);
  }
  double h = 0.0;
  for (int i = 0; i < dim; ++i)
    if (alpha[i] != 0.0) h += 1.0 / alpha[i];
  h = 2 * sqrt(fabs(h));
  return h;
}

/* compute_shear_rate: non_newtonian.hpp:23-29 (2D), 32-39 (3D), from the gradients
 * dI[k][j] = d I_j / d x_k (dI_dx, dI_dy, dI_dz); std::pow(x, 2) as written there. */
double compute_shear_rate(int dim, const double dI[3][MD]) {
  if (dim == 2) {
    const double dv1_1 = dI[0][1], dv2_1 = dI[0][2];
    const double dv1_2 = dI[1][1], dv2_2 = dI[1][2];
    return std::sqrt(std::pow(dv1_1, 2) + std::pow(dv2_2, 2) + 2 * std::pow(dv1_2 + dv2_1, 2));
  }
  const double dv1_1 = dI[0][1], dv2_1 = dI[0][2], dv3_1 = dI[0][3];
  const double dv1_2 = dI[1][1], dv2_2 = dI[1][2], dv3_2 = dI[1][3];
  const double dv1_3 = dI[2][1], dv2_3 = dI[2][2], dv3_3 = dI[2][3];
  return std::sqrt(std::pow(dv1_1, 2) + std::pow(dv2_2, 2) + std::pow(dv3_3, 2) + 2 * std::pow(dv1_2 + dv2_1, 2) +
                   2 * std::pow(dv1_3 + dv3_1, 2) + 2 * std::pow(dv2_3 + dv3_2, 2));
}

/* ------------------------------------------------------------------------- */
/* Properties: fluid_properties.hpp:199-227 (mix_of_ch), chemicals.hpp:43-47,
 * 258-264, base_mixture.hpp:50-65.                                            */
struct Props {
  double rho, mu, cp, cv, kappa, D, c, alpha, beta;
  double rho_c[GALES_MAX_COMP], e_c[GALES_MAX_COMP], D_c[GALES_MAX_COMP];
};

/* sr: the point's shear rate (non_newtonian.hpp:23-39); only magma viscosity models use
 * it (custom and ideal-gas chemicals ignore it, chemicals.hpp:19-49, 198-271). */
void properties(const gales_material_desc& mat, double p, double T, const double* Y, Props& o, double sr = 0.0) {
  const int nc = mat.nb_comp;
  o.rho = o.cv = o.cp = o.kappa = o.D = o.mu = o.c = o.alpha = o.beta = 0.0;
  if (gor_magma_active()) {
    // fluid_properties.hpp:171-200: mix_of_mix; the mixture's own chemical diffusivity
    // is not accumulated there and stays 0 from clear() (base_mixture.hpp:50-65)
    double f[8], cc[GALES_MAX_COMP][3];
    gor_magma_point(p, T, Y, sr, f, cc);
    o.rho = f[0]; o.mu = f[1]; o.cp = f[2]; o.cv = f[3]; o.kappa = f[4]; o.c = f[5];
    o.alpha = f[6]; o.beta = f[7];
    for (int c = 0; c < nc; ++c) {
      o.rho_c[c] = cc[c][0];
      o.e_c[c] = cc[c][1];
      o.D_c[c] = cc[c][2];
    }
    return;
  }
  double crho[GALES_MAX_COMP], cc[GALES_MAX_COMP], calpha[GALES_MAX_COMP], cbeta[GALES_MAX_COMP];
  for (int c = 0; c < nc; ++c) {
    const gales_chemical_desc& ch = mat.comp[c];
    double rho, cv, cp = ch.cp, mu = ch.mu, kappa = ch.kappa, sound, alpha, beta;
    if (ch.kind == GALES_CH_CUSTOM) {  // chemicals.hpp:23-47
      rho = ch.rho; alpha = ch.alpha; beta = ch.beta;
      sound = (beta == 0.0) ? 1.e20 : 1.0 / sqrt(rho * beta);
      cv = (beta == 0.0) ? cp : cp - T * alpha * alpha / (rho * beta);
    } else {  // chemicals.hpp:258-264
      rho = p / (ch.R * T);
      beta = 1.0 / p;
      alpha = 1.0 / T;
      sound = sqrt(ch.gamma * ch.R * T);
      cv = ch.cv;
    }
    crho[c] = rho; cc[c] = sound; calpha[c] = alpha; cbeta[c] = beta;
    o.rho += Y[c] / rho;
    o.mu += Y[c] * mu;
    o.cp += Y[c] * cp;
    o.cv += Y[c] * cv;
    o.kappa += Y[c] * kappa;
    o.D += Y[c] * ch.chemical_diffusivity;
    o.c += Y[c] / ((rho * rho) * (sound * sound));
    o.rho_c[c] = rho;
    o.e_c[c] = cv * T;
    o.D_c[c] = ch.chemical_diffusivity;
  }
  o.rho = 1. / o.rho;
  o.c = sqrt(1.0 / o.c);
  o.c /= o.rho;
  for (int c = 0; c < nc; ++c) {
    o.alpha += Y[c] * calpha[c] * o.rho / crho[c];
    o.beta += Y[c] * cbeta[c] * o.rho / crho[c];
  }
}

/* ------------------------------------------------------------------------- */
/* GALES::inverse (algorithm.hpp:399-416) = uBLAS lu_factorize + lu_substitute. */
int lu_inverse(int n, const double* A_in, double* inv) {
  double A[MD][MD];
  int pm[MD];
  for (int i = 0; i < n; ++i) {
    pm[i] = i;
    for (int j = 0; j < n; ++j) A[i][j] = A_in[i * n + j];
  }
  int singular = 0;
  for (int i = 0; i < n; ++i) {
    int imax = 0;
    double t = 0.0;
    for (int r = i; r < n; ++r) {
      const double u = fabs(A[r][i]);
      if (u > t) { imax = r - i; t = u; }
    }
    const int i_norm_inf = i + imax;
    if (A[i_norm_inf][i] != 0.0) {
      if (i_norm_inf != i) {
        pm[i] = i_norm_inf;
        for (int c = 0; c < n; ++c) std::swap(A[i][c], A[i_norm_inf][c]);
      }
      const double rcp = 1.0 / A[i][i];
      for (int r = i + 1; r < n; ++r) A[r][i] *= rcp;
    } else if (singular == 0) {
      singular = i + 1;
    }
    for (int r = i + 1; r < n; ++r)
      for (int c = i + 1; c < n; ++c) A[r][c] -= A[r][i] * A[i][c];
  }
  double X[MD][MD];
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) X[i][j] = (i == j) ? 1.0 : 0.0;
  for (int i = 0; i < n; ++i)
    if (pm[i] != i)
      for (int c = 0; c < n; ++c) std::swap(X[i][c], X[pm[i]][c]);
  for (int l = 0; l < n; ++l) {  // unit lower
    for (int r = 0; r < n; ++r) {
      const double t = X[r][l];
      if (t != 0.0)
        for (int m = r + 1; m < n; ++m) X[m][l] -= A[m][r] * t;
    }
  }
  for (int l = n - 1; l >= 0; --l) {  // upper
    for (int r = n - 1; r >= 0; --r) {
      const double t = X[r][l] /= A[r][r];
      if (t != 0.0)
        for (int m = r - 1; m >= 0; --m) X[m][l] -= A[m][r] * t;
    }
  }
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) inv[i * n + j] = X[i][j];
  return singular;
}

/* ------------------------------------------------------------------------- */
/* The element integral: fluid<ic_bc,2> (fluid_2d.hpp:22-1135), generic in dim. */
struct Ctx {
  ElemType et;
  const gales_material_desc* mat;
  const gales_setup_desc* setup;
  int dim, nc, nd, nen;
  double u_ref_inv[MD];
  double dt;
};

struct Fluxes {
  double DUDY[MD][MD], A[3][MD][MD], K[3][3][MD][MD], S0[MD][MD];
  double U[MD], Fadv[3][MD], Fdif[3][MD], S[MD];
};

/* assign(): fluid_2d.hpp:112-121 */
void assign(const Ctx& cx, const double* v, double& p, double* vel, double& T, double* Y) {
  p = v[0];
  for (int k = 0; k < cx.dim; ++k) vel[k] = v[1 + k];
  T = v[cx.dim + 1];
  double s = 0.0;
  for (int i = 0; i < cx.nc - 1; ++i) Y[i] = v[cx.dim + 2 + i];
  for (int i = 0; i < cx.nc - 1; ++i) s += Y[i];
  Y[cx.nc - 1] = 1.0 - s;
}

/* U(): fluid_2d.hpp:372-385 */
void conservative(const Ctx& cx, const Props& pr, const double* vel, double T, const double* Y,
                  double* u) {
  const double rho = pr.rho, cv = pr.cv;
  double v2 = 0.0;
  for (int k = 0; k < cx.dim; ++k) v2 += vel[k] * vel[k];
  const double E = cv * T + 0.5 * (v2);
  u[0] = rho;
  for (int k = 0; k < cx.dim; ++k) u[1 + k] = rho * vel[k];
  u[cx.dim + 1] = rho * E;
  for (int i = 0; i < cx.nc - 1; ++i) u[cx.dim + 2 + i] = rho * Y[i];
}

/* u_ref_inv(): fluid_2d.hpp:123-135 with Y_ref = 0.5 for every component */
void u_ref_inv(Ctx& cx) {
  double Y[GALES_MAX_COMP];
  for (int c = 0; c < cx.nc; ++c) Y[c] = 0.5;
  Props pr;
  properties(*cx.mat, cx.setup->p_ref, cx.setup->T_ref, Y, pr);
  double u[MD];
  conservative(cx, pr, cx.setup->v_ref, cx.setup->T_ref, Y, u);
  for (int i = 0; i < cx.nd; ++i) cx.u_ref_inv[i] = (u[i] < TOL) ? 0.0 : 1.0 / u[i];
}

/* matrix-vector product in uBLAS order */
inline void mv(int n, const double M[MD][MD], const double* x, double* y) {
  for (int i = 0; i < n; ++i) {
    double t = 0.0;
    for (int j = 0; j < n; ++j) t += M[i][j] * x[j];
    y[i] = t;
  }
}

/* flux_matrices_and_vectors(): fluid_2d.hpp:391-603 */
void fluxes(const Ctx& cx, const Props& pr, double p, const double* vel, double T, const double* Y,
            const double dI[3][MD], Fluxes& f) {
  const int dim = cx.dim, nc = cx.nc, nd = cx.nd;
  const int E_ = dim + 1, T_ = dim + 1;
  const double rho = pr.rho, cv = pr.cv, cp = pr.cp, alpha = pr.alpha, beta = pr.beta, mu = pr.mu,
               kappa = pr.kappa;
  double v2 = 0.0;
  for (int k = 0; k < dim; ++k) v2 += vel[k] * vel[k];
  const double E = cv * T + 0.5 * (v2);
  const double drho_dp = rho * beta;
  const double drho_dT = -rho * alpha;
  const double de_dp = (beta * p - alpha * T) / rho;
  const double de_dT = cp - p * alpha / rho;
  double drho_dY[GALES_MAX_COMP], dE_dY[GALES_MAX_COMP];
  for (int i = 0; i < nc - 1; ++i) {
    drho_dY[i] = -rho * rho * (1. / pr.rho_c[i] - 1 / pr.rho_c[nc - 1]);
    dE_dY[i] = pr.e_c[i] - pr.e_c[nc - 1];
  }
  const int Yo = dim + 2;
  memset(&f, 0, sizeof(Fluxes));
  // DUDY (fluid_2d.hpp:407-441)
  f.DUDY[0][0] = drho_dp;
  f.DUDY[0][T_] = drho_dT;
  for (int c = 0; c < nc - 1; ++c) f.DUDY[0][Yo + c] = drho_dY[c];
  for (int j = 0; j < dim; ++j) {
    f.DUDY[1 + j][0] = drho_dp * vel[j];
    f.DUDY[1 + j][1 + j] = rho;
    f.DUDY[1 + j][T_] = drho_dT * vel[j];
    for (int c = 0; c < nc - 1; ++c) f.DUDY[1 + j][Yo + c] = vel[j] * drho_dY[c];
  }
  f.DUDY[E_][0] = drho_dp * E + rho * de_dp;
  for (int j = 0; j < dim; ++j) f.DUDY[E_][1 + j] = rho * vel[j];
  f.DUDY[E_][T_] = drho_dT * E + rho * de_dT;
  for (int c = 0; c < nc - 1; ++c) f.DUDY[E_][Yo + c] = E * drho_dY[c] + rho * dE_dY[c];
  for (int i = 0; i < nc - 1; ++i) {
    f.DUDY[Yo + i][0] = drho_dp * Y[i];
    f.DUDY[Yo + i][T_] = drho_dT * Y[i];
    for (int c = 0; c < nc - 1; ++c) f.DUDY[Yo + i][Yo + c] = Y[i] * drho_dY[c];
  }
  for (int i = 0; i < nc - 1; ++i) f.DUDY[Yo + i][Yo + i] += rho;
  // A_k (fluid_2d.hpp:444-524)
  for (int k = 0; k < dim; ++k) {
    double (*A)[MD] = f.A[k];
    const double vk = vel[k];
    A[0][0] = drho_dp * vk;
    A[0][1 + k] = rho;
    A[0][T_] = drho_dT * vk;
    for (int c = 0; c < nc - 1; ++c) A[0][Yo + c] = drho_dY[c] * vk;
    for (int j = 0; j < dim; ++j) {
      const double vj = vel[j];
      if (j == k) {
        A[1 + j][0] = drho_dp * vk * vk + 1.0;
        A[1 + j][1 + k] = 2.0 * rho * vk;
        A[1 + j][T_] = drho_dT * vk * vk;
        for (int c = 0; c < nc - 1; ++c) A[1 + j][Yo + c] = drho_dY[c] * vk * vk;
      } else {
        A[1 + j][0] = drho_dp * vj * vk;
        A[1 + j][1 + k] = rho * vj;
        A[1 + j][1 + j] = rho * vk;
        A[1 + j][T_] = drho_dT * vj * vk;
        for (int c = 0; c < nc - 1; ++c) A[1 + j][Yo + c] = drho_dY[c] * vj * vk;
      }
    }
    A[E_][0] = vk + vk * (drho_dp * E + rho * de_dp);
    for (int j = 0; j < dim; ++j) {
      if (j == k)
        A[E_][1 + j] = p + rho * E + rho * vk * vk;
      else
        A[E_][1 + j] = rho * vel[std::min(j, k)] * vel[std::max(j, k)];
    }
    A[E_][T_] = vk * (drho_dT * E + rho * de_dT);
    for (int c = 0; c < nc - 1; ++c) A[E_][Yo + c] = (E * drho_dY[c] + rho * dE_dY[c]) * vk;
    for (int i = 0; i < nc - 1; ++i) {
      A[Yo + i][0] = drho_dp * Y[i] * vk;
      A[Yo + i][1 + k] = rho * Y[i];
      A[Yo + i][T_] = drho_dT * Y[i] * vk;
      for (int c = 0; c < nc - 1; ++c) A[Yo + i][Yo + c] = Y[i] * drho_dY[c] * vk;
    }
    for (int i = 0; i < nc - 1; ++i) A[Yo + i][Yo + i] += rho * vk;
  }
  // K_kl (fluid_2d.hpp:531-571)
  double H[GALES_MAX_COMP];
  for (int i = 0; i < nc; ++i) H[i] = pr.e_c[i] + p / pr.rho_c[i];
  const double lambda = -2.0 * mu / 3.0;
  for (int k = 0; k < dim; ++k)
    for (int l = 0; l < dim; ++l) {
      double (*K)[MD] = f.K[k][l];
      if (k == l) {
        for (int j = 0; j < dim; ++j) K[1 + j][1 + j] = (j == k) ? lambda + 2 * mu : mu;
        for (int m = 0; m < dim; ++m)
          K[E_][1 + m] = (m == k) ? (lambda + 2 * mu) * vel[k] : mu * vel[m];
        K[E_][T_] = kappa;
        for (int i = 0; i < nc - 1; ++i) {
          K[Yo + i][Yo + i] = rho * pr.D_c[i];
          K[E_][Yo + i] = rho * pr.D_c[i] * H[i];
        }
      } else {
        K[1 + k][1 + l] = lambda;
        K[1 + l][1 + k] = mu;
        K[E_][1 + k] = mu * vel[l];
        K[E_][1 + l] = lambda * vel[k];
      }
    }
  // S0 (fluid_2d.hpp:573-575)
  for (int k = 0; k < dim; ++k) f.S0[E_][1 + k] = rho * cx.setup->gravity[k];
  conservative(cx, pr, vel, T, Y, f.U);
  // F_adv (fluid_2d.hpp:581-595)
  for (int k = 0; k < dim; ++k) {
    const double vk = vel[k];
    f.Fadv[k][0] = rho * vk;
    for (int j = 0; j < dim; ++j) f.Fadv[k][1 + j] = (j == k) ? rho * vk * vk + p : rho * vk * vel[j];
    f.Fadv[k][E_] = vk * (rho * E + p);
    for (int i = 0; i < nc - 1; ++i) f.Fadv[k][Yo + i] = rho * vk * Y[i];
  }
  // S (fluid_2d.hpp:597-599)
  for (int k = 0; k < dim; ++k) f.S[1 + k] = rho * cx.setup->gravity[k];
  double gv = 0.0;
  for (int k = 0; k < dim; ++k) gv += cx.setup->gravity[k] * vel[k];
  f.S[E_] = rho * (gv);
  // F_dif = sum_l K_kl dI_l (fluid_2d.hpp:601-602)
  for (int k = 0; k < dim; ++k) {
    for (int l = 0; l < dim; ++l) {
      double t[MD];
      mv(nd, f.K[k][l], dI[l], t);
      for (int r = 0; r < nd; ++r) f.Fdif[k][r] = (l == 0) ? t[r] : f.Fdif[k][r] + t[r];
    }
  }
}

/* Stress component that K_al(E, v_m) carries (unique j, or -1). */
int energy_source(int a, int l, int m) {
  if (l == a && m == a) return a;
  if (l == a) return m;
  if (m == a) return l;
  if (m == l) return a;
  return -1;
}

/* Boundary flux variant: fluid_2d.hpp:610-868 (generic in dim). */
void fluxes_boundary(const Ctx& cx, const Props& pr, double p, const double* vel, double T,
                     const double* Y, const double dI[3][MD], const gales_side_bc& bc, Fluxes& f) {
  fluxes(cx, pr, p, vel, T, Y, dI, f);
  const int dim = cx.dim, nc = cx.nc;
  const int E_ = dim + 1, T_ = dim + 1, Yo = dim + 2;
  const double rho = pr.rho, cv = pr.cv, cp = pr.cp, alpha = pr.alpha, beta = pr.beta;
  double v2 = 0.0;
  for (int k = 0; k < dim; ++k) v2 += vel[k] * vel[k];
  const double E = cv * T + 0.5 * (v2);
  const double de_dp = (beta * p - alpha * T) / rho;
  const double de_dT = cp - p * alpha / rho;
  double dE_dY[GALES_MAX_COMP];
  for (int i = 0; i < nc - 1; ++i) dE_dY[i] = pr.e_c[i] - pr.e_c[nc - 1];
  // prescribed mass flux (fluid_2d.hpp:627-758); U_ and DUDY_ rebuilt there are not read by RM_b
  for (int k = 0; k < dim; ++k) {
    if (!(bc.mass_flux_mask >> k & 1u)) continue;
    const double mf = bc.mass_flux[k];
    for (int r = 0; r < MD; ++r) f.Fadv[k][r] = 0.0;
    f.Fadv[k][0] = mf;
    for (int j = 0; j < dim; ++j) f.Fadv[k][1 + j] = (j == k) ? mf * vel[j] + p : mf * vel[j];
    f.Fadv[k][E_] = mf * E + p * vel[k];
    for (int i = 0; i < nc - 1; ++i) f.Fadv[k][Yo + i] = mf * Y[i];
    double (*A)[MD] = f.A[k];
    for (int r = 0; r < MD; ++r)
      for (int c = 0; c < MD; ++c) A[r][c] = 0.0;
    A[1 + k][0] = 1.0;
    A[1 + k][1 + k] = mf;
    for (int j = 0; j < dim; ++j)
      if (j != k) A[1 + j][1 + j] = mf;
    A[E_][0] = vel[k] + mf * de_dp;
    for (int j = 0; j < dim; ++j) A[E_][1 + j] = (j == k) ? p + mf * vel[k] : mf * vel[j];
    A[E_][T_] = mf * de_dT;
    for (int c = 0; c < nc - 1; ++c) A[E_][Yo + c] = mf * dE_dY[c];
    for (int i = 0; i < nc - 1; ++i) A[Yo + i][Yo + i] = mf;
  }
  // physical stresses and fluxes (fluid_2d.hpp:761-817)
  const double lambda = -2.0 * pr.mu / 3.0;
  double div = 0.0;
  for (int k = 0; k < dim; ++k) div += dI[k][1 + k];
  double tau[3][3], q[3], J[3][GALES_MAX_COMP];
  for (int k = 0; k < dim; ++k)
    for (int j = 0; j < dim; ++j) {
      if (k == j)
        tau[k][j] = lambda * (div) + 2.0 * pr.mu * dI[k][1 + k];
      else
        tau[k][j] = pr.mu * (dI[std::max(k, j)][1 + std::min(k, j)] + dI[std::min(k, j)][1 + std::max(k, j)]);
    }
  for (int k = 0; k < dim; ++k) q[k] = -pr.kappa * dI[k][T_];
  for (int k = 0; k < dim; ++k)
    for (int i = 0; i < nc - 1; ++i) J[k][i] = rho * pr.D_c[i] * dI[k][Yo + i];
  for (int k = 0; k < dim; ++k)
    for (int j = k; j < dim; ++j)
      if (bc.tau_mask >> (k * 3 + j) & 1u) { tau[k][j] = bc.tau[k * 3 + j]; tau[j][k] = tau[k][j]; }
  for (int k = 0; k < dim; ++k)
    if (bc.q_mask >> k & 1u) q[k] = bc.q[k];
  for (int i = 0; i < nc - 1; ++i)
    for (int k = 0; k < dim; ++k)
      if (bc.J_mask >> (k * 8 + i) & 1u) J[k][i] = bc.J[k][i];
  double H[GALES_MAX_COMP];
  for (int i = 0; i < nc - 1; ++i) H[i] = pr.e_c[i] + p / pr.rho_c[i];
  for (int k = 0; k < dim; ++k) {
    double HJ = 0.0;
    for (int i = 0; i < nc - 1; ++i) HJ += H[i] * J[k][i];
    for (int j = 0; j < dim; ++j) f.Fdif[k][1 + j] = tau[k][j];
    double e = 0.0;
    for (int j = 0; j < dim; ++j) e = (j == 0) ? tau[k][j] * vel[j] : e + tau[k][j] * vel[j];
    f.Fdif[k][E_] = e - q[k] - HJ;
    for (int i = 0; i < nc - 1; ++i) f.Fdif[k][Yo + i] = J[k][i];
  }
  // zero the tangent entries of overridden fluxes (fluid_2d.hpp:819-867)
  for (int k = 0; k < dim; ++k)
    for (int j = k; j < dim; ++j) {
      if (!(bc.tau_mask >> (k * 3 + j) & 1u)) continue;
      for (int pass = 0; pass < (k == j ? 1 : 2); ++pass) {
        const int a = pass == 0 ? k : j, b = pass == 0 ? j : k;
        for (int l = 0; l < dim; ++l)
          for (int m = 0; m < dim; ++m) {
            f.K[a][l][1 + b][1 + m] = 0.0;
            if (energy_source(a, l, m) == b) f.K[a][l][E_][1 + m] = 0.0;
          }
      }
    }
  for (int k = 0; k < dim; ++k)
    if (bc.q_mask >> k & 1u) f.K[k][k][E_][T_] = 0.0;
  for (int i = 0; i < nc - 1; ++i)
    for (int k = 0; k < dim; ++k)
      if (bc.J_mask >> (k * 8 + i) & 1u) {
        f.K[k][k][Yo + i][Yo + i] = 0.0;
        f.K[k][k][E_][Yo + i] = 0.0;
      }
}

/* tau_matrix(): fluid_2d.hpp:877-1022; returns LU singular flag */
int tau_matrix(const Ctx& cx, const Quad& q, const Props& pr, const double* vel,
               const double dI[3][MD], const Fluxes& f, double tau[MD][MD]) {
  const int dim = cx.dim, nc = cx.nc, nd = cx.nd;
  const int E_ = dim + 1, Yo = dim + 2;
  for (int r = 0; r < MD; ++r)
    for (int c = 0; c < MD; ++c) tau[r][c] = 0.0;
  double v_nrm = 0.0;
  for (int k = 0; k < dim; ++k) v_nrm += vel[k] * vel[k];
  v_nrm = sqrt(v_nrm);
  if (v_nrm < TOL) return 0;
  const double c = pr.c, rho = pr.rho, mu = pr.mu, cv = pr.cv, kappa = pr.kappa, dt = cx.dt;
  double del_v[3][3];
  for (int i = 0; i < dim; ++i)
    for (int j = 0; j < dim; ++j) del_v[i][j] = dI[j][1 + i];
  const double h = compute_h(q, dim, vel, del_v);
  const gales_setup_desc& s = *cx.setup;
  double trG = 0.0;
  for (int k = 0; k < dim; ++k) trG += q.G[k][k];
  int singular = 0;
  auto finish_nondiag = [&]() {
    double A0[MD * MD], inv[MD * MD];
    for (int r = 0; r < nd; ++r)
      for (int cc = 0; cc < nd; ++cc) A0[r * nd + cc] = f.DUDY[r][cc];
    singular = lu_inverse(nd, A0, inv);
    double t[MD];
    for (int i = 0; i < nd; ++i) t[i] = tau[i][i];
    for (int r = 0; r < nd; ++r)
      for (int cc = 0; cc < nd; ++cc) tau[r][cc] = inv[r * nd + cc] * t[cc];
    if (v_nrm / c < 0.1) {
      // fluid_2d.hpp:953 in its own form: pow(pow(a,-1) + pow(b,-1), -1)
      tau[0][0] = pow(pow(tau[0][0], -1.0) + pow(rho * tau[1][1] * (trG), -1.0), -1.0);
      for (int cc = 1; cc < nd; ++cc) tau[0][cc] = 0.0;
    }
  };
  if (s.tau == GALES_TAU_NON_DIAG_COMP_2001) {
    const double alpha0 = 0.0, alpha1 = 0.0;  // the reference never fills its alpha vector
    double lambda_sqr = alpha0 * (v_nrm * v_nrm + c * c) + (alpha1) * 0.5 * c * c;
    lambda_sqr += 0.5 * c * sqrt(c * c * alpha1 * alpha1 + 16 * alpha0 * alpha0 * v_nrm * v_nrm);
    if (!s.steady_state) lambda_sqr += 4 / (dt * dt);
    const double lambda = 1.0 / sqrt(lambda_sqr) + h / (2 * v_nrm);
    const double use = s.steady_state ? lambda : std::min(dt * 0.5, lambda);
    tau[0][0] = use;
    for (int k = 0; k < dim; ++k) tau[1 + k][1 + k] = std::min(use, rho * h * h / (mu * 12));
    tau[E_][E_] = std::min(use, rho * h * h * cv / (kappa * 12));
    for (int i = 0; i < nc - 1; ++i) tau[Yo + i][Yo + i] = std::min(use, h * h / (pr.D_c[i] * 12));
    finish_nondiag();
  } else if (s.tau == GALES_TAU_NON_DIAG_COMP_2019) {
    double use;
    if (s.steady_state) use = h / (2.0 * (v_nrm + c)) + h / (2.0 * v_nrm);
    else use = std::min(dt * 0.5, h / (2.0 * (v_nrm + c)) + h / (2.0 * v_nrm));
    tau[0][0] = use;
    const double tm = std::min(use, h * h * rho / (12.0 * mu));
    for (int k = 0; k < dim; ++k) tau[1 + k][1 + k] = tm;
    tau[E_][E_] = std::min(use, h * h * rho * cv / (12.0 * kappa));
    for (int i = 0; i < nc - 1; ++i) tau[Yo + i][Yo + i] = std::min(use, h * h / (12.0 * pr.D_c[i]));
    finish_nondiag();
  } else if (s.tau == GALES_TAU_DIAG_INCOMP_2007) {
    double use = 0.0;
    for (int i = 0; i < dim; ++i)
      for (int j = 0; j < dim; ++j) use += q.G[i][j] * q.G[i][j];
    double vGv = 0.0;
    {
      double Gv[3];
      for (int i = 0; i < dim; ++i) {
        double t = 0.0;
        for (int j = 0; j < dim; ++j) t += q.G[i][j] * vel[j];
        Gv[i] = t;
      }
      for (int i = 0; i < dim; ++i) vGv += vel[i] * Gv[i];
    }
    const double nu = mu / rho;
    double tau_m = vGv + 9.0 * use * (nu * nu);
    if (!s.steady_state) tau_m += 4.0 / (dt * dt);
    tau_m = 1.0 / sqrt(tau_m);
    double gg = 0.0;
    for (int i = 0; i < dim; ++i) gg += q.g[i] * q.g[i];
    const double tau_c = 1.0 / (rho * tau_m * gg);
    const double de = kappa / (rho * cv);
    double tau_e = vGv + 9.0 * use * (de * de);
    if (!s.steady_state) tau_e += 4.0 / (dt * dt);
    tau_e = 1.0 / sqrt(tau_e);
    tau[0][0] = tau_c;
    for (int k = 0; k < dim; ++k) tau[1 + k][1 + k] = tau_m / rho;
    tau[E_][E_] = tau_e / (rho * cv);
    for (int i = 0; i < nc - 1; ++i) tau[Yo + i][Yo + i] = tau_m;
  } else if (s.tau == GALES_TAU_DIAG_2014) {
    for (int i = 0; i < nd; ++i) {
      const double a0 = f.DUDY[i][i];
      const double tt = 4.0 / (dt * dt) * (a0 * a0);
      double ta = 0.0, td = 0.0;
      for (int k = 0; k < dim; ++k)
        for (int l = 0; l < dim; ++l) {
          ta += q.G[k][l] * (f.A[k][i][i] * f.A[l][i][i]);
          td += q.G[k][l] * q.G[k][l] * (f.K[k][l][i][i] * f.K[k][l][i][i]);
        }
      tau[i][i] = pow(sqrt(tt) + sqrt(ta) + sqrt(td) + 1.e-8, -1.0);   // fluid_2d.hpp:1018
    }
    tau[0][0] = pow(tau[0][0] + rho * tau[1][1] * (trG), -1.0);          // fluid_2d.hpp:1020
  }
  return singular;
}

/* dc(): fluid_2d.hpp:1027-1065 */
void dc(const Ctx& cx, const Quad& q, const double dI[3][MD], const Fluxes& f, double shock[MD][MD]) {
  const int dim = cx.dim, nd = cx.nd, nen = cx.nen;
  for (int r = 0; r < MD; ++r)
    for (int c = 0; c < MD; ++c) shock[r][c] = 0.0;
  if (!cx.setup->dc_2006) return;
  double dU[3][MD];
  for (int k = 0; k < dim; ++k) mv(nd, f.DUDY, dI[k], dU[k]);
  double s = 0.0;
  for (int k = 0; k < dim; ++k) s += dU[k][0] * dU[k][0];
  const double del_rho_nrm = sqrt(s);
  if (del_rho_nrm < TOL) return;
  double J[3];
  for (int k = 0; k < dim; ++k) J[k] = dU[k][0] / del_rho_nrm;
  double h = 0.0;
  for (int i = 0; i < nen; ++i) {
    double t = 0.0;
    for (int k = 0; k < dim; ++k) t = (k == 0) ? J[0] * q.ds[0][i] : t + J[k] * q.ds[k][i];
    h += fabs(t);
  }
  if (h > TOL) h = 1.0 / h;
  else return;
  double Z[MD];
  for (int k = 0; k < dim; ++k) {
    double t[MD];
    mv(nd, f.A[k], dI[k], t);
    for (int r = 0; r < nd; ++r) Z[r] = (k == 0) ? t[r] : Z[r] + t[r];
  }
  for (int r = 0; r < nd; ++r) Z[r] = Z[r] - f.S[r];
  auto nrm_scaled = [&](const double* x) {
    double t = 0.0;
    for (int r = 0; r < nd; ++r) {
      const double u = cx.u_ref_inv[r] * x[r];
      t += u * u;
    }
    return sqrt(t);
  };
  const double Znrm = nrm_scaled(Z);
  const double Unrm = nrm_scaled(f.U);
  double use1 = 0.0;
  for (int k = 0; k < dim; ++k) {
    const double n = nrm_scaled(dU[k]);
    use1 += n * n;
  }
  const double a = cx.setup->dc_sharp;
  double nu = 0.0;
  // fluid_2d.hpp:1055-1057 in its own form: pow(use1, -0.5)
  if (a == 1.0) nu = Znrm * h * pow(use1, -0.5);
  else if (a == 2.0) nu = Znrm * h * h / Unrm;
  else if (a == 1.5) nu = Znrm * h * (pow(use1, -0.5) + h / Unrm) / 2.0;
  for (int r = 0; r < nd; ++r)
    for (int c = 0; c < nd; ++c) shock[r][c] = cx.setup->dc_scale_fact * (nu * f.DUDY[r][c]);
}

void gather(const Ctx& cx, const gales_mesh_desc& mesh, int64_t e, const double* I, const double* P,
            double X[8][3], double* Ie, double* Pe) {
  const int nen = cx.nen, nd = cx.nd, dim = cx.dim;
  for (int a = 0; a < nen; ++a) {
    const int64_t n = mesh.conn[e * nen + a];
    for (int d = 0; d < 3; ++d) X[a][d] = d < dim ? mesh.coords[n * dim + d] : 0.0;
    for (int k = 0; k < nd; ++k) {
      Ie[a * nd + k] = I[n * nd + k];
      Pe[a * nd + k] = P[n * nd + k];
    }
  }
}

struct ElemOut {
  int status = 0;
};

/* execute_i + RM_i: fluid_2d.hpp:171-202, 251-333.  m is (nen*nd)^2 row-major, r = -r_. */
int element_interior(const Ctx& cx, const double X[8][3], const double* Ie, const double* Pe,
                     double* m, double* r, bool want_m) {
  const int dim = cx.dim, nd = cx.nd, nen = cx.nen, n = nen * nd;
  const double dt = cx.dt;
  int status = 0;
  std::vector<double> r_(n, 0.0);
  if (want_m) std::fill(m, m + (size_t)n * n, 0.0);
  for (int iq = 0; iq < cx.et.nq; ++iq) {
    Quad q;
    make_quad(cx.et, X, cx.et.gp[iq], true, q);
    if (q.neg_jac) status |= GALES_ERR_NEG_JACOBIAN;
    const double JxW = q.JxW();
    double Pq[MD], Iq[MD], dI[3][MD];
    for (int j = 0; j < nd; ++j) {
      double a = 0.0;
      for (int i = 0; i < nen; ++i) a += q.sh[i] * Pe[nd * i + j];
      Pq[j] = a;
    }
    double p, vel[3] = {0, 0, 0}, T, Y[GALES_MAX_COMP];
    assign(cx, Pq, p, vel, T, Y);
    Props pr;
    properties(*cx.mat, p, T, Y, pr);
    double U_P[MD];
    conservative(cx, pr, vel, T, Y, U_P);
    for (int j = 0; j < nd; ++j) {
      double a = 0.0;
      for (int i = 0; i < nen; ++i) a += q.sh[i] * Ie[nd * i + j];
      Iq[j] = a;
    }
    for (int k = 0; k < dim; ++k)
      for (int j = 0; j < nd; ++j) {
        double a = 0.0;
        for (int i = 0; i < nen; ++i) a += q.ds[k][i] * Ie[nd * i + j];
        dI[k][j] = a;
      }
    assign(cx, Iq, p, vel, T, Y);
    properties(*cx.mat, p, T, Y, pr, compute_shear_rate(dim, dI));   // fluid_2d.hpp:193-194
    Fluxes f;
    fluxes(cx, pr, p, vel, T, Y, dI, f);
    // Galerkin residual (fluid_2d.hpp:253-262)
    for (int b = 0; b < nen; ++b)
      for (int jb = 0; jb < nd; ++jb) {
        double& R = r_[nd * b + jb];
        R += q.sh[b] * (f.U[jb] * JxW - U_P[jb] * JxW) / dt;
        for (int k = 0; k < dim; ++k) R -= q.ds[k][b] * f.Fadv[k][jb] * JxW;
        for (int k = 0; k < dim; ++k) R += q.ds[k][b] * f.Fdif[k][jb] * JxW;
        R -= q.sh[b] * f.S[jb] * JxW;
      }
    // Galerkin tangent (fluid_2d.hpp:264-277)
    if (want_m)
      for (int b = 0; b < nen; ++b)
        for (int jb = 0; jb < nd; ++jb)
          for (int a = 0; a < nen; ++a)
            for (int ja = 0; ja < nd; ++ja) {
              double& M = m[(size_t)(nd * b + jb) * n + nd * a + ja];
              M += q.sh[b] * f.DUDY[jb][ja] * q.sh[a] * JxW / dt;
              for (int k = 0; k < dim; ++k) M -= q.ds[k][b] * f.A[k][jb][ja] * q.sh[a] * JxW;
              for (int k = 0; k < dim; ++k)
                for (int l = 0; l < dim; ++l) M += q.ds[k][b] * f.K[k][l][jb][ja] * q.ds[l][a] * JxW;
              M -= q.sh[b] * f.S0[jb][ja] * q.sh[a] * JxW;
            }
    // least squares (fluid_2d.hpp:280-305)
    double tau[MD][MD];
    if (tau_matrix(cx, q, pr, vel, dI, f, tau)) status |= GALES_ERR_SINGULAR;
    double Res[MD];
    {
      double d[MD], t0[MD];
      for (int j = 0; j < nd; ++j) d[j] = (Iq[j] - Pq[j]) / dt;
      mv(nd, f.DUDY, d, t0);
      for (int j = 0; j < nd; ++j) Res[j] = t0[j];
      for (int k = 0; k < dim; ++k) {
        mv(nd, f.A[k], dI[k], t0);
        for (int j = 0; j < nd; ++j) Res[j] = Res[j] + t0[j];
      }
      for (int j = 0; j < nd; ++j) Res[j] = Res[j] - f.S[j];
    }
    auto first_part = [&](int b, double fp[MD][MD]) {
      for (int i = 0; i < nd; ++i)
        for (int j = 0; j < nd; ++j) {
          double t = f.A[0][i][j] * q.ds[0][b];
          for (int k = 1; k < dim; ++k) t = t + f.A[k][i][j] * q.ds[k][b];
          fp[i][j] = t - f.S0[i][j] * q.sh[b];
        }
    };
    auto mm = [&](const double Aa[MD][MD], const double Bb[MD][MD], double Cc[MD][MD]) {
      for (int i = 0; i < nd; ++i)
        for (int j = 0; j < nd; ++j) {
          double t = 0.0;
          for (int k = 0; k < nd; ++k) t += Aa[i][k] * Bb[k][j];
          Cc[i][j] = t;
        }
    };
    for (int b = 0; b < nen; ++b) {
      double fp[MD][MD], fpt[MD][MD], use[MD];
      first_part(b, fp);
      mm(fp, tau, fpt);
      mv(nd, fpt, Res, use);
      for (int jb = 0; jb < nd; ++jb) r_[nd * b + jb] += use[jb] * JxW;
    }
    if (want_m) {
      for (int a = 0; a < nen; ++a) {
        double Rm[MD][MD];
        for (int i = 0; i < nd; ++i)
          for (int j = 0; j < nd; ++j) {
            double t = f.DUDY[i][j] * q.sh[a] / dt;
            for (int k = 0; k < dim; ++k) t = t + f.A[k][i][j] * q.ds[k][a];
            Rm[i][j] = t - f.S0[i][j] * q.sh[a];
          }
        for (int b = 0; b < nen; ++b) {
          double fp[MD][MD], fpt[MD][MD], use[MD][MD];
          first_part(b, fp);
          mm(fp, tau, fpt);
          mm(fpt, Rm, use);
          for (int jb = 0; jb < nd; ++jb)
            for (int ja = 0; ja < nd; ++ja) m[(size_t)(nd * b + jb) * n + nd * a + ja] += use[jb][ja] * JxW;
        }
      }
    }
    // discontinuity capturing (fluid_2d.hpp:309-331)
    double shock[MD][MD];
    dc(cx, q, dI, f, shock);
    if (cx.setup->dc_2006) {
      double app[3][MD];
      for (int k = 0; k < dim; ++k) mv(nd, shock, dI[k], app[k]);
      for (int b = 0; b < nen; ++b)
        for (int jb = 0; jb < nd; ++jb)
          for (int k = 0; k < dim; ++k) r_[nd * b + jb] += q.ds[k][b] * app[k][jb] * JxW;
      if (want_m)
        for (int b = 0; b < nen; ++b)
          for (int jb = 0; jb < nd; ++jb)
            for (int a = 0; a < nen; ++a)
              for (int ja = 0; ja < nd; ++ja)
                for (int k = 0; k < dim; ++k)
                  m[(size_t)(nd * b + jb) * n + nd * a + ja] += q.ds[k][b] * shock[jb][ja] * q.ds[k][a] * JxW;
    }
  }
  for (int i = 0; i < n; ++i) r[i] = -r_[i];
  return status;
}

/* execute_b + RM_b: fluid_2d.hpp:209-245, 341-364.  sides: flags per local side (0 = off). */
int element_boundary(const Ctx& cx, const double X[8][3], const double* Ie, const int* side_flags,
                     double* m, double* r, bool want_m) {
  const int dim = cx.dim, nd = cx.nd, nen = cx.nen, n = nen * nd;
  int status = 0;
  std::vector<double> r_(n, 0.0);
  if (want_m) std::fill(m, m + (size_t)n * n, 0.0);
  for (int s = 0; s < cx.et.nsides; ++s) {
    const int flag = side_flags[s];
    if (flag <= 0) continue;
    const gales_side_bc& bc = cx.setup->side_bc[flag < GALES_MAX_FLAGS ? flag : 0];
    for (int iq = 0; iq < cx.et.nqs; ++iq) {
      Quad q;
      make_quad(cx.et, X, cx.et.sgp[s][iq], false, q);
      if (q.neg_jac) status |= GALES_ERR_NEG_JACOBIAN;
      double Iq[MD], dI[3][MD];
      for (int j = 0; j < nd; ++j) {
        double a = 0.0;
        for (int i = 0; i < nen; ++i) a += q.sh[i] * Ie[nd * i + j];
        Iq[j] = a;
      }
      for (int k = 0; k < dim; ++k)
        for (int j = 0; j < nd; ++j) {
          double a = 0.0;
          for (int i = 0; i < nen; ++i) a += q.ds[k][i] * Ie[nd * i + j];
          dI[k][j] = a;
        }
      double p, vel[3] = {0, 0, 0}, T, Y[GALES_MAX_COMP];
      assign(cx, Iq, p, vel, T, Y);
      Props pr;
      properties(*cx.mat, p, T, Y, pr, compute_shear_rate(dim, dI));   // fluid_2d.hpp:234-235
      Fluxes f;
      fluxes_boundary(cx, pr, p, vel, T, Y, dI, bc, f);
      for (int b = 0; b < nen; ++b)
        for (int j = 0; j < nd; ++j) {
          double& R = r_[nd * b + j];
          for (int k = 0; k < dim; ++k) R += q.sh[b] * f.Fadv[k][j] * q.JNxW(k);
          for (int k = 0; k < dim; ++k) R -= q.sh[b] * f.Fdif[k][j] * q.JNxW(k);
        }
      if (want_m)
        for (int b = 0; b < nen; ++b)
          for (int jb = 0; jb < nd; ++jb)
            for (int a = 0; a < nen; ++a)
              for (int ja = 0; ja < nd; ++ja) {
                double& M = m[(size_t)(nd * b + jb) * n + nd * a + ja];
                for (int k = 0; k < dim; ++k) M += q.sh[b] * f.A[k][jb][ja] * q.JNxW(k) * q.sh[a];
                for (int k = 0; k < dim; ++k)
                  for (int l = 0; l < dim; ++l)
                    M -= q.sh[b] * f.K[k][l][jb][ja] * q.JNxW(k) * q.ds[l][a];
              }
    }
  }
  for (int i = 0; i < n; ++i) r[i] = -r_[i];
  return status;
}

/* scatter::execute (scatter.hpp:37-98): Dirichlet rows, then SumIntoGlobalValues. */
void scatter(const Ctx& cx, const gales_mesh_desc& mesh, int64_t e, double* m, double* r,
             const int64_t* row_ptr, const int32_t* col, double* vals, double* rhs) {
  const int nen = cx.nen, nd = cx.nd, n = nen * nd;
  int64_t gid[8 * MD];
  bool blocked[8 * MD];
  for (int a = 0; a < nen; ++a) {
    const int64_t node = mesh.conn[e * nen + a];
    const int flag = mesh.node_flag ? mesh.node_flag[node] : 0;
    const uint32_t mask = (flag >= 0 && flag < GALES_MAX_FLAGS) ? cx.setup->dirichlet_mask[flag] : 0u;
    for (int k = 0; k < nd; ++k) {
      gid[a * nd + k] = node * nd + k;
      blocked[a * nd + k] = (mask >> k) & 1u;
    }
  }
  if (m) {
    double avg_val = 1.0;
    for (int i = 0; i < n; ++i) avg_val += m[(size_t)i * n + i];
    avg_val /= n;
    for (int i = 0; i < n; ++i)
      if (blocked[i]) {
        for (int j = 0; j < n; ++j) m[(size_t)i * n + j] = 0.0;
        m[(size_t)i * n + i] = avg_val;
        r[i] = avg_val * 0.0;
      }
  } else {
    for (int i = 0; i < n; ++i)
      if (blocked[i]) r[i] = 0.0;
  }
  for (int i = 0; i < n; ++i) rhs[gid[i]] += r[i];
  if (!m || !vals) return;
  for (int i = 0; i < n; ++i) {
    const int64_t row = gid[i];
    const int64_t lo = row_ptr[row], hi = row_ptr[row + 1];
    for (int j = 0; j < n; ++j) {
      const int32_t c = (int32_t)gid[j];
      const int32_t* pos = std::lower_bound(col + lo, col + hi, c);
      vals[pos - col] += m[(size_t)i * n + j];
    }
  }
}

bool init_ctx(Ctx& cx, const gales_mesh_desc* mesh, const gales_material_desc* mat,
              const gales_setup_desc* setup, double dt) {
  if (!make_elem_type(mesh->dim, mesh->nen, cx.et)) return false;
  cx.mat = mat;
  cx.setup = setup;
  cx.dim = mesh->dim;
  cx.nc = mat->nb_comp;
  cx.nd = 2 + cx.dim + cx.nc - 1;
  cx.nen = mesh->nen;
  cx.dt = dt;
  if (cx.nd > MD || cx.nc < 1 || cx.nc > GALES_MAX_COMP) return false;
  for (int i = 0; i < MD; ++i) cx.u_ref_inv[i] = 0.0;
  if (setup->dc_2006) u_ref_inv(cx);
  return true;
}

/* element -> local side flags (mesh.hpp:409-446 data) */
void side_table(const gales_mesh_desc& mesh, int nsides, std::vector<int32_t>& out) {
  out.assign((size_t)mesh.n_elements * nsides, 0);
  for (int64_t s = 0; s < mesh.n_bd_sides; ++s)
    out[(size_t)mesh.bd_side_el[s] * nsides + mesh.bd_side_local[s]] = mesh.bd_side_flag[s];
}

}  // namespace

extern "C" {

/* compute_shear_rate at a point from dI[k][j] = d I_j / d x_k (3 x GALES_MAX_ND). */
double gor_shear_rate(int dim, const double* dI) {
  double g[3][MD];
  for (int k = 0; k < 3; ++k)
    for (int j = 0; j < MD; ++j) g[k][j] = dI[k * MD + j];
  return compute_shear_rate(dim, g);
}

int gor_properties(const gales_material_desc* mat, double p, double T, const double* Y, double* out) {
  Props pr;
  properties(*mat, p, T, Y, pr);
  const double v[9] = {pr.rho, pr.mu, pr.cp, pr.cv, pr.kappa, pr.D, pr.c, pr.alpha, pr.beta};
  for (int i = 0; i < 9; ++i) out[i] = v[i];
  for (int c = 0; c < mat->nb_comp; ++c) {
    out[9 + 3 * c] = pr.rho_c[c];
    out[10 + 3 * c] = pr.e_c[c];
    out[11 + 3 * c] = pr.D_c[c];
  }
  return 0;
}

int gor_inverse(int n, const double* A, double* inv) { return lu_inverse(n, A, inv); }

/* out: sh[nen], dsh[dim][nen], J, JxW, G[dim][dim], g[dim], JN[dim] */
int gor_quad(int dim, int nen, const double* xe, const double* pt, int boundary, double* out) {
  ElemType et;
  if (!make_elem_type(dim, nen, et)) return GALES_ERR_UNSUPPORTED;
  double X[8][3] = {};
  for (int a = 0; a < nen; ++a)
    for (int d = 0; d < dim; ++d) X[a][d] = xe[a * dim + d];
  Quad q;
  make_quad(et, X, pt, !boundary, q);
  int o = 0;
  for (int a = 0; a < nen; ++a) out[o++] = q.sh[a];
  for (int k = 0; k < dim; ++k)
    for (int a = 0; a < nen; ++a) out[o++] = q.ds[k][a];
  out[o++] = q.J;
  out[o++] = q.JxW();
  for (int i = 0; i < dim; ++i)
    for (int j = 0; j < dim; ++j) out[o++] = q.G[i][j];
  for (int i = 0; i < dim; ++i) out[o++] = q.g[i];
  for (int i = 0; i < dim; ++i) out[o++] = q.JN[i] * q.W_bd;
  return q.neg_jac ? GALES_ERR_NEG_JACOBIAN : 0;
}

/* Gauss tables: pts[nq][3], side nodes, side points.  Returns nq. */
int gor_gauss(int dim, int nen, double* gp, int32_t* sides, double* sgp, int32_t* counts) {
  ElemType et;
  if (!make_elem_type(dim, nen, et)) return -1;
  for (int i = 0; i < et.nq; ++i)
    for (int d = 0; d < 3; ++d) gp[i * 3 + d] = et.gp[i][d];
  for (int s = 0; s < et.nsides; ++s)
    for (int j = 0; j < et.nsn; ++j) sides[s * et.nsn + j] = et.side[s][j];
  for (int s = 0; s < et.nsides; ++s)
    for (int j = 0; j < et.nqs; ++j)
      for (int d = 0; d < 3; ++d) sgp[(s * et.nqs + j) * 3 + d] = et.sgp[s][j][d];
  counts[0] = et.nq; counts[1] = et.nsides; counts[2] = et.nsn; counts[3] = et.nqs;
  return et.nq;
}

/* Node graph and scalar CSR of linear_system.hpp:46-63 on one rank. */
int64_t gor_pattern_count(const gales_mesh_desc* mesh, int nd, int64_t* nnz_nodes) {
  const int nen = mesh->nen;
  std::vector<std::vector<int32_t>> adj(mesh->n_nodes);
  for (int64_t e = 0; e < mesh->n_elements; ++e)
    for (int a = 0; a < nen; ++a)
      for (int b = 0; b < nen; ++b) adj[mesh->conn[e * nen + a]].push_back(mesh->conn[e * nen + b]);
  int64_t nn = 0;
  for (auto& v : adj) {
    std::sort(v.begin(), v.end());
    v.erase(std::unique(v.begin(), v.end()), v.end());
    nn += (int64_t)v.size();
  }
  *nnz_nodes = nn;
  return nn * nd * nd;
}

int gor_pattern(const gales_mesh_desc* mesh, int nd, int64_t* node_row_ptr, int32_t* node_col,
                int64_t* row_ptr, int32_t* col) {
  const int nen = mesh->nen;
  std::vector<std::vector<int32_t>> adj(mesh->n_nodes);
  for (int64_t e = 0; e < mesh->n_elements; ++e)
    for (int a = 0; a < nen; ++a)
      for (int b = 0; b < nen; ++b) adj[mesh->conn[e * nen + a]].push_back(mesh->conn[e * nen + b]);
  int64_t pos = 0;
  node_row_ptr[0] = 0;
  for (int64_t i = 0; i < mesh->n_nodes; ++i) {
    auto& v = adj[i];
    std::sort(v.begin(), v.end());
    v.erase(std::unique(v.begin(), v.end()), v.end());
    for (auto c : v) node_col[pos++] = c;
    node_row_ptr[i + 1] = pos;
  }
  if (row_ptr) {
    int64_t p = 0;
    row_ptr[0] = 0;
    for (int64_t i = 0; i < mesh->n_nodes; ++i)
      for (int k = 0; k < nd; ++k) {
        for (int64_t t = node_row_ptr[i]; t < node_row_ptr[i + 1]; ++t)
          for (int kk = 0; kk < nd; ++kk) {
            if (col) col[p] = node_col[t] * nd + kk;
            ++p;
          }
        row_ptr[i * nd + k + 1] = p;
      }
  }
  return 0;
}

/* Greedy colouring in element order: smallest colour unused by any element sharing a node. */
int gor_colouring(const gales_mesh_desc* mesh, int32_t* colour, int32_t* n_colours) {
  const int nen = mesh->nen;
  std::vector<std::vector<int64_t>> node_el(mesh->n_nodes);
  for (int64_t e = 0; e < mesh->n_elements; ++e)
    for (int a = 0; a < nen; ++a) node_el[mesh->conn[e * nen + a]].push_back(e);
  int32_t nc = 0;
  std::vector<int64_t> mark(1024, -1);
  for (int64_t e = 0; e < mesh->n_elements; ++e) colour[e] = -1;
  for (int64_t e = 0; e < mesh->n_elements; ++e) {
    for (int a = 0; a < nen; ++a)
      for (int64_t o : node_el[mesh->conn[e * nen + a]])
        if (colour[o] >= 0) {
          if ((size_t)colour[o] >= mark.size()) mark.resize(colour[o] * 2 + 1, -1);
          mark[colour[o]] = e;
        }
    int32_t c = 0;
    while ((size_t)c < mark.size() && mark[c] == e) ++c;
    if ((size_t)c >= mark.size()) mark.resize(c * 2 + 1, -1);
    colour[e] = c;
    nc = std::max(nc, c + 1);
  }
  *n_colours = nc;
  return 0;
}

/* One element's local block and residual before scatter (which: 0 interior, 1 boundary). */
int gor_element(const gales_mesh_desc* mesh, const gales_material_desc* mat,
                const gales_setup_desc* setup, const double* I, const double* P, double dt,
                int64_t e, int which, double* m, double* r) {
  Ctx cx;
  if (!init_ctx(cx, mesh, mat, setup, dt)) return GALES_ERR_UNSUPPORTED;
  double X[8][3];
  double Ie[8 * MD], Pe[8 * MD];
  gather(cx, *mesh, e, I, P, X, Ie, Pe);
  if (which == 0) return element_interior(cx, X, Ie, Pe, m, r, m != nullptr);
  std::vector<int32_t> st;
  side_table(*mesh, cx.et.nsides, st);
  int flags[6] = {0, 0, 0, 0, 0, 0};
  for (int s = 0; s < cx.et.nsides; ++s) flags[s] = st[(size_t)e * cx.et.nsides + s];
  return element_boundary(cx, X, Ie, flags, m, r, m != nullptr);
}

/* adaptive_time_criteria::f_mc (adaptive_time_step.hpp:183-260): per element, the first
 * smallest over its Gauss points of CFL/use, use = 2 max(2 mu/rho, kappa/(rho cv))/h^2
 * + v_tau/h with v_tau = |v|, or for Mach > 0.3 the acoustic form of 230-234; 1.2 dt
 * where |v| < DBL_EPSILON.  compute_del_v (356-374): del_v(i, j) = dI_j[1+i]. */
int gor_adaptive_dt(const gales_mesh_desc* mesh, const gales_material_desc* mat, const gales_setup_desc* setup,
                    const double* I, double dt, double cfl, double* dt_el) {
  Ctx cx;
  if (!init_ctx(cx, mesh, mat, setup, dt)) return GALES_ERR_UNSUPPORTED;
  const int dim = cx.dim, nd = cx.nd, nen = cx.nen;
  for (int64_t e = 0; e < mesh->n_elements; ++e) {
    double X[8][3];
    double Ie[8 * MD], Pe[8 * MD];
    gather(cx, *mesh, e, I, I, X, Ie, Pe);
    std::vector<double> dt_gp;
    for (int iq = 0; iq < cx.et.nq; ++iq) {
      Quad q;
      make_quad(cx.et, X, cx.et.gp[iq], true, q);
      double Iq[MD], dI[3][MD];
      for (int j = 0; j < nd; ++j) {
        double a = 0.0;
        for (int i = 0; i < nen; ++i) a += q.sh[i] * Ie[nd * i + j];
        Iq[j] = a;
      }
      for (int k = 0; k < dim; ++k)
        for (int j = 0; j < nd; ++j) {
          double a = 0.0;
          for (int i = 0; i < nen; ++i) a += q.ds[k][i] * Ie[nd * i + j];
          dI[k][j] = a;
        }
      double p, vel[3] = {0, 0, 0}, T, Y[GALES_MAX_COMP];
      assign(cx, Iq, p, vel, T, Y);
      Props pr;
      properties(*mat, p, T, Y, pr);
      double v_nrm = 0.0;
      for (int k = 0; k < dim; ++k) v_nrm += vel[k] * vel[k];
      v_nrm = sqrt(v_nrm);
      if (v_nrm < TOL) {
        dt_gp.push_back(1.2 * dt);
        continue;
      }
      double del_v[3][3];
      for (int i = 0; i < dim; ++i)
        for (int j = 0; j < dim; ++j) del_v[i][j] = dI[j][1 + i];
      const double h = compute_h(q, dim, vel, del_v);
      const double c = pr.c;
      double v_tau = v_nrm;
      const double Mach = v_nrm / c;
      if (Mach > 0.3) {
        if (dim == 2) v_tau = sqrt(v_nrm * v_nrm + 1.5 * c * c + c * sqrt(16.0 * v_nrm * v_nrm + c * c));
        else v_tau = sqrt(v_nrm * v_nrm + 2.0 * c * c + c * sqrt(4.0 * v_nrm * v_nrm + c * c));
      }
      const double use = 2.0 * std::max(2.0 * pr.mu / pr.rho, pr.kappa / (pr.rho * pr.cv)) / (h * h) + v_tau / h;
      dt_gp.push_back(cfl / use);
    }
    dt_el[e] = *std::min_element(dt_gp.begin(), dt_gp.end());
  }
  return 0;
}

/* fluid_assembly::execute (fluid_assembly.hpp:39-68).  vals may be NULL (residual only).
 * With colour != NULL, colours run in order and the elements of one colour run on
 * nthreads threads (no two share a node); otherwise elements run serially in order. */
int gor_assemble(const gales_mesh_desc* mesh, const gales_material_desc* mat,
                 const gales_setup_desc* setup, const double* I, const double* P, double dt,
                 const int64_t* row_ptr, const int32_t* col, double* vals, double* rhs,
                 int nthreads, const int32_t* colour, int32_t n_colours, int64_t* first_bad) {
  Ctx cx;
  if (!init_ctx(cx, mesh, mat, setup, dt)) return GALES_ERR_UNSUPPORTED;
  const int nd = cx.nd, n = cx.nen * nd;
  const int64_t n_rows = mesh->n_nodes * nd;
  if (vals) std::fill(vals, vals + row_ptr[n_rows], 0.0);
  std::fill(rhs, rhs + n_rows, 0.0);
  std::vector<int32_t> st;
  side_table(*mesh, cx.et.nsides, st);
  int status = 0;
  int64_t bad = -1;
  auto do_element = [&](int64_t e, std::vector<double>& m, std::vector<double>& r, int& st_out,
                        int64_t& bad_out) {
    double X[8][3];
    double Ie[8 * MD], Pe[8 * MD];
    gather(cx, *mesh, e, I, P, X, Ie, Pe);
    int s = element_interior(cx, X, Ie, Pe, m.data(), r.data(), vals != nullptr);
    scatter(cx, *mesh, e, vals ? m.data() : nullptr, r.data(), row_ptr, col, vals, rhs);
    if (mesh->el_on_boundary && mesh->el_on_boundary[e]) {
      int flags[6] = {0, 0, 0, 0, 0, 0};
      for (int k = 0; k < cx.et.nsides; ++k) flags[k] = st[(size_t)e * cx.et.nsides + k];
      s |= element_boundary(cx, X, Ie, flags, m.data(), r.data(), vals != nullptr);
      scatter(cx, *mesh, e, vals ? m.data() : nullptr, r.data(), row_ptr, col, vals, rhs);
    }
    if (s) {
      st_out |= s;
      if (bad_out < 0 || e < bad_out) bad_out = e;
    }
  };
  if (!colour) {
    std::vector<double> m((size_t)n * n), r(n);
    for (int64_t e = 0; e < mesh->n_elements; ++e) do_element(e, m, r, status, bad);
  } else {
    std::vector<std::vector<int64_t>> by(n_colours);
    for (int64_t e = 0; e < mesh->n_elements; ++e) by[colour[e]].push_back(e);
    if (nthreads < 1) nthreads = 1;
    for (int c = 0; c < n_colours; ++c) {
      const auto& list = by[c];
      const int64_t cnt = (int64_t)list.size();
#pragma omp parallel num_threads(nthreads)
      {
        std::vector<double> m((size_t)n * n), r(n);
        int s_loc = 0;
        int64_t bad_loc = -1;
#pragma omp for schedule(dynamic, 64)
        for (int64_t i = 0; i < cnt; ++i) do_element(list[i], m, r, s_loc, bad_loc);
#pragma omp critical
        {
          status |= s_loc;
          if (bad_loc >= 0 && (bad < 0 || bad_loc < bad)) bad = bad_loc;
        }
      }
    }
  }
  if (first_bad) *first_bad = bad;
  return status;
}

}  // extern "C"
