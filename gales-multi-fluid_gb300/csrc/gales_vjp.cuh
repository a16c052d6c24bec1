// Exact vector-Jacobian product of the assembled rhs, point level.
//
// The interior element residual of fluid_2d.hpp:251-305 at one quadrature point is
//   r_b += JxW [ N_b phi0 + sum_d dN_b/dx_d phi_d ]            with
//   phi0  = (U - U_P)/dt - S - S0 tau Res
//   phi_d = F_dif,d - F_adv,d + nu DUDY dI/dx_d + A_d tau Res
// (the least-squares weight FPT_b = (sum_d dN_b/dx_d A_d - N_b S0) tau split by node
// factor).  point_forward evaluates (phi0, phi_d) from the interpolated state Iq, its
// gradient dI and the previous level Pq in FP64 with every coefficient a function of
// the state and of the material parameters theta_c = (density parameter, mu_c, cp_c);
// point_reverse propagates cotangents (phi0_bar, phi_d_bar) back to Iq, dI and theta
// by hand-written reverse mode through tau (with compute_h and the DUDY inverse),
// the dc viscosity, the mixture EOS and U_P.  Nothing is stored between calls: the
// caller recomputes the point from the state.  The dc scaling u_ref_inv is itself a
// function of theta (fluid_2d.hpp:123-135, the mixture at p_ref, T_ref, Y_ref); its
// cotangent is returned in urib for the caller to fold into theta.
//
// Parameterisation (the derivative's meaning):
//   custom chemical (chemicals.hpp:19-49): theta = (rho_c, mu_c, cp_c); alpha, beta,
//     kappa fixed; cv_c = cp_c - T alpha^2/(rho_c beta) (beta != 0), else cp_c.
//   ideal gas (chemicals.hpp:198-271): theta = (M_c, mu_c, cp_c) with R_c = R_u/M_c,
//     cv_c = cp_c - R_c, gamma_c = cp_c/cv_c; kappa fixed.
// Everything here is __host__ __device__ so the same code can be checked on the CPU.
#pragma once

#include <cmath>

#include "gales_physics.cuh"

namespace gales {
namespace vjp {

#define GV_HD __host__ __device__ __forceinline__

constexpr double kRu = 8.314462;  // chemicals.hpp:229

template <int DIM, int NC>
struct Ctx {
  static constexpr int ND = Layout<DIM, NC>::ND;
  const DevChem* ch;
  double dt, inv_dt, dc_sharp, dc_scale;
  double gravity[3];
  const double* u_ref_inv;
  int tau, dc_2006, steady;
};

// Per point geometry used by tau and dc.
template <int DIM, int NEN>
struct PGeo {
  double G[DIM][DIM], trG;
  double ds[DIM][NEN];
};

template <int DIM>
GV_HD double dot(const double* a, const double* b) {
  double s = 0.0;
#pragma unroll
  for (int i = 0; i < DIM; ++i) s += a[i] * b[i];
  return s;
}

// ---------------------------------------------------------------------------
// Mixture EOS (fluid_properties.hpp:199-227) with its tape.
template <int NC>
struct Mix {
  double Y[NC];
  double r[NC], cvc[NC], c2t[NC];   // rho_c, cv_c, Y-free sound-speed term 1/(rho_c^2 s_c^2)
  double ac[NC], bc[NC];            // alpha_c, beta_c
  double irho, rho, mu, cp, cv, kappa, c2, c, alpha, beta;
};

// Component values at (p, T): rho_c, cv_c, 1/(rho_c^2 s_c^2), alpha_c, beta_c.
GV_HD void comp_eval(const DevChem& q, double p, double T, double& r, double& cvc, double& c2t, double& a,
                     double& b) {
  if (q.kind == GALES_CH_CUSTOM) {
    r = q.rho; a = q.alpha; b = q.beta;
    if (b == 0.0) {
      cvc = q.cp;
      c2t = 1.e-40 / (r * r);
    } else {
      cvc = q.cp - T * a * a / (r * b);
      c2t = b / r;                       // 1/(r^2 s^2) with s^2 = 1/(r b)
    }
  } else {
    const double R = q.R, g = q.cp / (q.cp - R);
    r = p / (R * T);
    a = 1.0 / T;
    b = 1.0 / p;
    cvc = q.cp - R;
    c2t = 1.0 / (r * r * g * R * T);
  }
}

// Adjoint of comp_eval: cotangents of (r, cvc, c2t, a, b) -> p, T and theta_c.
GV_HD void comp_rev(const DevChem& q, double p, double T, double rb, double cvb, double c2b, double ab, double bb,
                    double& pb, double& Tb, double* th) {
  if (q.kind == GALES_CH_CUSTOM) {
    const double r = q.rho, a = q.alpha, b = q.beta;
    th[2] += cvb;                                          // d cv/d cp
    if (b == 0.0) {
      th[0] += c2b * (-2.e-40 / (r * r * r));
    } else {
      Tb += cvb * (-a * a / (r * b));
      th[0] += cvb * (T * a * a / (r * r * b)) + c2b * (-b / (r * r));
    }
    th[0] += rb;
  } else {
    const double R = q.R, cp = q.cp, cv = cp - R, g = cp / cv;
    const double r = p / (R * T);
    // r = p/(R T)
    pb += rb / (R * T);
    Tb += rb * (-r / T);
    double Rb = rb * (-r / R);
    Tb += ab * (-1.0 / (T * T));
    pb += bb * (-1.0 / (p * p));
    // cv = cp - R
    th[2] += cvb;
    Rb -= cvb;
    // c2t = 1/(r^2 g R T) = R T/(g p^2) = R T cv/(cp p^2)
    const double c2t = R * T * cv / (cp * p * p);
    pb += c2b * (-2.0 * c2t / p);
    Tb += c2b * (c2t / T);
    // d/dR of R (cp - R) = cp - 2R ; d/dcp of cv/cp = R/cp^2
    Rb += c2b * (T * (cp - 2.0 * R) / (cp * p * p));
    th[2] += c2b * (R * T * R / (cp * cp * p * p));
    (void)g;
    // theta_0 = M, R = R_u/M: dR/dM = -R^2/R_u
    th[0] += Rb * (-R * R / kRu);
  }
}

template <int NC>
GV_HD void mix_forward(const DevChem* ch, double p, double T, const double* Y, Mix<NC>& m) {
  double irho = 0.0, mu = 0.0, cp = 0.0, cv = 0.0, kappa = 0.0, c2 = 0.0;
#pragma unroll
  for (int c = 0; c < NC; ++c) {
    m.Y[c] = Y[c];
    comp_eval(ch[c], p, T, m.r[c], m.cvc[c], m.c2t[c], m.ac[c], m.bc[c]);
    irho += Y[c] / m.r[c];
    mu += Y[c] * ch[c].mu;
    cp += Y[c] * ch[c].cp;
    cv += Y[c] * m.cvc[c];
    kappa += Y[c] * ch[c].kappa;
    c2 += Y[c] * m.c2t[c];
  }
  m.irho = irho;
  m.rho = 1.0 / irho;
  m.mu = mu; m.cp = cp; m.cv = cv; m.kappa = kappa; m.c2 = c2;
  m.c = irho / sqrt(c2);
  double al = 0.0, be = 0.0;
#pragma unroll
  for (int c = 0; c < NC; ++c) {
    al += Y[c] * m.ac[c] / m.r[c];
    be += Y[c] * m.bc[c] / m.r[c];
  }
  m.alpha = m.rho * al;
  m.beta = m.rho * be;
}

// Cotangents of the mixture outputs.
struct MixBar {
  double rho, mu, cp, cv, kappa, c, alpha, beta;
};

template <int NC>
GV_HD void mix_reverse(const DevChem* ch, double p, double T, const Mix<NC>& m, const MixBar& o, const double* rcb,
                       const double* cvcb, double& pb, double& Tb, double* Yb, double* th) {
  // outputs: rho = 1/irho, c = irho/sqrt(c2), alpha = rho*al, beta = rho*be (+ per-component
  // rho_c and cv_c cotangents rcb, cvcb from the coefficient layer)
  double al = m.alpha / m.rho, be = m.beta / m.rho;
  double rhob = o.rho + o.alpha * al + o.beta * be;
  const double alb = o.alpha * m.rho, beb = o.beta * m.rho;
  double irhob = -rhob * m.rho * m.rho + o.c / sqrt(m.c2);
  const double c2b = o.c * (-0.5 * m.irho / (m.c2 * sqrt(m.c2)));
#pragma unroll
  for (int c = 0; c < NC; ++c) {
    const double Yc = m.Y[c], r = m.r[c];
    double rb = rcb ? rcb[c] : 0.0;
    double cvb = (cvcb ? cvcb[c] : 0.0) + o.cv * Yc;
    double c2tb = c2b * Yc;
    double ab = alb * Yc / r, bb = beb * Yc / r;
    rb += -irhob * Yc / (r * r) - alb * Yc * m.ac[c] / (r * r) - beb * Yc * m.bc[c] / (r * r);
    Yb[c] += irhob / r + o.mu * ch[c].mu + o.cp * ch[c].cp + o.cv * m.cvc[c] + o.kappa * ch[c].kappa +
             c2b * m.c2t[c] + alb * m.ac[c] / r + beb * m.bc[c] / r;
    th[3 * c + 1] += o.mu * Yc;
    th[3 * c + 2] += o.cp * Yc;
    comp_rev(ch[c], p, T, rb, cvb, c2tb, ab, bb, pb, Tb, th + 3 * c);
  }
}

// ---------------------------------------------------------------------------
// Coefficient scalars (fluid_2d.hpp:393-404, 531-533) and the structure vectors of
// DUDY = w r0^T + rho M: w = (1, v, E, Y), r0 its first row, mE the energy row of M,
// u' = U + p e_E.
template <int DIM, int NC>
struct Cf {
  using L = Layout<DIM, NC>;
  static constexpr int ND = L::ND;
  double p, v[DIM], T, Y[NC];
  double rho, E, drho_dp, drho_dT, de_dp, de_dT, mu, lam, kappa, cv, cp;
  double drho_dY[L::NYA], dE_dY[L::NYA], H[L::NYA], rhoD[L::NYA], rhoDH[L::NYA];
  double w[ND], r0[ND], mE[ND];
};

template <int DIM, int NC>
struct CfBar {
  using L = Layout<DIM, NC>;
  static constexpr int ND = L::ND;
  double p, v[DIM], T, Y[NC];
  double rho, E, drho_dp, drho_dT, de_dp, de_dT, mu, lam, kappa;
  double drho_dY[L::NYA], dE_dY[L::NYA], rhoD[L::NYA], rhoDH[L::NYA];
  double w[ND], r0[ND], mE[ND];
};

template <int DIM, int NC>
GV_HD void coef_forward(const Mix<NC>& m, const DevChem* ch, double p, const double* v, double T, Cf<DIM, NC>& c) {
  using L = Layout<DIM, NC>;
  c.p = p; c.T = T;
#pragma unroll
  for (int k = 0; k < DIM; ++k) c.v[k] = v[k];
#pragma unroll
  for (int i = 0; i < NC; ++i) c.Y[i] = m.Y[i];
  const double rho = m.rho;
  c.rho = rho; c.cv = m.cv; c.cp = m.cp;
  c.E = m.cv * T + 0.5 * dot<DIM>(v, v);
  c.drho_dp = rho * m.beta;
  c.drho_dT = -rho * m.alpha;
  c.de_dp = (m.beta * p - m.alpha * T) / rho;
  c.de_dT = m.cp - p * m.alpha / rho;
  c.mu = m.mu;
  c.lam = -2.0 * m.mu / 3.0;
  c.kappa = m.kappa;
#pragma unroll
  for (int i = 0; i < NC - 1; ++i) {
    c.drho_dY[i] = -rho * rho * (1.0 / m.r[i] - 1.0 / m.r[NC - 1]);
    c.dE_dY[i] = m.cvc[i] * T - m.cvc[NC - 1] * T;
    c.H[i] = m.cvc[i] * T + p / m.r[i];
    c.rhoD[i] = rho * ch[i].D;
    c.rhoDH[i] = c.rhoD[i] * c.H[i];
  }
  c.w[0] = 1.0; c.r0[0] = c.drho_dp; c.mE[0] = c.de_dp;
#pragma unroll
  for (int k = 0; k < DIM; ++k) { c.w[1 + k] = v[k]; c.r0[1 + k] = 0.0; c.mE[1 + k] = v[k]; }
  c.w[L::iT] = c.E; c.r0[L::iT] = c.drho_dT; c.mE[L::iT] = c.de_dT;
#pragma unroll
  for (int i = 0; i < NC - 1; ++i) {
    c.w[L::iY + i] = m.Y[i]; c.r0[L::iY + i] = c.drho_dY[i]; c.mE[L::iY + i] = c.dE_dY[i];
  }
}

template <int DIM, int NC>
GV_HD void cfbar_zero(CfBar<DIM, NC>& b) {
  double* x = reinterpret_cast<double*>(&b);
  for (unsigned i = 0; i < sizeof(CfBar<DIM, NC>) / sizeof(double); ++i) x[i] = 0.0;
}

// Fold the structure-vector cotangents (w, r0, mE) into the scalar ones.
template <int DIM, int NC>
GV_HD void cfbar_fold(CfBar<DIM, NC>& b) {
  using L = Layout<DIM, NC>;
  b.drho_dp += b.r0[0]; b.de_dp += b.mE[0];
#pragma unroll
  for (int k = 0; k < DIM; ++k) b.v[k] += b.w[1 + k] + b.mE[1 + k];
  b.E += b.w[L::iT]; b.drho_dT += b.r0[L::iT]; b.de_dT += b.mE[L::iT];
#pragma unroll
  for (int i = 0; i < NC - 1; ++i) {
    b.Y[i] += b.w[L::iY + i]; b.drho_dY[i] += b.r0[L::iY + i]; b.dE_dY[i] += b.mE[L::iY + i];
  }
}

// Coefficient layer reverse: scalar cotangents -> mixture cotangents, per-component
// rho_c / cv_c cotangents, and direct state cotangents (p, v, T).
template <int DIM, int NC>
GV_HD void coef_reverse(const Mix<NC>& m, const DevChem* ch, const Cf<DIM, NC>& c, const CfBar<DIM, NC>& b,
                        MixBar& o, double* rcb, double* cvcb, double& pb, double* vb, double& Tb, double* Yb) {
  const double rho = m.rho, p = c.p, T = c.T;
  o = MixBar{0, 0, 0, 0, 0, 0, 0, 0};
#pragma unroll
  for (int i = 0; i < NC; ++i) { rcb[i] = 0.0; cvcb[i] = 0.0; }
  // E = cv T + |v|^2/2
  o.cv += b.E * T; Tb += b.E * m.cv;
#pragma unroll
  for (int k = 0; k < DIM; ++k) vb[k] += b.E * c.v[k] + b.v[k];
  pb += b.p; Tb += b.T;
#pragma unroll
  for (int i = 0; i < NC; ++i) Yb[i] += b.Y[i];
  o.rho += b.rho;
  // drho_dp = rho beta, drho_dT = -rho alpha
  o.rho += b.drho_dp * m.beta - b.drho_dT * m.alpha;
  o.beta += b.drho_dp * rho;
  o.alpha -= b.drho_dT * rho;
  // de_dp = (beta p - alpha T)/rho
  o.beta += b.de_dp * p / rho;
  o.alpha -= b.de_dp * T / rho;
  pb += b.de_dp * m.beta / rho;
  Tb -= b.de_dp * m.alpha / rho;
  o.rho -= b.de_dp * (m.beta * p - m.alpha * T) / (rho * rho);
  // de_dT = cp - p alpha/rho
  o.cp += b.de_dT;
  pb -= b.de_dT * m.alpha / rho;
  o.alpha -= b.de_dT * p / rho;
  o.rho += b.de_dT * p * m.alpha / (rho * rho);
  o.mu += b.mu - 2.0 * b.lam / 3.0;
  o.kappa += b.kappa;
#pragma unroll
  for (int i = 0; i < NC - 1; ++i) {
    const int n = NC - 1;
    // drho_dY = -rho^2 (1/r_i - 1/r_n)
    o.rho += b.drho_dY[i] * (-2.0 * rho * (1.0 / m.r[i] - 1.0 / m.r[n]));
    rcb[i] += b.drho_dY[i] * (rho * rho / (m.r[i] * m.r[i]));
    rcb[n] -= b.drho_dY[i] * (rho * rho / (m.r[n] * m.r[n]));
    // dE_dY = (cv_i - cv_n) T
    cvcb[i] += b.dE_dY[i] * T;
    cvcb[n] -= b.dE_dY[i] * T;
    Tb += b.dE_dY[i] * (m.cvc[i] - m.cvc[n]);
    // rhoD = rho D, rhoDH = rho D H with H = cv_i T + p/r_i
    o.rho += b.rhoD[i] * ch[i].D + b.rhoDH[i] * ch[i].D * c.H[i];
    const double Hb = b.rhoDH[i] * c.rhoD[i];
    cvcb[i] += Hb * T;
    Tb += Hb * m.cvc[i];
    pb += Hb / m.r[i];
    rcb[i] -= Hb * p / (m.r[i] * m.r[i]);
  }
}

// ---------------------------------------------------------------------------
// Bilinear forms with DUDY and A_d and their adjoints (weight s):
//   x^T DUDY y = (x.w)(r0.y) + rho (sum_{r in v,Y} x_r y_r + x_E mE.y)
//   x^T A_d y  = v_d x^T DUDY y + (x.u') y_{v_d} + (x_{v_d} + v_d x_E) y_p
template <int DIM, int NC>
GV_HD double xDy(const Cf<DIM, NC>& c, const double* x, const double* y) {
  using L = Layout<DIM, NC>;
  constexpr int ND = L::ND;
  double xw = 0.0, ry = 0.0, my = 0.0, d = 0.0;
#pragma unroll
  for (int j = 0; j < ND; ++j) {
    xw += x[j] * c.w[j];
    ry += c.r0[j] * y[j];
    my += c.mE[j] * y[j];
    if (j >= 1 && j != L::iT) d += x[j] * y[j];
  }
  return xw * ry + c.rho * (d + x[L::iT] * my);
}

template <int DIM, int NC>
GV_HD void Dy(const Cf<DIM, NC>& c, const double* y, double* out) {  // DUDY y
  using L = Layout<DIM, NC>;
  constexpr int ND = L::ND;
  double ry = 0.0, my = 0.0;
#pragma unroll
  for (int j = 0; j < ND; ++j) { ry += c.r0[j] * y[j]; my += c.mE[j] * y[j]; }
#pragma unroll
  for (int r = 0; r < ND; ++r) {
    double m = (r >= 1 && r != L::iT) ? y[r] : 0.0;
    if (r == L::iT) m = my;
    out[r] = c.w[r] * ry + c.rho * m;
  }
}

template <int DIM, int NC>
GV_HD void DTx(const Cf<DIM, NC>& c, const double* x, double* out) {  // DUDY^T x
  using L = Layout<DIM, NC>;
  constexpr int ND = L::ND;
  double xw = 0.0;
#pragma unroll
  for (int j = 0; j < ND; ++j) xw += x[j] * c.w[j];
#pragma unroll
  for (int j = 0; j < ND; ++j) {
    double m = (j >= 1 && j != L::iT) ? x[j] : 0.0;
    out[j] = c.r0[j] * xw + c.rho * (m + x[L::iT] * c.mE[j]);
  }
}

template <int DIM, int NC>
GV_HD void xDy_rev(const Cf<DIM, NC>& c, const double* x, const double* y, double s, CfBar<DIM, NC>& b) {
  using L = Layout<DIM, NC>;
  constexpr int ND = L::ND;
  double xw = 0.0, ry = 0.0, my = 0.0, d = 0.0;
#pragma unroll
  for (int j = 0; j < ND; ++j) {
    xw += x[j] * c.w[j];
    ry += c.r0[j] * y[j];
    my += c.mE[j] * y[j];
    if (j >= 1 && j != L::iT) d += x[j] * y[j];
  }
#pragma unroll
  for (int j = 0; j < ND; ++j) {
    b.w[j] += s * ry * x[j];
    b.r0[j] += s * xw * y[j];
    b.mE[j] += s * c.rho * x[L::iT] * y[j];
  }
  b.rho += s * (d + x[L::iT] * my);
}

template <int DIM, int NC>
GV_HD void Ay(const Cf<DIM, NC>& c, int d, const double* y, double* out) {  // A_d y
  using L = Layout<DIM, NC>;
  constexpr int ND = L::ND;
  Dy<DIM, NC>(c, y, out);
  const double vd = c.v[d];
#pragma unroll
  for (int r = 0; r < ND; ++r) {
    const double up = c.rho * c.w[r] + (r == L::iT ? c.p : 0.0);
    out[r] = vd * out[r] + up * y[1 + d];
  }
  out[1 + d] += y[0];
  out[L::iT] += vd * y[0];
}

template <int DIM, int NC>
GV_HD void ATx(const Cf<DIM, NC>& c, int d, const double* x, double* out) {  // A_d^T x
  using L = Layout<DIM, NC>;
  constexpr int ND = L::ND;
  DTx<DIM, NC>(c, x, out);
  const double vd = c.v[d];
  double xu = 0.0;
#pragma unroll
  for (int r = 0; r < ND; ++r) xu += x[r] * (c.rho * c.w[r] + (r == L::iT ? c.p : 0.0));
#pragma unroll
  for (int j = 0; j < ND; ++j) out[j] *= vd;
  out[1 + d] += xu;
  out[0] += x[1 + d] + vd * x[L::iT];
}

template <int DIM, int NC>
GV_HD void xAy_rev(const Cf<DIM, NC>& c, int d, const double* x, const double* y, double s, CfBar<DIM, NC>& b) {
  using L = Layout<DIM, NC>;
  constexpr int ND = L::ND;
  const double vd = c.v[d];
  b.v[d] += s * (xDy<DIM, NC>(c, x, y) + x[L::iT] * y[0]);
  xDy_rev<DIM, NC>(c, x, y, s * vd, b);
  double xw = 0.0;
#pragma unroll
  for (int r = 0; r < ND; ++r) xw += x[r] * c.w[r];
  const double t = s * y[1 + d];
  b.rho += t * xw;
#pragma unroll
  for (int r = 0; r < ND; ++r) b.w[r] += t * c.rho * x[r];
  b.p += t * x[L::iT];
}

// ---------------------------------------------------------------------------
// compute_h (quad.hpp:356-383, 701-739) with its tape and adjoint.
template <int DIM>
struct HTape {
  double nv, s0[DIM], acc[DIM], ip, s1[DIM], n1, s1n[DIM], s2[3], n2, s2n[3], alpha[3], Q;
  bool norm1, norm2;
};

template <int DIM>
GV_HD double quadform(const double (&G)[DIM][DIM], const double* s) {
  double r = 0.0;
#pragma unroll
  for (int i = 0; i < DIM; ++i) {
    double t = 0.0;
#pragma unroll
    for (int j = 0; j < DIM; ++j) t += G[i][j] * s[j];
    r += s[i] * t;
  }
  return r;
}

template <int DIM>
GV_HD void quadform_rev(const double (&G)[DIM][DIM], const double* s, double ab, double* sb) {
#pragma unroll
  for (int i = 0; i < DIM; ++i) {
    double t = 0.0;
#pragma unroll
    for (int j = 0; j < DIM; ++j) t += (G[i][j] + G[j][i]) * s[j];
    sb[i] += ab * t;
  }
}

template <int DIM>
GV_HD double compute_h_fwd(const double (&G)[DIM][DIM], const double* v, const double (&dv)[DIM][DIM],
                           HTape<DIM>& t) {
  t.nv = sqrt(dot<DIM>(v, v));
#pragma unroll
  for (int i = 0; i < DIM; ++i) t.s0[i] = v[i] / t.nv;
  t.alpha[0] = quadform<DIM>(G, t.s0);
#pragma unroll
  for (int i = 0; i < DIM; ++i) {
    double a = 0.0;
#pragma unroll
    for (int j = 0; j < DIM; ++j) a += dv[i][j] * v[j];
    t.acc[i] = a;
  }
  t.ip = dot<DIM>(t.acc, t.s0);
#pragma unroll
  for (int i = 0; i < DIM; ++i) t.s1[i] = t.acc[i] - t.ip * t.s0[i];
  t.n1 = sqrt(dot<DIM>(t.s1, t.s1));
  t.norm1 = t.n1 > kEps;
#pragma unroll
  for (int i = 0; i < DIM; ++i) t.s1n[i] = t.norm1 ? t.s1[i] / t.n1 : t.s1[i];
  t.alpha[1] = quadform<DIM>(G, t.s1n);
  t.alpha[2] = 0.0;
  t.norm2 = false;
  if constexpr (DIM == 3) {
    t.s2[0] = t.s0[1] * t.s1n[2] - t.s0[2] * t.s1n[1];
    t.s2[1] = t.s1n[0] * t.s0[2] - t.s1n[2] * t.s0[0];
    t.s2[2] = t.s0[0] * t.s1n[1] - t.s0[1] * t.s1n[0];
    t.n2 = sqrt(dot<3>(t.s2, t.s2));
    t.norm2 = t.n2 > kEps;
#pragma unroll
    for (int i = 0; i < 3; ++i) t.s2n[i] = t.norm2 ? t.s2[i] / t.n2 : t.s2[i];
    t.alpha[2] = quadform<DIM>(G, t.s2n);
  }
  double Q = 0.0;
#pragma unroll
  for (int i = 0; i < DIM; ++i)
    if (t.alpha[i] != 0.0) Q += 1.0 / t.alpha[i];
  t.Q = Q;
  return 2.0 * sqrt(fabs(Q));
}

template <int DIM>
GV_HD void normalise_rev(const double* sn, double n, bool norm, const double* snb, double* sb) {
  if (!norm) {
#pragma unroll
    for (int i = 0; i < DIM; ++i) sb[i] += snb[i];
    return;
  }
  const double pr = dot<DIM>(snb, sn);
#pragma unroll
  for (int i = 0; i < DIM; ++i) sb[i] += (snb[i] - pr * sn[i]) / n;
}

template <int DIM>
GV_HD void compute_h_rev(const double (&G)[DIM][DIM], const double* v, const double (&dv)[DIM][DIM],
                         const HTape<DIM>& t, double hb, double* vb, double (&dvb)[DIM][DIM]) {
  if (t.Q == 0.0) return;
  const double Qb = hb * (t.Q > 0.0 ? 1.0 : -1.0) / sqrt(fabs(t.Q));
  double s0b[DIM], s1nb[DIM], s1b[DIM], accb[DIM];
#pragma unroll
  for (int i = 0; i < DIM; ++i) { s0b[i] = 0.0; s1nb[i] = 0.0; s1b[i] = 0.0; accb[i] = 0.0; }
  if constexpr (DIM == 3) {
    if (t.alpha[2] != 0.0) {
      double s2nb[3] = {0, 0, 0}, s2b[3] = {0, 0, 0};
      quadform_rev<DIM>(G, t.s2n, -Qb / (t.alpha[2] * t.alpha[2]), s2nb);
      normalise_rev<3>(t.s2n, t.n2, t.norm2, s2nb, s2b);
      // s2 = s0 x s1n: s0b += s1n x s2b, s1nb += s2b x s0
      s0b[0] += t.s1n[1] * s2b[2] - t.s1n[2] * s2b[1];
      s0b[1] += t.s1n[2] * s2b[0] - t.s1n[0] * s2b[2];
      s0b[2] += t.s1n[0] * s2b[1] - t.s1n[1] * s2b[0];
      s1nb[0] += s2b[1] * t.s0[2] - s2b[2] * t.s0[1];
      s1nb[1] += s2b[2] * t.s0[0] - s2b[0] * t.s0[2];
      s1nb[2] += s2b[0] * t.s0[1] - s2b[1] * t.s0[0];
    }
  }
  if (t.alpha[1] != 0.0) quadform_rev<DIM>(G, t.s1n, -Qb / (t.alpha[1] * t.alpha[1]), s1nb);
  normalise_rev<DIM>(t.s1n, t.n1, t.norm1, s1nb, s1b);
  // s1 = acc - ip s0
  double ipb = 0.0;
#pragma unroll
  for (int i = 0; i < DIM; ++i) {
    accb[i] += s1b[i];
    ipb -= s1b[i] * t.s0[i];
    s0b[i] -= t.ip * s1b[i];
  }
  // ip = acc . s0
#pragma unroll
  for (int i = 0; i < DIM; ++i) {
    accb[i] += ipb * t.s0[i];
    s0b[i] += ipb * t.acc[i];
  }
  // acc = dv v
#pragma unroll
  for (int i = 0; i < DIM; ++i)
#pragma unroll
    for (int j = 0; j < DIM; ++j) {
      dvb[i][j] += accb[i] * v[j];
      vb[j] += accb[i] * dv[i][j];
    }
  if (t.alpha[0] != 0.0) quadform_rev<DIM>(G, t.s0, -Qb / (t.alpha[0] * t.alpha[0]), s0b);
  // s0 = v/|v|
  normalise_rev<DIM>(t.s0, t.nv, true, s0b, vb);
}

// ---------------------------------------------------------------------------
// DUDY^{-1} in closed form (dense), the 2x2 solve per column of DUDY = w r0^T + rho M.
template <int DIM, int NC>
GV_HD void dudy_inverse(const Cf<DIM, NC>& c, double (&X)[Layout<DIM, NC>::ND][Layout<DIM, NC>::ND]) {
  using L = Layout<DIM, NC>;
  constexpr int ND = L::ND;
  const double irho = 1.0 / c.rho;
  const double det = c.drho_dp * c.de_dT - c.drho_dT * c.de_dp;
#pragma unroll
  for (int col = 0; col < ND; ++col) {
    const double s = (col == 0) ? 1.0 : 0.0;
    double xv[DIM], xy[L::NYA];
#pragma unroll
    for (int j = 0; j < DIM; ++j) xv[j] = (((col == 1 + j) ? 1.0 : 0.0) - c.v[j] * s) * irho;
#pragma unroll
    for (int i = 0; i < NC - 1; ++i) xy[i] = (((col == L::iY + i) ? 1.0 : 0.0) - c.Y[i] * s) * irho;
    double R1 = s, R2 = (((col == L::iT) ? 1.0 : 0.0) - c.E * s) * irho;
#pragma unroll
    for (int j = 0; j < DIM; ++j) R2 -= c.v[j] * xv[j];
#pragma unroll
    for (int i = 0; i < NC - 1; ++i) {
      R1 -= c.drho_dY[i] * xy[i];
      R2 -= c.dE_dY[i] * xy[i];
    }
    X[0][col] = (R1 * c.de_dT - c.drho_dT * R2) / det;
    X[L::iT][col] = (c.drho_dp * R2 - c.de_dp * R1) / det;
#pragma unroll
    for (int j = 0; j < DIM; ++j) X[1 + j][col] = xv[j];
#pragma unroll
    for (int i = 0; i < NC - 1; ++i) X[L::iY + i][col] = xy[i];
  }
}

// ---------------------------------------------------------------------------
// The point residual (phi0, phi_d) and its reverse.
template <int DIM, int NEN, int NC>
struct PTape {
  using L = Layout<DIM, NC>;
  static constexpr int ND = L::ND;
  Mix<NC> m, mP;
  Cf<DIM, NC> c;
  double vP[DIM], TP, EP;
  double U[ND], UP[ND], S[ND];
  double dd[ND], Res[ND];
  // tau
  bool tau_on, lowm;
  HTape<DIM> ht;
  double vn, h, use, hv, td[ND], X[ND][ND], tau[ND][ND], tpre00, tpre11, Bm;
  int use_branch;            // 0: dt/2, 1: h/(2(v+c)) + h/(2v)
  int td_branch[ND];         // 0: use, 1: the capped term
  // dc
  bool dc_on;
  double dU[DIM][ND], grho[DIM], gn, Jv[DIM], sJ, hdc, AdI[ND], Z[ND], Zn, Un, use1, nrm[DIM], nu0, nu;
  double sg[NEN];
};

template <int DIM, int NEN, int NC>
GV_HD void point_forward(const Ctx<DIM, NC>& x, const PGeo<DIM, NEN>& q, const double* Iq,
                         const double (&dI)[DIM][Layout<DIM, NC>::ND], const double* Pq,
                         PTape<DIM, NEN, NC>& t, double* phi0, double (&phi)[DIM][Layout<DIM, NC>::ND]) {
  using L = Layout<DIM, NC>;
  constexpr int ND = L::ND;
  const double dt = x.dt;
  // primitive state at I and at P (fluid_2d.hpp:112-121)
  double p = Iq[0], T = Iq[L::iT], v[DIM], Y[NC], YP[NC];
  double sY = 0.0, sYP = 0.0;
#pragma unroll
  for (int k = 0; k < DIM; ++k) { v[k] = Iq[1 + k]; t.vP[k] = Pq[1 + k]; }
#pragma unroll
  for (int i = 0; i < NC - 1; ++i) {
    Y[i] = Iq[L::iY + i]; sY += Y[i];
    YP[i] = Pq[L::iY + i]; sYP += YP[i];
  }
  Y[NC - 1] = 1.0 - sY;
  YP[NC - 1] = 1.0 - sYP;
  t.TP = Pq[L::iT];
  mix_forward<NC>(x.ch, Pq[0], t.TP, YP, t.mP);
  mix_forward<NC>(x.ch, p, T, Y, t.m);
  coef_forward<DIM, NC>(t.m, x.ch, p, v, T, t.c);
  const Cf<DIM, NC>& c = t.c;
  // U, U_P, S and the mass term (fluid_2d.hpp:372-385, 597-599)
  t.EP = t.mP.cv * t.TP + 0.5 * dot<DIM>(t.vP, t.vP);
#pragma unroll
  for (int j = 0; j < ND; ++j) {
    t.U[j] = t.m.rho * c.w[j];
    double wP = (j == 0) ? 1.0 : (j < L::iT ? t.vP[j - 1] : (j == L::iT ? t.EP : YP[j - L::iY]));
    t.UP[j] = t.mP.rho * wP;
    t.S[j] = 0.0;
  }
  double gv = 0.0;
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    t.S[1 + d] = t.m.rho * x.gravity[d];
    gv += x.gravity[d] * v[d];
  }
  t.S[L::iT] = t.m.rho * gv;
  // least-squares residual Res = DUDY (I - P)/dt + sum_d A_d dI_d - S  (fluid_2d.hpp:282)
#pragma unroll
  for (int j = 0; j < ND; ++j) t.dd[j] = (Iq[j] - Pq[j]) / dt;
  Dy<DIM, NC>(c, t.dd, t.Res);
#pragma unroll
  for (int j = 0; j < ND; ++j) t.AdI[j] = 0.0;
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    double a[ND];
    Ay<DIM, NC>(c, d, dI[d], a);
#pragma unroll
    for (int j = 0; j < ND; ++j) t.AdI[j] += a[j];
  }
#pragma unroll
  for (int j = 0; j < ND; ++j) t.Res[j] += t.AdI[j] - t.S[j];
  // tau (fluid_2d.hpp:877-960), 2019 or none
#pragma unroll
  for (int r = 0; r < ND; ++r)
#pragma unroll
    for (int cc = 0; cc < ND; ++cc) t.tau[r][cc] = 0.0;
  t.vn = sqrt(dot<DIM>(v, v));
  t.tau_on = t.vn >= kEps && x.tau == GALES_TAU_NON_DIAG_COMP_2019;
  t.lowm = false;
  if (t.tau_on) {
    double dv[DIM][DIM];
#pragma unroll
    for (int a = 0; a < DIM; ++a)
#pragma unroll
      for (int d = 0; d < DIM; ++d) dv[a][d] = dI[d][1 + a];
    t.h = compute_h_fwd<DIM>(q.G, v, dv, t.ht);
    const double cs = t.m.c, h = t.h, vn = t.vn;
    t.hv = h / (2.0 * (vn + cs)) + h / (2.0 * vn);
    t.use_branch = (x.steady || t.hv <= dt * 0.5) ? 1 : 0;
    t.use = t.use_branch ? t.hv : dt * 0.5;
    const double use = t.use, rho = t.m.rho;
    double cap[ND];
    cap[0] = use;
#pragma unroll
    for (int d = 0; d < DIM; ++d) cap[1 + d] = h * h * rho / (12.0 * t.m.mu);
    cap[L::iT] = h * h * rho * t.m.cv / (12.0 * t.m.kappa);
#pragma unroll
    for (int i = 0; i < NC - 1; ++i) cap[L::iY + i] = h * h / (12.0 * x.ch[i].D);
    t.td_branch[0] = 0;
    t.td[0] = use;
#pragma unroll
    for (int j = 1; j < ND; ++j) {
      t.td_branch[j] = cap[j] < use ? 1 : 0;
      t.td[j] = t.td_branch[j] ? cap[j] : use;
    }
    dudy_inverse<DIM, NC>(c, t.X);
#pragma unroll
    for (int r = 0; r < ND; ++r)
#pragma unroll
      for (int cc = 0; cc < ND; ++cc) t.tau[r][cc] = t.X[r][cc] * t.td[cc];
    t.tpre00 = t.tau[0][0];
    t.tpre11 = t.tau[1][1];
    if (vn / cs < 0.1) {
      t.lowm = true;
      t.Bm = rho * t.tpre11 * q.trG;
      t.tau[0][0] = 1.0 / (1.0 / t.tpre00 + 1.0 / t.Bm);
#pragma unroll
      for (int cc = 1; cc < ND; ++cc) t.tau[0][cc] = 0.0;
    }
  }
  // dc viscosity (fluid_2d.hpp:1027-1065)
#pragma unroll
  for (int d = 0; d < DIM; ++d) Dy<DIM, NC>(c, dI[d], t.dU[d]);
  t.nu = 0.0;
  t.dc_on = false;
  if (x.dc_2006) {
    double s = 0.0;
#pragma unroll
    for (int d = 0; d < DIM; ++d) { t.grho[d] = t.dU[d][0]; s += t.grho[d] * t.grho[d]; }
    t.gn = sqrt(s);
    if (!(t.gn < kEps)) {
#pragma unroll
      for (int d = 0; d < DIM; ++d) t.Jv[d] = t.grho[d] / t.gn;
      double hs = 0.0;
#pragma unroll
      for (int i = 0; i < NEN; ++i) {
        double tt = 0.0;
#pragma unroll
        for (int d = 0; d < DIM; ++d) tt += t.Jv[d] * q.ds[d][i];
        t.sg[i] = tt >= 0.0 ? 1.0 : -1.0;
        hs += fabs(tt);
      }
      t.sJ = hs;
      if (hs > kEps) {
        t.dc_on = true;
        t.hdc = 1.0 / hs;
        double Zn = 0.0, Un = 0.0;
#pragma unroll
        for (int j = 0; j < ND; ++j) {
          t.Z[j] = x.u_ref_inv[j] * (t.AdI[j] - t.S[j]);
          const double u = x.u_ref_inv[j] * t.U[j];
          Zn += t.Z[j] * t.Z[j];
          Un += u * u;
        }
        t.Zn = sqrt(Zn);
        t.Un = sqrt(Un);
        double use1 = 0.0;
#pragma unroll
        for (int d = 0; d < DIM; ++d) {
          double n2 = 0.0;
#pragma unroll
          for (int j = 0; j < ND; ++j) {
            const double u = x.u_ref_inv[j] * t.dU[d][j];
            n2 += u * u;
          }
          t.nrm[d] = sqrt(n2);
          use1 += t.nrm[d] * t.nrm[d];
        }
        t.use1 = use1;
        const double a = x.dc_sharp, hd = t.hdc;
        double nu = 0.0;
        if (a == 1.0) nu = t.Zn * hd * (1.0 / sqrt(use1));
        else if (a == 2.0) nu = t.Zn * hd * hd / t.Un;
        else if (a == 1.5) nu = t.Zn * hd * ((1.0 / sqrt(use1)) + hd / t.Un) / 2.0;
        t.nu0 = nu;
        t.nu = x.dc_scale * nu;
      }
    }
  }
  // phi0 = rv - S0 tau Res,  phi_d = F_dif,d - F_adv,d + nu dU_d + A_d tau Res
  double wv[ND];
#pragma unroll
  for (int r = 0; r < ND; ++r) {
    double s = 0.0;
#pragma unroll
    for (int cc = 0; cc < ND; ++cc) s += t.tau[r][cc] * t.Res[cc];
    wv[r] = s;
  }
#pragma unroll
  for (int j = 0; j < ND; ++j) phi0[j] = (t.U[j] - t.UP[j]) / dt - t.S[j];
  {
    double s0w = 0.0;
#pragma unroll
    for (int d = 0; d < DIM; ++d) s0w += t.m.rho * x.gravity[d] * wv[1 + d];
    phi0[L::iT] -= s0w;
  }
  const double rho = t.m.rho, pp = c.p, E = c.E;
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    double aw[ND];
    Ay<DIM, NC>(c, d, wv, aw);
    // viscous stress row d
    double div = 0.0;
#pragma unroll
    for (int k = 0; k < DIM; ++k) div += dI[k][1 + k];
    double tsd[DIM];
#pragma unroll
    for (int j = 0; j < DIM; ++j) tsd[j] = c.mu * (dI[d][1 + j] + dI[j][1 + d]) + (j == d ? c.lam * div : 0.0);
    double fd[ND];
    fd[0] = 0.0;
#pragma unroll
    for (int j = 0; j < DIM; ++j) fd[1 + j] = tsd[j];
    double en = c.kappa * dI[d][L::iT];
#pragma unroll
    for (int j = 0; j < DIM; ++j) en += v[j] * tsd[j];
#pragma unroll
    for (int i = 0; i < NC - 1; ++i) {
      en += c.rhoDH[i] * dI[d][L::iY + i];
      fd[L::iY + i] = c.rhoD[i] * dI[d][L::iY + i];
    }
    fd[L::iT] = en;
    double fa[ND];
    fa[0] = rho * v[d];
#pragma unroll
    for (int j = 0; j < DIM; ++j) fa[1 + j] = rho * v[d] * v[j] + (j == d ? pp : 0.0);
    fa[L::iT] = v[d] * (rho * E + pp);
#pragma unroll
    for (int i = 0; i < NC - 1; ++i) fa[L::iY + i] = rho * v[d] * Y[i];
#pragma unroll
    for (int j = 0; j < ND; ++j) phi[d][j] = fd[j] - fa[j] + t.nu * t.dU[d][j] + aw[j];
  }
}

// Reverse of point_forward.  Outputs are accumulated (+=).
template <int DIM, int NEN, int NC>
GV_HD void point_reverse(const Ctx<DIM, NC>& x, const PGeo<DIM, NEN>& q, const double* Iq,
                         const double (&dI)[DIM][Layout<DIM, NC>::ND], const double* Pq,
                         const PTape<DIM, NEN, NC>& t, const double* phi0b,
                         const double (&phib)[DIM][Layout<DIM, NC>::ND], double* Ib,
                         double (&dIb)[DIM][Layout<DIM, NC>::ND], double* th, double* urib = nullptr) {
  using L = Layout<DIM, NC>;
  constexpr int ND = L::ND;
  const Cf<DIM, NC>& c = t.c;
  const double dt = x.dt, rho = t.m.rho;
  CfBar<DIM, NC> b;
  cfbar_zero<DIM, NC>(b);
  double Ub[ND], Sb[ND], Resb[ND], wvb[ND], nub = 0.0;
#pragma unroll
  for (int j = 0; j < ND; ++j) { Ub[j] = 0.0; Sb[j] = 0.0; Resb[j] = 0.0; wvb[j] = 0.0; }
  double dUb[DIM][ND];
#pragma unroll
  for (int d = 0; d < DIM; ++d)
#pragma unroll
    for (int j = 0; j < ND; ++j) dUb[d][j] = 0.0;
  // tau Res again
  double wv[ND];
#pragma unroll
  for (int r = 0; r < ND; ++r) {
    double s = 0.0;
#pragma unroll
    for (int cc = 0; cc < ND; ++cc) s += t.tau[r][cc] * t.Res[cc];
    wv[r] = s;
  }
  // ---- phi_d
  double div = 0.0;
#pragma unroll
  for (int k = 0; k < DIM; ++k) div += dI[k][1 + k];
  double divb = 0.0;
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    const double* pb = phib[d];
    // A_d wv
    double at[ND];
    ATx<DIM, NC>(c, d, pb, at);
#pragma unroll
    for (int j = 0; j < ND; ++j) wvb[j] += at[j];
    xAy_rev<DIM, NC>(c, d, pb, wv, 1.0, b);
    // nu dU_d
    double du = 0.0;
#pragma unroll
    for (int j = 0; j < ND; ++j) {
      du += pb[j] * t.dU[d][j];
      dUb[d][j] += t.nu * pb[j];
    }
    nub += du;
    // - F_adv,d
    const double vd = c.v[d];
    b.rho -= pb[0] * vd;
    b.v[d] -= pb[0] * rho;
#pragma unroll
    for (int j = 0; j < DIM; ++j) {
      // rho v_d v_j + p d_jd
      b.rho -= pb[1 + j] * vd * c.v[j];
      b.v[d] -= pb[1 + j] * rho * c.v[j];
      b.v[j] -= pb[1 + j] * rho * vd;
      if (j == d) b.p -= pb[1 + j];
    }
    // v_d (rho E + p)
    b.v[d] -= pb[L::iT] * (rho * c.E + c.p);
    b.rho -= pb[L::iT] * vd * c.E;
    b.E -= pb[L::iT] * vd * rho;
    b.p -= pb[L::iT] * vd;
#pragma unroll
    for (int i = 0; i < NC - 1; ++i) {
      b.rho -= pb[L::iY + i] * vd * c.Y[i];
      b.v[d] -= pb[L::iY + i] * rho * c.Y[i];
      b.Y[i] -= pb[L::iY + i] * rho * vd;
    }
    // F_dif,d: momentum rows tau_dj, energy row v.tau_d + kappa dT + sum rhoDH dY, species rhoD dY
    double tsd[DIM];
#pragma unroll
    for (int j = 0; j < DIM; ++j) tsd[j] = c.mu * (dI[d][1 + j] + dI[j][1 + d]) + (j == d ? c.lam * div : 0.0);
#pragma unroll
    for (int j = 0; j < DIM; ++j) {
      const double Phi = pb[1 + j] + pb[L::iT] * c.v[j];
      b.v[j] += pb[L::iT] * tsd[j];
      // tsd_j = mu (dI[d][1+j] + dI[j][1+d]) + [j==d] lam div
      b.mu += Phi * (dI[d][1 + j] + dI[j][1 + d]);
      dIb[d][1 + j] += Phi * c.mu;
      dIb[j][1 + d] += Phi * c.mu;
      if (j == d) {
        b.lam += Phi * div;
        divb += Phi * c.lam;
      }
    }
    b.kappa += pb[L::iT] * dI[d][L::iT];
    dIb[d][L::iT] += pb[L::iT] * c.kappa;
#pragma unroll
    for (int i = 0; i < NC - 1; ++i) {
      b.rhoDH[i] += pb[L::iT] * dI[d][L::iY + i];
      b.rhoD[i] += pb[L::iY + i] * dI[d][L::iY + i];
      dIb[d][L::iY + i] += pb[L::iT] * c.rhoDH[i] + pb[L::iY + i] * c.rhoD[i];
    }
  }
#pragma unroll
  for (int k = 0; k < DIM; ++k) dIb[k][1 + k] += divb;
  // ---- phi0 = (U - U_P)/dt - S - S0 wv
  double UPb[ND];
#pragma unroll
  for (int j = 0; j < ND; ++j) {
    Ub[j] += phi0b[j] / dt;
    UPb[j] = -phi0b[j] / dt;
    Sb[j] -= phi0b[j];
  }
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    b.rho -= phi0b[L::iT] * x.gravity[d] * wv[1 + d];
    wvb[1 + d] -= phi0b[L::iT] * rho * x.gravity[d];
  }
  // ---- dc viscosity: nu = dc_scale nu0(Zn, Un, hdc, use1)
  double AdIb[ND];
#pragma unroll
  for (int j = 0; j < ND; ++j) AdIb[j] = 0.0;
  if (t.dc_on && nub != 0.0) {
    const double a = x.dc_sharp, hd = t.hdc;
    const double nu0b = nub * x.dc_scale;
    double Znb = 0.0, Unb = 0.0, hdb = 0.0, use1b = 0.0;
    if (a == 1.0) {
      const double is = 1.0 / sqrt(t.use1);
      Znb = nu0b * hd * is;
      hdb = nu0b * t.Zn * is;
      use1b = nu0b * t.Zn * hd * (-0.5 * is / t.use1);
    } else if (a == 2.0) {
      Znb = nu0b * hd * hd / t.Un;
      hdb = nu0b * 2.0 * t.Zn * hd / t.Un;
      Unb = -nu0b * t.Zn * hd * hd / (t.Un * t.Un);
    } else if (a == 1.5) {
      const double is = 1.0 / sqrt(t.use1);
      const double inner = is + hd / t.Un;
      Znb = nu0b * hd * inner / 2.0;
      hdb = nu0b * t.Zn * (inner + hd / t.Un) / 2.0;
      Unb = -nu0b * t.Zn * hd * hd / (2.0 * t.Un * t.Un);
      use1b = nu0b * t.Zn * hd / 2.0 * (-0.5 * is / t.use1);
    }
    // Zn = |Z|, Z = u_ref_inv (AdI - S)
    if (t.Zn > 0.0) {
#pragma unroll
      for (int j = 0; j < ND; ++j) {
        const double g = Znb * t.Z[j] / t.Zn * x.u_ref_inv[j];
        AdIb[j] += g;
        Sb[j] -= g;
        if (urib) urib[j] += Znb * t.Z[j] / t.Zn * (t.AdI[j] - t.S[j]);
      }
    }
    // Un = |u_ref_inv U|
    if (t.Un > 0.0) {
#pragma unroll
      for (int j = 0; j < ND; ++j) {
        Ub[j] += Unb * x.u_ref_inv[j] * x.u_ref_inv[j] * t.U[j] / t.Un;
        if (urib) urib[j] += Unb * x.u_ref_inv[j] * t.U[j] * t.U[j] / t.Un;
      }
    }
    // use1 = sum_d |u_ref_inv dU_d|^2
#pragma unroll
    for (int d = 0; d < DIM; ++d)
#pragma unroll
      for (int j = 0; j < ND; ++j) {
        dUb[d][j] += use1b * 2.0 * x.u_ref_inv[j] * x.u_ref_inv[j] * t.dU[d][j];
        if (urib) urib[j] += use1b * 2.0 * x.u_ref_inv[j] * t.dU[d][j] * t.dU[d][j];
      }
    // hdc = 1/sJ, sJ = sum_i |J . dN_i|, J = grho/|grho|, grho_d = dU_d[0]
    const double sJb = -hdb / (t.sJ * t.sJ);
    double Jb[DIM];
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
      double sum = 0.0;
#pragma unroll
      for (int i = 0; i < NEN; ++i) sum += t.sg[i] * q.ds[d][i];
      Jb[d] = sJb * sum;
    }
    const double pr = dot<DIM>(Jb, t.Jv);
#pragma unroll
    for (int d = 0; d < DIM; ++d) dUb[d][0] += (Jb[d] - pr * t.Jv[d]) / t.gn;
  }
  // ---- tau: the loss term wv . wvb with wv = tau Res
#pragma unroll
  for (int cc = 0; cc < ND; ++cc) {
    double sum = 0.0;
#pragma unroll
    for (int r = 0; r < ND; ++r) sum += t.tau[r][cc] * wvb[r];
    Resb[cc] += sum;
  }
  double vb_h[DIM], dvb[DIM][DIM];
#pragma unroll
  for (int a = 0; a < DIM; ++a) {
    vb_h[a] = 0.0;
#pragma unroll
    for (int d = 0; d < DIM; ++d) dvb[a][d] = 0.0;
  }
  double cvb_tau = 0.0, csb_tau = 0.0;
  if (t.tau_on) {
    double taub[ND][ND];
#pragma unroll
    for (int r = 0; r < ND; ++r)
#pragma unroll
      for (int cc = 0; cc < ND; ++cc) taub[r][cc] = wvb[r] * t.Res[cc];
    if (t.lowm) {
      // tau00 = 1/(1/a + 1/B) with B = rho tau11 trG; row 0 off-diagonals set to zero
      const double t00 = t.tau[0][0];
      const double ab = taub[0][0] * (t00 / t.tpre00) * (t00 / t.tpre00);
      const double Bb = taub[0][0] * (t00 / t.Bm) * (t00 / t.Bm);
      taub[0][0] = ab;
#pragma unroll
      for (int cc = 1; cc < ND; ++cc) taub[0][cc] = 0.0;
      taub[1][1] += Bb * rho * q.trG;
      b.rho += Bb * t.tpre11 * q.trG;
    }
    // tau = X diag(td)
    double Xb[ND][ND], tdb[ND];
#pragma unroll
    for (int cc = 0; cc < ND; ++cc) {
      tdb[cc] = 0.0;
#pragma unroll
      for (int r = 0; r < ND; ++r) {
        Xb[r][cc] = taub[r][cc] * t.td[cc];
        tdb[cc] += taub[r][cc] * t.X[r][cc];
      }
    }
    // X = DUDY^{-1}: DUDY-bar = -X^T Xb X^T, folded into the coefficient cotangents
    // entry by entry through e_r^T DUDY e_c
    double T1[ND][ND];
#pragma unroll
    for (int r = 0; r < ND; ++r)
#pragma unroll
      for (int cc = 0; cc < ND; ++cc) {
        double sum = 0.0;
#pragma unroll
        for (int k = 0; k < ND; ++k) sum += t.X[k][r] * Xb[k][cc];
        T1[r][cc] = sum;
      }
#pragma unroll
    for (int r = 0; r < ND; ++r) {
      double Dbr[ND];
#pragma unroll
      for (int cc = 0; cc < ND; ++cc) {
        double sum = 0.0;
#pragma unroll
        for (int k = 0; k < ND; ++k) sum += T1[r][k] * t.X[cc][k];
        Dbr[cc] = -sum;
      }
      double er[ND];
#pragma unroll
      for (int k = 0; k < ND; ++k) er[k] = (k == r) ? 1.0 : 0.0;
      xDy_rev<DIM, NC>(c, er, Dbr, 1.0, b);
    }
    // td_0 = use, td_j = min(use, cap_j)
    const double h = t.h, vn = t.vn, cs = t.m.c;
    double useb = tdb[0], hb = 0.0;
#pragma unroll
    for (int j = 1; j < ND; ++j) {
      if (!t.td_branch[j]) {
        useb += tdb[j];
        continue;
      }
      if (j < L::iT) {
        const double cap = h * h * rho / (12.0 * t.m.mu);   // h^2 rho/(12 mu)
        hb += tdb[j] * 2.0 * cap / h;
        b.rho += tdb[j] * cap / rho;
        b.mu -= tdb[j] * cap / t.m.mu;
      } else if (j == L::iT) {
        const double cap = h * h * rho * t.m.cv / (12.0 * t.m.kappa);
        hb += tdb[j] * 2.0 * cap / h;
        b.rho += tdb[j] * cap / rho;
        cvb_tau += tdb[j] * cap / t.m.cv;
        b.kappa -= tdb[j] * cap / t.m.kappa;
      } else {
        const double cap = h * h / (12.0 * x.ch[j - L::iY].D);
        hb += tdb[j] * 2.0 * cap / h;
      }
    }
    double vnb = 0.0;
    if (t.use_branch) {
      // use = h/(2(vn + c)) + h/(2 vn)
      hb += useb * (1.0 / (2.0 * (vn + cs)) + 1.0 / (2.0 * vn));
      vnb += useb * (-h / (2.0 * (vn + cs) * (vn + cs)) - h / (2.0 * vn * vn));
      csb_tau += useb * (-h / (2.0 * (vn + cs) * (vn + cs)));
    }
    double dv[DIM][DIM];
#pragma unroll
    for (int a = 0; a < DIM; ++a)
#pragma unroll
      for (int d = 0; d < DIM; ++d) dv[a][d] = dI[d][1 + a];
    compute_h_rev<DIM>(q.G, c.v, dv, t.ht, hb, vb_h, dvb);
#pragma unroll
    for (int k = 0; k < DIM; ++k) vb_h[k] += vnb * c.v[k] / vn;
#pragma unroll
    for (int a = 0; a < DIM; ++a)
#pragma unroll
      for (int d = 0; d < DIM; ++d) dIb[d][1 + a] += dvb[a][d];
  }
  // ---- Res = DUDY dd + AdI - S
#pragma unroll
  for (int j = 0; j < ND; ++j) {
    AdIb[j] += Resb[j];
    Sb[j] -= Resb[j];
  }
  xDy_rev<DIM, NC>(c, Resb, t.dd, 1.0, b);
  {
    double ddb[ND];
    DTx<DIM, NC>(c, Resb, ddb);
#pragma unroll
    for (int j = 0; j < ND; ++j) Ib[j] += ddb[j] / dt;
  }
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    xAy_rev<DIM, NC>(c, d, AdIb, dI[d], 1.0, b);
    double at[ND];
    ATx<DIM, NC>(c, d, AdIb, at);
#pragma unroll
    for (int j = 0; j < ND; ++j) dIb[d][j] += at[j];
  }
  // dU_d = DUDY dI_d
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    xDy_rev<DIM, NC>(c, dUb[d], dI[d], 1.0, b);
    double at[ND];
    DTx<DIM, NC>(c, dUb[d], at);
#pragma unroll
    for (int j = 0; j < ND; ++j) dIb[d][j] += at[j];
  }
  // S = (0, rho g, rho g.v, 0)
  {
    double gv = 0.0;
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
      gv += x.gravity[d] * c.v[d];
      b.rho += Sb[1 + d] * x.gravity[d];
      b.v[d] += Sb[L::iT] * rho * x.gravity[d];
    }
    b.rho += Sb[L::iT] * gv;
  }
  // U = rho w
#pragma unroll
  for (int j = 0; j < ND; ++j) {
    b.rho += Ub[j] * c.w[j];
    b.w[j] += Ub[j] * rho;
  }
  cfbar_fold<DIM, NC>(b);
  // ---- coefficients -> mixture -> state and parameters
  MixBar o;
  double rcb[NC], cvcb[NC], pb = 0.0, Tb = 0.0, vb[DIM], Yb[NC];
#pragma unroll
  for (int k = 0; k < DIM; ++k) vb[k] = vb_h[k];
#pragma unroll
  for (int i = 0; i < NC; ++i) Yb[i] = 0.0;
  coef_reverse<DIM, NC>(t.m, x.ch, c, b, o, rcb, cvcb, pb, vb, Tb, Yb);
  o.cv += cvb_tau;
  o.c += csb_tau;
  mix_reverse<NC>(x.ch, c.p, c.T, t.m, o, rcb, cvcb, pb, Tb, Yb, th);
  // U_P = rho_P (1, v_P, E_P, Y_P): parameters only
  {
    MixBar oP{0, 0, 0, 0, 0, 0, 0, 0};
    double wP[ND];
#pragma unroll
    for (int j = 0; j < ND; ++j)
      wP[j] = (j == 0) ? 1.0 : (j < L::iT ? t.vP[j - 1] : (j == L::iT ? t.EP : t.mP.Y[j - L::iY]));
#pragma unroll
    for (int j = 0; j < ND; ++j) oP.rho += UPb[j] * wP[j];
    oP.cv += UPb[L::iT] * t.mP.rho * t.TP;
    double pPb = 0.0, TPb = 0.0, YPb[NC];
#pragma unroll
    for (int i = 0; i < NC; ++i) YPb[i] = 0.0;
    mix_reverse<NC>(x.ch, Pq[0], t.TP, t.mP, oP, nullptr, nullptr, pPb, TPb, YPb, th);
  }
  // state cotangents: p, v, T, Y_i (Y_nc = 1 - sum Y_i)
  Ib[0] += pb;
#pragma unroll
  for (int k = 0; k < DIM; ++k) Ib[1 + k] += vb[k];
  Ib[L::iT] += Tb;
#pragma unroll
  for (int i = 0; i < NC - 1; ++i) Ib[L::iY + i] += Yb[i] - Yb[NC - 1];
}

// ---------------------------------------------------------------------------
// Boundary point (execute_b, fluid_2d.hpp:341-349, 610-817): rb = sum_k (F_adv,k -
// F_dif,k) JNxW_k with the side's Neumann and mass-flux overrides, and its reverse.
template <int DIM, int NC>
struct BTape {
  using L = Layout<DIM, NC>;
  Mix<NC> m;
  Cf<DIM, NC> c;
  double ts[DIM][DIM], qf[DIM], Jf[DIM][L::NYA], div;
  bool tsf[DIM][DIM], qff[DIM], Jff[DIM][L::NYA];   // entry set by an override
};

template <int DIM, int NC>
GV_HD void bpoint_forward(const Ctx<DIM, NC>& x, const gales_side_bc& bc, const double* Iq,
                          const double (&dI)[DIM][Layout<DIM, NC>::ND], const double* JN, BTape<DIM, NC>& t,
                          double* rb) {
  using L = Layout<DIM, NC>;
  constexpr int ND = L::ND;
  double p = Iq[0], T = Iq[L::iT], v[DIM], Y[NC], sY = 0.0;
#pragma unroll
  for (int k = 0; k < DIM; ++k) v[k] = Iq[1 + k];
#pragma unroll
  for (int i = 0; i < NC - 1; ++i) { Y[i] = Iq[L::iY + i]; sY += Y[i]; }
  Y[NC - 1] = 1.0 - sY;
  mix_forward<NC>(x.ch, p, T, Y, t.m);
  coef_forward<DIM, NC>(t.m, x.ch, p, v, T, t.c);
  const Cf<DIM, NC>& c = t.c;
  const double rho = t.m.rho;
  double div = 0.0;
#pragma unroll
  for (int d = 0; d < DIM; ++d) div += dI[d][1 + d];
  t.div = div;
#pragma unroll
  for (int a = 0; a < DIM; ++a)
#pragma unroll
    for (int b = 0; b < DIM; ++b) {
      const int lo = a < b ? a : b, hi = a < b ? b : a;
      t.tsf[a][b] = (bc.tau_mask >> (lo * 3 + hi)) & 1u;
      if (t.tsf[a][b]) t.ts[a][b] = bc.tau[lo * 3 + hi];
      else if (a == b) t.ts[a][b] = c.lam * div + 2.0 * c.mu * dI[a][1 + a];
      else t.ts[a][b] = c.mu * (dI[hi][1 + lo] + dI[lo][1 + hi]);
    }
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    t.qff[d] = (bc.q_mask >> d) & 1u;
    t.qf[d] = t.qff[d] ? bc.q[d] : -c.kappa * dI[d][L::iT];
#pragma unroll
    for (int i = 0; i < NC - 1; ++i) {
      t.Jff[d][i] = (bc.J_mask >> (d * 8 + i)) & 1u;
      t.Jf[d][i] = t.Jff[d][i] ? bc.J[d][i] : rho * x.ch[i].D * dI[d][L::iY + i];
    }
  }
#pragma unroll
  for (int j = 0; j < ND; ++j) rb[j] = 0.0;
#pragma unroll
  for (int k = 0; k < DIM; ++k) {
    double fa[ND], fd[ND];
    if ((bc.mass_flux_mask >> k) & 1u) {
      const double mf = bc.mass_flux[k];
      fa[0] = mf;
#pragma unroll
      for (int j = 0; j < DIM; ++j) fa[1 + j] = mf * v[j] + (j == k ? p : 0.0);
      fa[L::iT] = mf * c.E + p * v[k];
#pragma unroll
      for (int i = 0; i < NC - 1; ++i) fa[L::iY + i] = mf * Y[i];
    } else {
      fa[0] = rho * v[k];
#pragma unroll
      for (int j = 0; j < DIM; ++j) fa[1 + j] = rho * v[k] * v[j] + (j == k ? p : 0.0);
      fa[L::iT] = v[k] * (rho * c.E + p);
#pragma unroll
      for (int i = 0; i < NC - 1; ++i) fa[L::iY + i] = rho * v[k] * Y[i];
    }
    fd[0] = 0.0;
    double en = -t.qf[k];
#pragma unroll
    for (int j = 0; j < DIM; ++j) {
      fd[1 + j] = t.ts[k][j];
      en += t.ts[k][j] * v[j];
    }
#pragma unroll
    for (int i = 0; i < NC - 1; ++i) {
      en -= c.H[i] * t.Jf[k][i];
      fd[L::iY + i] = t.Jf[k][i];
    }
    fd[L::iT] = en;
#pragma unroll
    for (int j = 0; j < ND; ++j) rb[j] += (fa[j] - fd[j]) * JN[k];
  }
}

template <int DIM, int NC>
GV_HD void bpoint_reverse(const Ctx<DIM, NC>& x, const gales_side_bc& bc, const double* Iq,
                          const double (&dI)[DIM][Layout<DIM, NC>::ND], const double* JN, const BTape<DIM, NC>& t,
                          const double* rbb, double* Ib, double (&dIb)[DIM][Layout<DIM, NC>::ND], double* th) {
  using L = Layout<DIM, NC>;
  constexpr int ND = L::ND;
  const Cf<DIM, NC>& c = t.c;
  const double rho = t.m.rho;
  CfBar<DIM, NC> b;
  cfbar_zero<DIM, NC>(b);
  double tsb[DIM][DIM], Hb[L::NYA];
#pragma unroll
  for (int a = 0; a < DIM; ++a)
#pragma unroll
    for (int e = 0; e < DIM; ++e) tsb[a][e] = 0.0;
#pragma unroll
  for (int i = 0; i < L::NYA; ++i) Hb[i] = 0.0;
#pragma unroll
  for (int k = 0; k < DIM; ++k) {
    double fab[ND], fdb[ND];
#pragma unroll
    for (int j = 0; j < ND; ++j) {
      fab[j] = rbb[j] * JN[k];
      fdb[j] = -rbb[j] * JN[k];
    }
    const double vk = c.v[k];
    if ((bc.mass_flux_mask >> k) & 1u) {
      const double mf = bc.mass_flux[k];
#pragma unroll
      for (int j = 0; j < DIM; ++j) {
        b.v[j] += fab[1 + j] * mf;
        if (j == k) b.p += fab[1 + j];
      }
      b.E += fab[L::iT] * mf;
      b.p += fab[L::iT] * vk;
      b.v[k] += fab[L::iT] * c.p;
#pragma unroll
      for (int i = 0; i < NC - 1; ++i) b.Y[i] += fab[L::iY + i] * mf;
    } else {
      b.rho += fab[0] * vk;
      b.v[k] += fab[0] * rho;
#pragma unroll
      for (int j = 0; j < DIM; ++j) {
        b.rho += fab[1 + j] * vk * c.v[j];
        b.v[k] += fab[1 + j] * rho * c.v[j];
        b.v[j] += fab[1 + j] * rho * vk;
        if (j == k) b.p += fab[1 + j];
      }
      b.v[k] += fab[L::iT] * (rho * c.E + c.p);
      b.rho += fab[L::iT] * vk * c.E;
      b.E += fab[L::iT] * vk * rho;
      b.p += fab[L::iT] * vk;
#pragma unroll
      for (int i = 0; i < NC - 1; ++i) {
        b.rho += fab[L::iY + i] * vk * c.Y[i];
        b.v[k] += fab[L::iY + i] * rho * c.Y[i];
        b.Y[i] += fab[L::iY + i] * rho * vk;
      }
    }
    // fd: (0, ts[k][:], ts[k].v - qf_k - sum_i H_i Jf_ki, Jf_k:)
#pragma unroll
    for (int j = 0; j < DIM; ++j) {
      tsb[k][j] += fdb[1 + j] + fdb[L::iT] * c.v[j];
      b.v[j] += fdb[L::iT] * t.ts[k][j];
    }
    const double qfb = -fdb[L::iT];
    if (!t.qff[k]) {
      b.kappa -= qfb * dI[k][L::iT];
      dIb[k][L::iT] -= qfb * c.kappa;
    }
#pragma unroll
    for (int i = 0; i < NC - 1; ++i) {
      Hb[i] -= fdb[L::iT] * t.Jf[k][i];
      const double Jb = -fdb[L::iT] * c.H[i] + fdb[L::iY + i];
      if (!t.Jff[k][i]) {
        b.rho += Jb * x.ch[i].D * dI[k][L::iY + i];
        dIb[k][L::iY + i] += Jb * rho * x.ch[i].D;
      }
    }
  }
  // stresses (symmetric overrides are constants)
#pragma unroll
  for (int a = 0; a < DIM; ++a)
#pragma unroll
    for (int e = 0; e < DIM; ++e) {
      if (t.tsf[a][e]) continue;
      const double g = tsb[a][e];
      if (a == e) {
        b.lam += g * t.div;
#pragma unroll
        for (int d = 0; d < DIM; ++d) dIb[d][1 + d] += g * c.lam;
        b.mu += g * 2.0 * dI[a][1 + a];
        dIb[a][1 + a] += g * 2.0 * c.mu;
      } else {
        const int lo = a < e ? a : e, hi = a < e ? e : a;
        b.mu += g * (dI[hi][1 + lo] + dI[lo][1 + hi]);
        dIb[hi][1 + lo] += g * c.mu;
        dIb[lo][1 + hi] += g * c.mu;
      }
    }
  cfbar_fold<DIM, NC>(b);
  MixBar o;
  double rcb[NC], cvcb[NC], pb = 0.0, Tb = 0.0, vb[DIM], Yb[NC];
#pragma unroll
  for (int k = 0; k < DIM; ++k) vb[k] = 0.0;
#pragma unroll
  for (int i = 0; i < NC; ++i) Yb[i] = 0.0;
  coef_reverse<DIM, NC>(t.m, x.ch, c, b, o, rcb, cvcb, pb, vb, Tb, Yb);
  // H_i = cv_i T + p/rho_i
#pragma unroll
  for (int i = 0; i < NC - 1; ++i) {
    cvcb[i] += Hb[i] * c.T;
    Tb += Hb[i] * t.m.cvc[i];
    pb += Hb[i] / t.m.r[i];
    rcb[i] -= Hb[i] * c.p / (t.m.r[i] * t.m.r[i]);
  }
  mix_reverse<NC>(x.ch, c.p, c.T, t.m, o, rcb, cvcb, pb, Tb, Yb, th);
  Ib[0] += pb;
#pragma unroll
  for (int k = 0; k < DIM; ++k) Ib[1 + k] += vb[k];
  Ib[L::iT] += Tb;
#pragma unroll
  for (int i = 0; i < NC - 1; ++i) Ib[L::iY + i] += Yb[i] - Yb[NC - 1];
}

#undef GV_HD

}  // namespace vjp
}  // namespace gales
