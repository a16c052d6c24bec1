// Magma mixture properties (mixtures.hpp:114-511, chemicals.hpp:56-271,
// GiordanoEtAlViscosityModel.hpp), point-wise, shared by the GPU kernel
// (gales_magma.cu) and a host build of the same code used by the CPU tests.
//
// Each magma's composition-only quantities (the melt's molar mass, volume and its
// derivatives, heat capacity, the viscosity model's seven composition parameters, the
// gas constants) are computed once at creation, in the reference constructors' order,
// and stored with pointers to the solubility tables.  The per-point work is the
// reference's properties() with the same operation order.  Out-of-table points clamp
// the index (no access outside the tables) and set a status bit; the reference stops.
#pragma once

#include <cmath>

#include "../../include/gales_asm.h"

#ifdef __CUDACC__
#define GALES_MAGMA_HD __host__ __device__ inline
#else
#define GALES_MAGMA_HD inline
#endif

namespace magma_mix {

struct DevMagma {
  double melt_M, melt_V, melt_dVdT, melt_dVdp, melt_cp, melt_kappa;
  double vol_M[2], vol_cp[2], vol_kappa[2];               // H2O(l), CO2(l)
  double gas_R[2], gas_gamma[2], gas_cv[2], gas_cp[2], gas_kappa[2];  // H2O(g), CO2(g)
  double visc_M, visc_P[7];                               // Giordano composition terms
  double wf_comp[3];                                      // melt, H2O, CO2 of the magma
  double crystal_vf, crystal_rho;
  int gas_on_mu, crystal_on_mu;
  int n_p, n_T;
  // custom_mix / ch_as_mix (kind != GALES_SUBMIX_MAGMA): the chemical's constants
  int kind, ch_kind;
  double ch_rho, ch_mu, ch_cp, ch_cv, ch_kappa, ch_alpha, ch_beta, ch_R, ch_gamma;
  const double* p_tab;
  const double* T_tab;
  const double* h2o_tab;
  const double* co2_tab;
};

struct Props {
  double rho, cv, cp, kappa, D, mu, c, alpha, beta;
};

// Host: composition constants in the reference constructors' order (melt():
// chemicals.hpp:62-103; GiordanoEtAlViscosityModel::set: GiordanoEtAlViscosityModel.hpp:36-83;
// ideal_gas("H2O"/"CO2"): chemicals.hpp:201-234).
inline void build_constants(const gales_magma_desc& d, DevMagma& g) {
  g.kind = d.kind;
  g.ch_kind = d.kind == GALES_SUBMIX_CUSTOM ? GALES_CH_CUSTOM : d.chemical.kind;
  g.ch_rho = d.chemical.rho;
  g.ch_mu = d.chemical.mu;
  g.ch_cp = d.chemical.cp;
  g.ch_cv = d.chemical.cv;
  g.ch_kappa = d.chemical.kappa;
  g.ch_alpha = d.chemical.alpha;
  g.ch_beta = d.chemical.beta;
  g.ch_R = d.chemical.R;
  g.ch_gamma = d.chemical.gamma;
  g.wf_comp[1] = d.h2o_wf;
  g.wf_comp[2] = d.co2_wf;
  g.wf_comp[0] = 1.0 - g.wf_comp[1] - g.wf_comp[2];
  double wf[10], mm[10], xf[10];
  double sum = 0.0;
  for (int i = 0; i < 10; ++i) sum += d.oxide_wf[i];
  for (int i = 0; i < 10; ++i) wf[i] = d.oxide_wf[i] / sum;
  static const double oxide_mm[10] = {60.084, 79.876, 101.956, 159.692, 71.846, 70.937, 40.304, 56.078, 61.979, 94.195};
  for (int i = 0; i < 10; ++i) mm[i] = oxide_mm[i] * 1.e-3;
  double M = 0.0;
  for (int i = 0; i < 10; ++i) M += wf[i] / mm[i];
  M = 1. / M;
  for (int i = 0; i < 10; ++i) xf[i] = wf[i] * M / mm[i];
  static const double dVdT[10] = {0.0, 7.24, 0.0, 9.09, 2.92, 0.0, 3.27, 3.74, 7.68, 12.08};
  static const double dVdp[10] = {-1.89, -2.31, -2.26, -2.53, -0.45, 0.0, 0.27, 0.34, -2.4, -6.75};
  static const double V0[10] = {26.86, 23.16, 37.42, 42.13, 13.65, 0.0, 11.69, 16.53, 28.88, 45.07};
  static const double cp0[10] = {1331.0, 1392.0, 1545.0, 1434.0, 1100.0, 0.0, 2424.0, 1781.0, 1651.0, 1030.0};
  double a = 0.0, b = 0.0, v = 0.0, c = 0.0;
  for (int i = 0; i < 10; ++i) a += xf[i] * (dVdT[i] * 1.e-9);
  for (int i = 0; i < 10; ++i) b += xf[i] * (dVdp[i] * 1.e-15);
  for (int i = 0; i < 10; ++i) v += xf[i] * (V0[i] * 1.e-6);
  for (int i = 0; i < 10; ++i) c += xf[i] * cp0[i];
  g.melt_M = M;
  g.melt_dVdT = a;
  g.melt_dVdp = b;
  g.melt_V = v;
  g.melt_cp = c;
  g.melt_kappa = d.melt_kappa;
  g.vol_M[0] = 0.01802;
  g.vol_M[1] = 0.04401;
  g.vol_cp[0] = d.h2o_l_cp;
  g.vol_cp[1] = d.co2_l_cp;
  g.vol_kappa[0] = d.h2o_l_kappa;
  g.vol_kappa[1] = d.co2_l_kappa;
  for (int k = 0; k < 2; ++k) {
    const double gm = 1.4, R = 8.314462 / (k == 0 ? 0.01802 : 0.04401);
    g.gas_gamma[k] = gm;
    g.gas_R[k] = R;
    g.gas_cv[k] = R / (gm - 1.0);
    g.gas_cp[k] = gm * g.gas_cv[k];
    g.gas_kappa[k] = 1.e-5 * g.gas_cp[k] / 0.72;
  }
  // viscosity model composition terms (mole percent of the anhydrous melt, Fe as FeO)
  double w[10], mg[10], m[10];
  for (int i = 0; i < 10; ++i) mg[i] = mm[i] * 1.e3;
  for (int i = 0; i < 10; ++i) w[i] = wf[i];
  w[4] = 0.9309 * (w[3] + w[4]);
  w[3] = 0.0;
  double s2 = 0.0;
  for (int i = 0; i < 10; ++i) s2 += w[i];
  for (int i = 0; i < 10; ++i) w[i] /= s2;
  double Mv = 0.0;
  for (int i = 0; i < 10; ++i) Mv += w[i] / mg[i];
  Mv = 1.0 / Mv;
  for (int i = 0; i < 10; ++i) m[i] = 100.0 * w[i] * Mv / mg[i];
  const double B[7] = {159.6, -173.3, 72.1, 75.7, -39.0, -84.1, 141.5};
  const double B1[3] = {-2.43, -0.91, 17.6};
  const double Cc[6] = {2.75, 15.7, 8.3, 10.2, -12.3, -99.5};
  g.visc_M = Mv;
  g.visc_P[0] = -4.55;
  g.visc_P[1] = B[0] * (m[0] + m[1]) + B[1] * m[2] + B[2] * (m[4] + m[5]) + B[3] * m[6] + B[4] * m[7] + B[5] * m[8];
  g.visc_P[2] = B1[0] * (m[0] + m[1]) * (m[4] + m[5] + m[6]) + B1[1] * (m[0] + m[1] + m[2]) * (m[8] + m[9]) +
                B1[2] * m[2] * (m[8] + m[9]);
  g.visc_P[3] = B1[1] * (m[0] + m[1] + m[2]);
  g.visc_P[4] = Cc[0] * m[0] + Cc[1] * (m[1] + m[2]) + Cc[2] * (m[4] + m[5] + m[6]) + Cc[3] * m[7] + Cc[4] * (m[8] + m[9]);
  g.visc_P[5] = 0.3 * (m[2] + m[4] + m[5] + m[6] + m[7]) * (m[8] + m[9]);
  g.visc_P[6] = 0.3 * (m[2] + m[4] + m[5] + m[6] + m[7]);
  g.crystal_vf = d.crystal_fraction;
  g.crystal_rho = d.crystal_rho;
  g.gas_on_mu = d.gas_on_mu;
  g.crystal_on_mu = d.crystal_on_mu;
  g.n_p = d.n_p;
  g.n_T = d.n_T;
}

// Linear interpolation on the equispaced pressure table (mixtures.hpp:342-356).
GALES_MAGMA_HD double lookup_p(const DevMagma& g, const double* y, double p, unsigned& st) {
  const double* pt = g.p_tab;
  const double dp = pt[1] - pt[0];
  const double f = floor((p - pt[0]) / dp);
  long long i = (long long)f;
  if (!(f >= 0.0) || i + 1 >= g.n_p) {
    st |= GALES_MAGMA_LOOKUP_RANGE;
    i = i < 0 ? 0 : (i > g.n_p - 2 ? g.n_p - 2 : i);
    if (!(f == f)) i = 0;
  }
  const double slope = (y[i + 1] - y[i]) / dp;
  return y[i] + slope * (p - pt[i]);
}

// Bilinear interpolation in (T, p) (mixtures.hpp:380-412): tables [n_T][n_p].
GALES_MAGMA_HD double lookup_Tp(const DevMagma& g, const double* m, double T, double p, unsigned& st) {
  const double* pt = g.p_tab;
  const double* Tt = g.T_tab;
  const double dp = fabs(pt[1] - pt[0]);
  const double dT = fabs(Tt[1] - Tt[0]);
  const double fp = floor(fabs(p - pt[0]) / dp), fT = floor(fabs(T - Tt[0]) / dT);
  long long pc = (long long)fp, Tr = (long long)fT;
  if (!(fp >= 0.0) || !(fT >= 0.0) || pc + 1 >= g.n_p || Tr + 1 >= g.n_T) {
    st |= GALES_MAGMA_LOOKUP_RANGE;
    pc = pc < 0 ? 0 : (pc > g.n_p - 2 ? g.n_p - 2 : pc);
    Tr = Tr < 0 ? 0 : (Tr > g.n_T - 2 ? g.n_T - 2 : Tr);
    if (!(fp == fp)) pc = 0;
    if (!(fT == fT)) Tr = 0;
  }
  const long long np = g.n_p;
  const double p1 = pt[pc], p2 = pt[pc + 1], T1 = Tt[Tr], T2 = Tt[Tr + 1];
  double mean = (T2 - T) * (p2 - p) * m[Tr * np + pc] + (T2 - T) * (p - p1) * m[Tr * np + pc + 1] +
                (T - T1) * (p2 - p) * m[(Tr + 1) * np + pc] + (T - T1) * (p - p1) * m[(Tr + 1) * np + pc + 1];
  mean /= dT * dp;
  return mean;
}

GALES_MAGMA_HD void melt_props(const DevMagma& g, double p, double T, Props& o) {
  const double mv = g.melt_V + g.melt_dVdT * (T - 1673.0) + g.melt_dVdp * (p - 1.e5);  // Lange-Carmichael
  o.alpha = 1. / mv * g.melt_dVdT;
  o.beta = -1. / mv * g.melt_dVdp;
  o.rho = g.melt_M / mv;
  o.c = 1.0 / sqrt(o.rho * o.beta);
  o.cp = g.melt_cp;
  o.kappa = g.melt_kappa;
  o.cv = g.melt_cp - T * o.alpha * o.alpha / (o.rho * o.beta);
  o.D = 1.e-10;
}

GALES_MAGMA_HD void volatile_props(const DevMagma& g, int k, double p, double T, Props& o) {
  // molar volume polynomial of the dissolved volatiles (chemicals.hpp:155-160)
  const double a[10] = {9.144e-06, 3.685e-09, 1.168e-11, -1.990e-15, 1.220e-16,
                        -1.945e-17, -1.580e-21, 4.680e-24, 1.144e-26, -3.960e-33};
  const double mole_vol = a[0] + a[1] * T + a[2] * T * T + a[3] * T * T * T + p * (a[4] + a[5] * T + a[6] * T * T) +
                          p * p * (a[7] + a[8] * T) + a[9] * p * p * p;
  o.rho = g.vol_M[k] / mole_vol;
  o.alpha = a[1] + 2 * a[2] * T + 3 * a[3] * T * T + p * (a[5] + 2 * a[6] * T) + p * p * a[8];
  o.alpha /= mole_vol;
  o.beta = -((a[4] + a[5] * T + a[6] * T * T) + 2 * p * (a[7] + a[8] * T) + 3 * a[9] * p * p);
  o.beta /= mole_vol;
  o.c = 1.0 / sqrt(o.rho * o.beta);
  o.cp = g.vol_cp[k];
  o.kappa = g.vol_kappa[k];
  o.cv = g.vol_cp[k] - T * o.alpha * o.alpha / (o.rho * o.beta);
  o.D = 1.e-10;
}

GALES_MAGMA_HD void gas_props(const DevMagma& g, int k, double p, double T, Props& o) {
  o.rho = p / (g.gas_R[k] * T);
  o.beta = 1.0 / p;
  o.alpha = 1.0 / T;
  o.c = sqrt(g.gas_gamma[k] * g.gas_R[k] * T);
  o.cv = g.gas_cv[k];
  o.cp = g.gas_cp[k];
  o.kappa = g.gas_kappa[k];
  o.D = 1.e-10;
}

// computeViscosity (GiordanoEtAlViscosityModel.hpp:88-116)
GALES_MAGMA_HD double giordano_mu(const DevMagma& g, double T, double wf_h2o_l, double wf_co2_l, unsigned& st) {
  const double b5 = -84.1, b6 = 141.5, c5 = -99.5;
  if (1.0 - wf_co2_l == 0.0) {
    st |= GALES_MAGMA_VISCOSITY;
    return 0.0;
  }
  const double new_wf_h2o = wf_h2o_l / (1 - wf_co2_l);
  double x = 1 + 18.015 * (1 - new_wf_h2o) / (new_wf_h2o * g.visc_M);
  x = 1.0 / x;
  const double x_no = 1 - x;
  const double pct = 100.0 * x;
  const double* P = g.visc_P;
  const double Bv = P[1] * x_no + P[2] * x_no * x_no + P[3] * x_no * pct + (b5 + b6) * pct + b6 * log(1 + pct);
  const double Cv = P[4] * x_no + c5 * log(1 + pct) + P[5] * x_no * x_no + P[6] * x_no * pct;
  if (T - Cv == 0.0) {
    st |= GALES_MAGMA_VISCOSITY;
    return 0.0;
  }
  return pow(10., P[0] + Bv / (T - Cv));
}

// magma_mixture::properties (mixtures.hpp:163-176, submix_of_comp 187-250).  fr
// (optional): wf_ph_[g], wf_[3], wf_[4], vf_ph_[g], vf_[3], vf_[4] (mixtures.hpp:225-258),
// the fractions secondary_dofs.hpp:113-131 reads.
GALES_MAGMA_HD void magma_props(const DevMagma& g, double p, double T, double sr, Props& o, double& vf_gas,
                            unsigned& st, double* fr = nullptr) {
  double wl1, wl2;
  if (g.n_T == 0) {
    wl1 = lookup_p(g, g.h2o_tab, p, st);
    wl2 = lookup_p(g, g.co2_tab, p, st);
  } else {
    wl1 = lookup_Tp(g, g.h2o_tab, T, p, st);
    wl2 = lookup_Tp(g, g.co2_tab, T, p, st);
  }
  const double wl0 = 1.0 - wl1 - wl2;
  double wf[5];
  wf[0] = g.wf_comp[0];
  const double wl_ph = wf[0] / wl0;
  wf[1] = wl1 * wl_ph;
  wf[2] = wl2 * wl_ph;
  wf[3] = g.wf_comp[1] - wf[1];
  wf[4] = g.wf_comp[2] - wf[2];
  Props ch[5];
  melt_props(g, p, T, ch[0]);
  volatile_props(g, 0, p, T, ch[1]);
  volatile_props(g, 1, p, T, ch[2]);
  gas_props(g, 0, p, T, ch[3]);
  gas_props(g, 1, p, T, ch[4]);
  double rho = 0.0;
#pragma unroll
  for (int c = 0; c < 5; ++c) rho += wf[c] / ch[c].rho;
  rho = 1. / rho;
  rho = (1.0 - g.crystal_vf) * rho + g.crystal_vf * g.crystal_rho;
  double cp = 0.0, cv = 0.0, alpha = 0.0, beta = 0.0, kappa = 0.0, D = 0.0, ss = 0.0;
#pragma unroll
  for (int c = 0; c < 5; ++c) {
    cp += wf[c] * ch[c].cp;
    cv += wf[c] * ch[c].cv;
    alpha += wf[c] * ch[c].alpha * rho / ch[c].rho;
    beta += wf[c] * ch[c].beta * rho / ch[c].rho;
    kappa += wf[c] * ch[c].kappa;
    D += wf[c] * ch[c].D;
    ss += wf[c] / (pow(ch[c].rho, 2) * pow(ch[c].c, 2));
  }
  double cs = sqrt(1. / ss);
  cs /= rho;
  const double vf3 = wf[3] * rho / ch[3].rho, vf4 = wf[4] * rho / ch[4].rho;
  vf_gas = vf3 + vf4;
  if (fr) {
    fr[0] = 1.0 - wl_ph;
    fr[1] = wf[3];
    fr[2] = wf[4];
    fr[3] = vf_gas;
    fr[4] = vf3;
    fr[5] = vf4;
  }
  double mu = giordano_mu(g, T, wl1, wl2, st);
  if (g.gas_on_mu == GALES_GAS_MU_ISHII_ZUBER) {
    mu = mu / (1.0 - vf_gas);
  } else if (g.gas_on_mu == GALES_GAS_MU_PAL_2003 && !(sr < 2.220446049250313e-16)) {
    const double bubble_radius = cbrt(3.0 / (4 * 3.142 * 1.e11));
    const double Ca = bubble_radius * mu * sr / 0.36;
    const double a = 2.4 * pow(Ca, 2);
    const double TT = pow(1.0 - a, -0.8) * pow(1.0 - vf_gas / 0.9999, -0.9999);
    double x = 1.e-5, F;
    int it = 0;
    do {
      F = pow(x, 5) / pow(1.0 - a * x * x, 4) - pow(TT, 5);
      const double Fp = 5 * pow(x, 4) / pow(1.0 - a * x * x, 4) + 8 * a * pow(x, 6) / pow(1.0 - a * x * x, 5);
      x -= F / Fp;
    } while (F < 1.e-9 && ++it < 200);
    if (it >= 200) st |= GALES_MAGMA_PAL_ITER;
    mu = mu * x;
  }
  if (g.crystal_on_mu == GALES_CRYSTAL_MU_EINSTEIN_ROSCOE) {
    mu = mu * pow(1.0 - 1.0 * g.crystal_vf, -2.5);
  } else if (g.crystal_on_mu == GALES_CRYSTAL_MU_CARICCHI) {
    const double s = sr < 2.220446049250313e-16 ? 1.e-6 : sr;
    const double ls = log10(s);
    const double phi_max = 0.066499 * tanh(0.913424 * ls + 3.850623) + 0.591806;
    const double delta = -6.301095 * tanh(0.818496 * ls + 2.86) + 7.462405;
    const double alpha_c = -0.000378 * tanh(1.148101 * ls + 3.92) + 0.999572;
    const double gamma = 3.987815 * tanh(0.8908 * ls + 3.24) + 5.099645;
    const double phi = g.crystal_vf;
    const double num = 1.0 + pow(phi / phi_max, delta);
    const double xx = sqrt(3.142) * phi / (2 * alpha_c * phi_max) * (1.0 + pow(phi / phi_max, gamma));
    const double den = pow(1.0 - alpha_c * erf(xx), 2.5 * phi_max);
    mu = mu * (num / den);
  }
  o.rho = rho;
  o.cp = cp;
  o.cv = cv;
  o.alpha = alpha;
  o.beta = beta;
  o.kappa = kappa;
  o.D = D;
  o.c = cs;
  o.mu = mu;
}

// A sub-mixture of any kind at (p, T): magma_mix above; custom_mix
// (custom_mixture, mixtures.hpp:69-101: constant properties, sound speed 1e20 or
// 1/sqrt(rho beta), cv = cp or cp - T alpha^2/(rho beta)); ch_as_mix (mixtures.hpp:25-53:
// the chemical's properties, chemicals.hpp:19-49 custom, 198-271 ideal gas).  The last
// two keep base_chemical's diffusivity 1e-10 (base_chemical.hpp:86; they never clear()
// it) and have no gas phase.
GALES_MAGMA_HD void sub_props(const DevMagma& g, double p, double T, double sr, Props& o, double& vf_gas,
                              unsigned& st, double* fr = nullptr) {
  if (g.kind == GALES_SUBMIX_MAGMA) {
    magma_props(g, p, T, sr, o, vf_gas, st, fr);
    return;
  }
  vf_gas = 0.0;
  if (fr)
    for (int k = 0; k < 6; ++k) fr[k] = 0.0;
  o.D = 1.e-10;
  if (g.ch_kind == GALES_CH_CUSTOM) {
    o.rho = g.ch_rho;
    o.mu = g.ch_mu;
    o.cp = g.ch_cp;
    o.kappa = g.ch_kappa;
    o.alpha = g.ch_alpha;
    o.beta = g.ch_beta;
    o.c = (o.beta == 0.0) ? 1.e20 : 1.0 / sqrt(o.rho * o.beta);
    o.cv = (o.beta == 0.0) ? o.cp : o.cp - T * o.alpha * o.alpha / (o.rho * o.beta);
  } else {
    o.rho = p / (g.ch_R * T);
    o.beta = 1.0 / p;
    o.alpha = 1.0 / T;
    o.c = sqrt(g.ch_gamma * g.ch_R * T);
    o.cv = g.ch_cv;
    o.cp = g.ch_cp;
    o.mu = g.ch_mu;
    o.kappa = g.ch_kappa;
  }
}

// One point of the mixture of sub-mixtures (fluid_properties.hpp:171-200):
// f = rho, mu, cp, cv, kappa, sound speed, alpha, beta; comp[c] = rho_c, cv_c T, chemical
// diffusivity, gas volume fraction.  Returns the status bits.
GALES_MAGMA_HD unsigned mix_point(const DevMagma* mg, int nc, double p, double T, const double* Y, double sr,
                                  double* f, double (*comp)[4]) {
  unsigned st = 0;
  double rho = 0, mu = 0, cp = 0, cv = 0, kappa = 0, ss = 0;
  double rho_c[GALES_MAX_COMP], alpha_c[GALES_MAX_COMP], beta_c[GALES_MAX_COMP];
  for (int c = 0; c < nc; ++c) {
    Props m;
    double vfg;
    sub_props(mg[c], p, T, sr, m, vfg, st);
    const double y = Y[c];
    rho += y / m.rho;
    mu += y * m.mu;
    cp += y * m.cp;
    cv += y * m.cv;
    kappa += y * m.kappa;
    ss += y / (pow(m.rho, 2) * pow(m.c, 2));
    rho_c[c] = m.rho;
    alpha_c[c] = m.alpha;
    beta_c[c] = m.beta;
    comp[c][0] = m.rho;
    comp[c][1] = m.cv * T;
    comp[c][2] = m.D;
    comp[c][3] = vfg;
  }
  rho = 1.0 / rho;
  double cs = sqrt(1. / ss);
  cs /= rho;
  double alpha = 0.0, beta = 0.0;
  for (int c = 0; c < nc; ++c) {
    alpha += Y[c] * alpha_c[c] * rho / rho_c[c];
    beta += Y[c] * beta_c[c] * rho / rho_c[c];
  }
  f[0] = rho;
  f[1] = mu;
  f[2] = cp;
  f[3] = cv;
  f[4] = kappa;
  f[5] = cs;
  f[6] = alpha;
  f[7] = beta;
  return st;
}

// secondary_dofs::execute's gas fractions (pp_vf_g, secondary_dofs.hpp:56-131) at one
// node (shear rate 0): out[2c] = vf_g_comp_c, out[2c + 1] = vf_comp_c for every magma c,
// then vf_g_on_total, vf_h2o_g_on_total, vf_co2_g_on_total, wf_g_on_total,
// wf_h2o_g_on_total, wf_co2_g_on_total (2 nc + 6 values).  Returns the status bits.
GALES_MAGMA_HD unsigned mix_fractions(const DevMagma* mg, int nc, double p, double T, const double* Y,
                                      double* out) {
  unsigned st = 0;
  double rho = 0.0, rho_c[GALES_MAX_COMP], fr[GALES_MAX_COMP][6];
  for (int c = 0; c < nc; ++c) {
    Props m;
    double vfg;
    sub_props(mg[c], p, T, 0.0, m, vfg, st, fr[c]);
    rho += Y[c] / m.rho;
    rho_c[c] = m.rho;
  }
  rho = 1.0 / rho;
  double vf_g = 0.0, vf_h2o = 0.0, vf_co2 = 0.0, wf_g = 0.0, wf_h2o = 0.0, wf_co2 = 0.0;
  for (int c = 0; c < nc; ++c) {
    const double vf_comp = Y[c] * rho / rho_c[c];
    out[2 * c] = fr[c][3] * vf_comp;
    out[2 * c + 1] = vf_comp;
    vf_g += fr[c][3] * vf_comp;
    vf_h2o += fr[c][4] * vf_comp;
    vf_co2 += fr[c][5] * vf_comp;
    wf_g += fr[c][0] * Y[c];
    wf_h2o += fr[c][1] * Y[c];
    wf_co2 += fr[c][2] * Y[c];
  }
  out[2 * nc] = vf_g;
  out[2 * nc + 1] = vf_h2o;
  out[2 * nc + 2] = vf_co2;
  out[2 * nc + 3] = wf_g;
  out[2 * nc + 4] = wf_h2o;
  out[2 * nc + 5] = wf_co2;
  return st;
}

}  // namespace magma_mix
