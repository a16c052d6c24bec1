/*
 * TEST INFRASTRUCTURE — NOT PART OF THE PRODUCT.
 *
 * CPU restatement ("oracle") of the magma mixture properties of GALES-multi-fluid, used
 * only by tests/ as the checker:
 *   - magma_mixture (src/fem/physical_props/fluid/mixtures.hpp:114-511): liquid-phase
 *     volatile fractions from the solubility lookup tables (1D in p, or bilinear in (T, p)),
 *     the five chemicals melt, H2O(l), CO2(l), H2O(g), CO2(g), their mass-weighted mixing,
 *     Giordano et al. (2008) viscosity and the gas (Ishii-Zuber, Pal 2003) and crystal
 *     (Einstein-Roscoe, Caricchi) corrections;
 *   - the chemicals melt (Lange-Carmichael volume, chemicals.hpp:56-145),
 *     dissolved_volatiles (chemicals.hpp:149-194) and named ideal gases (198-271);
 *   - GiordanoEtAlViscosityModel (GiordanoEtAlViscosityModel.hpp:36-116);
 *   - fluid_properties' mixture of sub-mixtures (fluid_properties.hpp:171-200).
 * The constants and operation orders are the reference's.  The chemicals (melt,
 * dissolved_volatiles, ideal_gas) and the Giordano model are pinned bit for bit against
 * the reference's own chemicals.hpp and GiordanoEtAlViscosityModel.hpp, compiled from its
 * checkout (ref_classes.cpp, tests/test_reference_pins.py).  The rest (the magma
 * mixture of mixtures.hpp, which needs Boost uBLAS) is UNPINNED: it cannot be built here
 * and the reference ships no expected values for it.
 * Pal 2003's Newton iteration (mixtures.hpp:266-289) loops while F < 1e-9; the
 * restatement stops after 200 steps and reports that.
 */
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <vector>

#include "../include/gales_asm.h"

namespace {

struct Chem {
  double rho = 0, cv = 0, cp = 0, kappa = 0, D = 1e-10, mu = 0, c = 0, alpha = 0, beta = 0;
};

struct Melt {
  double wf[10], mm[10], xf[10];
  double dVdT = 0, dVdp = 0, V = 0, M = 0, cp = 0, kappa = 0;
  void init(const double* oxide_wf, double k) {
    double sum = 0.0;
    for (int i = 0; i < 10; ++i) sum += oxide_wf[i];
    for (int i = 0; i < 10; ++i) wf[i] = oxide_wf[i] / sum;
    const double m0[10] = {60.084, 79.876, 101.956, 159.692, 71.846, 70.937, 40.304, 56.078, 61.979, 94.195};
    for (int i = 0; i < 10; ++i) mm[i] = m0[i] * 1.e-3;
    M = 0.0;
    for (int i = 0; i < 10; ++i) M += wf[i] / mm[i];
    M = 1. / M;
    for (int i = 0; i < 10; ++i) xf[i] = wf[i] * M / mm[i];
    const double dT[10] = {0.0, 7.24, 0.0, 9.09, 2.92, 0.0, 3.27, 3.74, 7.68, 12.08};
    dVdT = 0.0;
    for (int i = 0; i < 10; ++i) dVdT += xf[i] * (dT[i] * 1.e-9);
    const double dp[10] = {-1.89, -2.31, -2.26, -2.53, -0.45, 0.0, 0.27, 0.34, -2.4, -6.75};
    dVdp = 0.0;
    for (int i = 0; i < 10; ++i) dVdp += xf[i] * (dp[i] * 1.e-15);
    const double v0[10] = {26.86, 23.16, 37.42, 42.13, 13.65, 0.0, 11.69, 16.53, 28.88, 45.07};
    V = 0.0;
    for (int i = 0; i < 10; ++i) V += xf[i] * (v0[i] * 1.e-6);
    const double c0[10] = {1331.0, 1392.0, 1545.0, 1434.0, 1100.0, 0.0, 2424.0, 1781.0, 1651.0, 1030.0};
    cp = 0.0;
    for (int i = 0; i < 10; ++i) cp += xf[i] * c0[i];
    kappa = k;
  }
  void props(double p, double T, Chem& o) const {
    const double mv = V + dVdT * (T - 1673.0) + dVdp * (p - 1.e5);
    o.alpha = 1. / mv * dVdT;
    o.beta = -1. / mv * dVdp;
    o.rho = M / mv;
    o.c = 1.0 / std::sqrt(o.rho * o.beta);
    o.cp = cp;
    o.kappa = kappa;
    o.cv = cp - T * o.alpha * o.alpha / (o.rho * o.beta);
  }
};

struct Volatile {
  double M = 0, cp = 0, kappa = 0;
  double a[10] = {9.144e-06, 3.685e-09, 1.168e-11, -1.990e-15, 1.220e-16, -1.945e-17, -1.580e-21, 4.680e-24,
                  1.144e-26, -3.960e-33};
  void props(double p, double T, Chem& o) const {
    const double mole_vol = a[0] + a[1] * T + a[2] * T * T + a[3] * T * T * T + p * (a[4] + a[5] * T + a[6] * T * T) +
                            p * p * (a[7] + a[8] * T) + a[9] * p * p * p;
    o.rho = M / mole_vol;
    o.alpha = a[1] + 2 * a[2] * T + 3 * a[3] * T * T + p * (a[5] + 2 * a[6] * T) + p * p * a[8];
    o.alpha /= mole_vol;
    o.beta = -((a[4] + a[5] * T + a[6] * T * T) + 2 * p * (a[7] + a[8] * T) + 3 * a[9] * p * p);
    o.beta /= mole_vol;
    o.c = 1.0 / std::sqrt(o.rho * o.beta);
    o.cp = cp;
    o.kappa = kappa;
    o.cv = cp - T * o.alpha * o.alpha / (o.rho * o.beta);
  }
};

struct Gas {
  double M = 0, gamma = 1.4, R = 0, cv = 0, cp = 0, mu = 1e-5, kappa = 0;
  void init(double m) {
    M = m;
    gamma = 1.4;
    R = 8.314462 / M;
    cv = R / (gamma - 1.0);
    cp = gamma * cv;
    mu = 1.e-5;
    kappa = mu * cp / 0.72;
  }
  void props(double p, double T, Chem& o) const {
    o.rho = p / (R * T);
    o.beta = 1.0 / p;
    o.alpha = 1.0 / T;
    o.c = std::sqrt(gamma * R * T);
    o.cv = cv;
    o.cp = cp;
    o.kappa = kappa;
    o.mu = mu;
  }
};

struct Giordano {
  double M = 0.0, P[7] = {0, 0, 0, 0, 0, 0, 0};
  const double b[7] = {159.6, -173.3, 72.1, 75.7, -39.0, -84.1, 141.5};
  const double b1[3] = {-2.43, -0.91, 17.6};
  const double c[6] = {2.75, 15.7, 8.3, 10.2, -12.3, -99.5};
  void set(const double* oxide_wf, const double* oxide_mm) {
    double mm[10], w[10];
    for (int i = 0; i < 10; ++i) mm[i] = oxide_mm[i] * 1.e3;
    for (int i = 0; i < 10; ++i) w[i] = oxide_wf[i];
    w[4] = 0.9309 * (w[3] + w[4]);
    w[3] = 0.0;
    double sum = 0.0;
    for (int i = 0; i < 10; ++i) sum += w[i];
    for (int i = 0; i < 10; ++i) w[i] /= sum;
    M = 0.0;
    for (int i = 0; i < 10; ++i) M += w[i] / mm[i];
    M = 1.0 / M;
    double m[10];
    for (int i = 0; i < 10; ++i) m[i] = 100.0 * w[i] * M / mm[i];
    P[0] = -4.55;
    P[1] = b[0] * (m[0] + m[1]) + b[1] * m[2] + b[2] * (m[4] + m[5]) + b[3] * m[6] + b[4] * m[7] + b[5] * m[8];
    P[2] = b1[0] * (m[0] + m[1]) * (m[4] + m[5] + m[6]) + b1[1] * (m[0] + m[1] + m[2]) * (m[8] + m[9]) +
           b1[2] * m[2] * (m[8] + m[9]);
    P[3] = b1[1] * (m[0] + m[1] + m[2]);
    P[4] = c[0] * m[0] + c[1] * (m[1] + m[2]) + c[2] * (m[4] + m[5] + m[6]) + c[3] * m[7] + c[4] * (m[8] + m[9]);
    P[5] = 0.3 * (m[2] + m[4] + m[5] + m[6] + m[7]) * (m[8] + m[9]);
    P[6] = 0.3 * (m[2] + m[4] + m[5] + m[6] + m[7]);
  }
  // returns false on the reference's two error exits
  bool mu(double T, double wf_h2o_l, double wf_co2_l, double& out) const {
    const double h2o_mm = 18.015;
    if (1.0 - wf_co2_l == 0.0) return false;
    const double new_wf_h2o = wf_h2o_l / (1 - wf_co2_l);
    double x = 1 + h2o_mm * (1 - new_wf_h2o) / (new_wf_h2o * M);
    x = 1.0 / x;
    const double x_no = 1 - x;
    const double pct = 100.0 * x;
    const double A = P[0];
    const double B = P[1] * x_no + P[2] * x_no * x_no + P[3] * x_no * pct + (b[5] + b[6]) * pct + b[6] * std::log(1 + pct);
    const double C = P[4] * x_no + c[5] * std::log(1 + pct) + P[5] * x_no * x_no + P[6] * x_no * pct;
    if (T - C == 0.0) return false;
    out = std::pow(10., A + B / (T - C));
    return true;
  }
};

struct Magma {
  Melt melt;
  Volatile h2o_l, co2_l;
  Gas h2o_g, co2_g;
  Giordano visc;
  double wf_comp[3];
  double crystal_vf = 0, crystal_rho = 0;
  int gas_on_mu = 0, crystal_on_mu = 0;
  std::vector<double> p_tab, T_tab, h2o_tab, co2_tab;
  int kind = GALES_SUBMIX_MAGMA;   // magma_mix, custom_mix or ch_as_mix
  gales_chemical_desc ch{};        // custom_mix / ch_as_mix constants
};

// custom_mixture::properties (mixtures.hpp:69-101) and ch_as_mix::properties
// (mixtures.hpp:25-53) over custom_chemical (chemicals.hpp:19-49) or ideal_gas
// (chemicals.hpp:198-271).  The diffusivity is base_chemical's 1e-10 (base_chemical.hpp:86):
// neither class clears or copies it.
void submix_props(const Magma& g, double p, double T, Chem& o) {
  o = Chem();
  o.D = 1.e-10;
  const bool custom = g.kind == GALES_SUBMIX_CUSTOM || g.ch.kind == GALES_CH_CUSTOM;
  if (custom) {
    o.rho = g.ch.rho;
    o.mu = g.ch.mu;
    o.cp = g.ch.cp;
    o.alpha = g.ch.alpha;
    o.beta = g.ch.beta;
    o.kappa = g.ch.kappa;
    if (o.beta == 0.0) o.c = 1.e20;
    else o.c = 1.0 / std::sqrt(o.rho * o.beta);
    if (o.beta == 0.0) o.cv = o.cp;
    else o.cv = o.cp - T * o.alpha * o.alpha / (o.rho * o.beta);
  } else {
    o.rho = p / (g.ch.R * T);
    o.beta = 1.0 / p;
    o.alpha = 1.0 / T;
    o.c = std::sqrt(g.ch.gamma * g.ch.R * T);
    o.cv = g.ch.cv;
    o.cp = g.ch.cp;
    o.mu = g.ch.mu;
    o.kappa = g.ch.kappa;
  }
}

double interp1(double p, const std::vector<double>& pt, const std::vector<double>& y, bool& ok) {
  const double dp = pt[1] - pt[0];
  const std::size_t i = (std::size_t)(int)std::floor((p - pt[0]) / dp);
  if (i >= pt.size() || i + 1 >= pt.size()) {
    ok = false;
    return 0.0;
  }
  const double slope = (y[i + 1] - y[i]) / dp;
  return y[i] + slope * (p - pt[i]);
}

double interp2(double T, double p, const std::vector<double>& Tt, const std::vector<double>& pt,
               const std::vector<double>& m, bool& ok) {
  const double dp = std::fabs(pt[1] - pt[0]);
  const std::size_t pc = (std::size_t)(int)std::floor(std::fabs(p - pt[0]) / dp);
  const double dT = std::fabs(Tt[1] - Tt[0]);
  const std::size_t Tr = (std::size_t)(int)std::floor(std::fabs(T - Tt[0]) / dT);
  if (pc >= pt.size() || pc + 1 >= pt.size() || Tr >= Tt.size() || Tr + 1 >= Tt.size()) {
    ok = false;
    return 0.0;
  }
  const std::size_t np = pt.size();
  const double p1 = pt[pc], p2 = pt[pc + 1], T1 = Tt[Tr], T2 = Tt[Tr + 1];
  double mean = (T2 - T) * (p2 - p) * m[Tr * np + pc] + (T2 - T) * (p - p1) * m[Tr * np + pc + 1] +
                (T - T1) * (p2 - p) * m[(Tr + 1) * np + pc] + (T - T1) * (p - p1) * m[(Tr + 1) * np + pc + 1];
  mean /= dT * dp;
  return mean;
}

// status bits: 1 lookup out of range, 2 viscosity model division, 4 Pal 2003 not converged
// fr (optional): the phase and chemical fractions secondary_dofs.hpp:113-131 reads,
// wf_ph_[g], wf_[3], wf_[4], vf_ph_[g], vf_[3], vf_[4] (mixtures.hpp:225-258).
int magma_props(const Magma& g, double p, double T, double sr, Chem& o, double& vf_gas, double* fr = nullptr) {
  if (g.kind != GALES_SUBMIX_MAGMA) {
    submix_props(g, p, T, o);
    vf_gas = 0.0;
    if (fr)
      for (int k = 0; k < 6; ++k) fr[k] = 0.0;
    return 0;
  }
  int st = 0;
  bool ok = true;
  double wl[3];
  if (g.T_tab.empty()) {
    wl[1] = interp1(p, g.p_tab, g.h2o_tab, ok);
    wl[2] = interp1(p, g.p_tab, g.co2_tab, ok);
  } else {
    wl[1] = interp2(T, p, g.T_tab, g.p_tab, g.h2o_tab, ok);
    wl[2] = interp2(T, p, g.T_tab, g.p_tab, g.co2_tab, ok);
  }
  if (!ok) st |= 1;
  wl[0] = 1.0 - wl[1] - wl[2];
  double wf[5];
  wf[0] = g.wf_comp[0];
  const double wl_ph = wf[0] / wl[0];
  const double wg_ph = 1.0 - wl_ph;
  (void)wg_ph;
  wf[1] = wl[1] * wl_ph;
  wf[2] = wl[2] * wl_ph;
  wf[3] = g.wf_comp[1] - wf[1];
  wf[4] = g.wf_comp[2] - wf[2];
  Chem ch[5];
  g.melt.props(p, T, ch[0]);
  g.h2o_l.props(p, T, ch[1]);
  g.co2_l.props(p, T, ch[2]);
  g.h2o_g.props(p, T, ch[3]);
  g.co2_g.props(p, T, ch[4]);
  o = Chem();
  o.D = 0.0;
  o.rho = 0.0;
  for (int c = 0; c < 5; ++c) o.rho += wf[c] / ch[c].rho;
  o.rho = 1. / o.rho;
  o.rho = (1.0 - g.crystal_vf) * o.rho + g.crystal_vf * g.crystal_rho;
  double ss = 0.0;
  for (int c = 0; c < 5; ++c) {
    o.cp += wf[c] * ch[c].cp;
    o.cv += wf[c] * ch[c].cv;
    o.alpha += wf[c] * ch[c].alpha * o.rho / ch[c].rho;
    o.beta += wf[c] * ch[c].beta * o.rho / ch[c].rho;
    o.kappa += wf[c] * ch[c].kappa;
    o.D += wf[c] * ch[c].D;
    ss += wf[c] / (std::pow(ch[c].rho, 2) * std::pow(ch[c].c, 2));
  }
  o.c = std::sqrt(1. / ss);
  o.c /= o.rho;
  double vf[5];
  for (int c = 0; c < 5; ++c) vf[c] = wf[c] * o.rho / ch[c].rho;
  vf_gas = vf[3] + vf[4];
  if (fr) {
    fr[0] = wg_ph;
    fr[1] = wf[3];
    fr[2] = wf[4];
    fr[3] = vf_gas;
    fr[4] = vf[3];
    fr[5] = vf[4];
  }
  double mu = 0.0;
  if (!g.visc.mu(T, wl[1], wl[2], mu)) st |= 2;
  if (g.gas_on_mu == GALES_GAS_MU_ISHII_ZUBER) {
    mu = mu / (1.0 - vf_gas);
  } else if (g.gas_on_mu == GALES_GAS_MU_PAL_2003) {
    if (!(sr < std::numeric_limits<double>::epsilon())) {
      const double surface_tension = 0.36, bubble_number_density = 1.e11, max_volume_packing = 0.9999;
      const double bubble_radius = std::cbrt(3.0 / (4 * 3.142 * bubble_number_density));
      const double Ca = bubble_radius * mu * sr / surface_tension;
      const double a = 2.4 * std::pow(Ca, 2);
      const double TT = std::pow(1.0 - a, -0.8) * std::pow(1.0 - vf_gas / max_volume_packing, -max_volume_packing);
      double x = 1.e-5, F;
      int it = 0;
      do {
        F = std::pow(x, 5) / std::pow(1.0 - a * x * x, 4) - std::pow(TT, 5);
        const double Fp = 5 * std::pow(x, 4) / std::pow(1.0 - a * x * x, 4) + 8 * a * std::pow(x, 6) / std::pow(1.0 - a * x * x, 5);
        x -= F / Fp;
      } while (F < 1.e-9 && ++it < 200);
      if (it >= 200) st |= 4;
      mu = mu * x;
    }
  }
  if (g.crystal_on_mu == GALES_CRYSTAL_MU_EINSTEIN_ROSCOE) {
    mu = mu * std::pow(1.0 - 1.0 * g.crystal_vf, -2.5);
  } else if (g.crystal_on_mu == GALES_CRYSTAL_MU_CARICCHI) {
    double s = sr;
    if (s < std::numeric_limits<double>::epsilon()) s = 1.e-6;
    const double phi_max = 0.066499 * std::tanh(0.913424 * std::log10(s) + 3.850623) + 0.591806;
    const double delta = -6.301095 * std::tanh(0.818496 * std::log10(s) + 2.86) + 7.462405;
    const double alpha = -0.000378 * std::tanh(1.148101 * std::log10(s) + 3.92) + 0.999572;
    const double gamma = 3.987815 * std::tanh(0.8908 * std::log10(s) + 3.24) + 5.099645;
    const double phi = g.crystal_vf;
    const double num = 1.0 + std::pow(phi / phi_max, delta);
    const double x = std::sqrt(3.142) * phi / (2 * alpha * phi_max) * (1.0 + std::pow(phi / phi_max, gamma));
    const double den = std::pow(1.0 - alpha * std::erf(x), 2.5 * phi_max);
    mu = mu * (num / den);
  }
  o.mu = mu;
  return st;
}

void build(const gales_magma_desc& d, Magma& g) {
  g.kind = d.kind;
  g.ch = d.chemical;
  if (d.kind != GALES_SUBMIX_MAGMA) return;
  g.wf_comp[1] = d.h2o_wf;
  g.wf_comp[2] = d.co2_wf;
  g.wf_comp[0] = 1.0 - g.wf_comp[1] - g.wf_comp[2];
  g.melt.init(d.oxide_wf, d.melt_kappa);
  g.h2o_l.M = 0.01802;
  g.h2o_l.cp = d.h2o_l_cp;
  g.h2o_l.kappa = d.h2o_l_kappa;
  g.co2_l.M = 0.04401;
  g.co2_l.cp = d.co2_l_cp;
  g.co2_l.kappa = d.co2_l_kappa;
  g.h2o_g.init(0.01802);
  g.co2_g.init(0.04401);
  g.visc.set(g.melt.wf, g.melt.mm);
  g.crystal_vf = d.crystal_fraction;
  g.crystal_rho = d.crystal_rho;
  g.gas_on_mu = d.gas_on_mu;
  g.crystal_on_mu = d.crystal_on_mu;
  g.p_tab.assign(d.p_table, d.p_table + d.n_p);
  if (d.n_T > 0) {
    g.T_tab.assign(d.T_table, d.T_table + d.n_T);
    g.h2o_tab.assign(d.wf_l_h2o, d.wf_l_h2o + (size_t)d.n_T * d.n_p);
    g.co2_tab.assign(d.wf_l_co2, d.wf_l_co2 + (size_t)d.n_T * d.n_p);
  } else {
    g.h2o_tab.assign(d.wf_l_h2o, d.wf_l_h2o + d.n_p);
    g.co2_tab.assign(d.wf_l_co2, d.wf_l_co2 + d.n_p);
  }
}

std::vector<Magma> g_active;  // magmas that replace the chemicals in the assembly (gor_set_magma)

}  // namespace

// Used by the assembly restatement (gales_oracle.cpp) when magmas are set: the mixture
// of sub-mixtures at (p, T, Y) with shear rate sr, f = rho, mu, cp, cv, kappa, sound speed,
// alpha, beta; comp[c] = rho_c, cv_c T, D_c.  Returns the status bits.
bool gor_magma_active() { return !g_active.empty(); }

int gor_magma_point(double p, double T, const double* Y, double sr, double* f, double (*comp)[3]) {
  const int nc = (int)g_active.size();
  int st = 0;
  double rho = 0, mu = 0, cp = 0, cv = 0, kappa = 0, ss = 0;
  Chem m[GALES_MAX_COMP];
  for (int c = 0; c < nc; ++c) {
    double vfg = 0.0;
    st |= magma_props(g_active[c], p, T, sr, m[c], vfg);
    rho += Y[c] / m[c].rho;
    mu += Y[c] * m[c].mu;
    cp += Y[c] * m[c].cp;
    cv += Y[c] * m[c].cv;
    kappa += Y[c] * m[c].kappa;
    ss += Y[c] / (std::pow(m[c].rho, 2) * std::pow(m[c].c, 2));
    comp[c][0] = m[c].rho;
    comp[c][1] = m[c].cv * T;
    comp[c][2] = m[c].D;
  }
  rho = 1.0 / rho;
  double cs = std::sqrt(1. / ss);
  cs /= rho;
  double alpha = 0.0, beta = 0.0;
  for (int c = 0; c < nc; ++c) {
    alpha += Y[c] * m[c].alpha * rho / m[c].rho;
    beta += Y[c] * m[c].beta * rho / m[c].rho;
  }
  const double o[8] = {rho, mu, cp, cv, kappa, cs, alpha, beta};
  for (int k = 0; k < 8; ++k) f[k] = o[k];
  return st;
}

extern "C" {

// Replace the material's chemicals by nc magma mixtures in every later assembly,
// element and property call of the oracle (nc = 0 restores the chemicals).
int gor_set_magma(const gales_magma_desc* comps, int32_t nc) {
  g_active.clear();
  if (nc <= 0) return 0;
  g_active.resize(nc);
  for (int c = 0; c < nc; ++c) build(comps[c], g_active[c]);
  return 0;
}

// fluid_properties::properties, mix_of_mix branch (fluid_properties.hpp:171-200), for n
// points: out[f * n + i] with f = rho, mu, cp, cv, kappa, sound speed, alpha, beta;
// comp[(c * 4 + k) * n + i] with k = rho_c, e_c = cv_c T, D_c, gas volume fraction.
// Y[i * nc + c] holds all nc mass fractions.  Returns the OR of the status bits.
int gor_magma_properties(const gales_magma_desc* comps, int32_t nc, const double* p, const double* T,
                         const double* Y, const double* shear, int64_t n, double* out, double* comp) {
  std::vector<Magma> g(nc);
  for (int c = 0; c < nc; ++c) build(comps[c], g[c]);
  int st = 0;
  for (int64_t i = 0; i < n; ++i) {
    double rho = 0, mu = 0, cp = 0, cv = 0, kappa = 0, ss = 0, alpha = 0, beta = 0;
    std::vector<Chem> m(nc);
    for (int c = 0; c < nc; ++c) {
      double vfg = 0.0;
      st |= magma_props(g[c], p[i], T[i], shear ? shear[i] : 0.0, m[c], vfg);
      const double y = Y[i * nc + c];
      rho += y / m[c].rho;
      mu += y * m[c].mu;
      cp += y * m[c].cp;
      cv += y * m[c].cv;
      kappa += y * m[c].kappa;
      ss += y / (std::pow(m[c].rho, 2) * std::pow(m[c].c, 2));
      if (comp) {
        comp[(c * 4 + 0) * n + i] = m[c].rho;
        comp[(c * 4 + 1) * n + i] = m[c].cv * T[i];
        comp[(c * 4 + 2) * n + i] = m[c].D;
        comp[(c * 4 + 3) * n + i] = vfg;
      }
    }
    rho = 1.0 / rho;
    double c_s = std::sqrt(1. / ss);
    c_s /= rho;
    for (int c = 0; c < nc; ++c) {
      const double y = Y[i * nc + c];
      alpha += y * m[c].alpha * rho / m[c].rho;
      beta += y * m[c].beta * rho / m[c].rho;
    }
    const double f[8] = {rho, mu, cp, cv, kappa, c_s, alpha, beta};
    for (int k = 0; k < 8; ++k) out[k * n + i] = f[k];
  }
  return st;
}

}  // extern "C"

// The restated chemicals and viscosity model one at a time, for the pins against the
// reference's own classes (tests/test_reference_pins.py): out[0..8] = rho, mu, cp, cv,
// kappa, sound speed, alpha, beta, chemical diffusivity, set up as build() sets them up.
namespace {
void chem_out(const Chem& c, double* o) {
  const double v[9] = {c.rho, c.mu, c.cp, c.cv, c.kappa, c.c, c.alpha, c.beta, c.D};
  for (int k = 0; k < 9; ++k) o[k] = v[k];
}
}  // namespace

extern "C" int gor_melt_props(const double* oxide_wf, double kappa, double p, double T, double* out) {
  Melt m;
  m.init(oxide_wf, kappa);
  Chem c;
  m.props(p, T, c);
  chem_out(c, out);
  return 0;
}

// molar_mass 0.01802 (H2O) or 0.04401 (CO2), as build() sets them
extern "C" int gor_volatile_props(double molar_mass, double cp, double kappa, double p, double T, double* out) {
  Volatile v;
  v.M = molar_mass;
  v.cp = cp;
  v.kappa = kappa;
  Chem c;
  v.props(p, T, c);
  chem_out(c, out);
  return 0;
}

extern "C" int gor_gas_props(double molar_mass, double p, double T, double* out) {
  Gas g;
  g.init(molar_mass);
  Chem c;
  g.props(p, T, c);
  chem_out(c, out);
  return 0;
}

// Giordano viscosity of the melt of the given oxide weight fractions; -1 on the
// reference's error exits
extern "C" int gor_giordano_mu(const double* oxide_wf, double T, double wf_h2o_l, double wf_co2_l, double* mu) {
  Melt m;
  m.init(oxide_wf, 1.0);
  Giordano g;
  g.set(m.wf, m.mm);
  return g.mu(T, wf_h2o_l, wf_co2_l, *mu) ? 0 : -1;
}

// secondary_dofs::execute's gas fractions (pp_vf_g, secondary_dofs.hpp:56-131) at one
// node's (p, T, Y) with the set magmas, shear rate 0: out[2c] = vf_g_comp_c,
// out[2c + 1] = vf_comp_c for every magma c, then vf_g_on_total, vf_h2o_g_on_total,
// vf_co2_g_on_total, wf_g_on_total, wf_h2o_g_on_total, wf_co2_g_on_total.
extern "C" int gor_magma_fractions(double p, double T, const double* Y, double* out) {
  const int nc = (int)g_active.size();
  if (nc == 0) return -1;
  int st = 0;
  Chem m[GALES_MAX_COMP];
  double fr[GALES_MAX_COMP][6];
  double rho = 0.0;
  for (int c = 0; c < nc; ++c) {
    double vfg = 0.0;
    st |= magma_props(g_active[c], p, T, 0.0, m[c], vfg, fr[c]);
    rho += Y[c] / m[c].rho;   // fluid_properties.hpp:174, 185
  }
  rho = 1.0 / rho;
  double vf_g = 0.0, vf_h2o = 0.0, vf_co2 = 0.0, wf_g = 0.0, wf_h2o = 0.0, wf_co2 = 0.0;
  for (int c = 0; c < nc; ++c) {
    const double vf_comp = Y[c] * rho / m[c].rho;
    out[2 * c] = fr[c][3] * vf_comp;
    out[2 * c + 1] = vf_comp;
    vf_g += (fr[c][3]) * vf_comp;
    vf_h2o += (fr[c][4]) * vf_comp;
    vf_co2 += (fr[c][5]) * vf_comp;
    wf_g += (fr[c][0]) * Y[c];
    wf_h2o += (fr[c][1]) * Y[c];
    wf_co2 += (fr[c][2]) * Y[c];
  }
  const double tot[6] = {vf_g, vf_h2o, vf_co2, wf_g, wf_h2o, wf_co2};
  for (int k = 0; k < 6; ++k) out[2 * nc + k] = tot[k];
  return st;
}
