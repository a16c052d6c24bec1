// Point-level physics of the fluid_mc element integral, evaluated in FP64 at one
// quadrature point: mixture EOS, conservative variables, the frozen-coefficient
// matrices in structured (formula) form, the stabilisation parameter tau and the
// discontinuity-capturing viscosity.  Generic in the space dimension DIM and the
// number of components NC; ND = DIM + 1 + NC dofs per node, ordered
// (p, v_1..v_DIM, T, Y_1..Y_{NC-1}) with conservative rows (rho, rho v, rho E, rho Y).
//
// Reference: sim/fluid_mc/P0/fluid_2d.hpp (2D only; the 3D form here is the
// dimension-generic extension), src/fem/physical_props/fluid/fluid_properties.hpp,
// chemicals.hpp, src/fem/mesh/quad.hpp, src/fem/base/algorithm.hpp.
#pragma once

#include <cstdint>

#include "../../include/gales_asm.h"
#include "gales_magma.cuh"

namespace gales {

constexpr double kEps = 2.220446049250313e-16;  // DBL_EPSILON, fluid_2d.hpp:93

// The library is compiled without floating-point contraction (-fmad=false) so that
// the point-level physics performs exactly the IEEE operations of the reference, in
// its order.  This matters beyond rounding: compute_h (quad.hpp:367-375) decides
// between normalising and not normalising the cross-stream direction from a value
// that is pure rounding noise whenever the element's velocity field is rank one
// (e.g. every node but one on a no-slip wall), so only identical arithmetic takes
// identical branches.  The matrix-phase loops, whose summation order is already
// restructured, request fused multiply-adds explicitly through madd().
__device__ __forceinline__ double madd(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ float madd(float a, float b, float c) { return fmaf(a, b, c); }

struct DevChem {
  int32_t kind;
  int32_t pad;
  double rho, mu, cp, cv, kappa, alpha, beta, R, gamma, D;
  // reciprocals and ratios for the mixed form's EOS (filled on the host)
  double inv_rho, beta_over_rho, alpha_over_rho, cv_shift, inv_R, R_over_gamma, inv_D;
  double c2_coef;  // custom chemical: its 1/(rho_c^2 s_c^2) per unit Y_c
};

// The hardware conversions between binary64 and binary32 issue on the FP64 pipe,
// which the point stage already saturates, and a conversion kept for rare operands
// behind a branch is still issued (predicated off) for every value.  narrow_rn and
// widen are therefore integer-only, on the two 32-bit words of the binary64 value.

// Round-to-nearest-even narrowing of binary64 to binary32 (52-bit significand cut to
// 23 bits, ties to even, carry into the exponent, overflow to infinity, NaN kept
// quiet).  Results below the smallest normal binary32 (|x| < 2^-126) flush to a
// signed zero instead of a subnormal.
__device__ __forceinline__ float narrow_rn(double d) {
  const unsigned int hi = (unsigned int)__double2hiint(d), lo = (unsigned int)__double2loint(d);
  const unsigned int ah = hi & 0x7fffffffu, sign = hi & 0x80000000u;
  if (ah - 0x38100000u < 0x0fe00000u) {
    // binary64 exponent e64 in [897, 1150], a normal binary32 before rounding.  The
    // funnel shift of (hi:lo) by 3 holds the low 9 bits of e64 above the top 23
    // significand bits; subtracting 384 << 23 rebiases the exponent field modulo 2^9
    // (e64 - 896 < 256, so bit 31 ends clear).  Round to nearest even on the 29 dropped
    // bits: adding 2^28 - 1 + (bits & 1) to them carries into bit 29 exactly when they
    // exceed half, or equal half with bits odd; a carry out of the significand steps the
    // exponent (to infinity from the largest binade).
    unsigned int bits = __funnelshift_l(lo, hi, 3) - 0xc0000000u;
    bits += ((lo & 0x1fffffffu) + 0x0fffffffu + (bits & 1u)) >> 29;
    return __uint_as_float(bits | sign);
  }
  if (ah < 0x38100000u) return __uint_as_float(sign);       // below the binary32 normals
  if (ah >= 0x7ff00000u) {                                  // infinity or NaN (kept quiet)
    const unsigned int m = ((hi & 0xfffffu) << 3) | (lo >> 29);
    const bool nan = ((hi & 0xfffffu) | lo) != 0u;
    return __uint_as_float(sign | 0x7f800000u | (nan ? (m | 0x400000u) : 0u));
  }
  return __uint_as_float(sign | 0x7f800000u);               // finite beyond the range: overflow
}

// isfinite on the high word (integer pipe): the exponent field is not all ones
__device__ __forceinline__ bool finite_bits(double d) {
  return ((unsigned int)__double2hiint(d) & 0x7ff00000u) != 0x7ff00000u;
}

template <typename S>
__device__ __forceinline__ S to_s(double d) {
  if constexpr (sizeof(S) == 4) return narrow_rn(d);
  else return d;
}

template <int DIM, int NC>
struct Layout {
  static constexpr int ND = DIM + 1 + NC;
  static constexpr int iT = DIM + 1;   // T column == rho E row
  static constexpr int iY = DIM + 2;   // first Y column == first rho Y row
  static constexpr int NY = NC - 1;    // number of Y dofs
  static constexpr int NYA = NC > 1 ? NC - 1 : 1;  // array extent
};

// Mixture properties (fluid_properties.hpp:199-227; chemicals.hpp:43-47, 258-264).
template <int NC>
struct Props {
  double rho, mu, cp, cv, kappa, c, alpha, beta;
  double rho_c[NC], e_c[NC], D_c[NC];
  double irho_c[NC];  // 1/rho_c (mixed form only)
  double irho;        // 1/rho = sum_c Y_c/rho_c (mixed form only)
};

template <int NC>
__host__ __device__ __forceinline__ void mixture(const DevChem* ch, double p, double T, const double* Y,
                                                 Props<NC>& o) {
  double rho = 0.0, mu = 0.0, cp = 0.0, cv = 0.0, kappa = 0.0, c2 = 0.0;
  double calpha[NC], cbeta[NC];
#pragma unroll
  for (int c = 0; c < NC; ++c) {
    const DevChem& q = ch[c];
    double r, v, s, a, b;
    if (q.kind == GALES_CH_CUSTOM) {
      r = q.rho; a = q.alpha; b = q.beta;
      s = (b == 0.0) ? 1.e20 : 1.0 / sqrt(r * b);
      v = (b == 0.0) ? q.cp : q.cp - T * a * a / (r * b);
    } else {
      r = p / (q.R * T);
      b = 1.0 / p;
      a = 1.0 / T;
      s = sqrt(q.gamma * q.R * T);
      v = q.cv;
    }
    calpha[c] = a; cbeta[c] = b;
    rho += Y[c] / r;
    mu += Y[c] * q.mu;
    cp += Y[c] * q.cp;
    cv += Y[c] * v;
    kappa += Y[c] * q.kappa;
    c2 += Y[c] / ((r * r) * (s * s));
    o.rho_c[c] = r;
    o.e_c[c] = v * T;
    o.D_c[c] = q.D;
  }
  rho = 1. / rho;
  double c = sqrt(1.0 / c2);
  c /= rho;
  double alpha = 0.0, beta = 0.0;
#pragma unroll
  for (int c = 0; c < NC; ++c) {
    alpha += Y[c] * calpha[c] * rho / o.rho_c[c];
    beta += Y[c] * cbeta[c] * rho / o.rho_c[c];
  }
  o.rho = rho; o.mu = mu; o.cp = cp; o.cv = cv; o.kappa = kappa; o.c = c;
  o.alpha = alpha; o.beta = beta;
}

// The mixture in FP64 for the mixed form: state I in full (Props) and state P's rho
// and cv (what U(P) needs), from per-chemical ratios precomputed on the host and one
// division for both states.  A gas has 1/rho_c = R_c T/p, so
//   1/rho = (T G + p C)/p = D/p,   G = sum_gas Y_c R_c,  C = sum_custom Y_c/rho_c,
// and with r = 1/(p D D_P):  1/p = D D_P r,  rho = p^2 D_P r,  rho_P = p_P p D r.
// A gas's alpha_c/rho_c = R_c/p, beta_c/rho_c = R_c T/p^2 and 1/(rho_c^2 s_c^2) =
// (R_c/gamma_c) T/p^2, so the gas sums need 1/p alone.  A material without a gas
// (has_gas = 0) takes rho = 1/C, rho_P = 1/C_P and never divides by p.
template <int NC>
__device__ __forceinline__ void mixture_pair_fast(const DevChem* ch, bool has_gas, double pP, double TP,
                                                  const double* YP, double p, double T, const double* Y,
                                                  double& rhoP, double& cvP, Props<NC>& o) {
  double GP = 0.0, CP = 0.0, cvp = 0.0;
  double G = 0.0, GRg = 0.0, C = 0.0, mu = 0.0, cp = 0.0, cv = 0.0, kappa = 0.0;
  double c2 = 0.0, al = 0.0, be = 0.0;
#pragma unroll
  for (int c = 0; c < NC; ++c) {
    const DevChem& q = ch[c];
    double v;
    if (q.kind == GALES_CH_CUSTOM) {
      CP = fma(YP[c], q.inv_rho, CP);
      cvp = fma(YP[c], fma(-TP, q.cv_shift, q.cp), cvp);
      C = fma(Y[c], q.inv_rho, C);
      v = fma(-T, q.cv_shift, q.cp);
      c2 = fma(Y[c], q.c2_coef, c2);
      al = fma(Y[c], q.alpha_over_rho, al);
      be = fma(Y[c], q.beta_over_rho, be);
    } else {
      GP = fma(YP[c], q.R, GP);
      cvp = fma(YP[c], q.cv, cvp);
      G = fma(Y[c], q.R, G);
      GRg = fma(Y[c], q.R_over_gamma, GRg);
      v = q.cv;
    }
    mu = fma(Y[c], q.mu, mu);
    cp = fma(Y[c], q.cp, cp);
    cv = fma(Y[c], v, cv);
    kappa = fma(Y[c], q.kappa, kappa);
    o.e_c[c] = v * T;
    o.D_c[c] = q.D;
  }
  double rho, irho, ip;
  if (has_gas) {
    const double D = fma(T, G, p * C), DP = fma(TP, GP, pP * CP);
    const double r = 1.0 / (p * D * DP);
    ip = D * DP * r;
    rho = p * p * DP * r;
    rhoP = pP * p * D * r;
    irho = D * ip;
    const double ip2 = ip * ip;
    c2 = fma(GRg * T, ip2, c2);
    al = fma(G, ip, al);
    be = fma(G * T, ip2, be);
  } else {
    ip = 0.0;
    const double r = 1.0 / (C * CP);
    rho = CP * r;
    rhoP = C * r;
    irho = C;
  }
#pragma unroll
  for (int c = 0; c < NC; ++c) o.irho_c[c] = ch[c].kind == GALES_CH_CUSTOM ? ch[c].inv_rho : ch[c].R * T * ip;
  cvP = cvp;
  o.rho = rho; o.irho = irho; o.mu = mu; o.cp = cp; o.cv = cv; o.kappa = kappa;
  o.c = rsqrt(c2) * irho;
  o.alpha = rho * al;
  o.beta = rho * be;
}

// The equation of state a kernel instance is compiled for: the material's chemicals
// (custom_chemical / ideal_gas, mix_of_ch) or a mixture of magma sub-mixtures
// (mix_of_mix of magma_mix).  The chemical kernels are untouched by the magma ones.
constexpr int kEosChemicals = 0;
constexpr int kEosMagma = 1;

// The mixture of magma sub-mixtures at one point (fluid_properties.hpp:171-200 over
// magma_mixture::properties, mixtures.hpp:175-261), out of line: the evaluation (five
// chemicals per magma, table lookups, Giordano viscosity, gas and crystal corrections)
// is long, and one copy per kernel keeps the call sites small.  Returns the
// GALES_MAGMA_* bits.
static __device__ __noinline__ unsigned magma_point(const magma_mix::DevMagma* mg, int nc, double p, double T,
                                                    const double* Y, double sr, double* f, double (*comp)[4]) {
  return magma_mix::mix_point(mg, nc, p, T, Y, sr, f, comp);
}

// Props of the magma mixture; the mixture's own chemical diffusivity is not formed by
// fluid_properties' mix_of_mix (it stays 0 there), the components' are kept in D_c.
template <int NC>
__device__ __forceinline__ unsigned magma_mixture(const magma_mix::DevMagma* mg, double p, double T, const double* Y,
                                                  double sr, Props<NC>& o) {
  double f[8], comp[NC][4];
  const unsigned st = magma_point(mg, NC, p, T, Y, sr, f, comp);
  o.rho = f[0]; o.mu = f[1]; o.cp = f[2]; o.cv = f[3]; o.kappa = f[4]; o.c = f[5]; o.alpha = f[6]; o.beta = f[7];
#pragma unroll
  for (int c = 0; c < NC; ++c) {
    o.rho_c[c] = comp[c][0];
    o.e_c[c] = comp[c][1];
    o.D_c[c] = comp[c][2];
  }
  return st;
}

// compute_shear_rate (non_newtonian.hpp:23-29 in 2D, 32-39 in 3D) from the velocity
// gradient dv[i][j] = d v_i / d x_j; std::pow(x, 2) is the correctly rounded x*x.
template <int DIM>
__host__ __device__ __forceinline__ double shear_rate(const double (&dv)[DIM][DIM]) {
  if constexpr (DIM == 2) {
    const double a = dv[0][1] + dv[1][0];
    return sqrt(dv[0][0] * dv[0][0] + dv[1][1] * dv[1][1] + 2 * (a * a));
  } else {
    const double a = dv[0][1] + dv[1][0], b = dv[0][2] + dv[2][0], c = dv[1][2] + dv[2][1];
    return sqrt(dv[0][0] * dv[0][0] + dv[1][1] * dv[1][1] + dv[2][2] * dv[2][2] + 2 * (a * a) + 2 * (b * b) +
                2 * (c * c));
  }
}

// Only rho and cv (what U(P) needs); same operations as mixture().
template <int NC>
__device__ __forceinline__ void mixture_rho_cv(const DevChem* ch, double p, double T,
                                               const double* Y, double& rho_out, double& cv_out) {
  double rho = 0.0, cv = 0.0;
#pragma unroll
  for (int c = 0; c < NC; ++c) {
    const DevChem& q = ch[c];
    double r, v;
    if (q.kind == GALES_CH_CUSTOM) {
      r = q.rho;
      v = (q.beta == 0.0) ? q.cp : q.cp - T * q.alpha * q.alpha / (r * q.beta);
    } else {
      r = p / (q.R * T);
      v = q.cv;
    }
    rho += Y[c] / r;
    cv += Y[c] * v;
  }
  rho_out = 1. / rho;
  cv_out = cv;
}

// Scalars from which every frozen-coefficient matrix of the point is built
// (fluid_2d.hpp:393-404, 531-533).
template <int DIM, int NC, typename T = double>
struct Coef {
  using L = Layout<DIM, NC>;
  T p, v[DIM], T_, Y[NC];
  T rho, E, drho_dp, drho_dT, de_dp, de_dT, mu, lambda, kappa, c, cv;
  T drho_dY[L::NYA], dE_dY[L::NYA], rhoD[L::NYA], rhoDH[L::NYA];
};

template <int DIM, int NC>
__device__ __forceinline__ Coef<DIM, NC, float> narrow(const Coef<DIM, NC, double>& c) {
  using L = Layout<DIM, NC>;
  Coef<DIM, NC, float> f;
  f.p = narrow_rn(c.p); f.T_ = narrow_rn(c.T_);
#pragma unroll
  for (int k = 0; k < DIM; ++k) f.v[k] = narrow_rn(c.v[k]);
#pragma unroll
  for (int i = 0; i < NC; ++i) f.Y[i] = narrow_rn(c.Y[i]);
  f.rho = narrow_rn(c.rho); f.E = narrow_rn(c.E); f.drho_dp = narrow_rn(c.drho_dp); f.drho_dT = narrow_rn(c.drho_dT);
  f.de_dp = narrow_rn(c.de_dp); f.de_dT = narrow_rn(c.de_dT); f.mu = narrow_rn(c.mu); f.lambda = narrow_rn(c.lambda);
  f.kappa = narrow_rn(c.kappa); f.c = narrow_rn(c.c); f.cv = narrow_rn(c.cv);
#pragma unroll
  for (int i = 0; i < L::NYA; ++i) {
    f.drho_dY[i] = narrow_rn(c.drho_dY[i]); f.dE_dY[i] = narrow_rn(c.dE_dY[i]);
    f.rhoD[i] = narrow_rn(c.rhoD[i]); f.rhoDH[i] = narrow_rn(c.rhoDH[i]);
  }
  return f;
}

// assign(): fluid_2d.hpp:112-121
template <int DIM, int NC>
__device__ __forceinline__ void assign(const double* w, double& p, double* v, double& T, double* Y) {
  using L = Layout<DIM, NC>;
  p = w[0];
#pragma unroll
  for (int k = 0; k < DIM; ++k) v[k] = w[1 + k];
  T = w[L::iT];
  double s = 0.0;
#pragma unroll
  for (int i = 0; i < NC - 1; ++i) {
    Y[i] = w[L::iY + i];
    s += Y[i];
  }
  Y[NC - 1] = 1.0 - s;
}

template <int DIM>
__device__ __forceinline__ double vsq(const double* v) {
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < DIM; ++k) s += v[k] * v[k];
  return s;
}

// U(): fluid_2d.hpp:372-385
template <int DIM, int NC>
__device__ __forceinline__ void conservative(double rho, double cv, const double* v, double T,
                                             const double* Y, double* u) {
  using L = Layout<DIM, NC>;
  const double E = cv * T + 0.5 * (vsq<DIM>(v));
  u[0] = rho;
#pragma unroll
  for (int k = 0; k < DIM; ++k) u[1 + k] = rho * v[k];
  u[L::iT] = rho * E;
#pragma unroll
  for (int i = 0; i < NC - 1; ++i) u[L::iY + i] = rho * Y[i];
}

template <int DIM, int NC>
__device__ __forceinline__ void make_coef(const Props<NC>& pr, double p, const double* v, double T,
                                          const double* Y, Coef<DIM, NC>& c) {
  c.p = p; c.T_ = T;
#pragma unroll
  for (int k = 0; k < DIM; ++k) c.v[k] = v[k];
#pragma unroll
  for (int i = 0; i < NC; ++i) c.Y[i] = Y[i];
  const double rho = pr.rho;
  c.rho = rho;
  c.cv = pr.cv;
  c.E = pr.cv * T + 0.5 * (vsq<DIM>(v));
  c.drho_dp = rho * pr.beta;
  c.drho_dT = -rho * pr.alpha;
  c.de_dp = (pr.beta * p - pr.alpha * T) / rho;
  c.de_dT = pr.cp - p * pr.alpha / rho;
  c.mu = pr.mu;
  c.lambda = -2.0 * pr.mu / 3.0;
  c.kappa = pr.kappa;
  c.c = pr.c;
#pragma unroll
  for (int i = 0; i < NC - 1; ++i) {
    c.drho_dY[i] = -rho * rho * (1. / pr.rho_c[i] - 1 / pr.rho_c[NC - 1]);
    c.dE_dY[i] = pr.e_c[i] - pr.e_c[NC - 1];
    const double H = pr.e_c[i] + p / pr.rho_c[i];
    c.rhoD[i] = rho * pr.D_c[i];
    c.rhoDH[i] = rho * pr.D_c[i] * H;
  }
}

// make_coef for the mixed form, from mixture_pair_fast's reciprocals; vv = |v|^2.
template <int DIM, int NC>
__device__ __forceinline__ void make_coef_fast(const Props<NC>& pr, double p, const double* v, double vv,
                                               double T, const double* Y, Coef<DIM, NC>& c) {
  c.p = p; c.T_ = T;
#pragma unroll
  for (int k = 0; k < DIM; ++k) c.v[k] = v[k];
#pragma unroll
  for (int i = 0; i < NC; ++i) c.Y[i] = Y[i];
  const double rho = pr.rho, irho = pr.irho;
  c.rho = rho;
  c.cv = pr.cv;
  c.E = fma(pr.cv, T, 0.5 * vv);
  c.drho_dp = rho * pr.beta;
  c.drho_dT = -rho * pr.alpha;
  c.de_dp = fma(pr.beta, p, -pr.alpha * T) * irho;
  c.de_dT = fma(-p * pr.alpha, irho, pr.cp);
  c.mu = pr.mu;
  c.lambda = (-2.0 / 3.0) * pr.mu;
  c.kappa = pr.kappa;
  c.c = pr.c;
#pragma unroll
  for (int i = 0; i < NC - 1; ++i) {
    c.drho_dY[i] = -rho * rho * (pr.irho_c[i] - pr.irho_c[NC - 1]);
    c.dE_dY[i] = pr.e_c[i] - pr.e_c[NC - 1];
    const double H = fma(p, pr.irho_c[i], pr.e_c[i]);
    c.rhoD[i] = rho * pr.D_c[i];
    c.rhoDH[i] = c.rhoD[i] * H;
  }
}

// ---------------------------------------------------------------------------
// Matrix entries in formula form.  Each returns entry (r, col) of the matrix the
// reference builds densely (fluid_2d.hpp:407-575); zero where it has no entry.
// T is the arithmetic type (double for the FP64 form, float for the mixed form).

// DUDY (fluid_2d.hpp:407-441)
template <int DIM, int NC, typename T, typename C>
__device__ __forceinline__ T dudy_entry(const C& c, int r, int col) {
  using L = Layout<DIM, NC>;
  if (r == 0) {
    if (col == 0) return c.drho_dp;
    if (col == L::iT) return c.drho_dT;
    if (col >= L::iY) return c.drho_dY[col - L::iY];
    return T(0);
  }
  if (r < L::iT) {
    const int j = r - 1;
    if (col == 0) return c.drho_dp * c.v[j];
    if (col == r) return c.rho;
    if (col == L::iT) return c.drho_dT * c.v[j];
    if (col >= L::iY) return c.v[j] * c.drho_dY[col - L::iY];
    return T(0);
  }
  if (r == L::iT) {
    if (col == 0) return c.drho_dp * c.E + c.rho * c.de_dp;
    if (col < L::iT) return c.rho * c.v[col - 1];
    if (col == L::iT) return c.drho_dT * c.E + c.rho * c.de_dT;
    return c.E * c.drho_dY[col - L::iY] + c.rho * c.dE_dY[col - L::iY];
  }
  const int i = r - L::iY;
  if (col == 0) return c.drho_dp * c.Y[i];
  if (col == L::iT) return c.drho_dT * c.Y[i];
  if (col >= L::iY) {
    T x = c.Y[i] * c.drho_dY[col - L::iY];
    if (col == r) x += c.rho;
    return x;
  }
  return T(0);
}

// A_k (fluid_2d.hpp:444-524)
template <int DIM, int NC, typename T, typename C>
__device__ __forceinline__ T a_entry(const C& c, int k, int r, int col) {
  using L = Layout<DIM, NC>;
  const T vk = c.v[k];
  if (r == 0) {
    if (col == 0) return c.drho_dp * vk;
    if (col == 1 + k) return c.rho;
    if (col == L::iT) return c.drho_dT * vk;
    if (col >= L::iY) return c.drho_dY[col - L::iY] * vk;
    return T(0);
  }
  if (r < L::iT) {
    const int j = r - 1;
    const T vj = c.v[j];
    if (j == k) {
      if (col == 0) return c.drho_dp * vk * vk + T(1.0);
      if (col == 1 + k) return T(2.0) * c.rho * vk;
      if (col == L::iT) return c.drho_dT * vk * vk;
      if (col >= L::iY) return c.drho_dY[col - L::iY] * vk * vk;
      return T(0);
    }
    if (col == 0) return c.drho_dp * vj * vk;
    if (col == 1 + k) return c.rho * vj;
    if (col == 1 + j) return c.rho * vk;
    if (col == L::iT) return c.drho_dT * vj * vk;
    if (col >= L::iY) return c.drho_dY[col - L::iY] * vj * vk;
    return T(0);
  }
  if (r == L::iT) {
    if (col == 0) return vk + vk * (c.drho_dp * c.E + c.rho * c.de_dp);
    if (col < L::iT) {
      const int j = col - 1;
      if (j == k) return c.p + c.rho * c.E + c.rho * vk * vk;
      const int lo = j < k ? j : k, hi = j < k ? k : j;
      return c.rho * c.v[lo] * c.v[hi];
    }
    if (col == L::iT) return vk * (c.drho_dT * c.E + c.rho * c.de_dT);
    return (c.E * c.drho_dY[col - L::iY] + c.rho * c.dE_dY[col - L::iY]) * vk;
  }
  const int i = r - L::iY;
  if (col == 0) return c.drho_dp * c.Y[i] * vk;
  if (col == 1 + k) return c.rho * c.Y[i];
  if (col == L::iT) return c.drho_dT * c.Y[i] * vk;
  if (col >= L::iY) {
    T x = c.Y[i] * c.drho_dY[col - L::iY] * vk;
    if (col == r) x += c.rho * vk;
    return x;
  }
  return T(0);
}

// K_kl (fluid_2d.hpp:531-571)
template <int DIM, int NC, typename T, typename C>
__device__ __forceinline__ T k_entry(const C& c, int k, int l, int r, int col) {
  using L = Layout<DIM, NC>;
  if (r == 0 || col == 0) return T(0);
  if (k == l) {
    if (r < L::iT) {
      if (col != r) return T(0);
      return (r - 1 == k) ? c.lambda + T(2) * c.mu : c.mu;
    }
    if (r == L::iT) {
      if (col < L::iT) {
        const int m = col - 1;
        return (m == k) ? (c.lambda + T(2) * c.mu) * c.v[k] : c.mu * c.v[m];
      }
      if (col == L::iT) return c.kappa;
      return c.rhoDH[col - L::iY];
    }
    return (col == r) ? c.rhoD[r - L::iY] : T(0);
  }
  if (r == 1 + k && col == 1 + l) return c.lambda;
  if (r == 1 + l && col == 1 + k) return c.mu;
  if (r == L::iT) {
    if (col == 1 + k) return c.mu * c.v[l];
    if (col == 1 + l) return c.lambda * c.v[k];
  }
  return T(0);
}

// Structural nonzeros of DUDY, A_k and K_kl (the entries fluid_2d.hpp:407-571 sets).
// Evaluated at compile time inside fully unrolled loops, so products with structural
// zeros are never issued; dropping exact-zero terms leaves every finite sum unchanged.
template <int DIM, int NC>
__host__ __device__ constexpr bool dudy_nz(int r, int col) {
  using L = Layout<DIM, NC>;
  if (r == L::iT) return true;
  if (col == 0 || col == L::iT || col >= L::iY) return true;
  return r >= 1 && r < L::iT && col == r;
}

template <int DIM, int NC>
__host__ __device__ constexpr bool a_nz(int k, int r, int col) {
  using L = Layout<DIM, NC>;
  if (r == L::iT) return true;
  if (col == 0 || col == L::iT || col >= L::iY || col == 1 + k) return true;
  return r >= 1 && r < L::iT && col == r;
}

template <int DIM, int NC>
__host__ __device__ constexpr bool k_nz(int k, int l, int r, int col) {
  using L = Layout<DIM, NC>;
  if (r == 0 || col == 0) return false;
  if (k == l) {
    if (r < L::iT) return col == r;
    if (r == L::iT) return true;
    return col == r;
  }
  return (r == 1 + k && col == 1 + l) || (r == 1 + l && col == 1 + k) ||
         (r == L::iT && (col == 1 + k || col == 1 + l));
}

// y = DUDY x (and A_k x, K_kl x) in ascending column order, the order of a dense
// uBLAS prod(), skipping structural zeros.
template <int DIM, int NC, typename T, typename C>
__device__ __forceinline__ void dudy_mv(const C& c, const T* x, T* y) {
  using L = Layout<DIM, NC>;
#pragma unroll
  for (int r = 0; r < L::ND; ++r) {
    T t = T(0);
#pragma unroll
    for (int col = 0; col < L::ND; ++col)
      if (dudy_nz<DIM, NC>(r, col)) t += dudy_entry<DIM, NC, T>(c, r, col) * x[col];
    y[r] = t;
  }
}

template <int DIM, int NC, typename T, typename C>
__device__ __forceinline__ void a_mv(const C& c, int k, const T* x, T* y) {
  using L = Layout<DIM, NC>;
#pragma unroll
  for (int r = 0; r < L::ND; ++r) {
    T t = T(0);
#pragma unroll
    for (int col = 0; col < L::ND; ++col)
      if (a_nz<DIM, NC>(k, r, col)) t += a_entry<DIM, NC, T>(c, k, r, col) * x[col];
    y[r] = t;
  }
}

template <int DIM, int NC, typename T, typename C>
__device__ __forceinline__ void k_mv(const C& c, int k, int l, const T* x, T* y) {
  using L = Layout<DIM, NC>;
#pragma unroll
  for (int r = 0; r < L::ND; ++r) {
    T t = T(0);
#pragma unroll
    for (int col = 0; col < L::ND; ++col)
      if (k_nz<DIM, NC>(k, l, r, col)) t += k_entry<DIM, NC, T>(c, k, l, r, col) * x[col];
    y[r] = t;
  }
}

// GALES::inverse (algorithm.hpp:399-416): uBLAS lu_factorize (partial pivoting on
// the first max |.| of the column, reciprocal column scaling) + lu_substitute
// against the identity.  Returns nonzero if a zero pivot was met.
template <int N>
__device__ __forceinline__ int lu_inverse(double (&A)[N][N], double (&X)[N][N]) {
  int pm[N];
#pragma unroll
  for (int i = 0; i < N; ++i) pm[i] = i;
  int singular = 0;
#pragma unroll
  for (int i = 0; i < N; ++i) {
    int imax = i;
    double t = 0.0;
#pragma unroll
    for (int r = i; r < N; ++r) {
      const double u = fabs(A[r][i]);
      if (u > t) { imax = r; t = u; }
    }
    if (t == 0.0) imax = i;
    if (A[imax][i] != 0.0) {
      if (imax != i) {
        pm[i] = imax;
#pragma unroll
        for (int r = i + 1; r < N; ++r)
          if (r == imax)
#pragma unroll
            for (int c = 0; c < N; ++c) { const double s = A[i][c]; A[i][c] = A[r][c]; A[r][c] = s; }
      }
      const double rcp = 1.0 / A[i][i];
#pragma unroll
      for (int r = i + 1; r < N; ++r) A[r][i] *= rcp;
    } else if (singular == 0) {
      singular = i + 1;
    }
#pragma unroll
    for (int r = i + 1; r < N; ++r)
#pragma unroll
      for (int c = i + 1; c < N; ++c) A[r][c] -= A[r][i] * A[i][c];
  }
#pragma unroll
  for (int i = 0; i < N; ++i)
#pragma unroll
    for (int j = 0; j < N; ++j) X[i][j] = (i == j) ? 1.0 : 0.0;
#pragma unroll
  for (int i = 0; i < N; ++i)
#pragma unroll
    for (int r = i + 1; r < N; ++r)
      if (pm[i] == r)
#pragma unroll
        for (int c = 0; c < N; ++c) { const double s = X[i][c]; X[i][c] = X[r][c]; X[r][c] = s; }
#pragma unroll
  for (int l = 0; l < N; ++l)
#pragma unroll
    for (int r = 0; r < N; ++r) {
      const double t = X[r][l];
      if (t != 0.0)
#pragma unroll
        for (int m = r + 1; m < N; ++m) X[m][l] -= A[m][r] * t;
    }
#pragma unroll
  for (int l = N - 1; l >= 0; --l)
#pragma unroll
    for (int r = N - 1; r >= 0; --r) {
      const double t = X[r][l] /= A[r][r];
      if (t != 0.0)
#pragma unroll
        for (int m = r - 1; m >= 0; --m) X[m][l] -= A[m][r] * t;
    }
  return singular;
}

// tau = DUDY^{-1} diag(td) for the mixed form (fluid_2d.hpp:946-947), from the
// structure of DUDY = w r0^T + rho M.  The velocity and mass-fraction rows of
// DUDY^{-1} are (e_j - w_j e_p^T)/rho; the p and T rows come from the 2x2 system
// [drho_dp drho_dT; de_dp de_dT] per column.  Every other entry is zero (tau_nz).
// irho = 1/rho, idet = 1/(drho_dp de_dT - drho_dT de_dp) (tau_det gives the
// determinant).  low_mach applies the low-Mach form of the p row (fluid_2d.hpp:949-
// 958): tau[0][0] <- 1/(1/tau[0][0] + 1/b) with b = rho tau[1][1] tr(G) (rho_trG =
// rho tr(G)), tau[0][c] <- 0 for c > 0.  Each entry is formed in FP64 and stored in T.
template <int DIM, int NC>
__host__ __device__ constexpr bool tau_nz(int r, int cc) {
  return r == 0 || r == Layout<DIM, NC>::iT || cc == 0 || cc == r;
}

template <int DIM, int NC>
__device__ __forceinline__ double tau_det(const Coef<DIM, NC>& c) {
  return fma(c.drho_dp, c.de_dT, -c.drho_dT * c.de_dp);
}

template <int DIM, int NC, typename T>
__device__ __forceinline__ void tau_closed(const Coef<DIM, NC>& c, double irho, double idet, const double* td,
                                           bool low_mach, double rho_trG,
                                           T (&tau)[Layout<DIM, NC>::ND][Layout<DIM, NC>::ND]) {
  using L = Layout<DIM, NC>;
  const double q = irho * idet;
  // column p: R1 = 1 + (sum_i drho_dY_i Y_i)/rho, R2 = (|v|^2 - E + sum_i dE_dY_i Y_i)/rho
  double sY = 0.0, sE = -c.E;
#pragma unroll
  for (int j = 0; j < DIM; ++j) sE = fma(c.v[j], c.v[j], sE);
#pragma unroll
  for (int i = 0; i < NC - 1; ++i) {
    sY = fma(c.drho_dY[i], c.Y[i], sY);
    sE = fma(c.dE_dY[i], c.Y[i], sE);
  }
  const double R1 = fma(irho, sY, 1.0), R2 = irho * sE;
  const double t0 = td[0] * idet, ti = td[0] * irho;
  double t00 = fma(R1, c.de_dT, -c.drho_dT * R2) * t0;
  if (low_mach) {
    // 1/(1/a + 1/b) = a b/(a + b)
    const double b = rho_trG * (irho * td[1]);
    t00 = t00 * b / (t00 + b);
  }
  tau[0][0] = to_s<T>(t00);
  tau[L::iT][0] = to_s<T>(fma(c.drho_dp, R2, -c.de_dp * R1) * t0);
#pragma unroll
  for (int j = 0; j < DIM; ++j) {
    tau[1 + j][0] = to_s<T>(-c.v[j] * ti);
    tau[1 + j][1 + j] = to_s<T>(irho * td[1 + j]);
    const double a = q * td[1 + j] * c.v[j];
    tau[0][1 + j] = low_mach ? T(0) : to_s<T>(c.drho_dT * a);
    tau[L::iT][1 + j] = to_s<T>(-c.drho_dp * a);
  }
  tau[0][L::iT] = low_mach ? T(0) : to_s<T>(-c.drho_dT * q * td[L::iT]);
  tau[L::iT][L::iT] = to_s<T>(c.drho_dp * q * td[L::iT]);
#pragma unroll
  for (int i = 0; i < NC - 1; ++i) {
    const int y = L::iY + i;
    tau[y][0] = to_s<T>(-c.Y[i] * ti);
    tau[y][y] = to_s<T>(irho * td[y]);
    const double a = q * td[y];
    tau[0][y] = low_mach ? T(0) : to_s<T>(fma(c.drho_dT, c.dE_dY[i], -c.drho_dY[i] * c.de_dT) * a);
    tau[L::iT][y] = to_s<T>(fma(c.de_dp, c.drho_dY[i], -c.drho_dp * c.dE_dY[i]) * a);
  }
}

// compute_h: quad.hpp:356-383 (2D), 701-739 (3D).  dv[i][j] = d v_i / d x_j.
// IEEE multiply/add/subtract that are never fused into a multiply-add, whatever the
// translation unit's contraction setting: the steps of compute_h whose rounding
// decides its branches use them.
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub_rn(double a, double b) { return __dsub_rn(a, b); }

template <int DIM>
__device__ __forceinline__ double vsq_rn(const double* v) {
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < DIM; ++k) s = add_rn(s, mul_rn(v[k], v[k]));
  return s;
}

template <int DIM>
__device__ __forceinline__ double compute_h(const double (&G)[DIM][DIM], const double* v,
                                            const double (&dv)[DIM][DIM]) {
  double nrm_v = sqrt(vsq_rn<DIM>(v));
  double s0[DIM], s1[DIM], alpha[DIM];
#pragma unroll
  for (int i = 0; i < DIM; ++i) s0[i] = v[i] / nrm_v;
  auto quadform = [&](const double* s) {
    double Gs[DIM];
#pragma unroll
    for (int i = 0; i < DIM; ++i) {
      double t = 0.0;
#pragma unroll
      for (int j = 0; j < DIM; ++j) t = add_rn(t, mul_rn(G[i][j], s[j]));
      Gs[i] = t;
    }
    double r = 0.0;
#pragma unroll
    for (int i = 0; i < DIM; ++i) r = add_rn(r, mul_rn(s[i], Gs[i]));
    return r;
  };
  alpha[0] = quadform(s0);
  double acc[DIM];
#pragma unroll
  for (int i = 0; i < DIM; ++i) {
    double t = 0.0;
#pragma unroll
    for (int j = 0; j < DIM; ++j) t = add_rn(t, mul_rn(dv[i][j], v[j]));
    acc[i] = t;
  }
  double ip = 0.0;
#pragma unroll
  for (int i = 0; i < DIM; ++i) ip = add_rn(ip, mul_rn(acc[i], s0[i]));
#pragma unroll
  for (int i = 0; i < DIM; ++i) s1[i] = sub_rn(acc[i], mul_rn(ip, s0[i]));
  const double nrm_s1 = sqrt(vsq_rn<DIM>(s1));
  if (nrm_s1 > kEps)
#pragma unroll
    for (int i = 0; i < DIM; ++i) s1[i] /= nrm_s1;
  alpha[1] = quadform(s1);
  if constexpr (DIM == 3) {
    double s2[3];
    s2[0] = sub_rn(mul_rn(s0[1], s1[2]), mul_rn(s0[2], s1[1]));
    s2[1] = sub_rn(mul_rn(s1[0], s0[2]), mul_rn(s1[2], s0[0]));
    s2[2] = sub_rn(mul_rn(s0[0], s1[1]), mul_rn(s0[1], s1[0]));
    const double nrm_s2 = sqrt(vsq_rn<3>(s2));
    if (nrm_s2 > kEps)
#pragma unroll
      for (int i = 0; i < 3; ++i) s2[i] /= nrm_s2;
    alpha[2] = quadform(s2);
  }
  double h = 0.0;
#pragma unroll
  for (int i = 0; i < DIM; ++i)
    if (alpha[i] != 0.0) h = add_rn(h, 1.0 / alpha[i]);
  return 2 * sqrt(fabs(h));
}

template <int DIM>
__device__ __forceinline__ double qform_fma(const double (&G)[DIM][DIM], const double* s) {
  double r = 0.0;
#pragma unroll
  for (int i = 0; i < DIM; ++i) {
    double t = G[i][0] * s[0];
#pragma unroll
    for (int j = 1; j < DIM; ++j) t = fma(G[i][j], s[j], t);
    r = fma(s[i], t, r);
  }
  return r;
}

// compute_h for the mixed form, with fused operations and no normalisation but of v
// (iv = 1/|v| comes from the caller).  compute_h branches on |s1| > DBL_EPSILON, where
// s1 (the part of dv v normal to v) is rounding noise for a rank-one velocity field
// (every node but one at rest); there only the reference's exact operations take the
// reference's branch.  This routine decides the branch only when |s1| exceeds 1e-10
// |dv v| (and 1e3 DBL_EPSILON), far above what rounding can move, and so does the
// third direction |s0 x s1/|s1||; otherwise it returns with decided = false and the
// caller runs compute_h on the velocity and gradient formed with the reference's
// operations.  With w1 = s1 unnormalised and w2 = s0 x w1, alpha_1 = w1^T G w1/|w1|^2
// and alpha_2 = w2^T G w2/|w2|^2, so h = 1/alpha_0 + |w1|^2/A1 + |w2|^2/A2 takes one
// reciprocal square root at the end.  In 3D, where |w1| > 1e-3 |dv v| the basis
// {s0, w1/|w1|, w2/|w2|} is orthonormal to ~1e-13, and alpha_2 = tr G - alpha_0 -
// alpha_1 (the trace does not change under an orthonormal change of basis): then
// B2 = n1 alpha_2 = n1 (tr G - A0) - A1 replaces w2 and its quadratic form wherever
// alpha_2 > 1e-6 tr G, which keeps its rounding below ~1e-10 relative.
template <int DIM>
__device__ __forceinline__ double compute_h_fast(const double (&G)[DIM][DIM], double trG, const double* v,
                                                 double iv, const double (&dv)[DIM][DIM], bool& decided) {
  decided = false;
  double s0[DIM], acc[DIM], w1[DIM];
#pragma unroll
  for (int i = 0; i < DIM; ++i) s0[i] = v[i] * iv;
  double aa = 0.0, ip = 0.0;
#pragma unroll
  for (int i = 0; i < DIM; ++i) {
    double t = dv[i][0] * v[0];
#pragma unroll
    for (int j = 1; j < DIM; ++j) t = fma(dv[i][j], v[j], t);
    acc[i] = t;
    aa = fma(t, t, aa);
    ip = fma(t, s0[i], ip);
  }
  double n1 = 0.0;
#pragma unroll
  for (int i = 0; i < DIM; ++i) {
    w1[i] = fma(-ip, s0[i], acc[i]);
    n1 = fma(w1[i], w1[i], n1);
  }
  constexpr double kMin2 = 1.0e6 * kEps * kEps;  // (1e3 DBL_EPSILON)^2
  if (!(n1 > fmax(1.0e-20 * aa, kMin2))) return 0.0;
  const double A0 = qform_fma<DIM>(G, s0), A1 = qform_fma<DIM>(G, w1);
  double A2 = 0.0, n2 = 0.0;
  if constexpr (DIM == 3) {
    if (n1 > 1.0e-6 * aa) {
      const double B2 = fma(n1, trG - A0, -A1);
      if (B2 > 1.0e-6 * (n1 * trG) && A0 != 0.0 && A1 != 0.0) {
        decided = true;
        // 1/A0 + n1/A1 + n1/B2 = (A1 B2 + n1 A0 (B2 + A1)) / (A0 A1 B2), all terms > 0
        const double num = fma(A1, B2, (n1 * A0) * (B2 + A1)), den = A0 * A1 * B2;
        return 2.0 * num * rsqrt(num * den);
      }
    }
    double w2[3];
    w2[0] = fma(s0[1], w1[2], -s0[2] * w1[1]);
    w2[1] = fma(w1[0], s0[2], -w1[2] * s0[0]);
    w2[2] = fma(s0[0], w1[1], -s0[1] * w1[0]);
    n2 = fma(w2[0], w2[0], fma(w2[1], w2[1], w2[2] * w2[2]));
    if (!(n2 > kMin2 * n1)) return 0.0;
    A2 = qform_fma<DIM>(G, w2);
  }
  decided = true;
  if (DIM == 3 && A0 != 0.0 && A1 != 0.0 && A2 != 0.0) {
    // 2 sqrt|num/den| = 2 |num| / sqrt|num den|
    const double num = fma(A1, A2, A0 * fma(n1, A2, n2 * A1)), den = A0 * A1 * A2;
    return num == 0.0 ? 0.0 : 2.0 * fabs(num) * rsqrt(fabs(num * den));
  }
  double h = 0.0;
  if (A0 != 0.0) h += 1.0 / A0;
  if (A1 != 0.0) h += n1 / A1;
  if (DIM == 3 && A2 != 0.0) h += n2 / A2;
  return 2 * sqrt(fabs(h));
}

}  // namespace gales
