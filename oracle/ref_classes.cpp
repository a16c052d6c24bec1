/*
 * TEST INFRASTRUCTURE — NOT PART OF THE PRODUCT.
 *
 * The reference's own classes that compile here, built from its checkout by
 * oracle/build.py (build_ref) into oracle/_ref/libref_classes.so, so that the tests can
 * pin the oracle's restatement against the reference itself where the reference
 * compiles:
 *   - src/fem/physical_props/fluid/chemicals.hpp: custom_chemical (19-49), melt
 *     (56-145, Lange-Carmichael), dissolved_volatiles (149-194), ideal_gas (198-271),
 *     over base_chemical.hpp;
 *   - src/fem/physical_props/fluid/GiordanoEtAlViscosityModel.hpp (the magma viscosity),
 *     driven as magma_mixture drives it (mixtures.hpp:161, 180);
 *   - src/fem/mesh/element.hpp (over node.hpp and point.hpp): the element types' interior
 *     Gauss points, side node tables and side Gauss points (gauss_data).
 * The property headers need only the standard library, except two helpers that the reference
 * takes from base headers which include mpi.h and Boost: the Error macro
 * (src/fem/base/algorithm.hpp:42) and print_in_file (src/fem/base/print_tools.hpp).
 * Neither takes part in the arithmetic; stand-ins follow (Error throws, so the wrappers
 * report the reference's error exits as a return code; print_in_file does nothing).
 * The mixtures (mixtures.hpp) and the element integral need Boost uBLAS and Trilinos
 * and are not built.
 */
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <memory>
#include <numeric>
#include <stdexcept>
#include <string>
#include <vector>

namespace GALES {
template <class... A>
inline void print_in_file(A&&...) {}
inline void ref_error(const std::string& m) { throw std::runtime_error(m); }
}  // namespace GALES
#define Error(message) ref_error(message)

#include "chemicals.hpp"
#include "GiordanoEtAlViscosityModel.hpp"
#include "element.hpp"

namespace {

// out[0..8] = rho, mu, cp, cv, kappa, sound speed, alpha, beta, chemical diffusivity
void dump(const GALES::base_chemical& c, double* o) {
  o[0] = c.rho_;
  o[1] = c.mu_;
  o[2] = c.cp_;
  o[3] = c.cv_;
  o[4] = c.kappa_;
  o[5] = c.sound_speed_;
  o[6] = c.alpha_;
  o[7] = c.beta_;
  o[8] = c.chemical_diffusivity_;
}

}  // namespace

extern "C" {

int ref_custom_chemical(double rho, double mu, double cp, double kappa, double alpha, double beta, double p, double T,
                        double* out) {
  GALES::custom_chemical c(rho, mu, cp, kappa, alpha, beta);
  c.properties(p, T, 0.0);
  dump(c, out);
  return 0;
}

int ref_ideal_gas(double molar_mass, double gamma, double p, double T, double* out) {
  GALES::ideal_gas c(molar_mass, gamma);
  c.properties(p, T, 0.0);
  dump(c, out);
  return 0;
}

int ref_ideal_gas_named(const char* name, double p, double T, double* out) {
  GALES::ideal_gas c{std::string(name)};
  c.properties(p, T, 0.0);
  dump(c, out);
  return 0;
}

int ref_melt(const double* oxides_wf, double kappa, double p, double T, double* out) {
  GALES::melt c(std::vector<double>(oxides_wf, oxides_wf + 10), kappa);
  c.properties(p, T, 0.0);
  dump(c, out);
  return 0;
}

int ref_dissolved_volatile(const char* name, double cp, double kappa, double p, double T, double* out) {
  GALES::dissolved_volatiles c(std::string(name), cp, kappa);
  c.properties(p, T, 0.0);
  dump(c, out);
  return 0;
}

// The Giordano viscosity of a melt of the given oxide weight fractions at T with the
// dissolved H2O and CO2 weight fractions, set up from the melt as magma_mixture does.
// Returns 0, or -1 on the reference's error exits.
int ref_giordano(const double* oxides_wf, double T, double wf_h2o_l, double wf_co2_l, double* mu) {
  try {
    GALES::melt m(std::vector<double>(oxides_wf, oxides_wf + 10), 1.0);
    GALES::GiordanoEtAlViscosityModel g;
    g.set(m.oxides_wf(), m.oxides_molar_mass());
    *mu = g.computeViscosity(T, wf_h2o_l, wf_co2_l);
    return 0;
  } catch (const std::exception&) {
    return -1;
  }
}

// The element type's tables as gauss_data sets them: gp[i * 3 + d] interior points,
// sides[s * nsn + j] side node tables, sgp[(s * nqs + j) * 3 + d] side points (unused
// coordinates 0), counts = {nq, nsides, nsn, nqs}.  Returns nq, or -1 for an element
// the reference does not define.
int ref_element_tables(int dim, int nen, double* gp, int32_t* sides, double* sgp, int32_t* counts) {
  auto fill = [&](const auto& el, auto coords) {
    const int nq = el.nb_gp(), ns = el.nb_sides(), nsn = el.nb_side_nds();
    const int nqs = ns > 0 ? el.nb_side_gp(0) : 0;
    for (int i = 0; i < nq; ++i) coords(el.gp(i), gp + i * 3);
    for (int s = 0; s < ns; ++s)
      for (int j = 0; j < nsn; ++j) sides[s * nsn + j] = el.side(s, j);
    for (int s = 0; s < ns; ++s)
      for (int j = 0; j < nqs; ++j) coords(el.side_gp(s, j), sgp + (s * nqs + j) * 3);
    counts[0] = nq;
    counts[1] = ns;
    counts[2] = nsn;
    counts[3] = nqs;
    return nq;
  };
  if (dim == 2 && (nen == 3 || nen == 4)) {
    GALES::element<2> el(nen);
    return fill(el, [](const GALES::point<2>& p, double* o) { o[0] = p.get_x(); o[1] = p.get_y(); o[2] = 0.0; });
  }
  if (dim == 3 && (nen == 4 || nen == 8)) {
    GALES::element<3> el(nen);
    return fill(el, [](const GALES::point<3>& p, double* o) {
      o[0] = p.get_x();
      o[1] = p.get_y();
      o[2] = p.get_z();
    });
  }
  return -1;
}

}  // extern "C"
