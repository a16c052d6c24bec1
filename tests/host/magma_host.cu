// Host build of the magma property code the GPU kernel runs (gales_magma.cuh), for the
// CPU tests: the same functions, compiled for the host, over host arrays.
#include <cstdint>
#include <vector>

#include "../../gales-multi-fluid_gb300/csrc/gales_magma.cuh"

using namespace magma_mix;

extern "C" int magma_host_properties(const gales_magma_desc* comps, int32_t nc, const double* p, const double* T,
                                     const double* Y, const double* shear, int64_t n, double* out, double* comp) {
  std::vector<DevMagma> mg(nc);
  for (int c = 0; c < nc; ++c) {
    build_constants(comps[c], mg[c]);
    mg[c].p_tab = comps[c].p_table;
    mg[c].T_tab = comps[c].n_T > 0 ? comps[c].T_table : nullptr;
    mg[c].h2o_tab = comps[c].wf_l_h2o;
    mg[c].co2_tab = comps[c].wf_l_co2;
  }
  unsigned st = 0;
  for (int64_t i = 0; i < n; ++i) {
    double f[8], cc[GALES_MAX_COMP][4];
    st |= mix_point(mg.data(), nc, p[i], T[i], Y + i * nc, shear ? shear[i] : 0.0, f, cc);
    for (int k = 0; k < 8; ++k) out[k * n + i] = f[k];
    for (int c = 0; c < nc; ++c)
      for (int k = 0; k < 4; ++k) comp[(c * 4 + k) * n + i] = cc[c][k];
  }
  return (int)st;
}

// secondary_dofs' gas fractions (mix_fractions) at n points: out[k * n + i], 2 nc + 6 fields.
extern "C" int magma_host_fractions(const gales_magma_desc* comps, int32_t nc, const double* p, const double* T,
                                    const double* Y, int64_t n, double* out) {
  std::vector<DevMagma> mg(nc);
  for (int c = 0; c < nc; ++c) {
    build_constants(comps[c], mg[c]);
    mg[c].p_tab = comps[c].p_table;
    mg[c].T_tab = comps[c].n_T > 0 ? comps[c].T_table : nullptr;
    mg[c].h2o_tab = comps[c].wf_l_h2o;
    mg[c].co2_tab = comps[c].wf_l_co2;
  }
  unsigned st = 0;
  const int nf = 2 * nc + 6;
  for (int64_t i = 0; i < n; ++i) {
    double f[2 * GALES_MAX_COMP + 6];
    st |= mix_fractions(mg.data(), nc, p[i], T[i], Y + i * nc, f);
    for (int k = 0; k < nf; ++k) out[k * n + i] = f[k];
  }
  return (int)st;
}
