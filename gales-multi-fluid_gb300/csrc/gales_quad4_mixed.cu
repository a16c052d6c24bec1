// Kernel instances for the quad4 element (dim 2, 4 nodes, 4 interior points,
// 4 sides with 2 points each; element.hpp gauss_data tables).
#include "gales_launch.cuh"

namespace gales {

using D_quad4 = ElementDispatch<2, 4, 4, 4, 2>;

LaunchResult interior_quad4_mixed(const KParams& k, int nc, bool want_m, long long n, cudaStream_t st) {
  return D_quad4::interior<GALES_FORM_MIXED>(k, nc, want_m, n, st);
}

}  // namespace gales
