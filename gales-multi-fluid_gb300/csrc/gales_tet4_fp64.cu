// Kernel instances for the tet4 element (dim 3, 4 nodes, 4 interior points,
// 4 sides with 3 points each; element.hpp gauss_data tables).
#include "gales_launch.cuh"

namespace gales {

using D_tet4 = ElementDispatch<3, 4, 4, 4, 3>;

LaunchResult interior_tet4_fp64(const KParams& k, int nc, bool want_m, long long n, cudaStream_t st) {
  return D_tet4::interior<GALES_FORM_FP64>(k, nc, want_m, n, st);
}

LaunchResult boundary_tet4(const KParams& k, int nc, long long n, cudaStream_t st) {
  return D_tet4::boundary(k, nc, n, st);
}

}  // namespace gales
