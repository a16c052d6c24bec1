// Kernel instances for the tri3 element (dim 2, 3 nodes, 3 interior points,
// 3 sides with 2 points each; element.hpp gauss_data tables).
#include "gales_launch.cuh"

namespace gales {

using D_tri3 = ElementDispatch<2, 3, 3, 3, 2>;

LaunchResult interior_tri3_fp64(const KParams& k, int nc, bool want_m, long long n, cudaStream_t st) {
  return D_tri3::interior<GALES_FORM_FP64>(k, nc, want_m, n, st);
}

LaunchResult boundary_tri3(const KParams& k, int nc, long long n, cudaStream_t st) {
  return D_tri3::boundary(k, nc, n, st);
}

}  // namespace gales
