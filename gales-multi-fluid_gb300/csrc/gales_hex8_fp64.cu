// Kernel instances for the hex8 element (dim 3, 8 nodes, 8 interior points,
// 6 sides with 4 points each; element.hpp gauss_data tables).
#include "gales_launch.cuh"

namespace gales {

using D_hex8 = ElementDispatch<3, 8, 8, 6, 4>;

LaunchResult interior_hex8_fp64(const KParams& k, int nc, bool want_m, long long n, cudaStream_t st) {
  return D_hex8::interior<GALES_FORM_FP64>(k, nc, want_m, n, st);
}

LaunchResult boundary_hex8(const KParams& k, int nc, long long n, cudaStream_t st) {
  return D_hex8::boundary(k, nc, n, st);
}

}  // namespace gales
