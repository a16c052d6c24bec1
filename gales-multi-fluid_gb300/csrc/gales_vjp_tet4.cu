// Exact VJP kernel instances for the tet4 element.
#include "gales_launch.cuh"
#include "gales_vjp_kernels.cuh"

namespace gales {

LaunchResult vjp_interior_tet4(const KParams& k, int nc, long long n, cudaStream_t st) {
  return VjpDispatch<3, 4, 4, 4, 3>::interior(k, nc, n, st);
}

LaunchResult vjp_boundary_tet4(const KParams& k, int nc, long long n, cudaStream_t st) {
  return VjpDispatch<3, 4, 4, 4, 3>::boundary(k, nc, n, st);
}

}  // namespace gales
