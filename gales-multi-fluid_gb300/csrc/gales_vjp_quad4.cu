// Exact VJP kernel instances for the quad4 element.
#include "gales_launch.cuh"
#include "gales_vjp_kernels.cuh"

namespace gales {

LaunchResult vjp_interior_quad4(const KParams& k, int nc, long long n, cudaStream_t st) {
  return VjpDispatch<2, 4, 4, 4, 2>::interior(k, nc, n, st);
}

LaunchResult vjp_boundary_quad4(const KParams& k, int nc, long long n, cudaStream_t st) {
  return VjpDispatch<2, 4, 4, 4, 2>::boundary(k, nc, n, st);
}

}  // namespace gales
