// Exact VJP kernel instances for the tri3 element.
#include "gales_launch.cuh"
#include "gales_vjp_kernels.cuh"

namespace gales {

LaunchResult vjp_interior_tri3(const KParams& k, int nc, long long n, cudaStream_t st) {
  return VjpDispatch<2, 3, 3, 3, 2>::interior(k, nc, n, st);
}

LaunchResult vjp_boundary_tri3(const KParams& k, int nc, long long n, cudaStream_t st) {
  return VjpDispatch<2, 3, 3, 3, 2>::boundary(k, nc, n, st);
}

}  // namespace gales
