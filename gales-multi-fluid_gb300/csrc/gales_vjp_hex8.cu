// Exact VJP kernel instances for the hex8 element.
#include "gales_launch.cuh"
#include "gales_vjp_kernels.cuh"

namespace gales {

LaunchResult vjp_interior_hex8(const KParams& k, int nc, long long n, cudaStream_t st) {
  return VjpDispatch<3, 8, 8, 6, 4>::interior(k, nc, n, st);
}

LaunchResult vjp_boundary_hex8(const KParams& k, int nc, long long n, cudaStream_t st) {
  return VjpDispatch<3, 8, 8, 6, 4>::boundary(k, nc, n, st);
}

}  // namespace gales
