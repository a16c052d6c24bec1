// Kernel instances for the tri3 element with the magma EOS, mixed form (dim 2, 3 nodes,
// 3 interior points, 3 sides with 2 points each): interior pass and boundary pass.
#include "gales_launch.cuh"

namespace gales {

InteriorOps interior_ops_tri3_magma_mixed() {
  return InteriorDispatch<2, 3, 3, GALES_FORM_MIXED, kEosMagma>::ops();
}

LaunchResult boundary_tri3_magma_mixed(const KParams& k, int nc, long long n, cudaStream_t st) {
  return boundary_dispatch<2, 3, 3, 2, float, kEosMagma>(k, nc, n, st);
}

}  // namespace gales
