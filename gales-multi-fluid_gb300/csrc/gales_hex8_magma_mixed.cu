// Kernel instances for the hex8 element with the magma EOS, mixed form (dim 3, 8 nodes,
// 8 interior points, 6 sides with 4 points each): interior pass and boundary pass.
#include "gales_launch.cuh"

namespace gales {

InteriorOps interior_ops_hex8_magma_mixed() {
  return InteriorDispatch<3, 8, 8, GALES_FORM_MIXED, kEosMagma>::ops();
}

LaunchResult boundary_hex8_magma_mixed(const KParams& k, int nc, long long n, cudaStream_t st) {
  return boundary_dispatch<3, 8, 6, 4, float, kEosMagma>(k, nc, n, st);
}

}  // namespace gales
