// Kernel instances for the tet4 element with the magma EOS, mixed form (dim 3, 4 nodes,
// 4 interior points, 4 sides with 3 points each): interior pass and boundary pass.
#include "gales_launch.cuh"

namespace gales {

InteriorOps interior_ops_tet4_magma_mixed() {
  return InteriorDispatch<3, 4, 4, GALES_FORM_MIXED, kEosMagma>::ops();
}

LaunchResult boundary_tet4_magma_mixed(const KParams& k, int nc, long long n, cudaStream_t st) {
  return boundary_dispatch<3, 4, 4, 3, float, kEosMagma>(k, nc, n, st);
}

}  // namespace gales
