// Kernel instances for the tri3 element (dim 2, 3 nodes, 3 interior points,
// 3 sides with 2 points each; element.hpp gauss_data tables).
#include "gales_launch.cuh"

namespace gales {

InteriorOps interior_ops_tri3_mixed() { return InteriorDispatch<2, 3, 3, GALES_FORM_MIXED>::ops(); }

LaunchResult boundary_tri3_mixed(const KParams& k, int nc, long long n, cudaStream_t st) {
  return boundary_dispatch<2, 3, 3, 2, float>(k, nc, n, st);
}

}  // namespace gales
