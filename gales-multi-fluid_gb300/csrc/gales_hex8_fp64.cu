// Kernel instances for the hex8 element (dim 3, 8 nodes, 8 interior points,
// 6 sides with 4 points each; element.hpp gauss_data tables).
#include "gales_launch.cuh"

namespace gales {

InteriorOps interior_ops_hex8_fp64() { return InteriorDispatch<3, 8, 8, GALES_FORM_FP64>::ops(); }

LaunchResult boundary_hex8(const KParams& k, int nc, int form, long long n, cudaStream_t st) {
  if (form == GALES_FORM_MIXED) return boundary_hex8_mixed(k, nc, n, st);
  return boundary_dispatch<3, 8, 6, 4, double>(k, nc, n, st);
}

GeometryOps geometry_ops_hex8() { return GeometryDispatch<3, 8, 8>::ops(); }

BoundaryInfo boundary_info_hex8(int nc) { return BoundaryInfoDispatch<3, 8, 6, 4>::info(nc); }

LaunchResult adaptive_dt_hex8(const KParams& k, int nc, double cfl, double* dt_el, long long n, cudaStream_t st) {
  return adaptive_dt_dispatch<3, 8, 8>(k, nc, cfl, dt_el, n, st);
}

}  // namespace gales
