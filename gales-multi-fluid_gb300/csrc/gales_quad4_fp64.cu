// Kernel instances for the quad4 element (dim 2, 4 nodes, 4 interior points,
// 4 sides with 2 points each; element.hpp gauss_data tables).
#include "gales_launch.cuh"

namespace gales {

InteriorOps interior_ops_quad4_fp64() { return InteriorDispatch<2, 4, 4, GALES_FORM_FP64>::ops(); }

LaunchResult boundary_quad4(const KParams& k, int nc, int form, long long n, cudaStream_t st) {
  if (form == GALES_FORM_MIXED) return boundary_quad4_mixed(k, nc, n, st);
  return boundary_dispatch<2, 4, 4, 2, double>(k, nc, n, st);
}

GeometryOps geometry_ops_quad4() { return GeometryDispatch<2, 4, 4>::ops(); }

BoundaryInfo boundary_info_quad4(int nc) { return BoundaryInfoDispatch<2, 4, 4, 2>::info(nc); }

LaunchResult adaptive_dt_quad4(const KParams& k, int nc, double cfl, double* dt_el, long long n, cudaStream_t st) {
  return adaptive_dt_dispatch<2, 4, 4>(k, nc, cfl, dt_el, n, st);
}

}  // namespace gales
