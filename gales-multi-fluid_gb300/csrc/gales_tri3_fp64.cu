// Kernel instances for the tri3 element (dim 2, 3 nodes, 3 interior points,
// 3 sides with 2 points each; element.hpp gauss_data tables).
#include "gales_launch.cuh"

namespace gales {

InteriorOps interior_ops_tri3_fp64() { return InteriorDispatch<2, 3, 3, GALES_FORM_FP64>::ops(); }

LaunchResult boundary_tri3(const KParams& k, int nc, int form, long long n, cudaStream_t st) {
  if (form == GALES_FORM_MIXED) return boundary_tri3_mixed(k, nc, n, st);
  return boundary_dispatch<2, 3, 3, 2, double>(k, nc, n, st);
}

GeometryOps geometry_ops_tri3() { return GeometryDispatch<2, 3, 3>::ops(); }

BoundaryInfo boundary_info_tri3(int nc) { return BoundaryInfoDispatch<2, 3, 3, 2>::info(nc); }

LaunchResult adaptive_dt_tri3(const KParams& k, int nc, double cfl, double* dt_el, long long n, cudaStream_t st) {
  return adaptive_dt_dispatch<2, 3, 3>(k, nc, cfl, dt_el, n, st);
}

LaunchResult secondary_dofs_2d(const KParams& k, int nc, double* out, long long n, cudaStream_t st) {
  return secondary_dofs_dispatch<2>(k, nc, out, n, st);
}

}  // namespace gales
