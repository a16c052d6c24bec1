// Kernel instances for the tet4 element (dim 3, 4 nodes, 4 interior points,
// 4 sides with 3 points each; element.hpp gauss_data tables).
#include "gales_launch.cuh"

namespace gales {

InteriorOps interior_ops_tet4_fp64() { return InteriorDispatch<3, 4, 4, GALES_FORM_FP64>::ops(); }

LaunchResult boundary_tet4(const KParams& k, int nc, int form, long long n, cudaStream_t st) {
  if (form == GALES_FORM_MIXED) return boundary_tet4_mixed(k, nc, n, st);
  return boundary_dispatch<3, 4, 4, 3, double>(k, nc, n, st);
}

GeometryOps geometry_ops_tet4() { return GeometryDispatch<3, 4, 4>::ops(); }

BoundaryInfo boundary_info_tet4(int nc) { return BoundaryInfoDispatch<3, 4, 4, 3>::info(nc); }

LaunchResult adaptive_dt_tet4(const KParams& k, int nc, double cfl, double* dt_el, long long n, cudaStream_t st) {
  return adaptive_dt_dispatch<3, 4, 4>(k, nc, cfl, dt_el, n, st);
}

LaunchResult secondary_dofs_3d(const KParams& k, int nc, double* out, long long n, cudaStream_t st) {
  return secondary_dofs_dispatch<3>(k, nc, out, n, st);
}

}  // namespace gales
