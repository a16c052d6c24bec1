// Kernel instances for the tet4 element with the magma EOS, FP64 form (dim 3, 4 nodes, 4
// interior points, 4 sides with 3 points each): interior point stage, boundary pass,
// adaptive time step, and the nodal secondary variables and gas fractions of every 3D
// element type. The mixed form's instances are in gales_tet4_magma_mixed.cu.
#include "gales_launch.cuh"

namespace gales {

LaunchResult boundary_tet4_magma_mixed(const KParams&, int nc, long long n, cudaStream_t);

LaunchResult secondary_dofs_3d_magma(const KParams& k, int nc, double* out, long long n, cudaStream_t st) {
  return secondary_dofs_dispatch<3, kEosMagma>(k, nc, out, n, st);
}

LaunchResult magma_fractions_3d(const KParams& k, int nc, double* out, long long n, cudaStream_t st) {
  return magma_fractions_dispatch<3>(k, nc, out, n, st);
}

namespace {

LaunchResult boundary(const KParams& k, int nc, int form, long long n, cudaStream_t st) {
  if (form == GALES_FORM_MIXED) return boundary_tet4_magma_mixed(k, nc, n, st);
  return boundary_dispatch<3, 4, 4, 3, double, kEosMagma>(k, nc, n, st);
}

LaunchResult adaptive_dt(const KParams& k, int nc, double cfl, double* dt_el, long long n, cudaStream_t st) {
  return adaptive_dt_dispatch<3, 4, 4, kEosMagma>(k, nc, cfl, dt_el, n, st);
}

}  // namespace

InteriorOps interior_ops_tet4_magma_mixed();

MagmaOps magma_ops_tet4() {
  return {{InteriorDispatch<3, 4, 4, GALES_FORM_FP64, kEosMagma>::ops(), interior_ops_tet4_magma_mixed()},
          &boundary, &adaptive_dt, &secondary_dofs_3d_magma, &magma_fractions_3d};
}

}  // namespace gales
