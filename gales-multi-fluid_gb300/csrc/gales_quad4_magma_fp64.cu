// Kernel instances for the quad4 element with the magma EOS, FP64 form (dim 2, 4 nodes,
// 4 interior points, 4 sides with 2 points each): interior point stage, boundary pass,
// adaptive time step. The mixed form's instances are in gales_quad4_magma_mixed.cu.
#include "gales_launch.cuh"

namespace gales {

LaunchResult boundary_quad4_magma_mixed(const KParams&, int nc, long long n, cudaStream_t);

LaunchResult secondary_dofs_2d_magma(const KParams& k, int nc, double* out, long long n, cudaStream_t st);
LaunchResult magma_fractions_2d(const KParams& k, int nc, double* out, long long n, cudaStream_t st);

namespace {

LaunchResult boundary(const KParams& k, int nc, int form, long long n, cudaStream_t st) {
  if (form == GALES_FORM_MIXED) return boundary_quad4_magma_mixed(k, nc, n, st);
  return boundary_dispatch<2, 4, 4, 2, double, kEosMagma>(k, nc, n, st);
}

LaunchResult adaptive_dt(const KParams& k, int nc, double cfl, double* dt_el, long long n, cudaStream_t st) {
  return adaptive_dt_dispatch<2, 4, 4, kEosMagma>(k, nc, cfl, dt_el, n, st);
}

}  // namespace

InteriorOps interior_ops_quad4_magma_mixed();

MagmaOps magma_ops_quad4() {
  return {{InteriorDispatch<2, 4, 4, GALES_FORM_FP64, kEosMagma>::ops(), interior_ops_quad4_magma_mixed()},
          &boundary, &adaptive_dt, &secondary_dofs_2d_magma, &magma_fractions_2d};
}

}  // namespace gales
