// Kernel instances for the hex8 element with the magma EOS, FP64 form (dim 3, 8 nodes, 8
// interior points, 6 sides with 4 points each): interior point stage, boundary pass,
// adaptive time step. The mixed form's instances are in gales_hex8_magma_mixed.cu.
#include "gales_launch.cuh"

namespace gales {

LaunchResult boundary_hex8_magma_mixed(const KParams&, int nc, long long n, cudaStream_t);

LaunchResult secondary_dofs_3d_magma(const KParams& k, int nc, double* out, long long n, cudaStream_t st);
LaunchResult magma_fractions_3d(const KParams& k, int nc, double* out, long long n, cudaStream_t st);

namespace {

LaunchResult boundary(const KParams& k, int nc, int form, long long n, cudaStream_t st) {
  if (form == GALES_FORM_MIXED) return boundary_hex8_magma_mixed(k, nc, n, st);
  return boundary_dispatch<3, 8, 6, 4, double, kEosMagma>(k, nc, n, st);
}

LaunchResult adaptive_dt(const KParams& k, int nc, double cfl, double* dt_el, long long n, cudaStream_t st) {
  return adaptive_dt_dispatch<3, 8, 8, kEosMagma>(k, nc, cfl, dt_el, n, st);
}

}  // namespace

InteriorOps interior_ops_hex8_magma_mixed();

MagmaOps magma_ops_hex8() {
  return {{InteriorDispatch<3, 8, 8, GALES_FORM_FP64, kEosMagma>::ops(), interior_ops_hex8_magma_mixed()},
          &boundary, &adaptive_dt, &secondary_dofs_3d_magma, &magma_fractions_3d};
}

}  // namespace gales
