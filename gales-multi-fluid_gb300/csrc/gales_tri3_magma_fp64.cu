// Kernel instances for the tri3 element with the magma EOS, FP64 form (dim 2, 3 nodes, 3
// interior points, 3 sides with 2 points each): interior point stage, boundary pass,
// adaptive time step, and the nodal secondary variables and gas fractions of every 2D
// element type. The mixed form's instances are in gales_tri3_magma_mixed.cu.
#include "gales_launch.cuh"

namespace gales {

LaunchResult boundary_tri3_magma_mixed(const KParams&, int nc, long long n, cudaStream_t);

LaunchResult secondary_dofs_2d_magma(const KParams& k, int nc, double* out, long long n, cudaStream_t st) {
  return secondary_dofs_dispatch<2, kEosMagma>(k, nc, out, n, st);
}

LaunchResult magma_fractions_2d(const KParams& k, int nc, double* out, long long n, cudaStream_t st) {
  return magma_fractions_dispatch<2>(k, nc, out, n, st);
}

namespace {

LaunchResult boundary(const KParams& k, int nc, int form, long long n, cudaStream_t st) {
  if (form == GALES_FORM_MIXED) return boundary_tri3_magma_mixed(k, nc, n, st);
  return boundary_dispatch<2, 3, 3, 2, double, kEosMagma>(k, nc, n, st);
}

LaunchResult adaptive_dt(const KParams& k, int nc, double cfl, double* dt_el, long long n, cudaStream_t st) {
  return adaptive_dt_dispatch<2, 3, 3, kEosMagma>(k, nc, cfl, dt_el, n, st);
}

}  // namespace

InteriorOps interior_ops_tri3_magma_mixed();

MagmaOps magma_ops_tri3() {
  return {{InteriorDispatch<2, 3, 3, GALES_FORM_FP64, kEosMagma>::ops(), interior_ops_tri3_magma_mixed()},
          &boundary, &adaptive_dt, &secondary_dofs_2d_magma, &magma_fractions_2d};
}

}  // namespace gales
