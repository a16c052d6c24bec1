// Kernel dispatch for one element type (DIM, NEN): picks the template instance for
// the number of components and the numerical form.  Each element type lives in
// its own translation unit (gales_tri3.cu, gales_quad4.cu, gales_tet4.cu,
// gales_hex8.cu) so the library builds in parallel.
#pragma once

#include <type_traits>

#include "gales_kernels.cuh"

namespace gales {

struct LaunchResult {
  cudaError_t err;
  int launches;
};

template <int DIM, int NEN, int NC, int NQ, int FORM, typename S, bool WANT_M>
LaunchResult launch_interior_inst(const KParams& k, long long n_items, cudaStream_t st) {
  constexpr int EB = 8;
  using SM = InteriorSmem<DIM, NEN, NC, NQ, EB, S>;
  const size_t smem = sizeof(SM);
  auto fn = interior_kernel<DIM, NEN, NC, NQ, FORM, S, WANT_M>;
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return {e, 0};
  const long long blocks = (n_items + EB - 1) / EB;
  if (blocks == 0) return {cudaSuccess, 0};
  fn<<<(unsigned)blocks, 256, smem, st>>>(k);
  return {cudaGetLastError(), 1};
}

template <int DIM, int NEN, int NC, int NQ, int FORM>
LaunchResult launch_interior_nc(const KParams& k, bool want_m, long long n_items, cudaStream_t st) {
  using S = typename std::conditional<FORM == GALES_FORM_FP64, double, float>::type;
  if (want_m) return launch_interior_inst<DIM, NEN, NC, NQ, FORM, S, true>(k, n_items, st);
  return launch_interior_inst<DIM, NEN, NC, NQ, FORM, S, false>(k, n_items, st);
}

template <int DIM, int NEN, int NC, int NS, int NSQ>
LaunchResult launch_boundary_nc(const KParams& k, long long n_items, cudaStream_t st) {
  if (n_items == 0) return {cudaSuccess, 0};
  boundary_kernel<DIM, NEN, NC, NS, NSQ><<<(unsigned)n_items, 32, 0, st>>>(k);
  return {cudaGetLastError(), 1};
}

template <int DIM, int NEN, int NQ, int NS, int NSQ>
struct ElementDispatch {
  template <int FORM>
  static LaunchResult interior(const KParams& k, int nc, bool want_m, long long n, cudaStream_t st) {
    switch (nc) {
      case 1: return launch_interior_nc<DIM, NEN, 1, NQ, FORM>(k, want_m, n, st);
      case 2: return launch_interior_nc<DIM, NEN, 2, NQ, FORM>(k, want_m, n, st);
      case 3: return launch_interior_nc<DIM, NEN, 3, NQ, FORM>(k, want_m, n, st);
      case 4: return launch_interior_nc<DIM, NEN, 4, NQ, FORM>(k, want_m, n, st);
      default: return {cudaErrorInvalidValue, 0};
    }
  }
  static LaunchResult boundary(const KParams& k, int nc, long long n, cudaStream_t st) {
    switch (nc) {
      case 1: return launch_boundary_nc<DIM, NEN, 1, NS, NSQ>(k, n, st);
      case 2: return launch_boundary_nc<DIM, NEN, 2, NS, NSQ>(k, n, st);
      case 3: return launch_boundary_nc<DIM, NEN, 3, NS, NSQ>(k, n, st);
      case 4: return launch_boundary_nc<DIM, NEN, 4, NS, NSQ>(k, n, st);
      default: return {cudaErrorInvalidValue, 0};
    }
  }
};

// Entry points defined by the per-element translation units (<type>_fp64.cu holds the
// FP64 interior and the boundary kernels, <type>_mixed.cu the mixed interior kernels).
LaunchResult interior_tri3_fp64(const KParams&, int nc, bool want_m, long long n, cudaStream_t);
LaunchResult interior_tri3_mixed(const KParams&, int nc, bool want_m, long long n, cudaStream_t);
LaunchResult boundary_tri3(const KParams&, int nc, long long n, cudaStream_t);
LaunchResult interior_quad4_fp64(const KParams&, int nc, bool want_m, long long n, cudaStream_t);
LaunchResult interior_quad4_mixed(const KParams&, int nc, bool want_m, long long n, cudaStream_t);
LaunchResult boundary_quad4(const KParams&, int nc, long long n, cudaStream_t);
LaunchResult interior_tet4_fp64(const KParams&, int nc, bool want_m, long long n, cudaStream_t);
LaunchResult interior_tet4_mixed(const KParams&, int nc, bool want_m, long long n, cudaStream_t);
LaunchResult boundary_tet4(const KParams&, int nc, long long n, cudaStream_t);
LaunchResult interior_hex8_fp64(const KParams&, int nc, bool want_m, long long n, cudaStream_t);
LaunchResult interior_hex8_mixed(const KParams&, int nc, bool want_m, long long n, cudaStream_t);
LaunchResult boundary_hex8(const KParams&, int nc, long long n, cudaStream_t);

}  // namespace gales
