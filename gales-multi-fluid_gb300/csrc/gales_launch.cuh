// Kernel dispatch for one element type (DIM, NEN): picks the template instance for
// the number of components and the numerical form.  Each (element type, form)
// pair lives in its own translation unit (gales_<type>_<form>.cu) so the library
// builds in parallel; the boundary kernels are in the FP64 unit.
#pragma once

#include <type_traits>

#include "gales_kernels.cuh"

namespace gales {

struct LaunchResult {
  cudaError_t err;
  int launches;
};

template <int DIM, int NEN, int NC, int NQ, int FORM, int EOS = kEosChemicals>
struct InteriorInst {
  using S = typename std::conditional<FORM == GALES_FORM_FP64, double, float>::type;
  using Rec = QP<DIM, NEN, NC, S>;
  using RB = RecBlock<DIM, NEN, NC, NQ, S>;
  using SM = MatSmem<DIM, NEN, NC, NQ, S>;
  using M = MatShape<DIM, NEN, NC>;
  // record bytes per element, rounded up: (elements + 4) of them hold the blocks of a
  // chunk of elements
  static size_t rec_bytes() { return (RB::BYTES + M::EPC - 1) / M::EPC; }
  // resident point-kernel CTAs (128 threads) per SM
  static int point_occupancy() {
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, point_kernel<DIM, NEN, NC, NQ, FORM, S, EOS>, 128, 0) !=
        cudaSuccess)
      return 1;
    return nb > 0 ? nb : 1;
  }
  static LaunchResult point(const KParams& k, void* buf, long long first, long long n, cudaStream_t st) {
    if (n <= 0) return {cudaSuccess, 0};
    const long long threads = n * NQ;
    point_kernel<DIM, NEN, NC, NQ, FORM, S, EOS><<<(unsigned)((threads + 127) / 128), 128, 0, st>>>(
        k, reinterpret_cast<Rec*>(buf), first, n);
    return {cudaGetLastError(), 1};
  }
  // resident matrix CTAs per SM (set by prepare)
  static int& matrix_occupancy() {
    static int occ = 1;
    return occ;
  }
  // dynamic shared memory limits, set once per device before any launch (also before
  // a stream capture), and the matrix kernel's occupancy
  static cudaError_t prepare() {
    const int smem = (int)SM::BYTES;
    cudaError_t e = cudaFuncSetAttribute(matrix_kernel<DIM, NEN, NC, NQ, S, true>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    e = cudaFuncSetAttribute(matrix_kernel<DIM, NEN, NC, NQ, S, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             smem);
    if (e != cudaSuccess) return e;
    int nb = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, matrix_kernel<DIM, NEN, NC, NQ, S, true>, M::CTA, smem);
    if (e != cudaSuccess) return e;
    matrix_occupancy() = nb > 0 ? nb : 1;
    return cudaSuccess;
  }
  // persistent: at most (SMs x resident CTAs) CTAs, each looping over element groups
  static LaunchResult matrix(const KParams& k, bool want_m, const void* buf, long long first, long long n,
                             cudaStream_t st) {
    if (n <= 0) return {cudaSuccess, 0};
    const size_t smem = SM::BYTES;
    const long long groups = (n + M::EPC - 1) / M::EPC;
    const long long cap = (long long)(k.sms > 0 ? k.sms : 1) * matrix_occupancy();
    const unsigned blocks = (unsigned)(groups < cap ? groups : cap);
    const S* in = reinterpret_cast<const S*>(buf);
    if (want_m) matrix_kernel<DIM, NEN, NC, NQ, S, true><<<blocks, M::CTA, smem, st>>>(k, in, first, n);
    else matrix_kernel<DIM, NEN, NC, NQ, S, false><<<blocks, M::CTA, smem, st>>>(k, in, first, n);
    return {cudaGetLastError(), 1};
  }
};

template <int DIM, int NEN, int NC, int NS, int NSQ, typename S, int EOS = kEosChemicals>
cudaError_t prepare_boundary_nc() {
  return cudaFuncSetAttribute(boundary_kernel<DIM, NEN, NC, NS, NSQ, S, EOS>,
                              cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)sizeof(BoundarySmem<DIM, NEN, NC, NS, NSQ, S>));
}

// Boundary pass: with point records (k.bpt_rec) the point stage runs first, one thread
// per flagged side point; the element stage then reads the records.
template <int DIM, int NEN, int NC, int NS, int NSQ, typename S, int EOS = kEosChemicals>
LaunchResult launch_boundary_nc(const KParams& k, long long n_items, cudaStream_t st) {
  if (n_items == 0) return {cudaSuccess, 0};
  int launches = 0;
  if (k.bpt_rec && k.n_bpt > 0) {
    bpoint_kernel<DIM, NEN, NC, NS, NSQ, S, EOS><<<(unsigned)((k.n_bpt + 127) / 128), 128, 0, st>>>(k);
    ++launches;
  }
  const size_t smem = sizeof(BoundarySmem<DIM, NEN, NC, NS, NSQ, S>);
  boundary_kernel<DIM, NEN, NC, NS, NSQ, S, EOS><<<(unsigned)n_items, 32, smem, st>>>(k);
  return {cudaGetLastError(), launches + 1};
}

// Interior operations of one (element type, form): record bytes per element, point
// stage and matrix stage, for 1..4 components.
struct InteriorOps {
  cudaError_t (*prepare)(int nc);
  int (*point_occupancy)(int nc);
  size_t (*rec_bytes)(int nc);
  LaunchResult (*point)(const KParams&, int nc, void* buf, long long first, long long n, cudaStream_t);
  LaunchResult (*matrix)(const KParams&, int nc, bool want_m, const void* buf, long long first, long long n,
                         cudaStream_t);
};

#define GALES_NC_SWITCH(expr_nc, CALL) \
  switch (expr_nc) {                   \
    case 1: CALL(1);                   \
    case 2: CALL(2);                   \
    case 3: CALL(3);                   \
    case 4: CALL(4);                   \
    default: break;                    \
  }

template <int DIM, int NEN, int NQ, int FORM, int EOS = kEosChemicals>
struct InteriorDispatch {
  static cudaError_t prepare(int nc) {
#define GALES_C(NC) return InteriorInst<DIM, NEN, NC, NQ, FORM, EOS>::prepare()
    GALES_NC_SWITCH(nc, GALES_C)
#undef GALES_C
    return cudaErrorInvalidValue;
  }
  static int point_occupancy(int nc) {
#define GALES_C(NC) return InteriorInst<DIM, NEN, NC, NQ, FORM, EOS>::point_occupancy()
    GALES_NC_SWITCH(nc, GALES_C)
#undef GALES_C
    return 1;
  }
  static size_t rec_bytes(int nc) {
#define GALES_C(NC) return InteriorInst<DIM, NEN, NC, NQ, FORM, EOS>::rec_bytes()
    GALES_NC_SWITCH(nc, GALES_C)
#undef GALES_C
    return 0;
  }
  static LaunchResult point(const KParams& k, int nc, void* buf, long long first, long long n, cudaStream_t st) {
#define GALES_C(NC) return InteriorInst<DIM, NEN, NC, NQ, FORM, EOS>::point(k, buf, first, n, st)
    GALES_NC_SWITCH(nc, GALES_C)
#undef GALES_C
    return {cudaErrorInvalidValue, 0};
  }
  static LaunchResult matrix(const KParams& k, int nc, bool want_m, const void* buf, long long first, long long n,
                             cudaStream_t st) {
#define GALES_C(NC) return InteriorInst<DIM, NEN, NC, NQ, FORM, EOS>::matrix(k, want_m, buf, first, n, st)
    GALES_NC_SWITCH(nc, GALES_C)
#undef GALES_C
    return {cudaErrorInvalidValue, 0};
  }
  static InteriorOps ops() { return {&prepare, &point_occupancy, &rec_bytes, &point, &matrix}; }
};

// Boundary pass of one element type; S is the matrix arithmetic type of the form.
// n < 0 only prepares the kernel (shared-memory limit) and launches nothing.
template <int DIM, int NEN, int NS, int NSQ, typename S, int EOS = kEosChemicals>
LaunchResult boundary_dispatch(const KParams& k, int nc, long long n, cudaStream_t st) {
  if (n < 0) {
#define GALES_C(NC) return {prepare_boundary_nc<DIM, NEN, NC, NS, NSQ, S, EOS>(), 0}
    GALES_NC_SWITCH(nc, GALES_C)
#undef GALES_C
    return {cudaErrorInvalidValue, 0};
  }
#define GALES_C(NC) return launch_boundary_nc<DIM, NEN, NC, NS, NSQ, S, EOS>(k, n, st)
  GALES_NC_SWITCH(nc, GALES_C)
#undef GALES_C
  return {cudaErrorInvalidValue, 0};
}

// Adaptive time step (f_mc) per element of one element type.
template <int DIM, int NEN, int NQ, int EOS = kEosChemicals>
LaunchResult adaptive_dt_dispatch(const KParams& k, int nc, double cfl, double* dt_el, long long n, cudaStream_t st) {
  if (n <= 0) return {cudaSuccess, 0};
  const unsigned blocks = (unsigned)((n + 127) / 128);
#define GALES_C(NC)                                                                       \
  adaptive_dt_kernel<DIM, NEN, NC, NQ, EOS><<<blocks, 128, 0, st>>>(k, cfl, dt_el, n); \
  return {cudaGetLastError(), 1}
  GALES_NC_SWITCH(nc, GALES_C)
#undef GALES_C
  return {cudaErrorInvalidValue, 0};
}

// Secondary variables at the nodes (any element type of the dimension).
template <int DIM, int EOS = kEosChemicals>
LaunchResult secondary_dofs_dispatch(const KParams& k, int nc, double* out, long long n, cudaStream_t st) {
  if (n <= 0) return {cudaSuccess, 0};
  const unsigned blocks = (unsigned)((n + 127) / 128);
#define GALES_C(NC)                                                            \
  secondary_dofs_kernel<DIM, NC, EOS><<<blocks, 128, 0, st>>>(k, out, n); \
  return {cudaGetLastError(), 1}
  GALES_NC_SWITCH(nc, GALES_C)
#undef GALES_C
  return {cudaErrorInvalidValue, 0};
}

// Magma gas fractions at the nodes (pp_vf_g).
template <int DIM>
LaunchResult magma_fractions_dispatch(const KParams& k, int nc, double* out, long long n, cudaStream_t st) {
  if (n <= 0) return {cudaSuccess, 0};
  const unsigned blocks = (unsigned)((n + 127) / 128);
#define GALES_C(NC)                                                            \
  magma_fractions_kernel<DIM, NC><<<blocks, 128, 0, st>>>(k, out, n); \
  return {cudaGetLastError(), 1}
  GALES_NC_SWITCH(nc, GALES_C)
#undef GALES_C
  return {cudaErrorInvalidValue, 0};
}

// Every kernel of one element type compiled with the magma EOS (gales_<type>_magma.cu).
struct MagmaOps {
  InteriorOps interior[2];   // per form (FP64, mixed)
  LaunchResult (*boundary)(const KParams&, int nc, int form, long long n, cudaStream_t);
  LaunchResult (*adaptive_dt)(const KParams&, int nc, double cfl, double* dt_el, long long n, cudaStream_t);
  LaunchResult (*secondary_dofs)(const KParams&, int nc, double* out, long long n, cudaStream_t);
  LaunchResult (*fractions)(const KParams&, int nc, double* out, long long n, cudaStream_t);
};

// Boundary side-point geometry (handle creation) and record sizes.
struct BoundaryInfo {
  size_t bgeo_bytes;
  size_t rec_bytes[2];   // per form (FP64, mixed)
  LaunchResult (*geometry)(const KParams& k, void* out, cudaStream_t st);
};

template <int DIM, int NEN, int NS, int NSQ>
struct BoundaryInfoDispatch {
  static LaunchResult geometry(const KParams& k, void* out, cudaStream_t st) {
    if (k.n_bpt <= 0) return {cudaSuccess, 0};
    bgeo_kernel<DIM, NEN, NS, NSQ><<<(unsigned)((k.n_bpt + 127) / 128), 128, 0, st>>>(
        k, reinterpret_cast<BGeo<DIM, NEN>*>(out));
    return {cudaGetLastError(), 1};
  }
  static BoundaryInfo info(int nc) {
    BoundaryInfo b{sizeof(BGeo<DIM, NEN>), {0, 0}, &geometry};
#define GALES_C(NC)                                                      \
  b.rec_bytes[0] = sizeof(BPointRec<DIM, NEN, NC, double>);            \
  b.rec_bytes[1] = sizeof(BPointRec<DIM, NEN, NC, float>);             \
  break
    GALES_NC_SWITCH(nc, GALES_C)
#undef GALES_C
    return b;
  }
};

// Element geometry precompute (handle creation).
struct GeometryOps {
  size_t bytes_per_element;
  LaunchResult (*launch)(const double* coords, const int32_t* conn, const KParams& k, void* out, long long n_el,
                         cudaStream_t st);
};

template <int DIM, int NEN, int NQ>
struct GeometryDispatch {
  static constexpr int NG = geo_per_element<DIM, NEN>(NQ);
  static LaunchResult launch(const double* coords, const int32_t* conn, const KParams& k, void* out, long long n_el,
                             cudaStream_t st) {
    if (n_el <= 0) return {cudaSuccess, 0};
    const long long threads = n_el * NG;
    geometry_kernel<DIM, NEN, NQ><<<(unsigned)((threads + 127) / 128), 128, 0, st>>>(
        coords, conn, k, reinterpret_cast<ElemGeo<DIM, NEN>*>(out), n_el);
    return {cudaGetLastError(), 1};
  }
  static GeometryOps ops() { return {sizeof(ElemGeo<DIM, NEN>) * NG, &launch}; }
};

// Entry points defined by the per-element translation units.
InteriorOps interior_ops_tri3_fp64();
InteriorOps interior_ops_tri3_mixed();
LaunchResult boundary_tri3(const KParams&, int nc, int form, long long n, cudaStream_t);
LaunchResult boundary_tri3_mixed(const KParams&, int nc, long long n, cudaStream_t);
GeometryOps geometry_ops_tri3();
BoundaryInfo boundary_info_tri3(int nc);
LaunchResult adaptive_dt_tri3(const KParams&, int nc, double cfl, double* dt_el, long long n, cudaStream_t);
LaunchResult secondary_dofs_2d(const KParams&, int nc, double* out, long long n, cudaStream_t);
InteriorOps interior_ops_quad4_fp64();
InteriorOps interior_ops_quad4_mixed();
LaunchResult boundary_quad4(const KParams&, int nc, int form, long long n, cudaStream_t);
LaunchResult boundary_quad4_mixed(const KParams&, int nc, long long n, cudaStream_t);
GeometryOps geometry_ops_quad4();
BoundaryInfo boundary_info_quad4(int nc);
LaunchResult adaptive_dt_quad4(const KParams&, int nc, double cfl, double* dt_el, long long n, cudaStream_t);
InteriorOps interior_ops_tet4_fp64();
InteriorOps interior_ops_tet4_mixed();
LaunchResult boundary_tet4(const KParams&, int nc, int form, long long n, cudaStream_t);
LaunchResult boundary_tet4_mixed(const KParams&, int nc, long long n, cudaStream_t);
GeometryOps geometry_ops_tet4();
BoundaryInfo boundary_info_tet4(int nc);
LaunchResult adaptive_dt_tet4(const KParams&, int nc, double cfl, double* dt_el, long long n, cudaStream_t);
LaunchResult secondary_dofs_3d(const KParams&, int nc, double* out, long long n, cudaStream_t);
InteriorOps interior_ops_hex8_fp64();
InteriorOps interior_ops_hex8_mixed();
LaunchResult boundary_hex8(const KParams&, int nc, int form, long long n, cudaStream_t);
// exact VJP kernels (gales_vjp_<type>.cu)
LaunchResult vjp_interior_tri3(const KParams&, int nc, long long n, cudaStream_t);
LaunchResult vjp_boundary_tri3(const KParams&, int nc, long long n, cudaStream_t);
LaunchResult vjp_interior_quad4(const KParams&, int nc, long long n, cudaStream_t);
LaunchResult vjp_boundary_quad4(const KParams&, int nc, long long n, cudaStream_t);
LaunchResult vjp_interior_tet4(const KParams&, int nc, long long n, cudaStream_t);
LaunchResult vjp_boundary_tet4(const KParams&, int nc, long long n, cudaStream_t);
LaunchResult vjp_interior_hex8(const KParams&, int nc, long long n, cudaStream_t);
LaunchResult vjp_boundary_hex8(const KParams&, int nc, long long n, cudaStream_t);
LaunchResult boundary_hex8_mixed(const KParams&, int nc, long long n, cudaStream_t);
GeometryOps geometry_ops_hex8();
BoundaryInfo boundary_info_hex8(int nc);
LaunchResult adaptive_dt_hex8(const KParams&, int nc, double cfl, double* dt_el, long long n, cudaStream_t);
// The device array of a magma material's sub-mixtures, its count and its device
// (gales_magma.cu).
const magma_mix::DevMagma* magma_device_table(const gales_magma* m, int* nc, int* device);
MagmaOps magma_ops_tri3();
MagmaOps magma_ops_quad4();
MagmaOps magma_ops_tet4();
MagmaOps magma_ops_hex8();

}  // namespace gales
