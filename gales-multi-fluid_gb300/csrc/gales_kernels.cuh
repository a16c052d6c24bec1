// Element assembly kernels for fluid_mc (interior and boundary passes).
//
// Interior pass, two kernels per chunk of elements:
//   point_kernel  - one thread per (element, quadrature point): interpolation
//                   (quad.hpp:817-885), mixture EOS at P and I (fluid_2d.hpp:179-195),
//                   flux scalars (fluid_2d.hpp:391-603), tau (fluid_2d.hpp:877-1022)
//                   and the dc viscosity (fluid_2d.hpp:1027-1065), written as a point
//                   record in the form's arithmetic type S.
//   matrix_kernel - one warp per element (more for hexahedra), one lane per row of
//                   the element block: Galerkin, least-squares and dc terms of RM_i
//                   (fluid_2d.hpp:251-333) accumulated in registers over the points,
//                   then the Dirichlet row replacement of scatter::execute
//                   (scatter.hpp:62-78) and FP64 adds into the CSR values and rhs
//                   (scatter.hpp:96-97).
// Boundary kernel, one warp per boundary element: execute_b/RM_b
// (fluid_2d.hpp:209-245, 341-364, 610-868) and its own scatter pass
// (fluid_assembly.hpp:57-63), all in FP64.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include <type_traits>

#include "gales_physics.cuh"

namespace gales {

struct KParams {
  // mixture and flags
  DevChem ch[GALES_MAX_COMP];
  double dt;
  double dc_sharp, dc_scale;
  double gravity[3];
  double u_ref_inv[GALES_MAX_ND];
  double gp[8][3];
  double W_in, W_bd;
  int32_t tau, dc_2006, steady;
  int32_t has_gas;             // some component is an ideal gas (mixed-form EOS)
  const magma_mix::DevMagma* mg;  // magma sub-mixtures (kernels compiled with kEosMagma)
  int32_t n_sides, n_side_nodes, n_side_q;
  uint32_t dirichlet_mask[GALES_MAX_FLAGS];
  double sgp[6][4][3];
  // binary32 copies (round to nearest) of parameters the mixed form uses in FP32
  float gravity_f[3], u_ref_inv_f[GALES_MAX_ND], inv_dt_f, dc_scale_f;
  // mesh
  const double* coords;
  const int32_t* conn;
  const int32_t* node_flag;
  const int64_t* node_rp;      // node graph row pointers [n_nodes+1]
  const uint16_t* slot;        // [n_el][nen][nen]: position of node a in node b's graph row
  int64_t n_elements;
  const int32_t* el_list;      // optional element list (colour batch / boundary elements)
  int64_t n_list;
  const int8_t* bd_sides;      // [n_list][n_sides] side flags of the listed boundary elements
  const gales_side_bc* side_bc;  // [GALES_MAX_FLAGS]
  // state and outputs
  const double* I;
  const double* P;
  double* vals;
  double* rhs;
  double inv_dt;
  unsigned int* status;
  unsigned long long* first_bad;
  int32_t scatter_mode;        // 0 atomics, 1 plain read-modify-write (coloured batches)
  int32_t sms;                 // multiprocessors of the device (persistent grids)
  const void* geo;             // ElemGeo records (per element, or per element and point)
  double sh_tab[8][8];         // shape functions at the interior points [q][node]
  float sh_tab_f[8][8];        // the same rounded to binary32 (mixed form)
  double* local_m;             // element-level output [n_list][(nen*nd)^2] (no scatter) or null
  double* local_r;             // element-level output [n_list][nen*nd] (r = -r_) or null
  // vector-Jacobian products: lambda, g_state (+=) and g_params (+=); when vjp_lam is set
  // the matrix and boundary kernels contract their blocks with lambda instead of scattering
  const double* vjp_lam;
  double* vjp_g;
  double* vjp_th;
  // boundary points (flagged side points of the listed boundary elements): per-element
  // offsets [n_list+1], element slot and (side, point) index, precomputed geometry and
  // the point records of the boundary point stage; null for the fused boundary pass
  const int32_t* bpt_off;
  const int32_t* bpt_el;
  const int32_t* bpt_ip;
  const void* bgeo;
  void* bpt_rec;
  int64_t n_bpt;
  // arrays the point stage zeroes beside its own work (the first chunk's launch clears
  // A and b, whose first writers are the matrix and boundary stages after it)
  double* clear_p[2];
  int64_t clear_n[2];
};

__device__ __forceinline__ void flag_error(const KParams& k, unsigned int bits, long long e) {
  atomicOr(k.status, bits);
  atomicMin(k.first_bad, (unsigned long long)e);
}

template <typename S>
__device__ __forceinline__ void add_to(double* p, S v, int mode) {
  if (mode == 0) atomicAdd(p, (double)v);
  else *p += (double)v;
}

// ---------------------------------------------------------------------------
// Geometry at a point (quad.hpp).  dl: local derivatives; returns J.
template <int DIM, int NEN>
__device__ __forceinline__ void shape_local(const double* pt, double* sh, double (&dl)[DIM][NEN]) {
  if constexpr (DIM == 2 && NEN == 3) {
    const double xi = pt[0], eta = pt[1];
    sh[0] = 1.0 - xi - eta; sh[1] = xi; sh[2] = eta;
    dl[0][0] = -1.0; dl[1][0] = -1.0;
    dl[0][1] = 1.0;  dl[1][1] = 0.0;
    dl[0][2] = 0.0;  dl[1][2] = 1.0;
  } else if constexpr (DIM == 2 && NEN == 4) {
    const double xi = pt[0], eta = pt[1];
    sh[0] = 0.25 * (1.0 - xi) * (1.0 - eta);
    sh[1] = 0.25 * (1.0 + xi) * (1.0 - eta);
    sh[2] = 0.25 * (1.0 + xi) * (1.0 + eta);
    sh[3] = 0.25 * (1.0 - xi) * (1.0 + eta);
    dl[0][0] = -0.25 * (1. - eta); dl[1][0] = -0.25 * (1. - xi);
    dl[0][1] = 0.25 * (1. - eta);  dl[1][1] = -0.25 * (1. + xi);
    dl[0][2] = 0.25 * (1. + eta);  dl[1][2] = 0.25 * (1. + xi);
    dl[0][3] = -0.25 * (1. + eta); dl[1][3] = 0.25 * (1. - xi);
  } else if constexpr (DIM == 3 && NEN == 4) {
    const double xi = pt[0], eta = pt[1], zeta = pt[2];
    sh[0] = 1.0 - xi - eta - zeta; sh[1] = xi; sh[2] = eta; sh[3] = zeta;
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
      for (int i = 0; i < 4; ++i) dl[k][i] = (i == 0) ? -1.0 : ((i == k + 1) ? 1.0 : 0.0);
  } else {
    const double xi = pt[0], eta = pt[1], zeta = pt[2];
    const double sx[8] = {-1, 1, 1, -1, -1, 1, 1, -1};
    const double sy[8] = {-1, -1, 1, 1, -1, -1, 1, 1};
    const double sz[8] = {-1, -1, -1, -1, 1, 1, 1, 1};
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const double ax = sx[i] < 0 ? (1.0 - xi) : (1.0 + xi);
      const double ay = sy[i] < 0 ? (1.0 - eta) : (1.0 + eta);
      const double az = sz[i] < 0 ? (1.0 - zeta) : (1.0 + zeta);
      sh[i] = 0.125 * ax * ay * az;
      dl[0][i] = (sx[i] < 0 ? -0.125 : 0.125) * ay * az;
      dl[1][i] = (sy[i] < 0 ? -0.125 : 0.125) * ax * az;
      dl[2][i] = (sz[i] < 0 ? -0.125 : 0.125) * ax * ay;
    }
  }
}

// Mapping derivatives and global shape gradients; optionally metrics G, g and the
// boundary area vector JN (quad.hpp:196-345, 523-691).
template <int DIM, int NEN>
struct Geo {
  double sh[NEN], ds[DIM][NEN], J, G[DIM][DIM], g[DIM], JN[DIM];
};

template <int DIM, int NEN>
__device__ __forceinline__ void geometry(const double (&X)[NEN][DIM], const double* pt, bool interior,
                                         Geo<DIM, NEN>& o) {
  double dl[DIM][NEN];
  shape_local<DIM, NEN>(pt, o.sh, dl);
  if constexpr (DIM == 2) {
    double dx_dxi = 0.0, dx_deta = 0.0, dy_dxi = 0.0, dy_deta = 0.0;
#pragma unroll
    for (int i = 0; i < NEN; ++i) {
      dx_dxi += dl[0][i] * X[i][0];
      dx_deta += dl[1][i] * X[i][0];
      dy_dxi += dl[0][i] * X[i][1];
      dy_deta += dl[1][i] * X[i][1];
    }
    o.J = dx_dxi * dy_deta - dy_dxi * dx_deta;
    const double dxi_dx = (1 / o.J) * (dy_deta);
    const double deta_dx = (1 / o.J) * (-dy_dxi);
    const double dxi_dy = (1 / o.J) * (-dx_deta);
    const double deta_dy = (1 / o.J) * (dx_dxi);
#pragma unroll
    for (int i = 0; i < NEN; ++i) {
      o.ds[0][i] = dl[0][i] * dxi_dx + dl[1][i] * deta_dx;
      o.ds[1][i] = dl[0][i] * dxi_dy + dl[1][i] * deta_dy;
    }
    if (interior) {
      o.g[0] = dxi_dx + deta_dx;
      o.g[1] = dxi_dy + deta_dy;
      o.G[0][0] = dxi_dx * dxi_dx + deta_dx * deta_dx;
      o.G[1][1] = dxi_dy * dxi_dy + deta_dy * deta_dy;
      o.G[0][1] = dxi_dx * dxi_dy + deta_dx * deta_dy;
      o.G[1][0] = o.G[0][1];
    } else {
      const double xi = pt[0], eta = pt[1];
      o.JN[0] = 0.0; o.JN[1] = 0.0;
      if constexpr (NEN == 4) {
        if (eta == 1.0) { o.JN[0] = -dy_dxi; o.JN[1] = dx_dxi; }
        else if (eta == -1.0) { o.JN[0] = dy_dxi; o.JN[1] = -dx_dxi; }
        else if (xi == 1.0) { o.JN[0] = dy_deta; o.JN[1] = -dx_deta; }
        else if (xi == -1.0) { o.JN[0] = -dy_deta; o.JN[1] = dx_deta; }
      } else {
        if (xi == 0.0) { o.JN[0] = -dy_deta; o.JN[1] = dx_deta; }
        else if (eta == 0.0) { o.JN[0] = dy_dxi; o.JN[1] = -dx_dxi; }
        else { o.JN[0] = dy_deta - dy_dxi; o.JN[1] = dx_dxi - dx_deta; }
      }
    }
  } else {
    double a[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};  // a[i][j] = d x_i / d xi_j
#pragma unroll
    for (int n = 0; n < NEN; ++n)
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) a[i][j] += dl[j][n] * X[n][i];
    const double dx_dxi = a[0][0], dx_deta = a[0][1], dx_dzeta = a[0][2];
    const double dy_dxi = a[1][0], dy_deta = a[1][1], dy_dzeta = a[1][2];
    const double dz_dxi = a[2][0], dz_deta = a[2][1], dz_dzeta = a[2][2];
    o.J = dx_dxi * (dy_deta * dz_dzeta - dz_deta * dy_dzeta) -
          dy_dxi * (dx_deta * dz_dzeta - dz_deta * dx_dzeta) +
          dz_dxi * (dx_deta * dy_dzeta - dy_deta * dx_dzeta);
    const double iJ = 1 / o.J;
    const double dxi_dx = iJ * (dy_deta * dz_dzeta - dz_deta * dy_dzeta);
    const double deta_dx = iJ * (-dy_dxi * dz_dzeta + dz_dxi * dy_dzeta);
    const double dzeta_dx = iJ * (dy_dxi * dz_deta - dz_dxi * dy_deta);
    const double dxi_dy = iJ * (-dx_deta * dz_dzeta + dz_deta * dx_dzeta);
    const double deta_dy = iJ * (dx_dxi * dz_dzeta - dz_dxi * dx_dzeta);
    const double dzeta_dy = iJ * (-dx_dxi * dz_deta + dz_dxi * dx_deta);
    const double dxi_dz = iJ * (dx_deta * dy_dzeta - dy_deta * dx_dzeta);
    const double deta_dz = iJ * (-dx_dxi * dy_dzeta + dy_dxi * dx_dzeta);
    const double dzeta_dz = iJ * (dx_dxi * dy_deta - dy_dxi * dx_deta);
#pragma unroll
    for (int i = 0; i < NEN; ++i) {
      o.ds[0][i] = dl[0][i] * dxi_dx + dl[1][i] * deta_dx + dl[2][i] * dzeta_dx;
      o.ds[1][i] = dl[0][i] * dxi_dy + dl[1][i] * deta_dy + dl[2][i] * dzeta_dy;
      o.ds[2][i] = dl[0][i] * dxi_dz + dl[1][i] * deta_dz + dl[2][i] * dzeta_dz;
    }
    if (interior) {
      o.g[0] = dxi_dx + deta_dx + dzeta_dx;
      o.g[1] = dxi_dy + deta_dy + dzeta_dy;
      o.g[2] = dxi_dz + deta_dz + dzeta_dz;
      o.G[0][0] = dxi_dx * dxi_dx + deta_dx * deta_dx + dzeta_dx * dzeta_dx;
      o.G[1][1] = dxi_dy * dxi_dy + deta_dy * deta_dy + dzeta_dy * dzeta_dy;
      o.G[2][2] = dxi_dz * dxi_dz + deta_dz * deta_dz + dzeta_dz * dzeta_dz;
      o.G[0][1] = dxi_dx * dxi_dy + deta_dx * deta_dy + dzeta_dx * dzeta_dy;
      o.G[1][2] = dxi_dy * dxi_dz + deta_dy * deta_dz + dzeta_dy * dzeta_dz;
      o.G[0][2] = dxi_dz * dxi_dx + deta_dz * deta_dx + dzeta_dz * dzeta_dx;
      o.G[1][0] = o.G[0][1];
      o.G[2][1] = o.G[1][2];
      o.G[2][0] = o.G[0][2];
    } else {
      const double xi = pt[0], eta = pt[1], zeta = pt[2];
      double* JN = o.JN;
      JN[0] = JN[1] = JN[2] = 0.0;
      if constexpr (NEN == 8) {
        if (zeta == 1.0) {
          JN[0] = dy_dxi * dz_deta - dz_dxi * dy_deta;
          JN[1] = dz_dxi * dx_deta - dx_dxi * dz_deta;
          JN[2] = dx_dxi * dy_deta - dy_dxi * dx_deta;
        } else if (zeta == -1.0) {
          JN[0] = -dy_dxi * dz_deta + dz_dxi * dy_deta;
          JN[1] = -dz_dxi * dx_deta + dx_dxi * dz_deta;
          JN[2] = -dx_dxi * dy_deta + dy_dxi * dx_deta;
        } else if (eta == 1.0) {
          JN[0] = dy_dzeta * dz_dxi - dy_dxi * dz_dzeta;
          JN[1] = dz_dzeta * dx_dxi - dz_dxi * dx_dzeta;
          JN[2] = dx_dzeta * dy_dxi - dx_dxi * dy_dzeta;
        } else if (eta == -1.0) {
          JN[0] = -dy_dzeta * dz_dxi + dy_dxi * dz_dzeta;
          JN[1] = -dz_dzeta * dx_dxi + dz_dxi * dx_dzeta;
          JN[2] = -dx_dzeta * dy_dxi + dx_dxi * dy_dzeta;
        } else if (xi == 1.0) {
          JN[0] = dy_deta * dz_dzeta - dy_dzeta * dz_deta;
          JN[1] = dz_deta * dx_dzeta - dz_dzeta * dx_deta;
          JN[2] = dx_deta * dy_dzeta - dx_dzeta * dy_deta;
        } else if (xi == -1.0) {
          JN[0] = -dy_deta * dz_dzeta + dy_dzeta * dz_deta;
          JN[1] = -dz_deta * dx_dzeta + dz_dzeta * dx_deta;
          JN[2] = -dx_deta * dy_dzeta + dx_dzeta * dy_deta;
        }
      } else {
        if (xi == 0.0) {
          JN[0] = dz_deta * dy_dzeta - dy_deta * dz_dzeta;
          JN[1] = dx_deta * dz_dzeta - dz_deta * dx_dzeta;
          JN[2] = dy_deta * dx_dzeta - dx_deta * dy_dzeta;
        } else if (eta == 0.0) {
          JN[0] = dz_dzeta * dy_dxi - dy_dzeta * dz_dxi;
          JN[1] = dz_dxi * dx_dzeta - dx_dxi * dz_dzeta;
          JN[2] = dy_dzeta * dx_dxi - dx_dzeta * dy_dxi;
        } else if (zeta == 0.0) {
          JN[0] = dz_dxi * dy_deta - dy_dxi * dz_deta;
          JN[1] = dx_dxi * dz_deta - dx_deta * dz_dxi;
          JN[2] = dy_dxi * dx_deta - dx_dxi * dy_deta;
        } else {
          JN[0] = (dz_dzeta - dz_dxi) * (dy_deta - dy_dxi) - (dy_dzeta - dy_dxi) * (dz_deta - dz_dxi);
          JN[1] = (dx_dzeta - dx_dxi) * (dz_deta - dz_dxi) - (dx_deta - dx_dxi) * (dz_dzeta - dz_dxi);
          JN[2] = (dx_deta - dx_dxi) * (dy_dzeta - dy_dxi) - (dx_dzeta - dx_dxi) * (dy_deta - dy_dxi);
        }
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Per-quadrature-point record written by the point phase.  The record of point q of
// an element also carries the scatter descriptor of the element's node b = q (every
// element type here has as many interior points as nodes): the node, its CSR row
// length nd * (graph row length), its Dirichlet mask and, per trial node a, the unit
// offset u = node_rp(b) nd + slot(b, a), so that dof row jb of node b holds node a's
// columns from nd u + jb rowlen on.  The matrix stage then reads everything it needs
// from the record block.  Integers are stored as the bit patterns of S words.
template <int DIM, int NEN, int NC, typename S>
struct QP {
  using L = Layout<DIM, NC>;
  using Scalar = S;
  static constexpr int ND = L::ND;
  S sh[NEN], ds[DIM][NEN], JxW;
  S p, v[DIM], Y[NC], rho, E, drho_dp, drho_dT, de_dp, de_dT, mu, lambda, kappa;
  S drho_dY[L::NYA], dE_dY[L::NYA], rhoD[L::NYA], rhoDH[L::NYA];
  S tau[ND][ND];
  // structure vectors of DUDY = w r0^T + rho M and their products with tau:
  // w = (1, v, E, Y), z = r0^T tau, y = mE^T tau (mE: energy row of M), tg = g^T tau_v
  S w[ND], z[ND], y[ND], tg[ND];
  S nu;             // dc_scale_fact * nu_shoc (0 when dc is off or inactive)
  S rv[ND];         // coefficient of N_b:    (U - U_P)/dt - S
  S rf[DIM][ND];    // coefficient of dN_b/dx_k:  F_dif,k - F_adv,k + shock dI/dx_k
  S res[ND];        // least-squares residual Res (fluid_2d.hpp:282)
  S d_node, d_rowlen, d_blocked, d_off[NEN];  // scatter descriptor of node b = q (see above)
};

__device__ __forceinline__ float int_word(float, int32_t v) { return __int_as_float(v); }
__device__ __forceinline__ double int_word(double, int32_t v) { return __longlong_as_double((long long)v); }
__device__ __forceinline__ int32_t word_int(float w) { return __float_as_int(w); }
__device__ __forceinline__ int32_t word_int(double w) { return (int32_t)__double_as_longlong(w); }

// Lane layout of the matrix stage (see matrix_kernel); the point stage lays its
// records out in the matrix CTAs' blocks.
template <int DIM, int NEN, int NC>
struct MatShape {
  static constexpr int ND = Layout<DIM, NC>::ND;
  static constexpr int N = NEN * ND;                  // rows (and columns) of the block
  static constexpr int AG = NEN >= 8 ? 2 : 1;          // trial-node groups per row
  static constexpr int NA = NEN / AG;                  // trial nodes per lane
  static constexpr int LANES = N * AG;
  static constexpr int WPE = (LANES + 31) / 32;        // warps per element
  static constexpr int EPC = WPE == 1 ? 4 : (WPE == 2 ? 2 : 1);  // elements per CTA
  static constexpr int ET = WPE * 32;                  // threads per element
  static constexpr int CTA = EPC * ET;
  static constexpr int NS = N + 1;                     // stage row stride (doubles)
  static constexpr bool AFFINE = NEN == DIM + 1;
};

// Point records are stored in blocks of BP = (elements per matrix CTA) x NQ points, the
// points one matrix CTA group reads, word-major inside a block: word f of point p is at
// [f * BPS + p] with the odd stride BPS = BP + 1, so that the lanes of a matrix warp
// reading word f + i * nd of one point (the rows of tau) hit distinct banks.  A block
// is padded to a whole number of 16-byte units and is copied to shared memory as it
// lies (one bulk copy).  A warp of the point stage stores each word for its 32
// consecutive points as runs of BP contiguous words.
template <int DIM, int NEN, int NC, int NQ, typename S>
struct RecBlock {
  using QPT = QP<DIM, NEN, NC, S>;
  static constexpr int EPC = MatShape<DIM, NEN, NC>::EPC;
  static constexpr int BP = EPC * NQ;
  static constexpr int BPS = BP + 1;
  static constexpr int RW = (int)(sizeof(QPT) / sizeof(S));   // words per record
  static constexpr int V = (int)(16 / sizeof(S));
  static constexpr int WORDS = (RW * BPS + V - 1) / V * V;    // words per block
  static constexpr size_t BYTES = (size_t)WORDS * sizeof(S);
  static_assert(sizeof(QPT) % sizeof(S) == 0, "a record is a whole number of words");
};

// One point's words in a block being written (point stage) or read (matrix stage).
template <typename QPT, int BPS>
struct RecOut {
  using S = typename QPT::Scalar;
  S* __restrict__ blk;
  int p;
  __device__ __forceinline__ S& at(size_t off) const { return blk[(off / sizeof(S)) * BPS + p]; }
};
template <typename S, int BPS>
struct RecIn {
  const S* b;  // word 0 of the point
  __device__ __forceinline__ S operator[](int f) const { return b[f * BPS]; }
};
#define GALES_REC(m) out.at(offsetof(QPT, m))
#define GALES_RECA(m, i) out.at(offsetof(QPT, m) + (size_t)(i) * sizeof(S))
#define GALES_W(m) ((int)(offsetof(QPT, m) / sizeof(S)))

// Element geometry at the interior quadrature points, computed once at handle
// creation as the reference does at mesh load (mesh.hpp:468-495 builds a quad
// object per Gauss point): one record per element for simplices (affine map, the
// gradients, J and metrics are the same at every point), one per point otherwise.
template <int DIM, int NEN>
struct alignas(16) ElemGeo {
  double ds[DIM][NEN];
  double J;
  double G[DIM][DIM];
  double g[DIM];
  float ds_f[DIM][NEN];  // ds rounded to binary32 (narrow_rn), for the mixed form
};

template <int DIM, int NEN>
__host__ __device__ constexpr int geo_per_element(int nq) { return NEN == DIM + 1 ? 1 : nq; }

template <int DIM, int NEN, int NQ>
__global__ void __launch_bounds__(128) geometry_kernel(const double* __restrict__ coords,
                                                        const int32_t* __restrict__ conn, KParams k,
                                                        ElemGeo<DIM, NEN>* __restrict__ out, long long n_el) {
  constexpr int NG = geo_per_element<DIM, NEN>(NQ);
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long e = t / NG;
  const int iq = (int)(t % NG);
  if (e >= n_el) return;
  double X[NEN][DIM];
#pragma unroll
  for (int a = 0; a < NEN; ++a) {
    const int nd_ = conn[e * NEN + a];
#pragma unroll
    for (int d = 0; d < DIM; ++d) X[a][d] = coords[(long long)nd_ * DIM + d];
  }
  Geo<DIM, NEN> q;
  geometry<DIM, NEN>(X, k.gp[iq], true, q);
  ElemGeo<DIM, NEN>& o = out[e * NG + iq];
#pragma unroll
  for (int d = 0; d < DIM; ++d)
#pragma unroll
    for (int i = 0; i < NEN; ++i) {
      o.ds[d][i] = q.ds[d][i];
      o.ds_f[d][i] = narrow_rn(q.ds[d][i]);
    }
  o.J = q.J;
#pragma unroll
  for (int i = 0; i < DIM; ++i) {
    o.g[i] = q.g[i];
#pragma unroll
    for (int j = 0; j < DIM; ++j) o.G[i][j] = q.G[i][j];
  }
  if (!(q.J > 0.0)) flag_error(k, GALES_ERR_NEG_JACOBIAN, e);
}

// compute_h where its branches hang on rounding (rank-one velocity field): the point
// velocity and its gradient formed with the reference's operations (quad.hpp:817-885,
// unfused whatever the unit's contraction setting), then compute_h.  Rarely taken, so
// kept out of line.
template <int DIM, int NEN, int ND>
__device__ __noinline__ double compute_h_reference(const double* __restrict__ I, const int* nodes, const double* sh,
                                                   const ElemGeo<DIM, NEN>& q) {
  double ve[DIM], dve[DIM][DIM];
#pragma unroll
  for (int a = 0; a < DIM; ++a) {
    double x = 0.0;
#pragma unroll
    for (int i = 0; i < NEN; ++i) x = add_rn(x, mul_rn(sh[i], __ldg(I + (long long)nodes[i] * ND + 1 + a)));
    ve[a] = x;
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
      double b = 0.0;
#pragma unroll
      for (int i = 0; i < NEN; ++i) b = add_rn(b, mul_rn(q.ds[d][i], __ldg(I + (long long)nodes[i] * ND + 1 + a)));
      dve[a][d] = b;
    }
  }
  return compute_h<DIM>(q.G, ve, dve);
}

// Point phase for one (element, quadrature point).
//   GALES_FORM_FP64 : every step in FP64 with the reference's operations; tau uses
//                     the uBLAS-faithful LU inverse.
//   GALES_FORM_MIXED: FP64 for the mixture EOS and its derivatives, U - U_P, the
//                     element size h and tau with the closed-form DUDY inverse; the
//                     fluxes, least-squares residual and dc viscosity in FP32.
template <int DIM, int NEN, int NC, int NQ, int FORM, typename S, int BPS, int EOS = kEosChemicals>
__device__ void point_phase(const KParams& k, long long e, int iq, const RecOut<QP<DIM, NEN, NC, S>, BPS>& out) {
  using L = Layout<DIM, NC>;
  using QPT = QP<DIM, NEN, NC, S>;
  constexpr int ND = L::ND;
  constexpr int NG = geo_per_element<DIM, NEN>(NQ);
  using R = typename std::conditional<FORM == GALES_FORM_FP64, double, float>::type;
  static_assert(NQ == NEN, "point q carries the scatter descriptor of node q");
  int nodes[NEN];
#pragma unroll
  for (int a = 0; a < NEN; ++a) nodes[a] = __ldg(k.conn + e * NEN + a);
  {
    // scatter descriptor of node b = iq (see QP): its graph row, Dirichlet mask and the
    // positions of the element's nodes in that row (slot table)
    int nb = nodes[0];
#pragma unroll
    for (int a = 1; a < NEN; ++a) nb = (iq == a) ? nodes[a] : nb;
    const int64_t rr0 = __ldg(k.node_rp + nb), rr1 = __ldg(k.node_rp + nb + 1);
    const int fl = k.node_flag ? __ldg(k.node_flag + nb) : 0;
    const uint32_t blocked = (fl >= 0 && fl < GALES_MAX_FLAGS) ? k.dirichlet_mask[fl] : 0u;
    GALES_REC(d_node) = int_word(S(0), nb);
    GALES_REC(d_rowlen) = int_word(S(0), (int32_t)((rr1 - rr0) * ND));
    GALES_REC(d_blocked) = int_word(S(0), (int32_t)blocked);
    const uint16_t* sl = k.slot + ((long long)e * NEN + iq) * NEN;
#pragma unroll
    for (int a = 0; a < NEN; ++a) GALES_RECA(d_off, a) = int_word(S(0), (int32_t)(rr0 * ND + __ldg(sl + a)));
  }
  const ElemGeo<DIM, NEN>& q = reinterpret_cast<const ElemGeo<DIM, NEN>*>(k.geo)[e * NG + (NG == 1 ? 0 : iq)];
  double sh[NEN];
#pragma unroll
  for (int i = 0; i < NEN; ++i) sh[i] = k.sh_tab[iq][i];
  const double JxW = q.J * k.W_in;
  double Ie[NEN][ND], Pq[ND], Iq[ND];
#pragma unroll
  for (int i = 0; i < NEN; ++i)
#pragma unroll
    for (int j = 0; j < ND; ++j) Ie[i][j] = __ldg(k.I + (long long)nodes[i] * ND + j);
#pragma unroll
  for (int j = 0; j < ND; ++j) {
    Pq[j] = 0.0;
    Iq[j] = 0.0;
  }
#pragma unroll
  for (int i = 0; i < NEN; ++i) {
    const double* pi = k.P + (long long)nodes[i] * ND;
#pragma unroll
    for (int j = 0; j < ND; ++j) {
      if constexpr (FORM == GALES_FORM_FP64) {
        Pq[j] += sh[i] * __ldg(pi + j);
        Iq[j] += sh[i] * Ie[i][j];
      } else {
        // P and I are interpolated alike so that P == I gives U == U_P exactly
        Pq[j] = fma(sh[i], __ldg(pi + j), Pq[j]);
        Iq[j] = fma(sh[i], Ie[i][j], Iq[j]);
      }
    }
  }
  // (I - P)/dt at the point, in the form's type (the least-squares mass term)
  R dd[ND];
#pragma unroll
  for (int j = 0; j < ND; ++j) {
    if constexpr (FORM == GALES_FORM_FP64) dd[j] = (Iq[j] - Pq[j]) / k.dt;
    else dd[j] = narrow_rn(Iq[j] - Pq[j]) * k.inv_dt_f;
  }
  // gradients: FP64 in the FP64 form; FP32 of nodal differences in the mixed form
  // (sum_i dN_i/dx = 0, so sum_i dN_i (I_i - I_0) is the same gradient)
  R dI[DIM][ND];
  if constexpr (FORM == GALES_FORM_FP64) {
#pragma unroll
    for (int d = 0; d < DIM; ++d)
#pragma unroll
      for (int j = 0; j < ND; ++j) {
        double b = 0.0;
#pragma unroll
        for (int i = 0; i < NEN; ++i) b += q.ds[d][i] * Ie[i][j];
        dI[d][j] = b;
      }
  } else if constexpr (NEN == DIM + 1 && NQ >= 2 && NQ <= 32 && (32 % NQ) == 0) {
    // A simplex's gradient is the same at its NQ points, whose lanes are consecutive in
    // the warp: lane iq forms the columns j = iq, iq + NQ, ... of dI (its FP64 nodal
    // differences picked from its registers) and the lanes of the element exchange
    // them.  Same operations as the per-point form below.
    constexpr int NSL = (ND + NQ - 1) / NQ;
    const unsigned int lane = threadIdx.x & 31u;
    const unsigned int base = lane & ~(unsigned int)(NQ - 1);
    const unsigned int gmask = NQ == 32 ? 0xffffffffu : (((1u << NQ) - 1u) << base);
    float colv[NSL][DIM];
#pragma unroll
    for (int sl = 0; sl < NSL; ++sl) {
      const int jj = iq + NQ * sl;
      const int jc = jj < ND ? jj : ND - 1;
      float c[DIM];
#pragma unroll
      for (int d = 0; d < DIM; ++d) c[d] = 0.f;
#pragma unroll
      for (int i = 1; i < NEN; ++i) {
        double a = Ie[i][0], b0 = Ie[0][0];
#pragma unroll
        for (int j = 1; j < ND; ++j) {
          a = (jc == j) ? Ie[i][j] : a;
          b0 = (jc == j) ? Ie[0][j] : b0;
        }
        const float dif = narrow_rn(a - b0);
#pragma unroll
        for (int d = 0; d < DIM; ++d) c[d] = fmaf(q.ds_f[d][i], dif, c[d]);
      }
#pragma unroll
      for (int d = 0; d < DIM; ++d) colv[sl][d] = c[d];
    }
#pragma unroll
    for (int j = 0; j < ND; ++j)
#pragma unroll
      for (int d = 0; d < DIM; ++d) dI[d][j] = __shfl_sync(gmask, colv[j / NQ][d], (int)(base + j % NQ));
  } else {
#pragma unroll
    for (int d = 0; d < DIM; ++d)
#pragma unroll
      for (int j = 0; j < ND; ++j) dI[d][j] = 0.f;
#pragma unroll
    for (int i = 1; i < NEN; ++i)
#pragma unroll
      for (int j = 0; j < ND; ++j) {
        const float dif = narrow_rn(Ie[i][j] - Ie[0][j]);
#pragma unroll
        for (int d = 0; d < DIM; ++d) dI[d][j] = fmaf(q.ds_f[d][i], dif, dI[d][j]);
      }
  }
  // velocity gradient in FP64 (input of compute_h; fused in the mixed form, whose
  // compute_h falls back to the reference's operations where they matter)
  double dv[DIM][DIM];
  constexpr bool kShareDv = FORM == GALES_FORM_MIXED && NEN == DIM + 1 && NQ >= DIM && NQ <= 32 && (32 % NQ) == 0;
  if constexpr (kShareDv) {
    // A simplex's velocity gradient is the same at its NQ points, whose lanes are
    // consecutive in the warp (NQ divides 32): lane iq forms row a = min(iq, DIM - 1)
    // of dv (the element's shape gradients are the same in every lane; the lane picks
    // its velocity component from its registers) and the lanes of the element exchange
    // the rows.  Same operations as the per-point form below.
    const unsigned int lane = threadIdx.x & 31u;
    const unsigned int base = lane & ~(unsigned int)(NQ - 1);
    const unsigned int gmask = NQ == 32 ? 0xffffffffu : (((1u << NQ) - 1u) << base);
    const int am = iq < DIM ? iq : DIM - 1;
    double va[NEN];
#pragma unroll
    for (int i = 0; i < NEN; ++i) {
      double x = Ie[i][1];
#pragma unroll
      for (int a = 1; a < DIM; ++a) x = (am == a) ? Ie[i][1 + a] : x;
      va[i] = x;
    }
    double row[DIM];
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
      double b = q.ds[d][0] * va[0];
#pragma unroll
      for (int i = 1; i < NEN; ++i) b = fma(q.ds[d][i], va[i], b);
      row[d] = b;
    }
#pragma unroll
    for (int a = 0; a < DIM; ++a)
#pragma unroll
      for (int d = 0; d < DIM; ++d) dv[a][d] = __shfl_sync(gmask, row[d], (int)(base + (a < NQ ? a : NQ - 1)));
  } else {
#pragma unroll
    for (int a = 0; a < DIM; ++a)
#pragma unroll
      for (int d = 0; d < DIM; ++d) {
        if constexpr (FORM == GALES_FORM_FP64) {
          dv[a][d] = dI[d][1 + a];
        } else {
          double b = q.ds[d][0] * Ie[0][1 + a];
#pragma unroll
          for (int i = 1; i < NEN; ++i) b = fma(q.ds[d][i], Ie[i][1 + a], b);
          dv[a][d] = b;
        }
      }
  }
  // previous-level conservative vector U_P (props at P with shear rate 0) and the
  // current iterate's properties and U
  double p, v[DIM], T, Y[NC];
  double UP[ND], U[ND];
  Props<NC> pr;
  Coef<DIM, NC> c;
  double v_nrm, iv = 0.0;
  if constexpr (FORM == GALES_FORM_FP64) {
    assign<DIM, NC>(Pq, p, v, T, Y);
    if constexpr (EOS == kEosMagma) {
      // props at P with shear rate 0 (fluid_2d.hpp:186), at I with the point's shear
      // rate (fluid_2d.hpp:193-194)
      Props<NC> prP;
      unsigned st = magma_mixture<NC>(k.mg, p, T, Y, 0.0, prP);
      conservative<DIM, NC>(prP.rho, prP.cv, v, T, Y, UP);
      assign<DIM, NC>(Iq, p, v, T, Y);
      st |= magma_mixture<NC>(k.mg, p, T, Y, shear_rate<DIM>(dv), pr);
      if (st) flag_error(k, GALES_ERR_MAGMA, e);
    } else {
      double rhoP, cvP;
      mixture_rho_cv<NC>(k.ch, p, T, Y, rhoP, cvP);
      conservative<DIM, NC>(rhoP, cvP, v, T, Y, UP);
      assign<DIM, NC>(Iq, p, v, T, Y);
      mixture<NC>(k.ch, p, T, Y, pr);
    }
    make_coef<DIM, NC>(pr, p, v, T, Y, c);
    conservative<DIM, NC>(pr.rho, pr.cv, v, T, Y, U);
    v_nrm = sqrt(vsq<DIM>(v));
  } else {
    double pP, vP[DIM], TP, YP[NC];
    assign<DIM, NC>(Pq, pP, vP, TP, YP);
    assign<DIM, NC>(Iq, p, v, T, Y);
    double rhoP, cvP;
    if constexpr (EOS == kEosMagma) {
      Props<NC> prP;
      unsigned st = magma_mixture<NC>(k.mg, pP, TP, YP, 0.0, prP);
      st |= magma_mixture<NC>(k.mg, p, T, Y, shear_rate<DIM>(dv), pr);
      if (st) flag_error(k, GALES_ERR_MAGMA, e);
      rhoP = prP.rho;
      cvP = prP.cv;
      pr.irho = 1.0 / pr.rho;
#pragma unroll
      for (int i = 0; i < NC; ++i) pr.irho_c[i] = 1.0 / pr.rho_c[i];
    } else {
      mixture_pair_fast<NC>(k.ch, k.has_gas != 0, pP, TP, YP, p, T, Y, rhoP, cvP, pr);
    }
    conservative<DIM, NC>(rhoP, cvP, vP, TP, YP, UP);
    double vv = v[0] * v[0];
#pragma unroll
    for (int d = 1; d < DIM; ++d) vv = fma(v[d], v[d], vv);
    make_coef_fast<DIM, NC>(pr, p, v, vv, T, Y, c);
    U[0] = pr.rho;
#pragma unroll
    for (int d = 0; d < DIM; ++d) U[1 + d] = pr.rho * v[d];
    U[L::iT] = pr.rho * c.E;
#pragma unroll
    for (int i = 0; i < NC - 1; ++i) U[L::iY + i] = pr.rho * Y[i];
    iv = rsqrt(vv);
    v_nrm = vv > 0.0 ? vv * iv : 0.0;
  }
  const double dt = k.dt;
  // source S (gravity; fluid_2d.hpp:597-599) and the mass-term coefficient (U - U_P)/dt - S
  // the coefficients in the form's type R
  using CR = Coef<DIM, NC, R>;
  CR cr;
  if constexpr (FORM == GALES_FORM_FP64) cr = c;
  else cr = narrow<DIM, NC>(c);
  R SvR[ND];
#pragma unroll
  for (int r = 0; r < ND; ++r) SvR[r] = R(0);
  if constexpr (FORM == GALES_FORM_FP64) {
    double Sv[ND];
#pragma unroll
    for (int r = 0; r < ND; ++r) Sv[r] = 0.0;
    double gv = 0.0;
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
      Sv[1 + d] = pr.rho * k.gravity[d];
      gv += k.gravity[d] * v[d];
    }
    Sv[L::iT] = pr.rho * (gv);
#pragma unroll
    for (int j = 0; j < ND; ++j) {
      SvR[j] = Sv[j];
      GALES_RECA(rv, j) = (U[j] - UP[j]) / dt - Sv[j];
    }
  } else {
    const float rf = cr.rho;
    float gv = 0.f;
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
      const float gd = k.gravity_f[d];
      SvR[1 + d] = rf * gd;
      gv = fmaf(gd, cr.v[d], gv);
    }
    SvR[L::iT] = rf * gv;
    const float idt = k.inv_dt_f;
#pragma unroll
    for (int j = 0; j < ND; ++j) GALES_RECA(rv, j) = fmaf(narrow_rn(U[j] - UP[j]), idt, -SvR[j]);
  }
  R Ur[ND];  // U in the form's type (discontinuity capturing); U[0] = rho
#pragma unroll
  for (int j = 0; j < ND; ++j) Ur[j] = j == 0 ? cr.rho : to_s<R>(U[j]);
  // tau (fluid_2d.hpp:877-1022).  The branches give its diagonal parameters td; the FP64
  // form then forms DUDY^{-1} diag(td) by LU, the mixed form in closed form, narrowed to
  // FP32 entry by entry and only where it can be nonzero (tau_nz).
  R tau[ND][ND];
#pragma unroll
  for (int r = 0; r < ND; ++r)
#pragma unroll
    for (int cc = 0; cc < ND; ++cc) tau[r][cc] = R(0);
  if (v_nrm >= kEps && k.tau != GALES_TAU_NONE) {
    double h, idet = 0.0;
    bool have_idet = false;
    double trG = 0.0;
#pragma unroll
    for (int d = 0; d < DIM; ++d) trG += q.G[d][d];
    if constexpr (FORM == GALES_FORM_FP64) {
      h = compute_h<DIM>(q.G, v, dv);
    } else {
      bool decided;
      h = compute_h_fast<DIM>(q.G, trG, v, iv, dv, decided);
      if (!decided) h = compute_h_reference<DIM, NEN, ND>(k.I, nodes, sh, q);
    }
    const double cs = pr.c, rho = pr.rho, mu = pr.mu, cv = pr.cv, kappa = pr.kappa;
    double td[ND];
#pragma unroll
    for (int i = 0; i < ND; ++i) td[i] = 0.0;
    bool nondiag = false;
    if (k.tau == GALES_TAU_NON_DIAG_COMP_2001) {
      double lambda_sqr = 0.0 * (v_nrm * v_nrm + cs * cs) + (0.0) * 0.5 * cs * cs;
      lambda_sqr += 0.5 * cs * sqrt(cs * cs * 0.0 * 0.0 + 16 * 0.0 * 0.0 * v_nrm * v_nrm);
      if (!k.steady) lambda_sqr += 4 / (dt * dt);
      const double lam = 1.0 / sqrt(lambda_sqr) + h / (2 * v_nrm);
      const double use = k.steady ? lam : fmin(dt * 0.5, lam);
      td[0] = use;
#pragma unroll
      for (int d = 0; d < DIM; ++d) td[1 + d] = fmin(use, rho * h * h / (mu * 12));
      td[L::iT] = fmin(use, rho * h * h * cv / (kappa * 12));
#pragma unroll
      for (int i = 0; i < NC - 1; ++i) td[L::iY + i] = fmin(use, h * h / (pr.D_c[i] * 12));
      nondiag = true;
    } else if (FORM == GALES_FORM_MIXED && k.tau == GALES_TAU_NON_DIAG_COMP_2019) {
      // the same parameters with one division for 1/(|v|(|v|+c)), 1/(mu kappa) and
      // tau_closed's 1/det (mixed form): r = 1/(a b d) gives 1/a = b d r, ...
      const double a = v_nrm * (v_nrm + cs), bmk = mu * kappa, det = tau_det<DIM, NC>(c);
      const double ab = a * bmk, rr = 1.0 / (ab * det);
      const double ia = bmk * det * rr, imk = a * det * rr;
      idet = ab * rr;
      have_idet = true;
      const double hv = (0.5 * h) * fma(2.0, v_nrm, cs) * ia;
      const double use = k.steady ? hv : fmin(dt * 0.5, hv);
      const double hh12 = h * h * (1.0 / 12.0);
      td[0] = use;
      const double tm = fmin(use, hh12 * rho * kappa * imk);
#pragma unroll
      for (int d = 0; d < DIM; ++d) td[1 + d] = tm;
      td[L::iT] = fmin(use, hh12 * rho * cv * mu * imk);
#pragma unroll
      for (int i = 0; i < NC - 1; ++i)
        td[L::iY + i] = fmin(use, hh12 * (EOS == kEosMagma ? 1.0 / pr.D_c[i] : k.ch[i].inv_D));
      nondiag = true;
    } else if (k.tau == GALES_TAU_NON_DIAG_COMP_2019) {
      double use;
      if (k.steady) use = h / (2.0 * (v_nrm + cs)) + h / (2.0 * v_nrm);
      else use = fmin(dt * 0.5, h / (2.0 * (v_nrm + cs)) + h / (2.0 * v_nrm));
      td[0] = use;
      const double tm = fmin(use, h * h * rho / (12.0 * mu));
#pragma unroll
      for (int d = 0; d < DIM; ++d) td[1 + d] = tm;
      td[L::iT] = fmin(use, h * h * rho * cv / (12.0 * kappa));
#pragma unroll
      for (int i = 0; i < NC - 1; ++i) td[L::iY + i] = fmin(use, h * h / (12.0 * pr.D_c[i]));
      nondiag = true;
    } else if (k.tau == GALES_TAU_DIAG_INCOMP_2007) {
      double use = 0.0;
#pragma unroll
      for (int i = 0; i < DIM; ++i)
#pragma unroll
        for (int j = 0; j < DIM; ++j) use += q.G[i][j] * q.G[i][j];
      double vGv = 0.0;
#pragma unroll
      for (int i = 0; i < DIM; ++i) {
        double s = 0.0;
#pragma unroll
        for (int j = 0; j < DIM; ++j) s += q.G[i][j] * v[j];
        vGv += v[i] * s;
      }
      const double nu = mu / rho;
      double tau_m = vGv + 9.0 * use * (nu * nu);
      if (!k.steady) tau_m += 4.0 / (dt * dt);
      tau_m = 1.0 / sqrt(tau_m);
      double gg = 0.0;
#pragma unroll
      for (int i = 0; i < DIM; ++i) gg += q.g[i] * q.g[i];
      const double tau_c = 1.0 / (rho * tau_m * gg);
      const double de = kappa / (rho * cv);
      double tau_e = vGv + 9.0 * use * (de * de);
      if (!k.steady) tau_e += 4.0 / (dt * dt);
      tau_e = 1.0 / sqrt(tau_e);
      td[0] = tau_c;
#pragma unroll
      for (int d = 0; d < DIM; ++d) td[1 + d] = tau_m / rho;
      td[L::iT] = tau_e / (rho * cv);
#pragma unroll
      for (int i = 0; i < NC - 1; ++i) td[L::iY + i] = tau_m;
    } else if (k.tau == GALES_TAU_DIAG_2014) {
#pragma unroll
      for (int i = 0; i < ND; ++i) {
        const double a0 = dudy_entry<DIM, NC, double>(c, i, i);
        const double tt = 4.0 / (dt * dt) * (a0 * a0);
        double ta = 0.0, tk = 0.0;
#pragma unroll
        for (int kk = 0; kk < DIM; ++kk)
#pragma unroll
          for (int ll = 0; ll < DIM; ++ll) {
            const double ak = a_entry<DIM, NC, double>(c, kk, i, i);
            const double al = a_entry<DIM, NC, double>(c, ll, i, i);
            const double kv = k_entry<DIM, NC, double>(c, kk, ll, i, i);
            ta += q.G[kk][ll] * (ak * al);
            tk += q.G[kk][ll] * q.G[kk][ll] * (kv * kv);
          }
        td[i] = 1.0 / (sqrt(tt) + sqrt(ta) + sqrt(tk) + 1.e-8);
      }
      td[0] = 1.0 / (td[0] + rho * td[1] * (trG));
    }
    if (!nondiag) {
#pragma unroll
      for (int i = 0; i < ND; ++i) tau[i][i] = to_s<R>(td[i]);
    } else if constexpr (FORM == GALES_FORM_FP64) {
      double A0[ND][ND], Xinv[ND][ND];
#pragma unroll
      for (int r = 0; r < ND; ++r)
#pragma unroll
        for (int cc = 0; cc < ND; ++cc) A0[r][cc] = dudy_entry<DIM, NC, double>(c, r, cc);
      if (lu_inverse<ND>(A0, Xinv)) flag_error(k, GALES_ERR_SINGULAR, e);
#pragma unroll
      for (int r = 0; r < ND; ++r)
#pragma unroll
        for (int cc = 0; cc < ND; ++cc) tau[r][cc] = Xinv[r][cc] * td[cc];
      if (v_nrm / cs < 0.1) {
        tau[0][0] = 1.0 / (1.0 / tau[0][0] + 1.0 / (rho * tau[1][1] * (trG)));
#pragma unroll
        for (int cc = 1; cc < ND; ++cc) tau[0][cc] = 0.0;
      }
    } else {
      tau_closed<DIM, NC, R>(c, pr.irho, have_idet ? idet : 1.0 / tau_det<DIM, NC>(c), td,
                             v_nrm < 0.1 * cs, rho * trG, tau);
    }
  }
  {
    // z = r0^T tau, y = mE^T tau, tg = sum_d g_d tau[v_d] from the rounded tau (what the
    // matrix stage multiplies with), and w
    R zz[ND], yy[ND], gg[ND], gR[DIM];
#pragma unroll
    for (int d = 0; d < DIM; ++d) gR[d] = FORM == GALES_FORM_FP64 ? R(k.gravity[d]) : R(k.gravity_f[d]);
#pragma unroll
    for (int cc = 0; cc < ND; ++cc) zz[cc] = yy[cc] = gg[cc] = R(0);
#pragma unroll
    for (int r = 0; r < ND; ++r) {
      R r0r, mEr, gr;
      if (r == 0) { r0r = cr.drho_dp; mEr = cr.de_dp; gr = R(0); }
      else if (r < L::iT) { r0r = R(0); mEr = cr.v[r - 1]; gr = gR[(r - 1) % DIM]; }
      else if (r == L::iT) { r0r = cr.drho_dT; mEr = cr.de_dT; gr = R(0); }
      else { r0r = cr.drho_dY[r - L::iY]; mEr = cr.dE_dY[r - L::iY]; gr = R(0); }
#pragma unroll
      for (int cc = 0; cc < ND; ++cc) {
        if (FORM == GALES_FORM_MIXED && !tau_nz<DIM, NC>(r, cc)) {
          GALES_RECA(tau, (r) * ND + (cc)) = S(0);
          continue;
        }
        const R t = tau[r][cc];
        GALES_RECA(tau, (r) * ND + (cc)) = S(t);
        if (r < 1 || r >= L::iT) zz[cc] = madd(r0r, t, zz[cc]);
        yy[cc] = madd(mEr, t, yy[cc]);
        if (r >= 1 && r < L::iT) gg[cc] = madd(gr, t, gg[cc]);
      }
    }
#pragma unroll
    for (int cc = 0; cc < ND; ++cc) {
      GALES_RECA(z, cc) = S(zz[cc]);
      GALES_RECA(y, cc) = S(yy[cc]);
      GALES_RECA(tg, cc) = S(gg[cc]);
      GALES_RECA(w, cc) = S(cc == 0 ? R(1) : (cc < L::iT ? cr.v[cc - 1] : (cc == L::iT ? cr.E : cr.Y[cc - L::iY])));
    }
  }
  // fluxes, least-squares residual and dc in the form's type R
  R Res[ND], AdI[ND], t[ND];
  {
    dudy_mv<DIM, NC, R>(cr, dd, Res);
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
      a_mv<DIM, NC, R>(cr, d, dI[d], t);
#pragma unroll
      for (int j = 0; j < ND; ++j) {
        Res[j] = Res[j] + t[j];
        AdI[j] = (d == 0) ? t[j] : AdI[j] + t[j];
      }
    }
#pragma unroll
    for (int j = 0; j < ND; ++j) Res[j] = Res[j] - SvR[j];
  }
  // discontinuity capturing (fluid_2d.hpp:1027-1065)
  R nu = R(0);
  R dU[DIM][ND];
#pragma unroll
  for (int d = 0; d < DIM; ++d) dudy_mv<DIM, NC, R>(cr, dI[d], dU[d]);
  if (k.dc_2006) {
    R s = R(0);
#pragma unroll
    for (int d = 0; d < DIM; ++d) s += dU[d][0] * dU[d][0];
    const R del_rho_nrm = sqrt(s);
    if (!(del_rho_nrm < R(kEps))) {
      R Jv[DIM];
#pragma unroll
      for (int d = 0; d < DIM; ++d) Jv[d] = dU[d][0] / del_rho_nrm;
      R h = R(0);
#pragma unroll
      for (int i = 0; i < NEN; ++i) {
        R tt = Jv[0] * to_s<R>(q.ds[0][i]);
#pragma unroll
        for (int d = 1; d < DIM; ++d) tt = tt + Jv[d] * to_s<R>(q.ds[d][i]);
        h += fabs(tt);
      }
      if (h > R(kEps)) {
        h = R(1) / h;
        R Zn = R(0), Un = R(0), use1 = R(0);
#pragma unroll
        for (int j = 0; j < ND; ++j) {
          const R ui = FORM == GALES_FORM_FP64 ? R(k.u_ref_inv[j]) : R(k.u_ref_inv_f[j]);
          const R z = ui * (AdI[j] - SvR[j]);
          const R u = ui * Ur[j];
          Zn += z * z;
          Un += u * u;
        }
        Zn = sqrt(Zn);
        Un = sqrt(Un);
        const double a = k.dc_sharp;
        if (a == 1.0 || a == 1.5) {
#pragma unroll
          for (int d = 0; d < DIM; ++d) {
            R n2 = R(0);
#pragma unroll
            for (int j = 0; j < ND; ++j) {
              const R u = (FORM == GALES_FORM_FP64 ? R(k.u_ref_inv[j]) : R(k.u_ref_inv_f[j])) * dU[d][j];
              n2 += u * u;
            }
            const R n = sqrt(n2);
            use1 += n * n;
          }
        }
        if (a == 1.0) nu = Zn * h * (R(1) / sqrt(use1));
        else if (a == 2.0) nu = Zn * h * h / Un;
        else if (a == 1.5) nu = Zn * h * ((R(1) / sqrt(use1)) + h / Un) / R(2);
        nu = (FORM == GALES_FORM_FP64 ? R(k.dc_scale) : R(k.dc_scale_f)) * nu;
      }
    }
  }
  // F_dif - F_adv + shock dI (fluid_2d.hpp:253-262, 311-318)
  const R rhoR = cr.rho, pR = cr.p, ER = cr.E;
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    R fd[ND];
#pragma unroll
    for (int j = 0; j < ND; ++j) fd[j] = R(0);
#pragma unroll
    for (int l = 0; l < DIM; ++l) {
      k_mv<DIM, NC, R>(cr, d, l, dI[l], t);
#pragma unroll
      for (int j = 0; j < ND; ++j) fd[j] = (l == 0) ? t[j] : fd[j] + t[j];
    }
    const R vk = cr.v[d];
    R fa[ND];
    fa[0] = rhoR * vk;
#pragma unroll
    for (int j = 0; j < DIM; ++j) fa[1 + j] = (j == d) ? rhoR * vk * vk + pR : rhoR * vk * cr.v[j];
    fa[L::iT] = vk * (rhoR * ER + pR);
#pragma unroll
    for (int i = 0; i < NC - 1; ++i) fa[L::iY + i] = rhoR * vk * cr.Y[i];
#pragma unroll
    for (int j = 0; j < ND; ++j) GALES_RECA(rf, (d) * ND + (j)) = S(fd[j] - fa[j] + nu * dU[d][j]);
  }
  // write the record (the mixed form takes the coefficients already rounded in cr and
  // the shape data rounded once per mesh)
  if constexpr (FORM == GALES_FORM_MIXED) {
#pragma unroll
    for (int i = 0; i < NEN; ++i) {
      GALES_RECA(sh, i) = S(k.sh_tab_f[iq][i]);
#pragma unroll
      for (int d = 0; d < DIM; ++d) GALES_RECA(ds, (d) * NEN + (i)) = S(q.ds_f[d][i]);
    }
  } else {
#pragma unroll
    for (int i = 0; i < NEN; ++i) {
      GALES_RECA(sh, i) = to_s<S>(sh[i]);
#pragma unroll
      for (int d = 0; d < DIM; ++d) GALES_RECA(ds, (d) * NEN + (i)) = to_s<S>(q.ds[d][i]);
    }
  }
  GALES_REC(JxW) = to_s<S>(JxW);
  GALES_REC(p) = S(cr.p);
#pragma unroll
  for (int d = 0; d < DIM; ++d) GALES_RECA(v, d) = S(cr.v[d]);
#pragma unroll
  for (int i = 0; i < NC; ++i) GALES_RECA(Y, i) = S(cr.Y[i]);
  GALES_REC(rho) = S(cr.rho); GALES_REC(E) = S(cr.E);
  GALES_REC(drho_dp) = S(cr.drho_dp); GALES_REC(drho_dT) = S(cr.drho_dT);
  GALES_REC(de_dp) = S(cr.de_dp); GALES_REC(de_dT) = S(cr.de_dT);
  GALES_REC(mu) = S(cr.mu); GALES_REC(lambda) = S(cr.lambda); GALES_REC(kappa) = S(cr.kappa);
#pragma unroll
  for (int i = 0; i < L::NYA; ++i) {
    GALES_RECA(drho_dY, i) = S(cr.drho_dY[i]); GALES_RECA(dE_dY, i) = S(cr.dE_dY[i]);
    GALES_RECA(rhoD, i) = S(cr.rhoD[i]); GALES_RECA(rhoDH, i) = S(cr.rhoDH[i]);
  }
  GALES_REC(nu) = S(nu);
#pragma unroll
  for (int j = 0; j < ND; ++j) GALES_RECA(res, j) = S(Res[j]);
  if (!finite_bits(JxW) || !finite_bits(pr.rho) || !isfinite(nu)) flag_error(k, GALES_ERR_NONFINITE, e);
}

// Viscous/diffusive tangent contracted with the test-function gradient gb:
// sum_k gb_k K_kl(r, col), in closed form from the entries of K_kl
// (fluid_2d.hpp:531-571): K_kl(1+j, v_m) = mu d_lk d_mj + mu d_lj d_mk + lambda d_kj d_lm,
// K_kl(E, v_m) = sum_j v_j K_kl(1+j, v_m), K_kk(E, T) = kappa, K_kk(E, Y_i) = rho D_i H_i,
// K_kk(Y_i, Y_i) = rho D_i.  gbv = gb . v.
template <int DIM, int NC, typename S, typename C>
__device__ __forceinline__ S kd_entry(const C& c, const S* gb, S gbv, int l, int r, int col) {
  using L = Layout<DIM, NC>;
  if (r == 0 || col == 0) return S(0);
  if (r < L::iT) {
    if (col >= L::iT) return S(0);
    const int j = r - 1, m = col - 1;
    S x = S(0);
    if (m == j) x += c.mu * gb[l];
    if (l == j) x += c.mu * gb[m];
    if (l == m) x += c.lambda * gb[j];
    return x;
  }
  if (r == L::iT) {
    if (col < L::iT) {
      const int m = col - 1;
      S x = c.mu * (gb[l] * c.v[m] + c.v[l] * gb[m]);
      if (l == m) x += c.lambda * gbv;
      return x;
    }
    if (col == L::iT) return c.kappa * gb[l];
    return c.rhoDH[col - L::iY] * gb[l];
  }
  return (col == r) ? c.rhoD[r - L::iY] * gb[l] : S(0);
}

// Exact widening of binary32 to binary64 with 32-bit integer operations only (see
// narrow_rn): exponent rebias 127 -> 1023, the 23-bit significand split over the two
// words; subnormals normalised, infinities and NaN keep their payload.
__device__ __forceinline__ double widen_special(float f);
__device__ __forceinline__ double widen(float f) {
  // normal numbers and zeros: the exponent field shifted into place and rebiased by
  // (1023 - 127) << 20, the significand split over the two words
  const unsigned int u = __float_as_uint(f);
  const unsigned int a = u & 0x7fffffffu;
  if (a - 0x00800000u < 0x7f000000u || a == 0u) {
    const unsigned int hi = (a == 0u ? 0u : (a >> 3) + 0x38000000u) | (u & 0x80000000u);
    return __hiloint2double((int)hi, (int)(u << 29));
  }
  return widen_special(f);
}
// subnormals, infinities and NaN
__device__ __forceinline__ double widen_special(float f) {
  const unsigned int u = __float_as_uint(f);
  const unsigned int sign = u & 0x80000000u;
  const unsigned int ex = (u >> 23) & 0xffu;
  unsigned int m = u & 0x7fffffu, e64;
  if (ex - 1u < 254u) {
    e64 = ex + (1023u - 127u);
  } else if (ex == 0xffu) {
    e64 = 0x7ffu;
  } else if (m == 0u) {
    return __hiloint2double((int)sign, 0);
  } else {
    // subnormal m * 2^-149: leading one at bit p = 31 - clz(m)
    const int p = 31 - __clz((int)m);
    e64 = (unsigned int)(p - 149 + 1023);
    m = (m << (23 - p)) & 0x7fffffu;
  }
  return __hiloint2double((int)(sign | (e64 << 20) | (m >> 3)), (int)(m << 29));
}
__device__ __forceinline__ double widen(double d) { return d; }

// ---------------------------------------------------------------------------
// Interior pass, stage 1: one thread per (element, quadrature point) writes the
// point record of that point to a chunk buffer (L2-resident).  The mixed form is
// held to 128 registers (4 CTAs per SM): more warps hide the FP64 latency better
// than the spilled values cost.
template <int DIM, int NEN, int NC, int NQ, int FORM, typename S, int EOS = kEosChemicals>
__device__ __forceinline__ void point_block(const KParams& k, QP<DIM, NEN, NC, S>* __restrict__ out, long long first,
                                            long long n, int bid) {
  // chunk-local indices fit 32 bits (the host keeps a chunk's points below 2^31); 64-bit
  // divisions would issue on the FP64 pipe.  CTAs of 128 threads.
  const int t = bid * 128 + (int)threadIdx.x;
  const int li = t / NQ;
  const int iq = t - li * NQ;
  if (li >= n) return;
  const long long g = first + li;
  const long long e = k.el_list ? (long long)k.el_list[g] : g;
  using QPT = QP<DIM, NEN, NC, S>;
  using RB = RecBlock<DIM, NEN, NC, NQ, S>;
  const int blk = t / RB::BP;
  const RecOut<QPT, RB::BPS> o{reinterpret_cast<S*>(out) + (size_t)blk * (size_t)RB::WORDS, t - blk * RB::BP};
  point_phase<DIM, NEN, NC, NQ, FORM, S, RB::BPS, EOS>(k, e, iq, o);
}

// Resident point-stage CTAs the register budget is set for: 4 for the mixed form with
// the chemicals' EOS, 2 with the (out-of-line, register-hungry) magma EOS, 1 for FP64.
template <int FORM, int EOS>
constexpr int point_min_ctas() {
  return FORM == GALES_FORM_MIXED ? (EOS == kEosMagma ? 2 : 4) : 1;
}

// Zeroes k.clear_p[a][0 .. k.clear_n[a]) with every thread of the launch (grid-stride;
// 16-byte stores on the 16-byte-aligned body, scalar stores for an unaligned head and
// an odd tail).  A thread issues its stores after its point, so that they drain while
// the CTAs of later waves compute.
__device__ __forceinline__ void clear_arrays(const KParams& k) {
  const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long stride = (long long)gridDim.x * blockDim.x;
#pragma unroll 1
  for (int a = 0; a < 2; ++a) {
    double* p = k.clear_p[a];
    const long long n = k.clear_n[a];
    if (n <= 0) continue;
    const long long head = (reinterpret_cast<uintptr_t>(p) & 15u) != 0 ? 1 : 0;
    const long long body = n - head;
    if (tid == 0 && head) p[0] = 0.0;
    if (tid == 0 && (body & 1)) p[n - 1] = 0.0;
    double2* q = reinterpret_cast<double2*>(p + head);
#pragma unroll 1
    for (long long i = tid; i < body / 2; i += stride) q[i] = make_double2(0.0, 0.0);
  }
}

template <int DIM, int NEN, int NC, int NQ, int FORM, typename S, int EOS = kEosChemicals>
__global__ void __launch_bounds__(128, point_min_ctas<FORM, EOS>()) point_kernel(const KParams k, QP<DIM, NEN, NC, S>* __restrict__ out,
                                                     long long first, long long n) {
  point_block<DIM, NEN, NC, NQ, FORM, S, EOS>(k, out, first, n, (int)blockIdx.x);
  if (k.clear_n[0] > 0 || k.clear_n[1] > 0) clear_arrays(k);
}

// Interior pass, stage 2: element matrices.  Lane (b, r, g) owns row (b, r) of the
// element block (test node b, dof r) for the trial nodes of group g, and builds it
// per quadrature point (fluid_2d.hpp:264-331) from
//   JxW [ FPT_b RM_a + N_a X_b ]   with
//   WA_b  = sum_k dN_b/dx_k A_k
//   FPT_b = (WA_b - N_b S0) tau                       least-squares weight
//   RM_a  = N_a DUDY/dt + WA_a - N_a S0               least-squares operator
//   X_b   = N_b (DUDY/dt - S0) - WA_b                 Galerkin mass, source, advection
// plus the viscous/diffusive and dc terms sum_kl dN_b/dx_k K'_kl dN_a/dx_l with
// K'_kl = K_kl + nu d_kl DUDY.
// None of the nd x nd matrices is formed.  DUDY = w r0^T + rho M (w = (1, v, E, Y),
// r0 its first row, M zero but for the velocity and mass-fraction diagonal and the
// energy row mE), A_k = v_k DUDY + u' e_{v_k}^T + (e_{v_k} + v_k e_E) e_p^T with
// u' = U + p e_E, and S0 = e_E sigma^T with sigma = rho g on the velocity columns
// (fluid_2d.hpp:407-575).  With s_b = dN_b/dx . v these give, row r of the lane,
//   FPT_b[r]   = s_b (w_r z + rho Mtau[r]) + u'_r t_b + kappa_br tau[0] - N_b [r=E] rho t_g
//   (FPT_b RM_a)[r] = alpha_a (FPT_b DUDY)[r] + (FPT_b[r].u') gamma_a
//                     + (FPT_b[r].kappa_a) e_p - N_a FPT_b[r][E] sigma
//   X_b[r]     = beta_b DUDY[r] - u'_r gamma_b - kappa_br e_p - N_b [r=E] sigma
// where z = r0^T tau, Mtau = M tau, t_b = sum_k dN_b/dx_k tau[v_k], t_g = sum_k g_k
// tau[v_k], gamma_a = dN_a/dx on the velocity columns, kappa_a = dN_a/dx on the
// velocity rows + s_a e_E, alpha_a = N_a/dt + s_a, beta_b = N_b/dt - s_b.  K'_kl is
// applied in closed form from a few point scalars (mu, lambda, mu v, lambda v, kappa,
// rho D_i, rho D_i H_i) and nu DUDY: per point for non-affine elements, once from
// JxW-weighted sums for simplices (their shape gradients do not depend on the point).

// Per-point vectors t_b = sum_k dN_b/dx_k tau[v_k] shared by the lanes of an element
// (w, z, y and t_g come with the point record).
template <int DIM, int NEN, int NC, int NQ, typename S>
struct PointVecs {
  static constexpr int ND = Layout<DIM, NC>::ND;
  S tb[NQ][NEN][ND];
};

// Shared memory of one element slot of a matrix CTA: the per-point vectors t_b, the
// element block staged for the scatter (in the form's type; widened to FP64 as it is
// scattered), and the per-warp partial traces.
template <int DIM, int NEN, int NC, int NQ, typename S>
struct ElemSmem {
  using M = MatShape<DIM, NEN, NC>;
  PointVecs<DIM, NEN, NC, NQ, S> pv;
  S stage[M::N * M::NS];
  double wsum[M::WPE];
};

// Shared memory of a matrix CTA: two record blocks (the group being assembled and the
// next one, in flight), the element slots and the two transaction barriers of the
// blocks.  Offsets in bytes; every part 16-byte aligned.
template <int DIM, int NEN, int NC, int NQ, typename S>
struct MatSmem {
  using RB = RecBlock<DIM, NEN, NC, NQ, S>;
  using ES = ElemSmem<DIM, NEN, NC, NQ, S>;
  static constexpr size_t ES_BYTES = (sizeof(ES) + 15) / 16 * 16;
  static constexpr size_t OFF_ES = 2 * RB::BYTES;
  static constexpr size_t OFF_BAR = OFF_ES + (size_t)MatShape<DIM, NEN, NC>::EPC * ES_BYTES;
  static constexpr size_t BYTES = OFF_BAR + 16;
};

template <int WPE>
__device__ __forceinline__ void elem_sync(int el_in_cta) {
  if constexpr (WPE == 1) {
    __syncwarp();
  } else {
    asm volatile("bar.sync %0, %1;" ::"r"(el_in_cta + 1), "r"(WPE * 32) : "memory");
  }
}

// Point scalars entering K'_kl (JxW-weighted, summed over the points of a simplex).
template <int DIM, int NC, typename S>
struct KSums {
  using L = Layout<DIM, NC>;
  S mu, lambda, kappa, muv[DIM], lamv[DIM], rhoD[L::NYA], rhoDH[L::NYA];
};

// Adds sum_kl gb_k K_kl(r, :) ga_l to row r of one (b, a) block (the closed form of
// the contraction; fluid_2d.hpp:531-571), branch-free in r:
//   velocity row v_j: mu gb_m ga_j + lambda gb_j ga_m + mu (gb.ga) d_mj  on column v_m
//   energy row      : mu v_m (gb.ga) + gb_m (ga.mu v) + ga_m (gb.lambda v) on v_m,
//                     kappa (gb.ga) on T, rho D_i H_i (gb.ga) on Y_i
//   mass-fraction row Y_i: rho D_i (gb.ga) on Y_i.
template <int DIM, int NC, typename S>
__device__ __forceinline__ void add_viscous_row(S (&acc)[Layout<DIM, NC>::ND], int r, const KSums<DIM, NC, S>& ks,
                                                const S* gb, const S* ga) {
  using L = Layout<DIM, NC>;
  const bool cV = r >= 1 && r < L::iT, cE = r == L::iT;
  S gg = gb[0] * ga[0], gamv = ga[0] * ks.muv[0], gblv = gb[0] * ks.lamv[0];
  S gbj = S(0), gaj = S(0);
#pragma unroll
  for (int d = 1; d < DIM; ++d) {
    gg = madd(gb[d], ga[d], gg);
    gamv = madd(ga[d], ks.muv[d], gamv);
    gblv = madd(gb[d], ks.lamv[d], gblv);
  }
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    gbj = (r == 1 + d) ? gb[d] : gbj;
    gaj = (r == 1 + d) ? ga[d] : gaj;
  }
  const S p1 = cV ? ks.mu * gaj : (cE ? gamv : S(0));
  const S p2 = cV ? ks.lambda * gbj : (cE ? gblv : S(0));
  const S p3 = cV ? ks.mu * gg : S(0);
#pragma unroll
  for (int m = 0; m < DIM; ++m) {
    S x = madd(gb[m], p1, ga[m] * p2);
    if (cE) x = madd(ks.muv[m], gg, x);
    if (r == 1 + m) x += p3;
    acc[1 + m] += x;
  }
  acc[L::iT] = madd(cE ? ks.kappa : S(0), gg, acc[L::iT]);
#pragma unroll
  for (int y = 0; y < NC - 1; ++y) {
    const S q = cE ? ks.rhoDH[y] : ((r == L::iY + y) ? ks.rhoD[y] : S(0));
    acc[L::iY + y] = madd(q, gg, acc[L::iY + y]);
  }
}

// Element stage of one group of EPC elements (list positions first + li, li = grp EPC
// + ec) from their record block blk in shared memory; the lanes of slot ec build its
// rows.  Elements past n are skipped.
template <int DIM, int NEN, int NC, int NQ, typename S, bool WANT_M>
__device__ __forceinline__ void matrix_group(const KParams& k, const S* __restrict__ blk,
                                             ElemSmem<DIM, NEN, NC, NQ, S>& E, long long first, long long n,
                                             long long grp) {
  using L = Layout<DIM, NC>;
  using M = MatShape<DIM, NEN, NC>;
  using QPT = QP<DIM, NEN, NC, S>;
  using RB = RecBlock<DIM, NEN, NC, NQ, S>;
  constexpr int ND = M::ND, N = M::N, NA = M::NA, NT = N * N, WPE = M::WPE, ET = M::ET, NS = M::NS;
  constexpr int BPS = RB::BPS;
  constexpr int iT = L::iT, iY = L::iY;
  constexpr bool AFF = M::AFFINE;
  const int tid = threadIdx.x;
  const int ec = tid / ET;      // element slot in the CTA
  const int gl = tid % ET;      // thread index within the element
  const long long li = grp * M::EPC + ec;
  if (li >= n) return;          // whole element groups skip together
  const long long g = first + li;
  const S* el = blk + ec * NQ;  // word f of point q of this element: el[f * BPS + q]
  auto rec = [&](int q) { return RecIn<S, BPS>{el + q}; };
  // scatter descriptor words of node b (carried by point b)
  auto d_int = [&](int b, int f) { return word_int(el[f * BPS + b]); };
  S grav[DIM];
#pragma unroll
  for (int d = 0; d < DIM; ++d) grav[d] = S(k.gravity[d]);
  auto& pv = E.pv;
  // t_b per point
  for (int t = gl; t < NQ * NEN * ND; t += ET) {
    const int q = t / (NEN * ND), u = t % (NEN * ND), b = u / ND, col = u % ND;
    const RecIn<S, BPS> c = rec(q);
    S x = c[GALES_W(ds) + b] * c[GALES_W(tau) + ND + col];
#pragma unroll
    for (int d = 1; d < DIM; ++d) x = madd(c[GALES_W(ds) + d * NEN + b], c[GALES_W(tau) + (1 + d) * ND + col], x);
    pv.tb[q][b][col] = x;
  }
  elem_sync<WPE>(ec);
  const bool active = gl < M::LANES;
  const int row = active ? gl % N : 0;
  const int grp_a = active ? gl / N : 0;
  const int b = row / ND, r = row % ND;
  const int a0 = grp_a * NA;
  const bool cV = r >= 1 && r < iT, cE = r == iT, cvy = r >= 1 && r != iT;
  S acc[NA][ND];
#pragma unroll
  for (int i = 0; i < NA; ++i)
#pragma unroll
    for (int j = 0; j < ND; ++j) acc[i][j] = S(0);
  S racc = S(0);
  S Dnu[ND];
  KSums<DIM, NC, S> ksum;
  if constexpr (AFF) {
#pragma unroll
    for (int j = 0; j < ND; ++j) Dnu[j] = S(0);
    ksum.mu = ksum.lambda = ksum.kappa = S(0);
#pragma unroll
    for (int d = 0; d < DIM; ++d) ksum.muv[d] = ksum.lamv[d] = S(0);
#pragma unroll
    for (int y = 0; y < L::NYA; ++y) ksum.rhoD[y] = ksum.rhoDH[y] = S(0);
  }
  const S idt = S(k.inv_dt);
  const int mrow_f = cvy ? GALES_W(tau) + r * ND : GALES_W(y);
  for (int q = 0; q < NQ; ++q) {
    const RecIn<S, BPS> c = rec(q);
    const S rho = c[GALES_W(rho)], p = c[GALES_W(p)], jx = c[GALES_W(JxW)];
    S gb[DIM], vq[DIM];
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
      gb[d] = c[GALES_W(ds) + d * NEN + b];
      vq[d] = c[GALES_W(v) + d];
    }
    const S Nb = c[GALES_W(sh) + b];
    S sb = gb[0] * vq[0];
#pragma unroll
    for (int d = 1; d < DIM; ++d) sb = madd(gb[d], vq[d], sb);
    const S wr = c[GALES_W(w) + r];
    const S ur = madd(rho, wr, cE ? p : S(0));
    S gsel = S(0);
#pragma unroll
    for (int d = 0; d < DIM; ++d) gsel = (r == 1 + d) ? gb[d] : gsel;
    const S kap = (cE ? sb : S(0)) + gsel;
    // row r of FPT_b
    const S cz = sb * wr, cm = (r == 0) ? S(0) : sb * rho, cg = cE ? -Nb * rho : S(0);
    const S* tb = &pv.tb[q][b][0];
    S F[ND];
#pragma unroll
    for (int j = 0; j < ND; ++j) {
      S x = cz * c[GALES_W(z) + j];
      x = madd(cm, c[mrow_f + j], x);
      x = madd(ur, tb[j], x);
      x = madd(kap, c[GALES_W(tau) + j], x);
      F[j] = madd(cg, c[GALES_W(tg) + j], x);
    }
    // residual row: N_b rv + sum_k dN_b/dx_k rf_k + FPT_b Res (fluid_2d.hpp:253-262, 280-290)
    {
      S x = Nb * c[GALES_W(rv) + r];
#pragma unroll
      for (int d = 0; d < DIM; ++d) x = madd(gb[d], c[GALES_W(rf) + d * ND + r], x);
#pragma unroll
      for (int j = 0; j < ND; ++j) x = madd(F[j], c[GALES_W(res) + j], x);
      racc = madd(jx, x, racc);
    }
    if constexpr (WANT_M) {
      // FPT_b DUDY, DUDY row r, and the a-independent velocity-column terms
      S fw = F[0];
#pragma unroll
      for (int j = 1; j < ND; ++j) fw = madd(F[j], c[GALES_W(w) + j], fw);
      const S fu = madd(rho, fw, p * F[iT]);
      const S rF = rho * F[iT];
      S FD[ND], Dr[ND];
#pragma unroll
      for (int j = 0; j < ND; ++j) {
        S r0j, mEj;
        if (j == 0) { r0j = c[GALES_W(drho_dp)]; mEj = c[GALES_W(de_dp)]; }
        else if (j < iT) { r0j = S(0); mEj = vq[j - 1]; }
        else if (j == iT) { r0j = c[GALES_W(drho_dT)]; mEj = c[GALES_W(de_dT)]; }
        else { r0j = c[GALES_W(drho_dY) + j - iY]; mEj = c[GALES_W(dE_dY) + j - iY]; }
        S x = madd(rF, mEj, (j >= 1 && j != iT) ? rho * F[j] : S(0));
        FD[j] = (j >= 1 && j < iT) ? x : madd(fw, r0j, x);
        S dd = madd(cE ? rho : S(0), mEj, (cvy && r == j) ? rho : S(0));
        Dr[j] = (j >= 1 && j < iT) ? dd : madd(wr, r0j, dd);
      }
      S hv[DIM];
      const S fe = rho * (F[iT] + (cE ? Nb : S(0)));
#pragma unroll
      for (int d = 0; d < DIM; ++d) hv[d] = -madd(ur, gb[d], fe * grav[d]);
      const S beta = madd(Nb, idt, -sb);
      KSums<DIM, NC, S> ks;
      S nu_j = S(0);
      if constexpr (!AFF) {
        ks.mu = jx * c[GALES_W(mu)]; ks.lambda = jx * c[GALES_W(lambda)]; ks.kappa = jx * c[GALES_W(kappa)];
#pragma unroll
        for (int d = 0; d < DIM; ++d) { ks.muv[d] = ks.mu * vq[d]; ks.lamv[d] = ks.lambda * vq[d]; }
#pragma unroll
        for (int y = 0; y < L::NYA; ++y) {
          ks.rhoD[y] = jx * c[GALES_W(rhoD) + y];
          ks.rhoDH[y] = jx * c[GALES_W(rhoDH) + y];
        }
        nu_j = jx * c[GALES_W(nu)];
      }
#pragma unroll
      for (int ai = 0; ai < NA; ++ai) {
        const int a = a0 + ai;
        S ga[DIM];
#pragma unroll
        for (int d = 0; d < DIM; ++d) ga[d] = c[GALES_W(ds) + d * NEN + a];
        const S Na = c[GALES_W(sh) + a];
        S sa = ga[0] * vq[0];
#pragma unroll
        for (int d = 1; d < DIM; ++d) sa = madd(ga[d], vq[d], sa);
        S fk = sa * F[iT];
#pragma unroll
        for (int d = 0; d < DIM; ++d) fk = madd(ga[d], F[1 + d], fk);
        const S A1 = jx * madd(Na, idt, sa), A4 = jx * Na, A2 = A4 * beta, A3 = jx * fu;
        acc[ai][0] = madd(A1, FD[0], madd(A2, Dr[0], madd(jx, madd(-Na, kap, fk), acc[ai][0])));
#pragma unroll
        for (int d = 0; d < DIM; ++d)
          acc[ai][1 + d] = madd(A1, FD[1 + d], madd(A2, Dr[1 + d], madd(A3, ga[d], madd(A4, hv[d], acc[ai][1 + d]))));
#pragma unroll
        for (int j = iT; j < ND; ++j) acc[ai][j] = madd(A1, FD[j], madd(A2, Dr[j], acc[ai][j]));
        if constexpr (!AFF) {
          add_viscous_row<DIM, NC, S>(acc[ai], r, ks, gb, ga);
          S gg = gb[0] * ga[0];
#pragma unroll
          for (int d = 1; d < DIM; ++d) gg = madd(gb[d], ga[d], gg);
          const S gn = gg * nu_j;
#pragma unroll
          for (int j = 0; j < ND; ++j) acc[ai][j] = madd(gn, Dr[j], acc[ai][j]);
        }
      }
      if constexpr (AFF) {
        const S mu = c[GALES_W(mu)], lam = c[GALES_W(lambda)];
        const S jn = jx * c[GALES_W(nu)];
#pragma unroll
        for (int j = 0; j < ND; ++j) Dnu[j] = madd(jn, Dr[j], Dnu[j]);
        ksum.mu = madd(jx, mu, ksum.mu);
        ksum.lambda = madd(jx, lam, ksum.lambda);
        ksum.kappa = madd(jx, c[GALES_W(kappa)], ksum.kappa);
#pragma unroll
        for (int d = 0; d < DIM; ++d) {
          ksum.muv[d] = madd(jx * mu, vq[d], ksum.muv[d]);
          ksum.lamv[d] = madd(jx * lam, vq[d], ksum.lamv[d]);
        }
#pragma unroll
        for (int y = 0; y < L::NYA; ++y) {
          ksum.rhoD[y] = madd(jx, c[GALES_W(rhoD) + y], ksum.rhoD[y]);
          ksum.rhoDH[y] = madd(jx, c[GALES_W(rhoDH) + y], ksum.rhoDH[y]);
        }
      }
    }
  }
  if constexpr (WANT_M && AFF) {
    // viscous/diffusive and dc terms of a simplex, from the point sums
    const RecIn<S, BPS> c = rec(0);
    S gb[DIM];
#pragma unroll
    for (int d = 0; d < DIM; ++d) gb[d] = c[GALES_W(ds) + d * NEN + b];
#pragma unroll
    for (int ai = 0; ai < NA; ++ai) {
      S ga[DIM];
#pragma unroll
      for (int d = 0; d < DIM; ++d) ga[d] = c[GALES_W(ds) + d * NEN + a0 + ai];
      add_viscous_row<DIM, NC, S>(acc[ai], r, ksum, gb, ga);
      S gg = gb[0] * ga[0];
#pragma unroll
      for (int d = 1; d < DIM; ++d) gg = madd(gb[d], ga[d], gg);
#pragma unroll
      for (int j = 0; j < ND; ++j) acc[ai][j] = madd(gg, Dnu[j], acc[ai][j]);
    }
  }
  // Dirichlet rows (scatter.hpp:62-78) and scatter (scatter.hpp:96-97)
  const bool local = k.local_r != nullptr;
  const bool blk_row = !local && (((uint32_t)d_int(b, GALES_W(d_blocked)) >> r) & 1u);
  double avg = 0.0;
  if constexpr (WANT_M) {
    // avg_val = (1 + trace)/n (scatter.hpp:65-68), only where the element has a blocked
    // row (the same for every lane of the element)
    uint32_t any_blocked = 0u;
#pragma unroll
    for (int i = 0; i < NEN; ++i) any_blocked |= (uint32_t)d_int(i, GALES_W(d_blocked));
    const bool need_avg = !local && any_blocked != 0u;
    double tr = 0.0;
    if (need_avg) {
      S dg = S(0);
#pragma unroll
      for (int ai = 0; ai < NA; ++ai)
#pragma unroll
        for (int j = 0; j < ND; ++j) dg = (a0 + ai == b && j == r) ? acc[ai][j] : dg;
      tr = active ? widen(dg) : 0.0;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) tr += __shfl_xor_sync(0xffffffffu, tr, o);
      if constexpr (WPE > 1) {
        if ((gl & 31) == 0) E.wsum[gl >> 5] = tr;
      }
    }
    elem_sync<WPE>(ec);
    if (need_avg) {
      if constexpr (WPE > 1) {
        tr = E.wsum[0];
#pragma unroll
        for (int w = 1; w < WPE; ++w) tr += E.wsum[w];
      }
      avg = (1.0 + tr) * (1.0 / N);
    }
    if (active) {
      S* srow = E.stage + row * NS + a0 * ND;
#pragma unroll
      for (int ai = 0; ai < NA; ++ai)
#pragma unroll
        for (int j = 0; j < ND; ++j) srow[ai * ND + j] = acc[ai][j];
    }
    elem_sync<WPE>(ec);
  }
  // staged entry (row rw, column cx) as scattered: a blocked row (Dirichlet) is avg on
  // the diagonal and zero elsewhere (scatter.hpp:62-78)
  auto staged = [&](int rw, int cx) -> double {
    const int bn = rw / ND, jr = rw - bn * ND;
    if (!local && ((((uint32_t)d_int(bn, GALES_W(d_blocked))) >> jr) & 1u)) return rw == cx ? avg : 0.0;
    return widen(E.stage[rw * NS + cx]);
  };
  if (WANT_M && k.vjp_lam) {
    // frozen-tangent VJP: g += K^T lambda for this element's block (Dirichlet rows included)
    for (int cx = gl; cx < N; cx += ET) {
      double sum = 0.0;
      for (int rw = 0; rw < N; ++rw)
        sum += __ldg(k.vjp_lam + (long long)d_int(rw / ND, GALES_W(d_node)) * ND + rw % ND) * staged(rw, cx);
      if (sum != 0.0) atomicAdd(k.vjp_g + (long long)d_int(cx / ND, GALES_W(d_node)) * ND + cx % ND, sum);
    }
    return;
  }
  if (local) {  // element-level output of execute_i (fluid_2d.hpp:200-201): m = m_, r = -r_
    if (active && grp_a == 0) k.local_r[g * N + row] = widen(-racc);
    if (WANT_M && k.local_m)
      for (int t = gl; t < NT; t += ET) k.local_m[g * NT + t] = widen(E.stage[(t / N) * NS + t % N]);
    return;
  }
  const int mode = k.scatter_mode;
  if (active && grp_a == 0 && !blk_row)
    add_to(k.rhs + (long long)d_int(b, GALES_W(d_node)) * ND + r, widen(-racc), mode);
  if constexpr (WANT_M) {
    // One block row per warp step: lane l covers columns l, l+32, ... of the row; node
    // sb_'s dof row jb holds node a's columns from nd off(sb_, a) + jb rowlen on, so
    // consecutive lanes write the contiguous nd-runs.
    constexpr int CH = (N + 31) / 32;   // column passes per row
    const int lane = gl & 31, warp = gl >> 5;
#pragma unroll
    for (int h = 0; h < CH; ++h) {
      const int cx = lane + 32 * h;
      if (cx >= N) break;
      const int a = cx / ND, ja = cx - a * ND;
      for (int sb_ = 0; sb_ < NEN; ++sb_) {
        const int64_t rl = d_int(sb_, GALES_W(d_rowlen));
        const uint32_t bl = (uint32_t)d_int(sb_, GALES_W(d_blocked));
        double* rowp = k.vals + (int64_t)d_int(sb_, GALES_W(d_off) + a) * ND + (int64_t)warp * rl + ja;
        const int64_t step = (int64_t)WPE * rl;
        for (int jb = warp; jb < ND; jb += WPE, rowp += step) {
          if ((bl >> jb) & 1u) {  // blocked row: avg on its diagonal only
            if (cx == sb_ * ND + jb) add_to(rowp, avg, mode);
            continue;
          }
          const double val = widen(E.stage[(sb_ * ND + jb) * NS + cx]);
          if ((__double2hiint(val) & 0x7fffffff) | __double2loint(val)) add_to(rowp, val, mode);
        }
      }
    }
  }
}

// Bulk copies of record blocks into shared memory with transaction barriers
// (cp.async.bulk and mbarrier, sm_90+).  Every wait is bounded.
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0u;
}
// Bounded wait on phase `parity` of a transaction barrier: false after kMbarTries
// polls (each poll may suspend the thread for a while), far beyond any bulk copy.
constexpr long long kMbarTries = 1ll << 24;
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  for (long long i = 0; i < kMbarTries; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

// Interior pass, stage 2 (persistent): CTA c assembles the element groups c, c + grid,
// ... of the n listed elements whose records start at `in`.  One thread issues the bulk
// copy of the next group's record block into the second buffer before the CTA works
// on the current one, so the copy overlaps the element arithmetic.  A barrier wait
// that runs out (it cannot on a working device) sets GALES_ERR_TIMEOUT, waits (again
// bounded) for the other buffer's copy and ends the CTA.
template <int DIM, int NEN, int NC, int NQ, typename S, bool WANT_M>
__global__ void __launch_bounds__(MatShape<DIM, NEN, NC>::CTA)
    matrix_kernel(const KParams k, const S* __restrict__ in, long long first, long long n) {
  using RB = RecBlock<DIM, NEN, NC, NQ, S>;
  using SM = MatSmem<DIM, NEN, NC, NQ, S>;
  using ES = ElemSmem<DIM, NEN, NC, NQ, S>;
  constexpr int EPC = MatShape<DIM, NEN, NC>::EPC, ET = MatShape<DIM, NEN, NC>::ET;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  S* buf[2] = {reinterpret_cast<S*>(smem_raw), reinterpret_cast<S*>(smem_raw + RB::BYTES)};
  ES& E = *reinterpret_cast<ES*>(smem_raw + SM::OFF_ES + (size_t)(threadIdx.x / ET) * SM::ES_BYTES);
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem_raw + SM::OFF_BAR);
  const long long ngroups = (n + EPC - 1) / EPC;
  if (threadIdx.x == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    mbar_fence_init();
  }
  __syncthreads();
  long long grp = blockIdx.x;
  if (threadIdx.x == 0 && grp < ngroups) bulk_load(buf[0], in + grp * RB::WORDS, (uint32_t)RB::BYTES, &bar[0]);
  for (int it = 0; grp < ngroups; ++it, grp += gridDim.x) {
    const int cur = it & 1;
    const long long nxt = grp + gridDim.x;
    if (threadIdx.x == 0 && nxt < ngroups)
      bulk_load(buf[cur ^ 1], in + nxt * RB::WORDS, (uint32_t)RB::BYTES, &bar[cur ^ 1]);
    const bool ok = mbar_wait(&bar[cur], (uint32_t)((it >> 1) & 1));
    if (__syncthreads_or(!ok)) {
      if (threadIdx.x == 0) {
        flag_error(k, GALES_ERR_TIMEOUT, first + grp * EPC);
        if (nxt < ngroups) mbar_wait(&bar[cur ^ 1], (uint32_t)(((it + 1) >> 1) & 1));
      }
      return;
    }
    matrix_group<DIM, NEN, NC, NQ, S, WANT_M>(k, buf[cur], E, first, n, grp);
    __syncthreads();  // the buffer and the element slots are free again
  }
}

// ---------------------------------------------------------------------------
// Adaptive time step of the multicomponent solver, adaptive_time_criteria::f_mc
// (adaptive_time_step.hpp:183-260): one thread per element, FP64 with the reference's
// operations in order (this is instantiated in the FP64 units, without contraction).
// At each Gauss point: interpolate I and its gradient, the mixture at shear rate 0,
// |v| (uBLAS norm_2); 1.2 dt where |v| < DBL_EPSILON, else with h = compute_h(v, dv)
// (compute_del_v, 356-374) and v_tau = |v| (or, for Mach > 0.3,
// sqrt(|v|^2 + 1.5 c^2 + c sqrt(16|v|^2 + c^2)) in 2D, sqrt(|v|^2 + 2 c^2 +
// c sqrt(4|v|^2 + c^2)) in 3D), use = 2 max(2 mu/rho, kappa/(rho cv))/h^2 + v_tau/h and
// CFL/use.  dt_el[e] = the first smallest of the element's values (min_element).
template <int DIM, int NEN, int NC, int NQ, int EOS = kEosChemicals>
__global__ void __launch_bounds__(128) adaptive_dt_kernel(const KParams k, double cfl, double* __restrict__ dt_el,
                                                          long long n) {
  using L = Layout<DIM, NC>;
  constexpr int ND = L::ND;
  constexpr int NG = geo_per_element<DIM, NEN>(NQ);
  const long long e = (long long)blockIdx.x * 128 + threadIdx.x;
  if (e >= n) return;
  int nodes[NEN];
#pragma unroll
  for (int a = 0; a < NEN; ++a) nodes[a] = __ldg(k.conn + e * NEN + a);
  double Ie[NEN][ND];
#pragma unroll
  for (int i = 0; i < NEN; ++i)
#pragma unroll
    for (int j = 0; j < ND; ++j) Ie[i][j] = __ldg(k.I + (long long)nodes[i] * ND + j);
  double best = 0.0;
  for (int iq = 0; iq < NQ; ++iq) {
    const ElemGeo<DIM, NEN>& q = reinterpret_cast<const ElemGeo<DIM, NEN>*>(k.geo)[e * NG + (NG == 1 ? 0 : iq)];
    double Iq[ND], dI[DIM][ND];
#pragma unroll
    for (int j = 0; j < ND; ++j) {
      double a = 0.0;
#pragma unroll
      for (int i = 0; i < NEN; ++i) a += k.sh_tab[iq][i] * Ie[i][j];
      Iq[j] = a;
#pragma unroll
      for (int d = 0; d < DIM; ++d) {
        double b = 0.0;
#pragma unroll
        for (int i = 0; i < NEN; ++i) b += q.ds[d][i] * Ie[i][j];
        dI[d][j] = b;
      }
    }
    double p, v[DIM], T, Y[NC];
    assign<DIM, NC>(Iq, p, v, T, Y);
    Props<NC> pr;
    if constexpr (EOS == kEosMagma) {  // shear rate 0 (adaptive_time_step.hpp:197, 226)
      if (magma_mixture<NC>(k.mg, p, T, Y, 0.0, pr)) flag_error(k, GALES_ERR_MAGMA, e);
    } else {
      mixture<NC>(k.ch, p, T, Y, pr);
    }
    const double v_nrm = sqrt(vsq<DIM>(v));
    double dtg;
    if (v_nrm < kEps) {
      dtg = 1.2 * k.dt;
    } else {
      double dv[DIM][DIM];
#pragma unroll
      for (int a = 0; a < DIM; ++a)
#pragma unroll
        for (int d = 0; d < DIM; ++d) dv[a][d] = dI[d][1 + a];
      const double h = compute_h<DIM>(q.G, v, dv);
      const double c = pr.c;
      double v_tau = v_nrm;
      const double mach = v_nrm / c;
      if (mach > 0.3) {
        if (DIM == 2) v_tau = sqrt(v_nrm * v_nrm + 1.5 * c * c + c * sqrt(16.0 * v_nrm * v_nrm + c * c));
        else v_tau = sqrt(v_nrm * v_nrm + 2.0 * c * c + c * sqrt(4.0 * v_nrm * v_nrm + c * c));
      }
      const double m1 = 2.0 * pr.mu / pr.rho, m2 = pr.kappa / (pr.rho * pr.cv);
      const double mx = (m1 < m2) ? m2 : m1;  // std::max
      const double use = 2.0 * mx / (h * h) + v_tau / h;
      dtg = cfl / use;
    }
    if (iq == 0 || dtg < best) best = dtg;
  }
  dt_el[e] = best;
}

// Secondary variables at the nodes, secondary_dofs::execute (secondary_dofs.hpp:56-101):
// the mixture properties of every node's state at shear rate 0, written word-major:
// out[f * n + node] for f = rho, mu, cp, cv, alpha, beta, kappa, sound speed (the
// order of 146-153).  FP64 with the reference's operations (FP64 units).
template <int DIM, int NC, int EOS = kEosChemicals>
__global__ void __launch_bounds__(128) secondary_dofs_kernel(const KParams k, double* __restrict__ out, long long n) {
  using L = Layout<DIM, NC>;
  const long long i = (long long)blockIdx.x * 128 + threadIdx.x;
  if (i >= n) return;
  double w[L::ND];
#pragma unroll
  for (int j = 0; j < L::ND; ++j) w[j] = __ldg(k.I + i * L::ND + j);
  double p, v[DIM], T, Y[NC];
  assign<DIM, NC>(w, p, v, T, Y);
  Props<NC> pr;
  if constexpr (EOS == kEosMagma) {  // shear rate 0 (secondary_dofs.hpp:85)
    if (magma_mixture<NC>(k.mg, p, T, Y, 0.0, pr)) flag_error(k, GALES_ERR_MAGMA, i);
  } else {
    mixture<NC>(k.ch, p, T, Y, pr);
  }
  const double f[8] = {pr.rho, pr.mu, pr.cp, pr.cv, pr.alpha, pr.beta, pr.kappa, pr.c};
#pragma unroll
  for (int q = 0; q < 8; ++q) out[q * n + i] = f[q];
}

// The magma gas fractions of secondary_dofs::execute (pp_vf_g, secondary_dofs.hpp:
// 113-131) at every node, shear rate 0, written word-major: out[f * n + node] for
// f = vf_g_comp_c, vf_comp_c (c = 0..NC-1, interleaved), then vf_g_on_total,
// vf_h2o_g_on_total, vf_co2_g_on_total, wf_g_on_total, wf_h2o_g_on_total,
// wf_co2_g_on_total.  FP64 with the reference's operations (magma units).
template <int DIM, int NC>
__global__ void __launch_bounds__(128) magma_fractions_kernel(const KParams k, double* __restrict__ out, long long n) {
  using L = Layout<DIM, NC>;
  const long long i = (long long)blockIdx.x * 128 + threadIdx.x;
  if (i >= n) return;
  double w[L::ND];
#pragma unroll
  for (int j = 0; j < L::ND; ++j) w[j] = __ldg(k.I + i * L::ND + j);
  double p, v[DIM], T, Y[NC];
  assign<DIM, NC>(w, p, v, T, Y);
  double f[2 * NC + 6];
  if (magma_mix::mix_fractions(k.mg, NC, p, T, Y, f)) flag_error(k, GALES_ERR_MAGMA, i);
#pragma unroll
  for (int q = 0; q < 2 * NC + 6; ++q) out[q * n + i] = f[q];
}

// ---------------------------------------------------------------------------
// Boundary pass helpers (fluid_2d.hpp:610-868): boundary-modified A_k and K_kl.

// Entry of the boundary-modified K_kl (fluid_2d.hpp:819-867).
template <int DIM>
__device__ __forceinline__ int energy_source(int a, int l, int m) {
  if (l == a && m == a) return a;
  if (l == a) return m;
  if (m == a) return l;
  if (m == l) return a;
  return -1;
}

template <int DIM, int NC, typename T>
__device__ __forceinline__ T k_entry_bd(const Coef<DIM, NC, T>& c, const gales_side_bc& bc, int k,
                                             int l, int r, int col) {
  using L = Layout<DIM, NC>;
  T x = k_entry<DIM, NC, T>(c, k, l, r, col);
  if (x == T(0)) return x;
  auto tau_set = [&](int i, int j) {
    const int lo = i < j ? i : j, hi = i < j ? j : i;
    return (bc.tau_mask >> (lo * 3 + hi)) & 1u;
  };
  if (r >= 1 && r < L::iT && col >= 1 && col < L::iT) {
    if (tau_set(k, r - 1)) return T(0);
  }
  if (r == L::iT && col >= 1 && col < L::iT) {
    const int j = energy_source<DIM>(k, l, col - 1);
    if (j >= 0 && tau_set(k, j)) return T(0);
  }
  if (k == l && r == L::iT && col == L::iT && ((bc.q_mask >> k) & 1u)) return T(0);
  if (k == l && col >= L::iY) {
    const int i = col - L::iY;
    if (((bc.J_mask >> (k * 8 + i)) & 1u) && (r == col || r == L::iT)) return T(0);
  }
  return x;
}

template <int DIM, int NC, typename T>
__device__ __forceinline__ T a_entry_bd(const Coef<DIM, NC, T>& c, const gales_side_bc& bc, int k, int r, int col) {
  using L = Layout<DIM, NC>;
  if (!((bc.mass_flux_mask >> k) & 1u)) return a_entry<DIM, NC, T>(c, k, r, col);
  const T mf = T(bc.mass_flux[k]);
  if (r == 1 + k && col == 0) return T(1);
  if (r >= 1 && r < L::iT && col == r) return mf;
  if (r == L::iT) {
    if (col == 0) return c.v[k] + mf * c.de_dp;
    if (col < L::iT) return (col - 1 == k) ? c.p + mf * c.v[k] : mf * c.v[col - 1];
    if (col == L::iT) return mf * c.de_dT;
    return mf * c.dE_dY[col - L::iY];
  }
  if (r >= L::iY && col == r) return mf;
  return T(0);
}

// BA and BK of one boundary point from its narrowed coefficients and area vector,
// every entry at a compile-time (row, column), so that the entry functions fold to
// their closed forms; one thread per point (the boundary point stage).  dst_* may be
// global or shared memory.
template <int DIM, int NC, typename S>
__device__ __forceinline__ void bpoint_blocks(const Coef<DIM, NC, S>& c, const S* JNxW, const gales_side_bc& bc,
                                              S (*BA)[Layout<DIM, NC>::ND], S (*BK)[Layout<DIM, NC>::ND][Layout<DIM, NC>::ND]) {
  constexpr int ND = Layout<DIM, NC>::ND;
#pragma unroll
  for (int r = 0; r < ND; ++r)
#pragma unroll
    for (int col = 0; col < ND; ++col) {
      S x = S(0);
#pragma unroll
      for (int d = 0; d < DIM; ++d) x = madd(a_entry_bd<DIM, NC, S>(c, bc, d, r, col), JNxW[d], x);
      BA[r][col] = x;
    }
#pragma unroll
  for (int l = 0; l < DIM; ++l)
#pragma unroll
    for (int r = 0; r < ND; ++r)
#pragma unroll
      for (int col = 0; col < ND; ++col) {
        S x = S(0);
#pragma unroll
        for (int d = 0; d < DIM; ++d) x = madd(k_entry_bd<DIM, NC, S>(c, bc, d, l, r, col), JNxW[d], x);
        BK[l][r][col] = x;
      }
}

// Per boundary point data (one side quadrature point): the state coefficients, the
// area vector, shape data and the boundary residual vector
//   rb = sum_k (F_adv,k - F_dif,k) JNxW_k                       (fluid_2d.hpp:343-349)
template <int DIM, int NEN, int NC, typename S>
struct alignas(16) BPoint {
  using L = Layout<DIM, NC>;
  static constexpr int ND = L::ND;
  Coef<DIM, NC, S> c;
  S sh[NEN], ds[DIM][NEN], JNxW[DIM];
  double shr[NEN], rb[ND];
  int flag;
};

// A boundary point's record: its data and its two matrices
//   BA = sum_k A'_k JNxW_k,  BK_l = sum_k K'_kl JNxW_k
// (A' and K' with the side's prescribed fluxes, fluid_2d.hpp:610-817), in S.
template <int DIM, int NEN, int NC, typename S>
struct alignas(16) BPointRec {
  static constexpr int ND = Layout<DIM, NC>::ND;
  BPoint<DIM, NEN, NC, S> pt;
  S BA[ND][ND];
  S BK[DIM][ND][ND];
};

template <int DIM, int NEN, int NC, int NS, int NSQ, typename S>
struct BoundarySmem {
  static constexpr int ND = Layout<DIM, NC>::ND, N = NEN * ND;
  static constexpr int MS = N + 1;   // row stride of m: rows and columns bank-conflict free
  BPointRec<DIM, NEN, NC, S> pt[NS * NSQ];
  S m[N * MS];           // element block accumulator
  double r[N];
  double wsum;
  int64_t rowbase[NEN];
  int32_t rowlen[NEN];
  uint32_t blocked[NEN];
  uint16_t slot[NEN][NEN];
};

// Boundary point physics (fluid_2d.hpp:341-349, 610-817) at one side point with
// the given geometry (shape values, gradients, JN W_bd): the coefficients, shape data
// and the boundary residual rb = sum_k (F_adv,k - F_dif,k) JNxW_k, in FP64.
template <int DIM, int NEN, int NC, typename S, int EOS = kEosChemicals>
__device__ __forceinline__ void bpoint_phase(const KParams& k, const int* nodes, int flag, const double* sh,
                                             const double (&ds)[DIM][NEN], const double* JNxW,
                                             BPoint<DIM, NEN, NC, S>& P, long long e) {
  using L = Layout<DIM, NC>;
  constexpr int ND = L::ND;
  const gales_side_bc& bc = k.side_bc[flag < GALES_MAX_FLAGS ? flag : 0];
  P.flag = flag;
  double Ie[NEN][ND];
#pragma unroll
  for (int a = 0; a < NEN; ++a)
#pragma unroll
    for (int j = 0; j < ND; ++j) Ie[a][j] = __ldg(k.I + (long long)nodes[a] * ND + j);
#pragma unroll
  for (int d = 0; d < DIM; ++d) P.JNxW[d] = to_s<S>(JNxW[d]);
#pragma unroll
  for (int i = 0; i < NEN; ++i) {
    P.sh[i] = to_s<S>(sh[i]);
    P.shr[i] = sh[i];
#pragma unroll
    for (int d = 0; d < DIM; ++d) P.ds[d][i] = to_s<S>(ds[d][i]);
  }
  double Iq[ND], dI[DIM][ND];
#pragma unroll
  for (int j = 0; j < ND; ++j) {
    double a = 0.0;
#pragma unroll
    for (int i = 0; i < NEN; ++i) a += sh[i] * Ie[i][j];
    Iq[j] = a;
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
      double b = 0.0;
#pragma unroll
      for (int i = 0; i < NEN; ++i) b += ds[d][i] * Ie[i][j];
      dI[d][j] = b;
    }
  }
  double p, v[DIM], T, Y[NC];
  assign<DIM, NC>(Iq, p, v, T, Y);
  Props<NC> pr;
  if constexpr (EOS == kEosMagma) {  // the side point's shear rate (fluid_2d.hpp:234-235)
    double dv[DIM][DIM];
#pragma unroll
    for (int a = 0; a < DIM; ++a)
#pragma unroll
      for (int d = 0; d < DIM; ++d) dv[a][d] = dI[d][1 + a];
    if (magma_mixture<NC>(k.mg, p, T, Y, shear_rate<DIM>(dv), pr)) flag_error(k, GALES_ERR_MAGMA, e);
  } else {
    mixture<NC>(k.ch, p, T, Y, pr);
  }
  Coef<DIM, NC> c;
  make_coef<DIM, NC>(pr, p, v, T, Y, c);
  if constexpr (sizeof(S) == 4) P.c = narrow<DIM, NC>(c);
  else P.c = c;
  // advective flux (fluid_2d.hpp:581-595), mass-flux override (fluid_2d.hpp:674-680, 732-738)
  double Fa[DIM][ND], Fd[DIM][ND];
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    const double vk = v[d];
    if ((bc.mass_flux_mask >> d) & 1u) {
      const double mf = bc.mass_flux[d];
      Fa[d][0] = mf;
#pragma unroll
      for (int j = 0; j < DIM; ++j) Fa[d][1 + j] = (j == d) ? mf * v[j] + p : mf * v[j];
      Fa[d][L::iT] = mf * c.E + p * v[d];
#pragma unroll
      for (int i = 0; i < NC - 1; ++i) Fa[d][L::iY + i] = mf * Y[i];
    } else {
      Fa[d][0] = pr.rho * vk;
#pragma unroll
      for (int j = 0; j < DIM; ++j) Fa[d][1 + j] = (j == d) ? pr.rho * vk * vk + p : pr.rho * vk * v[j];
      Fa[d][L::iT] = vk * (pr.rho * c.E + p);
#pragma unroll
      for (int i = 0; i < NC - 1; ++i) Fa[d][L::iY + i] = pr.rho * vk * Y[i];
    }
  }
  // diffusive flux from stresses with Neumann overrides (fluid_2d.hpp:761-817)
  {
    const double lambda = -2.0 * pr.mu / 3.0;
    double div = 0.0;
#pragma unroll
    for (int d = 0; d < DIM; ++d) div += dI[d][1 + d];
    double ts[DIM][DIM], qf[DIM], Jf[DIM][L::NYA];
#pragma unroll
    for (int a = 0; a < DIM; ++a)
#pragma unroll
      for (int b = 0; b < DIM; ++b) {
        if (a == b) ts[a][b] = lambda * (div) + 2.0 * pr.mu * dI[a][1 + a];
        else {
          const int lo = a < b ? a : b, hi = a < b ? b : a;
          ts[a][b] = pr.mu * (dI[hi][1 + lo] + dI[lo][1 + hi]);
        }
      }
#pragma unroll
    for (int d = 0; d < DIM; ++d) qf[d] = -pr.kappa * dI[d][L::iT];
#pragma unroll
    for (int d = 0; d < DIM; ++d)
#pragma unroll
      for (int i = 0; i < NC - 1; ++i) Jf[d][i] = pr.rho * pr.D_c[i] * dI[d][L::iY + i];
#pragma unroll
    for (int a = 0; a < DIM; ++a)
#pragma unroll
      for (int b = a; b < DIM; ++b)
        if ((bc.tau_mask >> (a * 3 + b)) & 1u) { ts[a][b] = bc.tau[a * 3 + b]; ts[b][a] = ts[a][b]; }
#pragma unroll
    for (int d = 0; d < DIM; ++d)
      if ((bc.q_mask >> d) & 1u) qf[d] = bc.q[d];
#pragma unroll
    for (int i = 0; i < NC - 1; ++i)
#pragma unroll
      for (int d = 0; d < DIM; ++d)
        if ((bc.J_mask >> (d * 8 + i)) & 1u) Jf[d][i] = bc.J[d][i];
    double H[L::NYA];
#pragma unroll
    for (int i = 0; i < NC - 1; ++i) H[i] = pr.e_c[i] + p / pr.rho_c[i];
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
      double HJ = 0.0;
#pragma unroll
      for (int i = 0; i < NC - 1; ++i) HJ += H[i] * Jf[d][i];
      Fd[d][0] = 0.0;
#pragma unroll
      for (int j = 0; j < DIM; ++j) Fd[d][1 + j] = ts[d][j];
      double en = ts[d][0] * v[0];
#pragma unroll
      for (int j = 1; j < DIM; ++j) en = en + ts[d][j] * v[j];
      Fd[d][L::iT] = en - qf[d] - HJ;
#pragma unroll
      for (int i = 0; i < NC - 1; ++i) Fd[d][L::iY + i] = Jf[d][i];
    }
  }
#pragma unroll
  for (int j = 0; j < ND; ++j) {
    double x = Fa[0][j] * JNxW[0];
#pragma unroll
    for (int d = 1; d < DIM; ++d) x = madd(Fa[d][j], JNxW[d], x);
#pragma unroll
    for (int d = 0; d < DIM; ++d) x = madd(-Fd[d][j], JNxW[d], x);
    P.rb[j] = x;
  }
}

// Side-point geometry of the listed boundary elements' flagged sides, once per mesh.
template <int DIM, int NEN>
struct alignas(16) BGeo {
  double sh[NEN], ds[DIM][NEN], JNxW[DIM];
};

template <int DIM, int NEN, int NS, int NSQ>
__global__ void __launch_bounds__(128) bgeo_kernel(const KParams k, BGeo<DIM, NEN>* __restrict__ out) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= k.n_bpt) return;
  const int li = k.bpt_el[t], ip = k.bpt_ip[t], s = ip / NSQ, iq = ip % NSQ;
  const long long e = k.el_list[li];
  double X[NEN][DIM];
#pragma unroll
  for (int a = 0; a < NEN; ++a) {
    const int nd_ = __ldg(k.conn + e * NEN + a);
#pragma unroll
    for (int d = 0; d < DIM; ++d) X[a][d] = __ldg(k.coords + (long long)nd_ * DIM + d);
  }
  Geo<DIM, NEN> q;
  geometry<DIM, NEN>(X, k.sgp[s][iq], false, q);
  if (!(q.J > 0.0)) flag_error(k, GALES_ERR_NEG_JACOBIAN, e);
  BGeo<DIM, NEN>& o = out[t];
#pragma unroll
  for (int i = 0; i < NEN; ++i) {
    o.sh[i] = q.sh[i];
#pragma unroll
    for (int d = 0; d < DIM; ++d) o.ds[d][i] = q.ds[d][i];
  }
#pragma unroll
  for (int d = 0; d < DIM; ++d) o.JNxW[d] = q.JN[d] * k.W_bd;
}

// Boundary pass, stage 1: one thread per flagged side point writes its point record.
template <int DIM, int NEN, int NC, int NS, int NSQ, typename S, int EOS = kEosChemicals>
__global__ void __launch_bounds__(128) bpoint_kernel(const KParams k) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= k.n_bpt) return;
  const int li = k.bpt_el[t], ip = k.bpt_ip[t];
  const long long e = k.el_list[li];
  int nodes[NEN];
#pragma unroll
  for (int a = 0; a < NEN; ++a) nodes[a] = __ldg(k.conn + e * NEN + a);
  const BGeo<DIM, NEN>& g = reinterpret_cast<const BGeo<DIM, NEN>*>(k.bgeo)[t];
  double sh[NEN], ds[DIM][NEN], JN[DIM];
#pragma unroll
  for (int i = 0; i < NEN; ++i) {
    sh[i] = g.sh[i];
#pragma unroll
    for (int d = 0; d < DIM; ++d) ds[d][i] = g.ds[d][i];
  }
#pragma unroll
  for (int d = 0; d < DIM; ++d) JN[d] = g.JNxW[d];
  BPoint<DIM, NEN, NC, S> P;
  const int flag = (int)k.bd_sides[li * NS + ip / NSQ];
  bpoint_phase<DIM, NEN, NC, S, EOS>(k, nodes, flag, sh, ds, JN, P, e);
  BPointRec<DIM, NEN, NC, S>& O = reinterpret_cast<BPointRec<DIM, NEN, NC, S>*>(k.bpt_rec)[t];
  O.pt = P;
  bpoint_blocks<DIM, NC, S>(P.c, P.JNxW, k.side_bc[flag < GALES_MAX_FLAGS ? flag : 0], O.BA, O.BK);
}

// Boundary pass, one warp per listed boundary element.  Lanes first evaluate one
// side quadrature point each (thread per point, FP64: geometry, EOS, fluxes and the
// boundary residual), then build BA and BK entry-parallel per point in the form's
// matrix type S and accumulate
//   m_ba += N_b (N_a BA - sum_l dN_a/dx_l BK_l)                 (fluid_2d.hpp:351-363)
// before the element's own Dirichlet pass and scatter (fluid_assembly.hpp:57-63).
template <int DIM, int NEN, int NC, int NS, int NSQ, typename S, int EOS = kEosChemicals>
__global__ void __launch_bounds__(32) boundary_kernel(const KParams k) {
  using L = Layout<DIM, NC>;
  constexpr int ND = L::ND;
  constexpr int N = NEN * ND;
  constexpr int NT = N * N;
  using BS = BoundarySmem<DIM, NEN, NC, NS, NSQ, S>;
  constexpr int MS = BS::MS;
  using BR = BPointRec<DIM, NEN, NC, S>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  BS& B = *reinterpret_cast<BS*>(smem_raw);
  const int lane = threadIdx.x;
  const long long li = blockIdx.x;
  if (li >= k.n_list) return;
  const long long e = k.el_list[li];
  int nodes[NEN];
#pragma unroll
  for (int a = 0; a < NEN; ++a) nodes[a] = __ldg(k.conn + e * NEN + a);
  for (int t = lane; t < N * MS; t += 32) B.m[t] = S(0);
  for (int t = lane; t < N; t += 32) B.r[t] = 0.0;
  // rows of the element's nodes and the element's slot table, for the scatter
  if (lane < NEN) {
    const int fl = k.node_flag ? __ldg(k.node_flag + nodes[lane]) : 0;
    B.blocked[lane] = (fl >= 0 && fl < GALES_MAX_FLAGS) ? k.dirichlet_mask[fl] : 0u;
    const int64_t r0 = __ldg(k.node_rp + nodes[lane]), r1 = __ldg(k.node_rp + nodes[lane] + 1);
    B.rowbase[lane] = r0 * (int64_t)(ND * ND);
    B.rowlen[lane] = (int32_t)((r1 - r0) * ND);
  }
  for (int t = lane; t < NEN * NEN; t += 32) B.slot[t / NEN][t % NEN] = __ldg(k.slot + e * NEN * NEN + t);
  // (1) point physics and matrices: from the boundary point records of this element
  // when the boundary point stage ran (k.bpt_rec), otherwise one lane per (side, point)
  if (k.bpt_rec) {
    for (int t = lane; t < NS * NSQ; t += 32) B.pt[t].pt.flag = 0;
    __syncwarp();
    const int p0 = k.bpt_off[li], p1 = k.bpt_off[li + 1];
    static_assert(sizeof(BR) % 16 == 0, "point record must be int4-aligned");
    constexpr int W4 = sizeof(BR) / 16;
    for (int t = lane; t < (p1 - p0) * W4; t += 32) {
      const int pt = p0 + t / W4, w = t % W4;
      reinterpret_cast<int4*>(&B.pt[k.bpt_ip[pt]])[w] =
          reinterpret_cast<const int4*>(reinterpret_cast<const BR*>(k.bpt_rec) + pt)[w];
    }
  } else if (lane < NS * NSQ) {
    const int s = lane / NSQ, iq = lane % NSQ;
    const int flag = k.bd_sides[li * NS + s];
    BPoint<DIM, NEN, NC, S>& P = B.pt[lane].pt;
    P.flag = flag;
    if (flag > 0) {
      double X[NEN][DIM];
#pragma unroll
      for (int a = 0; a < NEN; ++a)
#pragma unroll
        for (int d = 0; d < DIM; ++d) X[a][d] = __ldg(k.coords + (long long)nodes[a] * DIM + d);
      Geo<DIM, NEN> q;
      geometry<DIM, NEN>(X, k.sgp[s][iq], false, q);
      if (!(q.J > 0.0)) flag_error(k, GALES_ERR_NEG_JACOBIAN, e);
      double JNxW[DIM];
#pragma unroll
      for (int d = 0; d < DIM; ++d) JNxW[d] = q.JN[d] * k.W_bd;
      bpoint_phase<DIM, NEN, NC, S, EOS>(k, nodes, flag, q.sh, q.ds, JNxW, P, e);
      bpoint_blocks<DIM, NC, S>(P.c, P.JNxW, k.side_bc[flag < GALES_MAX_FLAGS ? flag : 0], B.pt[lane].BA,
                                B.pt[lane].BK);
    }
  }
  __syncwarp();
  // (2) per flagged point, the block m_ba += N_b (N_a BA - sum_l dN_a/dx_l BK_l) and the
  // residual.  Lane l owns block rows l, l + 32, ...: its row's BA and BK rows are read
  // once per point, the columns run at compile time; a block of at most 32 rows is
  // accumulated in registers, a larger one in shared memory.
  constexpr int RPL = (N + 31) / 32;
  constexpr bool kRegs = N <= 32;
  S acc[kRegs ? N : 1];
#pragma unroll
  for (int c = 0; c < (kRegs ? N : 1); ++c) acc[c] = S(0);
  for (int ip = 0; ip < NS * NSQ; ++ip) {
    const BR& R = B.pt[ip];
    const BPoint<DIM, NEN, NC, S>& P = R.pt;
    if (P.flag <= 0) continue;
#pragma unroll
    for (int rr = 0; rr < RPL; ++rr) {
      const int row = lane + 32 * rr;
      if (row < N) {
        const int b = row / ND, jb = row - (row / ND) * ND;
        const S shb = P.sh[b];
        S ba[ND], bk[DIM][ND];
#pragma unroll
        for (int ja = 0; ja < ND; ++ja) {
          ba[ja] = R.BA[jb][ja];
#pragma unroll
          for (int l = 0; l < DIM; ++l) bk[l][ja] = R.BK[l][jb][ja];
        }
#pragma unroll
        for (int a = 0; a < NEN; ++a) {
          const S sha = P.sh[a];
          S dsa[DIM];
#pragma unroll
          for (int l = 0; l < DIM; ++l) dsa[l] = P.ds[l][a];
#pragma unroll
          for (int ja = 0; ja < ND; ++ja) {
            S x = sha * ba[ja];
#pragma unroll
            for (int l = 0; l < DIM; ++l) x = madd(-dsa[l], bk[l][ja], x);
            if constexpr (kRegs) acc[a * ND + ja] = madd(shb, x, acc[a * ND + ja]);
            else B.m[row * MS + a * ND + ja] = madd(shb, x, B.m[row * MS + a * ND + ja]);
          }
        }
      }
    }
    for (int t = lane; t < N; t += 32) B.r[t] = madd(P.shr[t / ND], P.rb[t % ND], B.r[t]);
    __syncwarp();
  }
  if constexpr (kRegs) {
    if (lane < N)
#pragma unroll
      for (int c = 0; c < N; ++c) B.m[lane * MS + c] = acc[c];
    __syncwarp();
  }
  if (k.local_r) {  // element-level output of execute_b: m = m_, r = -r_
    for (int t = lane; t < N; t += 32) k.local_r[li * N + t] = -B.r[t];
    if (k.local_m)
      for (int t = lane; t < NT; t += 32) k.local_m[li * NT + t] = widen(B.m[(t / N) * MS + t % N]);
    return;
  }
  // second scatter pass with its own Dirichlet average avg = (1 + trace)/n
  // (scatter.hpp:62-78), formed only where the element has a blocked row
  uint32_t any_blocked = 0u;
#pragma unroll
  for (int a = 0; a < NEN; ++a) any_blocked |= B.blocked[a];
  double avg = 0.0;
  if (any_blocked != 0u || k.vjp_lam) {
    double tr = 0.0;
    for (int i = lane; i < N; i += 32) tr += widen(B.m[i * MS + i]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) tr += __shfl_xor_sync(0xffffffffu, tr, o);
    avg = (1.0 + tr) * (1.0 / N);
  }
  if (k.vjp_lam) {
    // frozen-tangent VJP: g += K^T lambda for this element's boundary block
    for (int cx = lane; cx < N; cx += 32) {
      double sum = 0.0;
      for (int rw = 0; rw < N; ++rw) {
        const int b = rw / ND, jb = rw % ND;
        const double val = ((B.blocked[b] >> jb) & 1u) ? (rw == cx ? avg : 0.0) : widen(B.m[rw * MS + cx]);
        sum += __ldg(k.vjp_lam + (long long)nodes[b] * ND + jb) * val;
      }
      if (sum != 0.0) atomicAdd(k.vjp_g + (long long)nodes[cx / ND] * ND + cx % ND, sum);
    }
    return;
  }
  const int mode = k.scatter_mode;
  for (int t = lane; t < N; t += 32) {
    const int b = t / ND, jb = t % ND;
    if (!((B.blocked[b] >> jb) & 1u)) add_to(k.rhs + (long long)nodes[b] * ND + jb, -B.r[t], mode);
  }
  if (k.vals) {
    // lane = column (a, ja): one block row per step, consecutive lanes on consecutive
    // columns of node a's run in the row
    constexpr int CH = (N + 31) / 32;
#pragma unroll
    for (int h = 0; h < CH; ++h) {
      const int cx = lane + 32 * h;
      if (cx >= N) break;
      const int a = cx / ND, ja = cx - (cx / ND) * ND;
#pragma unroll
      for (int bq = 0; bq < NEN; ++bq) {
        const uint32_t bl = B.blocked[bq];
        const int64_t rl = B.rowlen[bq];
        double* rowp = k.vals + B.rowbase[bq] + (int64_t)B.slot[bq][a] * ND + ja;
#pragma unroll
        for (int jb = 0; jb < ND; ++jb, rowp += rl) {
          const int row = bq * ND + jb;
          double val;
          if ((bl >> jb) & 1u) {
            if (row != cx) continue;
            val = avg;
          } else {
            val = widen(B.m[row * MS + cx]);
          }
          if ((__double2hiint(val) & 0x7fffffff) | __double2loint(val)) add_to(rowp, val, mode);
        }
      }
    }
  }
}

}  // namespace gales
