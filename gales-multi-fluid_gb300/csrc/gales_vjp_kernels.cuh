// Exact VJP kernels: lambda^T d(rhs)/d(I, theta) of the assembled rhs, recomputing
// every point from the state (nothing stored between the forward and the reverse).
//   vjp_interior_kernel - one thread per (element, interior point): the element's
//                         interpolated cotangents Lambda0 = sum_b N_b lambda_b and
//                         Lambda_d = sum_b dN_b/dx_d lambda_b seed the point reverse;
//                         the state cotangents go back to the nodes with N_a and
//                         dN_a/dx_d (FP64 atomics), the parameter cotangents are
//                         reduced per warp.
//   vjp_boundary_kernel - one thread per (boundary element, side point) for the
//                         boundary fluxes of execute_b.
// Rows under a Dirichlet constraint are zero in the rhs whatever the state
// (scatter.hpp:70-78), so their lambda entries are masked out.  k.vjp_th receives the
// parameter cotangents [3 nc] followed by the u_ref_inv cotangents [nd].
#pragma once

#include "gales_kernels.cuh"
#include "gales_vjp.cuh"

namespace gales {

template <int DIM, int NC>
__device__ __forceinline__ void vjp_ctx(const KParams& k, vjp::Ctx<DIM, NC>& x) {
  x.ch = k.ch;
  x.dt = k.dt;
  x.inv_dt = k.inv_dt;
  x.dc_sharp = k.dc_sharp;
  x.dc_scale = k.dc_scale;
  for (int d = 0; d < 3; ++d) x.gravity[d] = k.gravity[d];
  x.u_ref_inv = k.u_ref_inv;
  x.tau = k.tau;
  x.dc_2006 = k.dc_2006;
  x.steady = k.steady;
}

// lambda of node nd_, masked by its Dirichlet flags; returns whether any entry is nonzero
template <int ND>
__device__ __forceinline__ bool masked_lambda(const KParams& k, int nd_, double* lam) {
  const int fl = k.node_flag ? __ldg(k.node_flag + nd_) : 0;
  const uint32_t blk = (fl >= 0 && fl < GALES_MAX_FLAGS) ? k.dirichlet_mask[fl] : 0u;
  bool any = false;
#pragma unroll
  for (int j = 0; j < ND; ++j) {
    const double l = ((blk >> j) & 1u) ? 0.0 : __ldg(k.vjp_lam + (long long)nd_ * ND + j);
    lam[j] = l;
    any |= l != 0.0;
  }
  return any;
}

// Warp sums of per-thread cotangents added to k.vjp_th[off + i].
template <int NP>
__device__ __forceinline__ void reduce_params(const KParams& k, const double (&th)[NP], int off) {
  if (!k.vjp_th) return;
#pragma unroll
  for (int i = 0; i < NP; ++i) {
    double x = th[i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    if ((threadIdx.x & 31) == 0 && x != 0.0) atomicAdd(k.vjp_th + off + i, x);
  }
}

template <int DIM, int NEN, int NC, int NQ>
__global__ void __launch_bounds__(128) vjp_interior_kernel(const KParams k, long long n) {
  using L = Layout<DIM, NC>;
  constexpr int ND = L::ND;
  constexpr int NG = geo_per_element<DIM, NEN>(NQ);
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long li = t / NQ;
  const int iq = (int)(t % NQ);
  double th[3 * NC], urib[ND];
#pragma unroll
  for (int i = 0; i < 3 * NC; ++i) th[i] = 0.0;
#pragma unroll
  for (int j = 0; j < ND; ++j) urib[j] = 0.0;
  if (li < n) {
    const long long e = k.el_list ? (long long)k.el_list[li] : li;
    int nodes[NEN];
    double lam[NEN][ND];
    bool any = false;
#pragma unroll
    for (int a = 0; a < NEN; ++a) {
      nodes[a] = __ldg(k.conn + e * NEN + a);
      any |= masked_lambda<ND>(k, nodes[a], lam[a]);
    }
    if (any) {
      const ElemGeo<DIM, NEN>& g = reinterpret_cast<const ElemGeo<DIM, NEN>*>(k.geo)[e * NG + (NG == 1 ? 0 : iq)];
      vjp::PGeo<DIM, NEN> pg;
      pg.trG = 0.0;
#pragma unroll
      for (int i = 0; i < DIM; ++i) {
#pragma unroll
        for (int j = 0; j < DIM; ++j) pg.G[i][j] = g.G[i][j];
        pg.trG += g.G[i][i];
#pragma unroll
        for (int a = 0; a < NEN; ++a) pg.ds[i][a] = g.ds[i][a];
      }
      const double JxW = g.J * k.W_in;
      double Iq[ND], Pq[ND], dI[DIM][ND], L0[ND], Ld[DIM][ND];
#pragma unroll
      for (int j = 0; j < ND; ++j) {
        Iq[j] = 0.0; Pq[j] = 0.0; L0[j] = 0.0;
#pragma unroll
        for (int d = 0; d < DIM; ++d) { dI[d][j] = 0.0; Ld[d][j] = 0.0; }
      }
#pragma unroll
      for (int a = 0; a < NEN; ++a) {
        const double sh = k.sh_tab[iq][a];
#pragma unroll
        for (int j = 0; j < ND; ++j) {
          const double Ia = __ldg(k.I + (long long)nodes[a] * ND + j);
          Iq[j] += sh * Ia;
          Pq[j] += sh * __ldg(k.P + (long long)nodes[a] * ND + j);
          L0[j] += sh * lam[a][j];
#pragma unroll
          for (int d = 0; d < DIM; ++d) {
            dI[d][j] += g.ds[d][a] * Ia;
            Ld[d][j] += g.ds[d][a] * lam[a][j];
          }
        }
      }
      // the rhs is -r: cotangents of (phi0, phi_d) are -JxW (Lambda0, Lambda_d)
#pragma unroll
      for (int j = 0; j < ND; ++j) {
        L0[j] *= -JxW;
#pragma unroll
        for (int d = 0; d < DIM; ++d) Ld[d][j] *= -JxW;
      }
      vjp::Ctx<DIM, NC> x;
      vjp_ctx<DIM, NC>(k, x);
      vjp::PTape<DIM, NEN, NC> tp;
      double phi0[ND], phi[DIM][ND], Ib[ND], dIb[DIM][ND];
      vjp::point_forward<DIM, NEN, NC>(x, pg, Iq, dI, Pq, tp, phi0, phi);
#pragma unroll
      for (int j = 0; j < ND; ++j) {
        Ib[j] = 0.0;
#pragma unroll
        for (int d = 0; d < DIM; ++d) dIb[d][j] = 0.0;
      }
      vjp::point_reverse<DIM, NEN, NC>(x, pg, Iq, dI, Pq, tp, L0, Ld, Ib, dIb, th, urib);
#pragma unroll
      for (int a = 0; a < NEN; ++a) {
        const double sh = k.sh_tab[iq][a];
#pragma unroll
        for (int j = 0; j < ND; ++j) {
          double v = sh * Ib[j];
#pragma unroll
          for (int d = 0; d < DIM; ++d) v += g.ds[d][a] * dIb[d][j];
          if (v != 0.0) atomicAdd(k.vjp_g + (long long)nodes[a] * ND + j, v);
        }
      }
    }
  }
  reduce_params<3 * NC>(k, th, 0);
  reduce_params<ND>(k, urib, 3 * NC);
}

template <int DIM, int NEN, int NC, int NS, int NSQ>
__global__ void __launch_bounds__(128) vjp_boundary_kernel(const KParams k) {
  using L = Layout<DIM, NC>;
  constexpr int ND = L::ND;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long li = t / (NS * NSQ);
  const int ip = (int)(t % (NS * NSQ)), s = ip / NSQ, iq = ip % NSQ;
  double th[3 * NC];
#pragma unroll
  for (int i = 0; i < 3 * NC; ++i) th[i] = 0.0;
  const int flag = li < k.n_list ? k.bd_sides[li * NS + s] : 0;
  if (flag > 0) {
    const long long e = k.el_list[li];
    const gales_side_bc& bc = k.side_bc[flag < GALES_MAX_FLAGS ? flag : 0];
    int nodes[NEN];
    double lam[NEN][ND];
    bool any = false;
#pragma unroll
    for (int a = 0; a < NEN; ++a) {
      nodes[a] = __ldg(k.conn + e * NEN + a);
      any |= masked_lambda<ND>(k, nodes[a], lam[a]);
    }
    if (any) {
      double X[NEN][DIM];
#pragma unroll
      for (int a = 0; a < NEN; ++a)
#pragma unroll
        for (int d = 0; d < DIM; ++d) X[a][d] = __ldg(k.coords + (long long)nodes[a] * DIM + d);
      Geo<DIM, NEN> q;
      geometry<DIM, NEN>(X, k.sgp[s][iq], false, q);
      double JN[DIM];
#pragma unroll
      for (int d = 0; d < DIM; ++d) JN[d] = q.JN[d] * k.W_bd;
      double Iq[ND], dI[DIM][ND], rbb[ND];
#pragma unroll
      for (int j = 0; j < ND; ++j) {
        Iq[j] = 0.0; rbb[j] = 0.0;
#pragma unroll
        for (int d = 0; d < DIM; ++d) dI[d][j] = 0.0;
      }
#pragma unroll
      for (int a = 0; a < NEN; ++a)
#pragma unroll
        for (int j = 0; j < ND; ++j) {
          const double Ia = __ldg(k.I + (long long)nodes[a] * ND + j);
          Iq[j] += q.sh[a] * Ia;
          rbb[j] -= q.sh[a] * lam[a][j];       // the rhs carries -r of execute_b
#pragma unroll
          for (int d = 0; d < DIM; ++d) dI[d][j] += q.ds[d][a] * Ia;
        }
      vjp::Ctx<DIM, NC> x;
      vjp_ctx<DIM, NC>(k, x);
      vjp::BTape<DIM, NC> tp;
      double rb[ND], Ib[ND], dIb[DIM][ND];
      vjp::bpoint_forward<DIM, NC>(x, bc, Iq, dI, JN, tp, rb);
#pragma unroll
      for (int j = 0; j < ND; ++j) {
        Ib[j] = 0.0;
#pragma unroll
        for (int d = 0; d < DIM; ++d) dIb[d][j] = 0.0;
      }
      vjp::bpoint_reverse<DIM, NC>(x, bc, Iq, dI, JN, tp, rbb, Ib, dIb, th);
#pragma unroll
      for (int a = 0; a < NEN; ++a)
#pragma unroll
        for (int j = 0; j < ND; ++j) {
          double v = q.sh[a] * Ib[j];
#pragma unroll
          for (int d = 0; d < DIM; ++d) v += q.ds[d][a] * dIb[d][j];
          if (v != 0.0) atomicAdd(k.vjp_g + (long long)nodes[a] * ND + j, v);
        }
    }
  }
  reduce_params<3 * NC>(k, th, 0);
}

// Launchers for one element type.
template <int DIM, int NEN, int NQ, int NS, int NSQ>
struct VjpDispatch {
  static LaunchResult interior(const KParams& k, int nc, long long n, cudaStream_t st) {
    if (n <= 0) return {cudaSuccess, 0};
    const unsigned blocks = (unsigned)((n * NQ + 127) / 128);
#define GALES_C(NC)                                                      \
  vjp_interior_kernel<DIM, NEN, NC, NQ><<<blocks, 128, 0, st>>>(k, n); \
  return {cudaGetLastError(), 1}
    GALES_NC_SWITCH(nc, GALES_C)
#undef GALES_C
    return {cudaErrorInvalidValue, 0};
  }
  static LaunchResult boundary(const KParams& k, int nc, long long n, cudaStream_t st) {
    if (n <= 0) return {cudaSuccess, 0};
    const unsigned blocks = (unsigned)((n * NS * NSQ + 127) / 128);
#define GALES_C(NC)                                                          \
  vjp_boundary_kernel<DIM, NEN, NC, NS, NSQ><<<blocks, 128, 0, st>>>(k); \
  return {cudaGetLastError(), 1}
    GALES_NC_SWITCH(nc, GALES_C)
#undef GALES_C
    return {cudaErrorInvalidValue, 0};
  }
};

}  // namespace gales
