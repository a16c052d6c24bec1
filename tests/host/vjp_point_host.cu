// Host-side instances of the point-level VJP (gales_vjp.cuh) for the CPU tests:
// the same __host__ __device__ code the GPU kernel runs, called from ctypes.
#include "../../gales-multi-fluid_gb300/csrc/gales_vjp.cuh"

using namespace gales;

namespace {

// scal: dt, dc_sharp, dc_scale, gravity[3], tau, dc_2006, steady  (9 doubles)
template <int DIM, int NEN, int NC>
void fill(const DevChem* ch, const double* scal, const double* uri, const double* G, const double* ds,
          vjp::Ctx<DIM, NC>& x, vjp::PGeo<DIM, NEN>& q) {
  x.ch = ch;
  x.dt = scal[0];
  x.inv_dt = 1.0 / scal[0];
  x.dc_sharp = scal[1];
  x.dc_scale = scal[2];
  for (int d = 0; d < 3; ++d) x.gravity[d] = scal[3 + d];
  x.tau = (int)scal[6];
  x.dc_2006 = (int)scal[7];
  x.steady = (int)scal[8];
  x.u_ref_inv = uri;
  q.trG = 0.0;
  for (int i = 0; i < DIM; ++i) {
    for (int j = 0; j < DIM; ++j) q.G[i][j] = G[i * DIM + j];
    q.trG += q.G[i][i];
  }
  for (int d = 0; d < DIM; ++d)
    for (int a = 0; a < NEN; ++a) q.ds[d][a] = ds[d * NEN + a];
}

template <int DIM, int NEN, int NC>
void fwd(const DevChem* ch, const double* scal, const double* uri, const double* G, const double* ds,
         const double* Iq, const double* dIf, const double* Pq, double* phi0, double* phif) {
  constexpr int ND = Layout<DIM, NC>::ND;
  vjp::Ctx<DIM, NC> x;
  vjp::PGeo<DIM, NEN> q;
  fill<DIM, NEN, NC>(ch, scal, uri, G, ds, x, q);
  double dI[DIM][ND], phi[DIM][ND];
  for (int d = 0; d < DIM; ++d)
    for (int j = 0; j < ND; ++j) dI[d][j] = dIf[d * ND + j];
  vjp::PTape<DIM, NEN, NC> t;
  vjp::point_forward<DIM, NEN, NC>(x, q, Iq, dI, Pq, t, phi0, phi);
  for (int d = 0; d < DIM; ++d)
    for (int j = 0; j < ND; ++j) phif[d * ND + j] = phi[d][j];
}

template <int DIM, int NEN, int NC>
void rev(const DevChem* ch, const double* scal, const double* uri, const double* G, const double* ds,
         const double* Iq, const double* dIf, const double* Pq, const double* phi0b, const double* phibf, double* Ib,
         double* dIbf, double* th) {
  constexpr int ND = Layout<DIM, NC>::ND;
  vjp::Ctx<DIM, NC> x;
  vjp::PGeo<DIM, NEN> q;
  fill<DIM, NEN, NC>(ch, scal, uri, G, ds, x, q);
  double dI[DIM][ND], phi[DIM][ND], phib[DIM][ND], dIb[DIM][ND], phi0[ND];
  for (int d = 0; d < DIM; ++d)
    for (int j = 0; j < ND; ++j) {
      dI[d][j] = dIf[d * ND + j];
      phib[d][j] = phibf[d * ND + j];
      dIb[d][j] = 0.0;
    }
  vjp::PTape<DIM, NEN, NC> t;
  vjp::point_forward<DIM, NEN, NC>(x, q, Iq, dI, Pq, t, phi0, phi);
  vjp::point_reverse<DIM, NEN, NC>(x, q, Iq, dI, Pq, t, phi0b, phib, Ib, dIb, th);
  for (int d = 0; d < DIM; ++d)
    for (int j = 0; j < ND; ++j) dIbf[d * ND + j] = dIb[d][j];
}

template <int DIM, int NC>
void bfwd(const DevChem* ch, const double* scal, const double* uri, const gales_side_bc* bc, const double* Iq,
          const double* dIf, const double* JN, double* rb) {
  constexpr int ND = Layout<DIM, NC>::ND;
  vjp::Ctx<DIM, NC> x;
  vjp::PGeo<DIM, 1> q;
  const double G[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1}, ds[3] = {0, 0, 0};
  fill<DIM, 1, NC>(ch, scal, uri, G, ds, x, q);
  double dI[DIM][ND];
  for (int d = 0; d < DIM; ++d)
    for (int j = 0; j < ND; ++j) dI[d][j] = dIf[d * ND + j];
  vjp::BTape<DIM, NC> t;
  vjp::bpoint_forward<DIM, NC>(x, *bc, Iq, dI, JN, t, rb);
}

template <int DIM, int NC>
void brev(const DevChem* ch, const double* scal, const double* uri, const gales_side_bc* bc, const double* Iq,
          const double* dIf, const double* JN, const double* rbb, double* Ib, double* dIbf, double* th) {
  constexpr int ND = Layout<DIM, NC>::ND;
  vjp::Ctx<DIM, NC> x;
  vjp::PGeo<DIM, 1> q;
  const double G[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1}, ds[3] = {0, 0, 0};
  fill<DIM, 1, NC>(ch, scal, uri, G, ds, x, q);
  double dI[DIM][ND], dIb[DIM][ND], rb[ND];
  for (int d = 0; d < DIM; ++d)
    for (int j = 0; j < ND; ++j) { dI[d][j] = dIf[d * ND + j]; dIb[d][j] = 0.0; }
  vjp::BTape<DIM, NC> t;
  vjp::bpoint_forward<DIM, NC>(x, *bc, Iq, dI, JN, t, rb);
  vjp::bpoint_reverse<DIM, NC>(x, *bc, Iq, dI, JN, t, rbb, Ib, dIb, th);
  for (int d = 0; d < DIM; ++d)
    for (int j = 0; j < ND; ++j) dIbf[d * ND + j] = dIb[d][j];
}

}  // namespace

#define GV_BINST(DIM, NC)                                                                                     \
  extern "C" void bp_forward_##DIM##_##NC(const DevChem* ch, const double* scal, const double* uri,          \
                                          const gales_side_bc* bc, const double* Iq, const double* dI,        \
                                          const double* JN, double* rb) {                                     \
    bfwd<DIM, NC>(ch, scal, uri, bc, Iq, dI, JN, rb);                                                         \
  }                                                                                                           \
  extern "C" void bp_reverse_##DIM##_##NC(const DevChem* ch, const double* scal, const double* uri,          \
                                          const gales_side_bc* bc, const double* Iq, const double* dI,        \
                                          const double* JN, const double* rbb, double* Ib, double* dIb,       \
                                          double* th) {                                                       \
    brev<DIM, NC>(ch, scal, uri, bc, Iq, dI, JN, rbb, Ib, dIb, th);                                           \
  }

GV_BINST(3, 3)
GV_BINST(2, 2)
GV_BINST(3, 4)
GV_BINST(3, 1)

#define GV_INST(DIM, NEN, NC)                                                                               \
  extern "C" void pt_forward_##DIM##_##NEN##_##NC(const DevChem* ch, const double* scal, const double* uri, \
                                                  const double* G, const double* ds, const double* Iq,      \
                                                  const double* dI, const double* Pq, double* phi0,         \
                                                  double* phi) {                                            \
    fwd<DIM, NEN, NC>(ch, scal, uri, G, ds, Iq, dI, Pq, phi0, phi);                                         \
  }                                                                                                         \
  extern "C" void pt_reverse_##DIM##_##NEN##_##NC(                                                          \
      const DevChem* ch, const double* scal, const double* uri, const double* G, const double* ds,          \
      const double* Iq, const double* dI, const double* Pq, const double* phi0b, const double* phib,        \
      double* Ib, double* dIb, double* th) {                                                                \
    rev<DIM, NEN, NC>(ch, scal, uri, G, ds, Iq, dI, Pq, phi0b, phib, Ib, dIb, th);                          \
  }

GV_INST(3, 4, 3)
GV_INST(3, 4, 1)
GV_INST(2, 3, 2)
GV_INST(3, 8, 4)
