// Host side of the C ABI declared in include/gales_asm.h.
//
// The handle replaces, for one rank and one GPU, the objects the reference's
// assembly reads and fills: linear_system's FECrsGraph (linear_system.hpp:40-66),
// the per-element dof gids of scatter::execute (scatter.hpp:44-57), the Dirichlet
// policy of fluid_dofs_ic_bc (fluid_dofs_ic_bc.hpp:86-117) and the fluid
// integral's constructor state (u_ref_inv, fluid_2d.hpp:123-135).  Everything the
// kernels read lives in device memory owned by the handle; the caller owns the
// state and output buffers.
#include <cuda_runtime.h>

#include <algorithm>
#include <functional>
#include <atomic>
#include <cfloat>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <mutex>
#include <thread>
#include <vector>

#include "../../include/gales_asm.h"
#include "gales_launch.cuh"

using namespace gales;

namespace {

struct ElemInfo {
  int nq, nsides, nsn, nqs;
  double gp[8][3];
  double sgp[6][4][3];
  double W_in, W_bd;
};

// Gauss tables of element.hpp:63-176 (2D) and 360-477 (3D), weights of
// quad.hpp:165-186 and 497-513.
bool elem_info(int dim, int nen, ElemInfo& o) {
  memset(&o, 0, sizeof(o));
  if (dim == 2 && nen == 3) {
    o.nq = 3; o.nsides = 3; o.nsn = 2; o.nqs = 2;
    const double g[3][2] = {{1.0 / 6.0, 1.0 / 6.0}, {4.0 / 6.0, 1.0 / 6.0}, {1.0 / 6.0, 4.0 / 6.0}};
    for (int i = 0; i < 3; ++i) { o.gp[i][0] = g[i][0]; o.gp[i][1] = g[i][1]; }
    const double gm = 0.5 * (1.0 - 1.0 / sqrt(3.0)), gpl = 0.5 * (1.0 + 1.0 / sqrt(3.0));
    const double s[3][2][2] = {{{gpl, 1.0 - gpl}, {gm, 1.0 - gm}}, {{0.0, gpl}, {0.0, gm}}, {{gm, 0.0}, {gpl, 0.0}}};
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 2; ++j) { o.sgp[i][j][0] = s[i][j][0]; o.sgp[i][j][1] = s[i][j][1]; }
    o.W_in = 1.0 / 6.0; o.W_bd = 1.0 / 2.0;
    return true;
  }
  if (dim == 2 && nen == 4) {
    o.nq = 4; o.nsides = 4; o.nsn = 2; o.nqs = 2;
    const double gm = -1.0 / sqrt(3.0), gpl = 1.0 / sqrt(3.0);
    const double g[4][2] = {{gm, gm}, {gpl, gm}, {gpl, gpl}, {gm, gpl}};
    for (int i = 0; i < 4; ++i) { o.gp[i][0] = g[i][0]; o.gp[i][1] = g[i][1]; }
    const double s[4][2][2] = {{{gm, -1.0}, {gpl, -1.0}}, {{1.0, gm}, {1.0, gpl}},
                               {{gpl, 1.0}, {gm, 1.0}}, {{-1.0, gpl}, {-1.0, gm}}};
    for (int i = 0; i < 4; ++i)
      for (int j = 0; j < 2; ++j) { o.sgp[i][j][0] = s[i][j][0]; o.sgp[i][j][1] = s[i][j][1]; }
    o.W_in = 1.0; o.W_bd = 1.0;
    return true;
  }
  if (dim == 3 && nen == 4) {
    o.nq = 4; o.nsides = 4; o.nsn = 3; o.nqs = 3;
    const double a = 0.1381966011250105, b = 0.5854101966249685;
    const double g[4][3] = {{a, a, a}, {b, a, a}, {a, b, a}, {a, a, b}};
    for (int i = 0; i < 4; ++i)
      for (int d = 0; d < 3; ++d) o.gp[i][d] = g[i][d];
    const double t = 1.0 / 6.0, f = 4.0 / 6.0;
    const double s[4][3][3] = {{{f, t, t}, {t, f, t}, {t, t, f}},
                               {{0.0, t, t}, {0.0, t, f}, {0.0, f, t}},
                               {{t, 0.0, t}, {f, 0.0, t}, {t, 0.0, f}},
                               {{t, t, 0.0}, {t, f, 0.0}, {f, t, 0.0}}};
    for (int i = 0; i < 4; ++i)
      for (int j = 0; j < 3; ++j)
        for (int d = 0; d < 3; ++d) o.sgp[i][j][d] = s[i][j][d];
    o.W_in = 1.0 / 24.0; o.W_bd = 1.0 / 6.0;
    return true;
  }
  if (dim == 3 && nen == 8) {
    o.nq = 8; o.nsides = 6; o.nsn = 4; o.nqs = 4;
    const double m = -1.0 / sqrt(3.0), p = 1.0 / sqrt(3.0);
    const double g[8][3] = {{m, m, m}, {p, m, m}, {p, p, m}, {m, p, m}, {m, m, p}, {p, m, p}, {p, p, p}, {m, p, p}};
    for (int i = 0; i < 8; ++i)
      for (int d = 0; d < 3; ++d) o.gp[i][d] = g[i][d];
    const double s[6][4][3] = {{{m, m, 1.0}, {p, m, 1.0}, {p, p, 1.0}, {m, p, 1.0}},
                               {{m, m, -1.0}, {m, p, -1.0}, {p, p, -1.0}, {p, m, -1.0}},
                               {{-1.0, m, m}, {-1.0, m, p}, {-1.0, p, p}, {-1.0, p, m}},
                               {{1.0, m, m}, {1.0, p, m}, {1.0, p, p}, {1.0, m, p}},
                               {{p, 1.0, m}, {m, 1.0, m}, {m, 1.0, p}, {p, 1.0, p}},
                               {{p, -1.0, m}, {p, -1.0, p}, {m, -1.0, p}, {m, -1.0, m}}};
    for (int i = 0; i < 6; ++i)
      for (int j = 0; j < 4; ++j)
        for (int d = 0; d < 3; ++d) o.sgp[i][j][d] = s[i][j][d];
    o.W_in = 1.0; o.W_bd = 1.0;
    return true;
  }
  return false;
}

template <typename T>
struct DevBuf {
  T* p = nullptr;
  size_t n = 0;
  cudaError_t alloc(size_t count) {
    if (count <= n && p) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
    if (count == 0) return cudaSuccess;
    cudaError_t e = cudaMalloc(&p, count * sizeof(T));
    if (e == cudaSuccess) n = count;
    return e;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
};

int hw_threads() {
  unsigned n = std::thread::hardware_concurrency();
  return n == 0 ? 1 : (int)std::min(n, 32u);
}

template <typename F>
void parallel_for(int64_t n, F f) {
  const int nt = (int)std::min<int64_t>(hw_threads(), std::max<int64_t>(1, n / 4096));
  if (nt <= 1) {
    f(0, n);
    return;
  }
  std::vector<std::thread> th;
  const int64_t chunk = (n + nt - 1) / nt;
  for (int t = 0; t < nt; ++t) {
    const int64_t lo = t * chunk, hi = std::min(n, lo + chunk);
    if (lo >= hi) break;
    th.emplace_back([=] { f(lo, hi); });
  }
  for (auto& x : th) x.join();
}

// Scratch of the exact VJP: the theta and u_ref_inv cotangents.
constexpr int kVjpAux = 3 * GALES_MAX_COMP + GALES_MAX_ND;
// Chunks of the interior pass.  On this GPU an FP64 instruction occupies the FMA
// pipe that the FP32 instructions issue to, so the FP64-bound point stage and the
// FP32 matrix stage gain nothing from sharing an SM: each chunk runs the point kernel
// over all its elements, then the persistent matrix kernel, on the caller's stream.
// Chunks are as large as kRecordBytes of point records allow (the whole mesh for the
// 1.0M-tet workload), so that few launch tails remain; the records go through DRAM,
// which the compute-bound stages leave mostly idle.  A host-buffer call cuts the pass
// into chunks that shrink toward its end, after each of which the finished CSR rows
// are copied.
constexpr size_t kRecordBytes = size_t(3) << 30;
constexpr int kCopyTail = 64;    // smallest host-buffer chunk: n / kCopyTail elements
constexpr int kCopyEvents = 24;  // row copies per host-buffer assembly (at most)

GeometryOps geometry_ops(int dim, int nen) {
  if (dim == 2 && nen == 3) return geometry_ops_tri3();
  if (dim == 2 && nen == 4) return geometry_ops_quad4();
  if (dim == 3 && nen == 4) return geometry_ops_tet4();
  return geometry_ops_hex8();
}

// Shape functions at a reference point (quad.hpp:153-187, 476-514); products and sums
// only, so host and device evaluate them identically.
void shape_values(int dim, int nen, const double* pt, double* sh) {
  const double xi = pt[0], eta = pt[1], zeta = pt[2];
  if (dim == 2 && nen == 3) {
    sh[0] = 1.0 - xi - eta; sh[1] = xi; sh[2] = eta;
  } else if (dim == 2 && nen == 4) {
    sh[0] = 0.25 * (1.0 - xi) * (1.0 - eta);
    sh[1] = 0.25 * (1.0 + xi) * (1.0 - eta);
    sh[2] = 0.25 * (1.0 + xi) * (1.0 + eta);
    sh[3] = 0.25 * (1.0 - xi) * (1.0 + eta);
  } else if (dim == 3 && nen == 4) {
    sh[0] = 1.0 - xi - eta - zeta; sh[1] = xi; sh[2] = eta; sh[3] = zeta;
  } else {
    const double sx[8] = {-1, 1, 1, -1, -1, 1, 1, -1};
    const double sy[8] = {-1, -1, 1, 1, -1, -1, 1, 1};
    const double sz[8] = {-1, -1, -1, -1, 1, 1, 1, 1};
    for (int i = 0; i < 8; ++i) {
      const double ax = sx[i] < 0 ? (1.0 - xi) : (1.0 + xi);
      const double ay = sy[i] < 0 ? (1.0 - eta) : (1.0 + eta);
      const double az = sz[i] < 0 ? (1.0 - zeta) : (1.0 + zeta);
      sh[i] = 0.125 * ax * ay * az;
    }
  }
}

InteriorOps interior_ops(int dim, int nen, int form) {
  const bool f64 = form == GALES_FORM_FP64;
  if (dim == 2 && nen == 3) return f64 ? interior_ops_tri3_fp64() : interior_ops_tri3_mixed();
  if (dim == 2 && nen == 4) return f64 ? interior_ops_quad4_fp64() : interior_ops_quad4_mixed();
  if (dim == 3 && nen == 4) return f64 ? interior_ops_tet4_fp64() : interior_ops_tet4_mixed();
  return f64 ? interior_ops_hex8_fp64() : interior_ops_hex8_mixed();
}

}  // namespace

struct gales_asm {
  int device = 0;
  int dim = 0, nen = 0, nc = 0, nd = 0;
  int64_t n_nodes = 0, n_el = 0, n_rows = 0, nnz = 0, nnz_nodes = 0;
  ElemInfo ei;
  gales_material_desc mat;
  gales_setup_desc setup;
  double u_ref_inv[GALES_MAX_ND];
  // host copies
  std::vector<int32_t> conn;
  std::vector<int32_t> node_flag;
  std::vector<int64_t> node_rp;
  std::vector<int32_t> node_col;
  std::vector<int64_t> row_ptr;   // scalar CSR, built on request
  std::vector<int32_t> col;
  std::vector<int32_t> colour;
  int32_t n_colours = 0;
  std::vector<int32_t> colour_order;  // elements sorted by colour
  std::vector<int32_t> sweep;         // elements along a Morton curve of their centroids
  // host-buffer calls: elements grouped by the bucket of their lowest node (Morton order
  // inside a bucket), so that finished CSR rows form a growing prefix that is copied to
  // the host while later chunks run
  std::vector<int32_t> sweep_rows;
  std::vector<int64_t> bucket_end;    // end (exclusive) of each bucket in sweep_rows
  int64_t bucket_nodes = 1;
  std::vector<int64_t> colour_off;
  std::vector<int32_t> bd_list;
  std::vector<int8_t> bd_sides;
  std::vector<int8_t> el_sides;  // side flags of every element [n_el][nsides]
  // flagged side points of the boundary elements, grouped by element
  std::vector<int32_t> bpt_off, bpt_el, bpt_ip;
  // device
  DevBuf<double> d_coords;
  DevBuf<int32_t> d_conn, d_node_flag, d_colour_order, d_bd_list, d_sweep, d_sweep_rows;
  DevBuf<int64_t> d_node_rp;
  DevBuf<uint16_t> d_slot;
  DevBuf<int8_t> d_bd_sides;
  DevBuf<int32_t> d_bpt_off, d_bpt_el, d_bpt_ip;
  DevBuf<unsigned char> d_bgeo, d_bpt_rec;
  DevBuf<gales_side_bc> d_side_bc;
  DevBuf<unsigned int> d_status;
  DevBuf<unsigned long long> d_first_bad;
  DevBuf<double> s_I, s_P, s_vals, s_rhs, s_aux, s_lam, s_th;  // staging for host pointers
  DevBuf<double> d_vjp;                          // theta and u_ref_inv cotangents of the exact VJP
  double* h_vjp = nullptr;                       // pinned copy of d_vjp
  unsigned int* h_status = nullptr;              // pinned
  unsigned long long* h_first_bad = nullptr;
  double* h_aux = nullptr;                       // pinned scalar
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  cudaEvent_t evp[4] = {nullptr, nullptr, nullptr, nullptr};  // clear | interior | boundary | end
  cudaEvent_t evs[2] = {nullptr, nullptr};  // end of the first chunk's point and matrix stages
  int32_t scatter_mode = GALES_SCATTER_ATOMIC;
  // interior pass: point-record chunk buffers (scratch) and, for the FP64 form, two
  // internal streams
  InteriorOps ops[2];
  // magma mixtures (gales_asm_set_magma): the kernels compiled with the magma EOS replace
  // ops[] while a magma material is attached; ops_ch keeps the chemicals' kernels
  InteriorOps ops_ch[2];
  const magma_mix::DevMagma* mg = nullptr;
  MagmaOps mops{};
  DevBuf<unsigned char> qpbuf;          // point records of one chunk
  long long chunk_elems[2] = {1, 1};   // elements per chunk, per form
  long long chunk_default[2] = {1, 1};  // the chunk the record buffer was sized for
  int sms = 1;                          // multiprocessors of the device
  DevBuf<unsigned char> d_geo;   // element geometry at the interior points (mesh.hpp:468-495)
  cudaStream_t bst = nullptr;                  // boundary pass, concurrent with the interior
  cudaStream_t cst = nullptr;                  // device-to-host copies of finished CSR rows
  cudaEvent_t ev_copy[kCopyEvents] = {};
  cudaEvent_t ev_cjoin = nullptr;
  cudaEvent_t ev_bfork = nullptr, ev_bjoin = nullptr;
  int status = 0;
  int64_t first_bad = -1;
  double last_ms = 0.0;
  int64_t launches = 0;
  std::string err;
};

namespace {

int fail(gales_asm* h, int code, const std::string& msg) {
  if (h) {
    h->err = msg;
    h->status = code;
  }
  return code;
}

int cuda_fail(gales_asm* h, cudaError_t e, const char* what) {
  return fail(h, GALES_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define CK(h, call, what)                          \
  do {                                             \
    cudaError_t e__ = (call);                      \
    if (e__ != cudaSuccess) return cuda_fail(h, e__, what); \
  } while (0)

bool is_device_ptr(const void* p) {
  if (!p) return false;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// Page-locked host memory (cudaHostAlloc or registered): copies into it run
// asynchronously, so they may overlap the assembly.
bool is_pinned_host_ptr(const void* p) {
  if (!p) return false;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeHost;
}

// Reference fluid properties at the dc_2006 reference state (fluid_2d.hpp:123-135):
// props at (p_ref, T_ref, Y = 0.5 for every component), U at v_ref.
void u_ref_inv_from(gales_asm* h, double rho, double cv);

void compute_u_ref_inv(gales_asm* h) {
  for (int i = 0; i < GALES_MAX_ND; ++i) h->u_ref_inv[i] = 0.0;
  if (!h->setup.dc_2006) return;
  const int nc = h->nc;
  const double p = h->setup.p_ref, T = h->setup.T_ref;
  double rho = 0.0, cv = 0.0;
  for (int c = 0; c < nc; ++c) {
    const gales_chemical_desc& q = h->mat.comp[c];
    double r, v;
    if (q.kind == GALES_CH_CUSTOM) {
      r = q.rho;
      v = (q.beta == 0.0) ? q.cp : q.cp - T * q.alpha * q.alpha / (r * q.beta);
    } else {
      r = p / (q.R * T);
      v = q.cv;
    }
    rho += 0.5 / r;
    cv += 0.5 * v;
  }
  rho = 1. / rho;
  u_ref_inv_from(h, rho, cv);
}

// U at (rho, cv, T_ref, v_ref, Y_ref = 0.5) and its inverse where U >= DBL_EPSILON.
void u_ref_inv_from(gales_asm* h, double rho, double cv) {
  for (int i = 0; i < GALES_MAX_ND; ++i) h->u_ref_inv[i] = 0.0;
  if (!h->setup.dc_2006) return;
  const int nc = h->nc, dim = h->dim;
  const double T = h->setup.T_ref;
  double v2 = 0.0;
  for (int k = 0; k < dim; ++k) v2 += h->setup.v_ref[k] * h->setup.v_ref[k];
  const double E = cv * T + 0.5 * (v2);
  double u[GALES_MAX_ND];
  u[0] = rho;
  for (int k = 0; k < dim; ++k) u[1 + k] = rho * h->setup.v_ref[k];
  u[dim + 1] = rho * E;
  for (int i = 0; i < nc - 1; ++i) u[dim + 2 + i] = rho * 0.5;
  for (int i = 0; i < h->nd; ++i) h->u_ref_inv[i] = (u[i] < DBL_EPSILON) ? 0.0 : 1.0 / u[i];
}

// Reverse of compute_u_ref_inv: the cotangents urib of u_ref_inv = 1/U_ref, with U_ref
// the conservative vector of the mixture at (p_ref, T_ref, v_ref, Y_ref = 0.5), folded
// into the parameter cotangents th (theta_c = (density parameter, mu_c, cp_c); the
// density parameter of an ideal gas is its molar mass, R = R_u/M, cv = cp - R).
void u_ref_inv_reverse(const gales_asm* h, const double* urib, double* th) {
  if (!h->setup.dc_2006) return;
  const int nc = h->nc, dim = h->dim;
  const double p = h->setup.p_ref, T = h->setup.T_ref;
  double irho = 0.0, cv = 0.0, r[GALES_MAX_COMP], vc[GALES_MAX_COMP];
  for (int c = 0; c < nc; ++c) {
    const gales_chemical_desc& q = h->mat.comp[c];
    if (q.kind == GALES_CH_CUSTOM) {
      r[c] = q.rho;
      vc[c] = (q.beta == 0.0) ? q.cp : q.cp - T * q.alpha * q.alpha / (r[c] * q.beta);
    } else {
      r[c] = p / (q.R * T);
      vc[c] = q.cv;
    }
    irho += 0.5 / r[c];
    cv += 0.5 * vc[c];
  }
  const double rho = 1.0 / irho;
  double v2 = 0.0;
  for (int k = 0; k < dim; ++k) v2 += h->setup.v_ref[k] * h->setup.v_ref[k];
  const double E = cv * T + 0.5 * v2;
  // u = (rho, rho v_ref, rho E, rho/2 ...); u_ref_inv = 1/u where u >= eps
  double rhob = 0.0, Eb = 0.0;
  for (int j = 0; j < h->nd; ++j) {
    const double uri = h->u_ref_inv[j];
    if (uri == 0.0) continue;
    const double ub = -urib[j] * uri * uri;
    if (j == 0) rhob += ub;
    else if (j <= dim) rhob += ub * h->setup.v_ref[j - 1];
    else if (j == dim + 1) { rhob += ub * E; Eb += ub * rho; }
    else rhob += ub * 0.5;
  }
  const double cvb = Eb * T;
  for (int c = 0; c < nc; ++c) {
    const gales_chemical_desc& q = h->mat.comp[c];
    const double rb = rhob * rho * rho * 0.5 / (r[c] * r[c]);
    const double vb = 0.5 * cvb;
    if (q.kind == GALES_CH_CUSTOM) {
      th[3 * c + 0] += rb;
      if (q.beta != 0.0) th[3 * c + 0] += vb * T * q.alpha * q.alpha / (r[c] * r[c] * q.beta);
      th[3 * c + 2] += vb;
    } else {
      double Rb = rb * (-r[c] / q.R) - vb;
      th[3 * c + 2] += vb;
      th[3 * c + 0] += Rb * (-q.R * q.R / 8.314462);
    }
  }
}

// Node graph of linear_system.hpp:46-63 on one rank: sorted unique neighbours.
void build_graph(gales_asm* h) {
  const int nen = h->nen;
  const int64_t nn = h->n_nodes, ne = h->n_el;
  std::vector<int64_t> cnt(nn + 1, 0);
  for (int64_t e = 0; e < ne; ++e)
    for (int a = 0; a < nen; ++a) cnt[h->conn[e * nen + a] + 1] += 1;
  for (int64_t i = 0; i < nn; ++i) cnt[i + 1] += cnt[i];
  std::vector<int64_t> el_of(cnt[nn]);
  {
    std::vector<int64_t> fill(cnt.begin(), cnt.end() - 1);
    for (int64_t e = 0; e < ne; ++e)
      for (int a = 0; a < nen; ++a) el_of[fill[h->conn[e * nen + a]]++] = e;
  }
  std::vector<int32_t> deg(nn, 0);
  std::vector<std::vector<int32_t>> rows(nn);
  parallel_for(nn, [&](int64_t lo, int64_t hi) {
    std::vector<int32_t> tmp;
    for (int64_t i = lo; i < hi; ++i) {
      tmp.clear();
      for (int64_t t = cnt[i]; t < cnt[i + 1]; ++t) {
        const int64_t e = el_of[t];
        for (int b = 0; b < nen; ++b) tmp.push_back(h->conn[e * nen + b]);
      }
      std::sort(tmp.begin(), tmp.end());
      tmp.erase(std::unique(tmp.begin(), tmp.end()), tmp.end());
      rows[i] = tmp;
      deg[i] = (int32_t)tmp.size();
    }
  });
  h->node_rp.assign(nn + 1, 0);
  for (int64_t i = 0; i < nn; ++i) h->node_rp[i + 1] = h->node_rp[i] + deg[i];
  h->nnz_nodes = h->node_rp[nn];
  h->node_col.resize(h->nnz_nodes);
  parallel_for(nn, [&](int64_t lo, int64_t hi) {
    for (int64_t i = lo; i < hi; ++i) {
      std::copy(rows[i].begin(), rows[i].end(), h->node_col.begin() + h->node_rp[i]);
      std::vector<int32_t>().swap(rows[i]);
    }
  });
  h->nnz = h->nnz_nodes * (int64_t)h->nd * h->nd;
}

// Greedy colouring in element order (the oracle states the same rule).
void build_colouring(gales_asm* h) {
  const int nen = h->nen;
  const int64_t nn = h->n_nodes, ne = h->n_el;
  std::vector<int64_t> cnt(nn + 1, 0);
  for (int64_t e = 0; e < ne; ++e)
    for (int a = 0; a < nen; ++a) cnt[h->conn[e * nen + a] + 1] += 1;
  for (int64_t i = 0; i < nn; ++i) cnt[i + 1] += cnt[i];
  std::vector<int64_t> el_of(cnt[nn]);
  {
    std::vector<int64_t> fill(cnt.begin(), cnt.end() - 1);
    for (int64_t e = 0; e < ne; ++e)
      for (int a = 0; a < nen; ++a) el_of[fill[h->conn[e * nen + a]]++] = e;
  }
  h->colour.assign(ne, -1);
  std::vector<int64_t> mark(64, -1);
  int32_t ncol = 0;
  for (int64_t e = 0; e < ne; ++e) {
    for (int a = 0; a < nen; ++a) {
      const int32_t n = h->conn[e * nen + a];
      for (int64_t t = cnt[n]; t < cnt[n + 1]; ++t) {
        const int32_t c = h->colour[el_of[t]];
        if (c >= 0) {
          if ((size_t)c >= mark.size()) mark.resize(2 * c + 1, -1);
          mark[c] = e;
        }
      }
    }
    int32_t c = 0;
    while ((size_t)c < mark.size() && mark[c] == e) ++c;
    if ((size_t)c >= mark.size()) mark.resize(2 * c + 1, -1);
    h->colour[e] = c;
    ncol = std::max(ncol, c + 1);
  }
  h->n_colours = ncol;
  h->colour_off.assign(ncol + 1, 0);
  for (int64_t e = 0; e < ne; ++e) h->colour_off[h->colour[e] + 1] += 1;
  for (int c = 0; c < ncol; ++c) h->colour_off[c + 1] += h->colour_off[c];
  h->colour_order.resize(ne);
  std::vector<int64_t> fill(h->colour_off.begin(), h->colour_off.end() - 1);
  for (int64_t e = 0; e < ne; ++e) h->colour_order[fill[h->colour[e]]++] = (int32_t)e;
}

// Processing order of the atomic scatter: elements sorted by the Morton code of their
// centroid (21 bits per axis in 3D, 32 in 2D, over the mesh bounding box).  Elements
// that follow one another then share nodes, so the CSR rows they add into stay in L2
// while a chunk runs.  The order changes only the order of the FP64 additions.
uint64_t spread_bits(uint64_t x, int dim) {
  if (dim == 2) {
    x &= 0xffffffffull;
    x = (x | (x << 16)) & 0x0000ffff0000ffffull;
    x = (x | (x << 8)) & 0x00ff00ff00ff00ffull;
    x = (x | (x << 4)) & 0x0f0f0f0f0f0f0f0full;
    x = (x | (x << 2)) & 0x3333333333333333ull;
    x = (x | (x << 1)) & 0x5555555555555555ull;
    return x;
  }
  x &= 0x1fffffull;
  x = (x | (x << 32)) & 0x1f00000000ffffull;
  x = (x | (x << 16)) & 0x1f0000ff0000ffull;
  x = (x | (x << 8)) & 0x100f00f00f00f00full;
  x = (x | (x << 4)) & 0x10c30c30c30c30c3ull;
  x = (x | (x << 2)) & 0x1249249249249249ull;
  return x;
}

void build_sweep(gales_asm* h, const double* coords) {
  const int dim = h->dim, nen = h->nen;
  double lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
  for (int d = 0; d < dim; ++d) lo[d] = hi[d] = coords[d];
  for (int64_t i = 0; i < h->n_nodes; ++i)
    for (int d = 0; d < dim; ++d) {
      lo[d] = std::min(lo[d], coords[i * dim + d]);
      hi[d] = std::max(hi[d], coords[i * dim + d]);
    }
  const double levels = dim == 3 ? 2097151.0 : 4294967295.0;
  std::vector<std::pair<uint64_t, int32_t>> key((size_t)h->n_el);
  parallel_for(h->n_el, [&](int64_t a, int64_t b) {
    for (int64_t e = a; e < b; ++e) {
      uint64_t code = 0;
      for (int d = 0; d < dim; ++d) {
        double c = 0.0;
        for (int n = 0; n < nen; ++n) c += coords[(int64_t)h->conn[e * nen + n] * dim + d];
        c /= nen;
        const double ext = hi[d] - lo[d];
        double u = ext > 0.0 ? (c - lo[d]) / ext : 0.0;
        u = std::min(1.0, std::max(0.0, u));
        code |= spread_bits((uint64_t)(u * levels), dim) << d;
      }
      key[e] = {code, (int32_t)e};
    }
  });
  std::sort(key.begin(), key.end());
  h->sweep.resize(h->n_el);
  for (int64_t e = 0; e < h->n_el; ++e) h->sweep[e] = key[e].second;
  // bucket of the lowest node of every element; stable sort of the Morton order by it
  h->bucket_nodes = std::max<int64_t>(1, (h->n_nodes + 127) / 128);
  const int64_t nb = (h->n_nodes + h->bucket_nodes - 1) / h->bucket_nodes;
  std::vector<int64_t> count(nb + 1, 0);
  std::vector<int32_t> bucket(h->n_el);
  for (int64_t e = 0; e < h->n_el; ++e) {
    int32_t lo_node = h->conn[e * nen];
    for (int n = 1; n < nen; ++n) lo_node = std::min(lo_node, h->conn[e * nen + n]);
    bucket[e] = (int32_t)(lo_node / h->bucket_nodes);
    ++count[bucket[e] + 1];
  }
  for (int64_t b = 0; b < nb; ++b) count[b + 1] += count[b];
  h->bucket_end.assign(count.begin() + 1, count.end());
  h->sweep_rows.resize(h->n_el);
  std::vector<int64_t> pos(count.begin(), count.end() - 1);
  for (int64_t i = 0; i < h->n_el; ++i) {
    const int32_t e = h->sweep[i];
    h->sweep_rows[pos[bucket[e]]++] = e;
  }
}

int validate(gales_asm* h, const gales_mesh_desc* m, const gales_material_desc* mat,
             const gales_setup_desc* s) {
  if (!m || !mat || !s) return fail(h, GALES_ERR_BAD_INPUT, "null descriptor");
  if (!elem_info(m->dim, m->nen, h->ei))
    return fail(h, GALES_ERR_UNSUPPORTED, "unsupported element (dim, nen)");
  if (mat->nb_comp < 1 || mat->nb_comp > 4)
    return fail(h, GALES_ERR_UNSUPPORTED, "nb_comp must be 1..4");
  if (m->n_nodes <= 0 || m->n_elements < 0 || !m->coords || (!m->conn && m->n_elements > 0))
    return fail(h, GALES_ERR_BAD_INPUT, "empty or null mesh arrays");
  if (m->n_nodes >= INT32_MAX) return fail(h, GALES_ERR_BAD_INPUT, "n_nodes exceeds int32 node ids");
  for (int64_t i = 0; i < m->n_elements * m->nen; ++i)
    if (m->conn[i] < 0 || m->conn[i] >= m->n_nodes)
      return fail(h, GALES_ERR_BAD_INPUT, "connectivity entry out of range at " + std::to_string(i));
  if (m->n_bd_sides > 0 && (!m->bd_side_el || !m->bd_side_local || !m->bd_side_flag))
    return fail(h, GALES_ERR_BAD_INPUT, "null boundary side arrays");
  for (int64_t i = 0; i < m->n_bd_sides; ++i) {
    if (m->bd_side_el[i] < 0 || m->bd_side_el[i] >= m->n_elements)
      return fail(h, GALES_ERR_BAD_INPUT, "boundary side element out of range");
    if (m->bd_side_local[i] < 0 || m->bd_side_local[i] >= h->ei.nsides)
      return fail(h, GALES_ERR_BAD_INPUT, "boundary side local index out of range");
    if (m->bd_side_flag[i] <= 0 || m->bd_side_flag[i] >= GALES_MAX_FLAGS)
      return fail(h, GALES_ERR_BAD_INPUT, "boundary side flag must be in 1..31");
  }
  for (int c = 0; c < mat->nb_comp; ++c) {
    const int k = mat->comp[c].kind;
    if (k != GALES_CH_CUSTOM && k != GALES_CH_IDEAL_GAS)
      return fail(h, GALES_ERR_UNSUPPORTED, "unknown chemical kind");
  }
  const int t = s->tau;
  if (t != GALES_TAU_NONE && t != 2001 && t != 2019 && t != 2007 && t != 2014)
    return fail(h, GALES_ERR_BAD_INPUT, "unknown tau variant");
  return 0;
}

}  // namespace

namespace {
KParams base_params(gales_asm* h, double dt);
LaunchResult dispatch_boundary(gales_asm* h, const KParams& k, int form, long long n, cudaStream_t st);

BoundaryInfo boundary_info(int dim, int nen, int nc) {
  if (dim == 2 && nen == 3) return boundary_info_tri3(nc);
  if (dim == 2 && nen == 4) return boundary_info_quad4(nc);
  if (dim == 3 && nen == 4) return boundary_info_tet4(nc);
  return boundary_info_hex8(nc);
}

// The boundary-point tables of the handle's boundary element list (k.el_list must be
// the handle's boundary list).
void set_boundary_points(gales_asm* h, KParams& k) {
  k.bpt_off = h->d_bpt_off.p;
  k.bpt_el = h->d_bpt_el.p;
  k.bpt_ip = h->d_bpt_ip.p;
  k.bgeo = h->d_bgeo.p;
  k.bpt_rec = h->bpt_el.empty() ? nullptr : h->d_bpt_rec.p;
  k.n_bpt = (int64_t)h->bpt_el.size();
}
}  // namespace

extern "C" {

void gales_chemical_custom(gales_chemical_desc* c, double rho, double mu, double cp, double kappa,
                           double alpha, double beta) {
  memset(c, 0, sizeof(*c));
  c->kind = GALES_CH_CUSTOM;
  c->rho = rho; c->mu = mu; c->cp = cp; c->kappa = kappa; c->alpha = alpha; c->beta = beta;
  c->cv = cp;
  c->chemical_diffusivity = 1.e-10;
}

void gales_chemical_ideal_gas(gales_chemical_desc* c, double molar_mass, double gamma) {
  memset(c, 0, sizeof(*c));
  c->kind = GALES_CH_IDEAL_GAS;
  c->R = 8.314462 / molar_mass;
  c->gamma = gamma;
  c->cv = c->R / (gamma - 1.0);
  c->cp = gamma * c->cv;
  c->mu = 1.e-5;
  c->kappa = c->mu * c->cp / 0.72;
  c->chemical_diffusivity = 1.e-10;
}

void gales_setup_default(gales_setup_desc* s, int32_t dim) {
  memset(s, 0, sizeof(*s));
  s->tau = GALES_TAU_NON_DIAG_COMP_2019;
  s->dc_2006 = 1;
  s->steady_state = 0;
  s->dc_sharp = 2.0;
  s->dc_scale_fact = 1.0;
  if (dim == 2) s->gravity[1] = -9.81;
  s->p_ref = 70.e6;
  s->T_ref = 1300.0;
}

int gales_asm_create(const gales_mesh_desc* m, const gales_material_desc* mat,
                     const gales_setup_desc* s, int device, gales_asm** out) {
  if (!out) return GALES_ERR_BAD_INPUT;
  *out = nullptr;
  gales_asm* h = new gales_asm();
  int rc = validate(h, m, mat, s);
  if (rc) {
    // keep the message reachable through a handle-less error path
    fprintf(stderr, "gales_asm_create: %s\n", h->err.c_str());
    delete h;
    return rc;
  }
  h->device = device;
  h->dim = m->dim; h->nen = m->nen; h->nc = mat->nb_comp;
  h->nd = 2 + h->dim + h->nc - 1;
  h->n_nodes = m->n_nodes; h->n_el = m->n_elements;
  h->n_rows = h->n_nodes * h->nd;
  h->mat = *mat;
  h->setup = *s;
  h->conn.assign(m->conn, m->conn + m->n_elements * m->nen);
  h->node_flag.assign(h->n_nodes, 0);
  if (m->node_flag) std::copy(m->node_flag, m->node_flag + h->n_nodes, h->node_flag.begin());
  compute_u_ref_inv(h);
  build_graph(h);
  // per-element slot table: position of node a within node b's graph row
  std::vector<uint16_t> slot((size_t)h->n_el * h->nen * h->nen);
  bool slot_ok = true;
  for (int64_t i = 0; i < h->n_nodes; ++i)
    if (h->node_rp[i + 1] - h->node_rp[i] > 65535) slot_ok = false;
  if (!slot_ok) {
    int code = fail(h, GALES_ERR_UNSUPPORTED, "node degree above 65535");
    fprintf(stderr, "gales_asm_create: %s\n", h->err.c_str());
    delete h;
    return code;
  }
  {
    const int nen = h->nen;
    parallel_for(h->n_el, [&](int64_t lo, int64_t hi) {
      for (int64_t e = lo; e < hi; ++e)
        for (int b = 0; b < nen; ++b) {
          const int32_t nb = h->conn[e * nen + b];
          const int32_t* r0 = h->node_col.data() + h->node_rp[nb];
          const int32_t* r1 = h->node_col.data() + h->node_rp[nb + 1];
          for (int a = 0; a < nen; ++a) {
            const int32_t na = h->conn[e * nen + a];
            slot[((size_t)e * nen + b) * nen + a] = (uint16_t)(std::lower_bound(r0, r1, na) - r0);
          }
        }
    });
  }
  build_colouring(h);
  build_sweep(h, m->coords);
  // boundary elements (fluid_assembly.hpp:57) and their side flags (mesh.hpp:409-446)
  {
    std::vector<int32_t> pos(h->n_el, -1);
    if (m->el_on_boundary)
      for (int64_t e = 0; e < h->n_el; ++e)
        if (m->el_on_boundary[e]) {
          pos[e] = (int32_t)h->bd_list.size();
          h->bd_list.push_back((int32_t)e);
        }
    h->bd_sides.assign(h->bd_list.size() * h->ei.nsides, 0);
    h->el_sides.assign((size_t)h->n_el * h->ei.nsides, 0);
    for (int64_t i = 0; i < m->n_bd_sides; ++i)
      h->el_sides[(size_t)m->bd_side_el[i] * h->ei.nsides + m->bd_side_local[i]] = (int8_t)m->bd_side_flag[i];
    for (int64_t i = 0; i < m->n_bd_sides; ++i) {
      const int32_t e = m->bd_side_el[i];
      if (pos[e] >= 0) h->bd_sides[(size_t)pos[e] * h->ei.nsides + m->bd_side_local[i]] = (int8_t)m->bd_side_flag[i];
    }
    h->bpt_off.assign(h->bd_list.size() + 1, 0);
    for (size_t li = 0; li < h->bd_list.size(); ++li) {
      for (int sd = 0; sd < h->ei.nsides; ++sd)
        if (h->bd_sides[li * h->ei.nsides + sd] > 0)
          for (int q = 0; q < h->ei.nqs; ++q) {
            h->bpt_el.push_back((int32_t)li);
            h->bpt_ip.push_back(sd * h->ei.nqs + q);
          }
      h->bpt_off[li + 1] = (int32_t)h->bpt_el.size();
    }
  }
  cudaError_t ce = cudaSetDevice(device);
  auto bail = [&](cudaError_t e, const char* what) {
    fprintf(stderr, "gales_asm_create: %s: %s\n", what, cudaGetErrorString(e));
    gales_asm_destroy(h);
    return GALES_ERR_CUDA;
  };
  if (ce != cudaSuccess) return bail(ce, "cudaSetDevice");
#define UP(buf, src, count, what)                                                              \
  do {                                                                                         \
    cudaError_t e_ = buf.alloc(count);                                                         \
    if (e_ != cudaSuccess) return bail(e_, what);                                              \
    if ((count) > 0) {                                                                         \
      e_ = cudaMemcpy(buf.p, src, (count) * sizeof(*buf.p), cudaMemcpyHostToDevice);           \
      if (e_ != cudaSuccess) return bail(e_, what);                                            \
    }                                                                                          \
  } while (0)
  UP(h->d_coords, m->coords, (size_t)h->n_nodes * h->dim, "coords");
  UP(h->d_conn, h->conn.data(), h->conn.size(), "conn");
  UP(h->d_node_flag, h->node_flag.data(), h->node_flag.size(), "node_flag");
  UP(h->d_node_rp, h->node_rp.data(), h->node_rp.size(), "node_rp");
  UP(h->d_slot, slot.data(), slot.size(), "slot");
  UP(h->d_colour_order, h->colour_order.data(), h->colour_order.size(), "colour_order");
  UP(h->d_sweep, h->sweep.data(), h->sweep.size(), "sweep");
  UP(h->d_sweep_rows, h->sweep_rows.data(), h->sweep_rows.size(), "row-order sweep");
  UP(h->d_bd_list, h->bd_list.data(), h->bd_list.size(), "bd_list");
  UP(h->d_bd_sides, h->bd_sides.data(), h->bd_sides.size(), "bd_sides");
  UP(h->d_bpt_off, h->bpt_off.data(), h->bpt_off.size(), "bpt_off");
  UP(h->d_bpt_el, h->bpt_el.data(), h->bpt_el.size(), "bpt_el");
  UP(h->d_bpt_ip, h->bpt_ip.data(), h->bpt_ip.size(), "bpt_ip");
  UP(h->d_side_bc, h->setup.side_bc, (size_t)GALES_MAX_FLAGS, "side_bc");
#undef UP
  if ((ce = h->d_status.alloc(1)) != cudaSuccess) return bail(ce, "status");
  if ((ce = h->d_first_bad.alloc(1)) != cudaSuccess) return bail(ce, "first_bad");
  if ((ce = cudaMallocHost(&h->h_status, sizeof(unsigned int))) != cudaSuccess) return bail(ce, "pinned");
  if ((ce = cudaMallocHost(&h->h_first_bad, sizeof(unsigned long long))) != cudaSuccess) return bail(ce, "pinned");
  if ((ce = cudaMallocHost(&h->h_aux, sizeof(double))) != cudaSuccess) return bail(ce, "pinned");
  if ((ce = cudaMallocHost(&h->h_vjp, kVjpAux * sizeof(double))) != cudaSuccess) return bail(ce, "pinned");
  if ((ce = cudaEventCreate(&h->ev0)) != cudaSuccess) return bail(ce, "event");
  if ((ce = cudaEventCreate(&h->ev1)) != cudaSuccess) return bail(ce, "event");
  for (int i = 0; i < 4; ++i)
    if ((ce = cudaEventCreate(&h->evp[i])) != cudaSuccess) return bail(ce, "event");
  for (int i = 0; i < 2; ++i)
    if ((ce = cudaEventCreate(&h->evs[i])) != cudaSuccess) return bail(ce, "event");
  if ((ce = cudaEventCreateWithFlags(&h->ev_bfork, cudaEventDisableTiming)) != cudaSuccess) return bail(ce, "event");
  if ((ce = cudaEventCreateWithFlags(&h->ev_bjoin, cudaEventDisableTiming)) != cudaSuccess) return bail(ce, "event");
  if ((ce = cudaStreamCreateWithFlags(&h->bst, cudaStreamNonBlocking)) != cudaSuccess) return bail(ce, "stream");
  if ((ce = cudaStreamCreateWithFlags(&h->cst, cudaStreamNonBlocking)) != cudaSuccess) return bail(ce, "stream");
  for (int i = 0; i < kCopyEvents; ++i)
    if ((ce = cudaEventCreateWithFlags(&h->ev_copy[i], cudaEventDisableTiming)) != cudaSuccess) return bail(ce, "event");
  if ((ce = cudaEventCreateWithFlags(&h->ev_cjoin, cudaEventDisableTiming)) != cudaSuccess) return bail(ce, "event");
  h->ops[GALES_FORM_FP64] = interior_ops(h->dim, h->nen, GALES_FORM_FP64);
  h->ops[GALES_FORM_MIXED] = interior_ops(h->dim, h->nen, GALES_FORM_MIXED);
  h->ops_ch[GALES_FORM_FP64] = h->ops[GALES_FORM_FP64];
  h->ops_ch[GALES_FORM_MIXED] = h->ops[GALES_FORM_MIXED];
  // the scatter descriptors in the point records hold CSR offsets in units of nd
  // values as 32-bit integers
  if (h->nnz_nodes * (int64_t)h->nd >= (int64_t(1) << 31)) {
    fprintf(stderr, "gales_asm_create: %lld node-graph entries x %d dofs exceed the 32-bit scatter offsets\n",
            (long long)h->nnz_nodes, h->nd);
    gales_asm_destroy(h);
    return GALES_ERR_UNSUPPORTED;
  }
  {  // chunk size per form (kRecordBytes of point records, a multiple of four elements);
     // one record buffer for the larger
    int sms = 0;
    if ((ce = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device)) != cudaSuccess)
      return bail(ce, "device attribute");
    h->sms = sms;
    size_t bytes = 0;
    for (int f = 0; f < 2; ++f) {
      const size_t rb = h->ops[f].rec_bytes(h->nc);
      if (rb == 0) continue;
      const long long cap = std::max<long long>(4, (long long)(kRecordBytes / rb) / 4 * 4);
      h->chunk_elems[f] = std::max<long long>(1, std::min<long long>(cap, std::max<int64_t>(h->n_el, 1)));
      h->chunk_default[f] = h->chunk_elems[f];
      // records are written in blocks of (elements per matrix CTA, at most 4) elements
      bytes = std::max(bytes, rb * (size_t)(h->chunk_elems[f] + 4));
    }
    if ((ce = h->qpbuf.alloc(std::max<size_t>(bytes, 16))) != cudaSuccess) return bail(ce, "point-record buffer");
  }
  for (int f = 0; f < 2; ++f) {  // kernel attributes, once, outside any stream capture
    if ((ce = h->ops[f].prepare(h->nc)) != cudaSuccess) return bail(ce, "kernel attributes");
    KParams k0;
    memset(&k0, 0, sizeof(k0));
    LaunchResult r = dispatch_boundary(h, k0, f, -1, 0);
    if (r.err != cudaSuccess) return bail(r.err, "kernel attributes");
  }
  {  // element geometry, once per mesh; an inverted element fails here as it does at mesh load
    GeometryOps g = geometry_ops(h->dim, h->nen);
    if ((ce = h->d_geo.alloc(g.bytes_per_element * (size_t)h->n_el)) != cudaSuccess) return bail(ce, "geometry");
    KParams k = base_params(h, 1.0);
    if ((ce = cudaMemset(h->d_status.p, 0, sizeof(unsigned int))) != cudaSuccess) return bail(ce, "status");
    if ((ce = cudaMemset(h->d_first_bad.p, 0xff, sizeof(unsigned long long))) != cudaSuccess) return bail(ce, "status");
    LaunchResult r = g.launch(h->d_coords.p, h->d_conn.p, k, h->d_geo.p, h->n_el, 0);
    if (r.err != cudaSuccess) return bail(r.err, "geometry kernel");
    h->launches += r.launches;
    if ((ce = cudaDeviceSynchronize()) != cudaSuccess) return bail(ce, "geometry kernel");
    unsigned int st = 0;
    unsigned long long fb = 0;
    cudaMemcpy(&st, h->d_status.p, sizeof(st), cudaMemcpyDeviceToHost);
    cudaMemcpy(&fb, h->d_first_bad.p, sizeof(fb), cudaMemcpyDeviceToHost);
    if (st) {
      fprintf(stderr, "gales_asm_create: Jacobian is not positive at element %llu (quad.hpp:215-218)\n", fb);
      gales_asm_destroy(h);
      return (int)st;
    }
  }
  {  // boundary side-point geometry and the point-record buffer of the boundary pass
    const BoundaryInfo bi = boundary_info(h->dim, h->nen, h->nc);
    const size_t nb = h->bpt_el.size();
    if ((ce = h->d_bgeo.alloc(bi.bgeo_bytes * nb)) != cudaSuccess) return bail(ce, "boundary geometry");
    const size_t rec = std::max(bi.rec_bytes[0], bi.rec_bytes[1]);
    if ((ce = h->d_bpt_rec.alloc(rec * nb)) != cudaSuccess) return bail(ce, "boundary records");
    KParams k = base_params(h, 1.0);
    k.el_list = h->d_bd_list.p;
    k.n_list = (int64_t)h->bd_list.size();
    k.bd_sides = h->d_bd_sides.p;
    set_boundary_points(h, k);
    LaunchResult r = bi.geometry(k, h->d_bgeo.p, 0);
    if (r.err != cudaSuccess) return bail(r.err, "boundary geometry kernel");
    h->launches += r.launches;
    if ((ce = cudaDeviceSynchronize()) != cudaSuccess) return bail(ce, "boundary geometry kernel");
    unsigned int st = 0;
    unsigned long long fb = 0;
    cudaMemcpy(&st, h->d_status.p, sizeof(st), cudaMemcpyDeviceToHost);
    cudaMemcpy(&fb, h->d_first_bad.p, sizeof(fb), cudaMemcpyDeviceToHost);
    if (st) {
      fprintf(stderr, "gales_asm_create: boundary Jacobian is not positive at element %llu (quad.hpp:215-218)\n", fb);
      gales_asm_destroy(h);
      return (int)st;
    }
  }
  cudaMemset(h->d_status.p, 0, sizeof(unsigned int));
  cudaMemset(h->d_first_bad.p, 0xff, sizeof(unsigned long long));
  *out = h;
  return 0;
}

void gales_asm_destroy(gales_asm* h) {
  if (!h) return;
  cudaSetDevice(h->device);
  h->d_coords.release(); h->d_conn.release(); h->d_node_flag.release();
  h->d_colour_order.release(); h->d_bd_list.release(); h->d_node_rp.release(); h->d_sweep.release();
  h->d_sweep_rows.release();
  h->d_slot.release(); h->d_bd_sides.release(); h->d_side_bc.release();
  h->d_bpt_off.release(); h->d_bpt_el.release(); h->d_bpt_ip.release(); h->d_bgeo.release(); h->d_bpt_rec.release();
  h->d_status.release(); h->d_first_bad.release(); h->d_geo.release();
  h->s_I.release(); h->s_P.release(); h->s_vals.release(); h->s_rhs.release(); h->s_aux.release();
  h->s_lam.release(); h->s_th.release();
  if (h->h_status) cudaFreeHost(h->h_status);
  if (h->h_first_bad) cudaFreeHost(h->h_first_bad);
  if (h->h_aux) cudaFreeHost(h->h_aux);
  if (h->h_vjp) cudaFreeHost(h->h_vjp);
  h->d_vjp.release();
  if (h->ev0) cudaEventDestroy(h->ev0);
  if (h->ev1) cudaEventDestroy(h->ev1);
  for (int i = 0; i < 4; ++i)
    if (h->evp[i]) cudaEventDestroy(h->evp[i]);
  for (int i = 0; i < 2; ++i)
    if (h->evs[i]) cudaEventDestroy(h->evs[i]);
  if (h->ev_bfork) cudaEventDestroy(h->ev_bfork);
  if (h->ev_bjoin) cudaEventDestroy(h->ev_bjoin);
  if (h->bst) cudaStreamDestroy(h->bst);
  if (h->cst) cudaStreamDestroy(h->cst);
  for (int i = 0; i < kCopyEvents; ++i)
    if (h->ev_copy[i]) cudaEventDestroy(h->ev_copy[i]);
  if (h->ev_cjoin) cudaEventDestroy(h->ev_cjoin);
  h->qpbuf.release();
  delete h;
}

int gales_asm_pattern(gales_asm* h, int64_t* n_rows, int64_t* nnz, const int64_t** row_ptr,
                      const int32_t** col) {
  if (!h) return GALES_ERR_BAD_INPUT;
  if (h->nnz > INT64_MAX / 2) return fail(h, GALES_ERR_UNSUPPORTED, "nnz overflow");
  if (h->row_ptr.empty()) {
    const int nd = h->nd;
    if ((int64_t)h->n_nodes * nd > INT32_MAX) return fail(h, GALES_ERR_UNSUPPORTED, "column ids exceed int32");
    h->row_ptr.resize(h->n_rows + 1);
    h->col.resize(h->nnz);
    h->row_ptr[0] = 0;
    for (int64_t i = 0; i < h->n_nodes; ++i) {
      const int64_t deg = h->node_rp[i + 1] - h->node_rp[i];
      for (int k = 0; k < nd; ++k) h->row_ptr[i * nd + k + 1] = h->node_rp[i] * nd * nd + (k + 1) * deg * nd;
    }
    parallel_for(h->n_nodes, [&](int64_t lo, int64_t hi) {
      for (int64_t i = lo; i < hi; ++i)
        for (int k = 0; k < nd; ++k) {
          int64_t p = h->row_ptr[i * nd + k];
          for (int64_t t = h->node_rp[i]; t < h->node_rp[i + 1]; ++t)
            for (int kk = 0; kk < nd; ++kk) h->col[p++] = h->node_col[t] * nd + kk;
        }
    });
  }
  if (n_rows) *n_rows = h->n_rows;
  if (nnz) *nnz = h->nnz;
  if (row_ptr) *row_ptr = h->row_ptr.data();
  if (col) *col = h->col.data();
  return 0;
}

int gales_asm_node_graph(gales_asm* h, int64_t* n_nodes, int64_t* nnz_nodes, const int64_t** node_row_ptr,
                         const int32_t** node_col) {
  if (!h) return GALES_ERR_BAD_INPUT;
  if (n_nodes) *n_nodes = h->n_nodes;
  if (nnz_nodes) *nnz_nodes = h->nnz_nodes;
  if (node_row_ptr) *node_row_ptr = h->node_rp.data();
  if (node_col) *node_col = h->node_col.data();
  return 0;
}

int gales_asm_colouring(gales_asm* h, int32_t* n_colours, const int32_t** colour) {
  if (!h) return GALES_ERR_BAD_INPUT;
  if (n_colours) *n_colours = h->n_colours;
  if (colour) *colour = h->colour.data();
  return 0;
}

int gales_asm_set_scatter(gales_asm* h, int32_t mode) {
  if (!h) return GALES_ERR_BAD_INPUT;
  if (mode != GALES_SCATTER_ATOMIC && mode != GALES_SCATTER_COLOURED)
    return fail(h, GALES_ERR_BAD_INPUT, "unknown scatter mode");
  h->scatter_mode = mode;
  return 0;
}

int gales_asm_set_chunk(gales_asm* h, int64_t elements) {
  if (!h) return GALES_ERR_BAD_INPUT;
  if (elements < 0) return fail(h, GALES_ERR_BAD_INPUT, "negative chunk size");
  for (int f = 0; f < 2; ++f) {
    if (elements == 0) {
      h->chunk_elems[f] = h->chunk_default[f];
    } else {
      const long long c = std::max<long long>(4, (long long)elements / 4 * 4);
      h->chunk_elems[f] = std::min<long long>(c, h->chunk_default[f]);
    }
  }
  return 0;
}

}  // extern "C"

namespace {

void fill_chem(const gales_chemical_desc& q, DevChem& d) {
  d.kind = q.kind;
  d.rho = q.rho; d.mu = q.mu; d.cp = q.cp; d.cv = q.cv; d.kappa = q.kappa;
  d.alpha = q.alpha; d.beta = q.beta; d.R = q.R; d.gamma = q.gamma; d.D = q.chemical_diffusivity;
  // ratios used by the mixed form's EOS
  d.inv_rho = q.kind == GALES_CH_CUSTOM ? 1.0 / q.rho : 0.0;
  d.beta_over_rho = q.kind == GALES_CH_CUSTOM ? q.beta / q.rho : 0.0;
  d.alpha_over_rho = q.kind == GALES_CH_CUSTOM ? q.alpha / q.rho : 0.0;
  d.cv_shift = (q.kind == GALES_CH_CUSTOM && q.beta != 0.0) ? q.alpha * q.alpha / (q.rho * q.beta) : 0.0;
  d.inv_R = q.kind == GALES_CH_IDEAL_GAS ? 1.0 / q.R : 0.0;
  d.R_over_gamma = q.kind == GALES_CH_IDEAL_GAS ? q.R / q.gamma : 0.0;
  d.inv_D = 1.0 / q.chemical_diffusivity;
  // 1/(rho^2 s^2) with s = 1/sqrt(rho beta), or 1e20 when beta = 0 (chemicals.hpp:43-47)
  d.c2_coef = q.kind == GALES_CH_CUSTOM ? (q.beta == 0.0 ? 1.e-40 * d.inv_rho * d.inv_rho : q.beta / q.rho) : 0.0;
}

KParams base_params(gales_asm* h, double dt) {
  KParams k;
  memset(&k, 0, sizeof(k));
  k.mg = h->mg;
  for (int c = 0; c < h->nc; ++c) {
    const gales_chemical_desc& q = h->mat.comp[c];
    fill_chem(q, k.ch[c]);
    if (q.kind == GALES_CH_IDEAL_GAS) k.has_gas = 1;
  }
  k.dt = dt;
  k.inv_dt = 1.0 / dt;
  k.dc_sharp = h->setup.dc_sharp;
  k.dc_scale = h->setup.dc_scale_fact;
  for (int d = 0; d < 3; ++d) k.gravity[d] = h->setup.gravity[d];
  for (int i = 0; i < GALES_MAX_ND; ++i) k.u_ref_inv[i] = h->u_ref_inv[i];
  for (int d = 0; d < 3; ++d) k.gravity_f[d] = (float)k.gravity[d];
  for (int i = 0; i < GALES_MAX_ND; ++i) k.u_ref_inv_f[i] = (float)k.u_ref_inv[i];
  k.inv_dt_f = (float)k.inv_dt;
  k.dc_scale_f = (float)k.dc_scale;
  memcpy(k.gp, h->ei.gp, sizeof(k.gp));
  memcpy(k.sgp, h->ei.sgp, sizeof(k.sgp));
  k.W_in = h->ei.W_in;
  for (int q = 0; q < h->ei.nq; ++q) {
    shape_values(h->dim, h->nen, h->ei.gp[q], k.sh_tab[q]);
    for (int i = 0; i < 8; ++i) k.sh_tab_f[q][i] = (float)k.sh_tab[q][i];  // round to nearest, as narrow_rn
  }
  k.geo = h->d_geo.p;
  k.W_bd = h->ei.W_bd;
  k.tau = h->setup.tau;
  k.dc_2006 = h->setup.dc_2006;
  k.steady = h->setup.steady_state;
  k.n_sides = h->ei.nsides;
  k.n_side_nodes = h->ei.nsn;
  k.n_side_q = h->ei.nqs;
  for (int i = 0; i < GALES_MAX_FLAGS; ++i) k.dirichlet_mask[i] = h->setup.dirichlet_mask[i];
  k.coords = h->d_coords.p;
  k.conn = h->d_conn.p;
  k.node_flag = h->d_node_flag.p;
  k.node_rp = h->d_node_rp.p;
  k.slot = h->d_slot.p;
  k.n_elements = h->n_el;
  k.side_bc = h->d_side_bc.p;
  k.status = h->d_status.p;
  k.first_bad = h->d_first_bad.p;
  k.sms = h->sms;
  return k;
}

// Device-to-host copy of the CSR values of a host-buffer call while the interior pass
// runs: with the elements in row order (sweep_rows), the node rows [0, K) are final
// once every element whose lowest node is below K has been assembled (an element adds
// only into the rows of its own nodes), i.e. once the buckets of those nodes are done;
// the boundary pass (another stream) must have finished too.  After a launch that
// finishes a large enough prefix, an event on the assembly stream releases the copy of
// the new rows on the copy stream.
struct RowCopy {
  double* host_vals;
  const double* dev_vals;
  int64_t copied_nodes = 0;   // node rows already sent
  size_t bucket = 0;          // first unfinished bucket
  int events = 0;             // copy events used
};

int copy_finished_rows(gales_asm* h, RowCopy& rc, int64_t elements_done, bool last, cudaStream_t st) {
  while (rc.bucket < h->bucket_end.size() && h->bucket_end[rc.bucket] <= elements_done) ++rc.bucket;
  const int64_t k = last ? h->n_nodes : std::min<int64_t>(h->n_nodes, (int64_t)rc.bucket * h->bucket_nodes);
  const int64_t piece = std::max<int64_t>(1, h->n_nodes / (kCopyEvents - 2));
  if (k <= rc.copied_nodes || (!last && k - rc.copied_nodes < piece)) return 0;
  if (rc.events >= kCopyEvents) return 0;
  cudaEvent_t ev = h->ev_copy[rc.events++];
  CK(h, cudaEventRecord(ev, st), "event");
  CK(h, cudaStreamWaitEvent(h->cst, ev, 0), "stream wait");
  const int64_t nd2 = (int64_t)h->nd * h->nd;
  const int64_t a = h->node_rp[rc.copied_nodes] * nd2, b = h->node_rp[k] * nd2;
  CK(h, cudaMemcpyAsync(rc.host_vals + a, rc.dev_vals + a, (size_t)(b - a) * sizeof(double), cudaMemcpyDeviceToHost,
                        h->cst),
     "copy rows");
  rc.copied_nodes = k;
  return 0;
}

// Interior pass over n listed elements (k.el_list, or elements 0..n-1): per chunk the
// point kernel, then the matrix kernel, on the caller's stream, with the optional
// device-to-host copy of finished rows (rc) after each chunk.  The arrays k.clear_*
// names are zeroed by the first chunk's point kernel only; after_first_point runs on
// the host once that launch is enqueued (before the first matrix launch).
int run_interior(gales_asm* h, const KParams& k, int form, bool want_m, long long n, cudaStream_t st,
                 RowCopy* rc = nullptr, bool stage_events = false,
                 const std::function<int()>* after_first_point = nullptr) {
  const InteriorOps& ops = h->ops[form];
  const size_t rb = ops.rec_bytes(h->nc);
  if (rb == 0) return fail(h, GALES_ERR_UNSUPPORTED, "no interior kernel for this element/component count");
  const long long chunk = h->chunk_elems[form];
  // host-buffer calls: chunks that shrink toward the end of the pass (a third of what
  // remains, down to n / 64), so that the rows copied after the last chunk are few
  const long long tail = std::max<long long>(4, (n + kCopyTail - 1) / kCopyTail / 4 * 4);
  void* buf = h->qpbuf.p;
  KParams kl;  // the later chunks' parameters: nothing left to clear
  const KParams* kp = &k;
  long long first = 0;
  for (long long c = 0; first < n; ++c) {
    long long cnt = chunk;
    if (rc) {
      const long long rem = n - first;
      cnt = rem <= 2 * tail ? rem : std::max(tail, (rem / 3 + 3) / 4 * 4);
      cnt = std::min(cnt, chunk);
    }
    cnt = std::min(cnt, n - first);
    LaunchResult r = ops.point(*kp, h->nc, buf, first, cnt, st);
    if (r.err != cudaSuccess) return cuda_fail(h, r.err, "point kernel");
    h->launches += r.launches;
    if (c == 0) {
      if (stage_events) CK(h, cudaEventRecord(h->evs[0], st), "event");
      if (after_first_point) {
        const int e = (*after_first_point)();
        if (e) return e;
      }
      if (k.clear_n[0] > 0 || k.clear_n[1] > 0) {
        kl = k;
        kl.clear_n[0] = kl.clear_n[1] = 0;
        kp = &kl;
      }
    }
    r = ops.matrix(*kp, h->nc, want_m, buf, first, cnt, st);
    if (r.err != cudaSuccess) return cuda_fail(h, r.err, "matrix kernel");
    h->launches += r.launches;
    if (stage_events && c == 0) CK(h, cudaEventRecord(h->evs[1], st), "event");
    if (rc) {
      const int e = copy_finished_rows(h, *rc, first + cnt, first + cnt >= n, st);
      if (e) return e;
    }
    first += cnt;
  }
  return 0;
}

LaunchResult dispatch_boundary(gales_asm* h, const KParams& k, int form, long long n, cudaStream_t st) {
  if (h->mg) return h->mops.boundary(k, h->nc, form, n, st);
  if (h->dim == 2 && h->nen == 3) return boundary_tri3(k, h->nc, form, n, st);
  if (h->dim == 2 && h->nen == 4) return boundary_quad4(k, h->nc, form, n, st);
  if (h->dim == 3 && h->nen == 4) return boundary_tet4(k, h->nc, form, n, st);
  return boundary_hex8(k, h->nc, form, n, st);
}

LaunchResult dispatch_adaptive_dt(gales_asm* h, const KParams& k, double cfl, double* dt_el, long long n,
                                  cudaStream_t st) {
  if (h->mg) return h->mops.adaptive_dt(k, h->nc, cfl, dt_el, n, st);
  if (h->dim == 2 && h->nen == 3) return adaptive_dt_tri3(k, h->nc, cfl, dt_el, n, st);
  if (h->dim == 2 && h->nen == 4) return adaptive_dt_quad4(k, h->nc, cfl, dt_el, n, st);
  if (h->dim == 3 && h->nen == 4) return adaptive_dt_tet4(k, h->nc, cfl, dt_el, n, st);
  return adaptive_dt_hex8(k, h->nc, cfl, dt_el, n, st);
}

LaunchResult dispatch_vjp(gales_asm* h, const KParams& k, bool boundary, long long n, cudaStream_t st) {
  if (h->dim == 2 && h->nen == 3) return boundary ? vjp_boundary_tri3(k, h->nc, n, st) : vjp_interior_tri3(k, h->nc, n, st);
  if (h->dim == 2 && h->nen == 4)
    return boundary ? vjp_boundary_quad4(k, h->nc, n, st) : vjp_interior_quad4(k, h->nc, n, st);
  if (h->dim == 3 && h->nen == 4) return boundary ? vjp_boundary_tet4(k, h->nc, n, st) : vjp_interior_tet4(k, h->nc, n, st);
  return boundary ? vjp_boundary_hex8(k, h->nc, n, st) : vjp_interior_hex8(k, h->nc, n, st);
}

// ||b||_2 of a vector (residual_check.hpp:48-51): per-block sums of squares in a fixed
// order, then one block adds the partials, so the result does not depend on timing.
constexpr int kNormBlocks = 256;

__global__ void __launch_bounds__(256) norm_partial_kernel(const double* __restrict__ x, long long n,
                                                            double* __restrict__ part) {
  __shared__ double sh[256];
  double s = 0.0;
  for (long long i = (long long)blockIdx.x * 256 + threadIdx.x; i < n; i += (long long)gridDim.x * 256)
    s = fma(x[i], x[i], s);
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

__global__ void __launch_bounds__(256) norm_final_kernel(double* part) {
  __shared__ double sh[256];
  sh[threadIdx.x] = part[threadIdx.x];
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[kNormBlocks] = sqrt(sh[0]);
}

// Zero fill of the CSR values and the rhs before the scatter adds into them, as a
// kernel of the library (one counted launch each, visible with the other kernels in a
// profile; it runs at copy bandwidth like cudaMemsetAsync).  16-byte stores on the
// 16-byte-aligned body, scalar stores for an unaligned head and an odd tail.
__global__ void __launch_bounds__(256) zero_kernel(double* __restrict__ p, long long n) {
  const long long head = (reinterpret_cast<uintptr_t>(p) & 15u) != 0 ? 1 : 0;
  const long long tid = (long long)blockIdx.x * 256 + threadIdx.x, stride = (long long)gridDim.x * 256;
  if (n <= 0) return;
  if (tid == 0 && head) p[0] = 0.0;
  const long long body = n - head;
  double2* q = reinterpret_cast<double2*>(p + head);
  for (long long i = tid; i < body / 2; i += stride) q[i] = make_double2(0.0, 0.0);
  if (tid == 0 && body > 0 && (body & 1)) p[n - 1] = 0.0;
}

cudaError_t launch_zero(double* p, long long n, int sms, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  const long long want = (n / 2 + 255) / 256;
  const int blocks = (int)std::max<long long>(1, std::min<long long>(want, 4LL * std::max(sms, 1)));
  zero_kernel<<<blocks, 256, 0, st>>>(p, n);
  return cudaGetLastError();
}

// First smallest value of x[0..n) (min_element), in two launches: per-block minima,
// then the minimum of those (partials kept in index order).
constexpr int kMinBlocks = 256;
__global__ void __launch_bounds__(256) min_partial_kernel(const double* __restrict__ x, long long n,
                                                          double* __restrict__ part) {
  __shared__ double sh[256];
  __shared__ int has[256];
  double m = 0.0;
  int any = 0;
  for (long long i = (long long)blockIdx.x * 256 + threadIdx.x; i < n; i += (long long)gridDim.x * 256) {
    const double v = x[i];
    if (!any || v < m) m = v;
    any = 1;
  }
  sh[threadIdx.x] = m;
  has[threadIdx.x] = any;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o && has[threadIdx.x + o] && (!has[threadIdx.x] || sh[threadIdx.x + o] < sh[threadIdx.x])) {
      sh[threadIdx.x] = sh[threadIdx.x + o];
      has[threadIdx.x] = 1;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    part[blockIdx.x] = sh[0];
    part[kMinBlocks + blockIdx.x] = has[0] ? 1.0 : 0.0;
  }
}

__global__ void __launch_bounds__(256) min_final_kernel(double* part) {
  __shared__ double sh[256];
  __shared__ int has[256];
  sh[threadIdx.x] = part[threadIdx.x];
  has[threadIdx.x] = part[kMinBlocks + threadIdx.x] != 0.0;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o && has[threadIdx.x + o] && (!has[threadIdx.x] || sh[threadIdx.x + o] < sh[threadIdx.x])) {
      sh[threadIdx.x] = sh[threadIdx.x + o];
      has[threadIdx.x] = 1;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) part[2 * kMinBlocks] = sh[0];
}

cudaError_t launch_norm2(const double* x, long long n, double* part, cudaStream_t st) {
  norm_partial_kernel<<<kNormBlocks, 256, 0, st>>>(x, n, part);
  norm_final_kernel<<<1, 256, 0, st>>>(part);
  return cudaGetLastError();
}

// Device-side body of one assembly on device pointers (no host synchronisation).
// With enqueue_only the call records no timing events and leaves the status word
// alone (it accumulates until gales_asm_sync), so it may be captured into a graph.
int run_assembly(gales_asm* h, const double* dI, const double* dP, double dt, int form, double* dvals,
                 double* drhs, cudaStream_t st, bool enqueue_only = false, RowCopy* rc = nullptr) {
  KParams k = base_params(h, dt);
  k.I = dI;
  k.P = dP;
  k.vals = dvals;
  k.rhs = drhs;
  k.scatter_mode = (h->scatter_mode == GALES_SCATTER_COLOURED) ? 1 : 0;
  const bool want_m = dvals != nullptr;
  const bool timed = !enqueue_only;
  if (timed) CK(h, cudaEventRecord(h->evp[0], st), "event");
  if (!enqueue_only) {
    CK(h, cudaMemsetAsync(h->d_status.p, 0, sizeof(unsigned int), st), "memset status");
    CK(h, cudaMemsetAsync(h->d_first_bad.p, 0xff, sizeof(unsigned long long), st), "memset first_bad");
  }
  // A and b start at zero.  A device-buffer call with the atomic scatter whose interior
  // pass is one chunk has its point kernel clear them beside its own work (it neither
  // reads nor writes them; the matrix and boundary stages, their first writers, come
  // after it); otherwise a clear kernel runs first.  Over several chunks the first
  // chunk's point kernel is too short to hide the clear.  A host-buffer call keeps the
  // clear kernel so that its boundary pass can start at once: the rows finished by the
  // first chunk are copied only once the boundary pass is done, and copying is what
  // bounds that call.
  const bool atomic = h->scatter_mode != GALES_SCATTER_COLOURED;
  const bool fold_clear = atomic && h->n_el > 0 && h->n_el <= h->chunk_elems[form] && rc == nullptr;
  if (fold_clear) {
    k.clear_p[0] = dvals;
    k.clear_n[0] = dvals ? h->nnz : 0;
    k.clear_p[1] = drhs;
    k.clear_n[1] = h->n_rows;
  } else {
    if (dvals) {
      CK(h, launch_zero(dvals, h->nnz, h->sms, st), "zero vals");
      ++h->launches;
    }
    CK(h, launch_zero(drhs, h->n_rows, h->sms, st), "zero rhs");
    ++h->launches;
  }
  if (timed) CK(h, cudaEventRecord(h->evp[1], st), "event");
  // boundary pass (fluid_assembly.hpp:57-63): always atomics, since boundary elements
  // of one colour may still share nodes.  With the atomic interior scatter the two
  // passes only add into A and b, so the boundary pass runs on its own stream beside
  // the interior chunks, from the end of the first point launch when that launch
  // clears A and b, else from the start; with the coloured (plain read-modify-write)
  // scatter it waits for the interior.
  const bool has_bd = !h->bd_list.empty();
  const bool bd_concurrent = has_bd && atomic;
  KParams kb = k;
  kb.scatter_mode = 0;
  kb.el_list = h->d_bd_list.p;
  kb.n_list = (int64_t)h->bd_list.size();
  kb.bd_sides = h->d_bd_sides.p;
  kb.clear_n[0] = kb.clear_n[1] = 0;
  set_boundary_points(h, kb);
  const std::function<int()> fork_boundary = [&]() -> int {
    CK(h, cudaEventRecord(h->ev_bfork, st), "event");
    CK(h, cudaStreamWaitEvent(h->bst, h->ev_bfork, 0), "stream wait");
    LaunchResult r = dispatch_boundary(h, kb, form, kb.n_list, h->bst);
    if (r.err != cudaSuccess) return cuda_fail(h, r.err, "boundary kernel");
    h->launches += r.launches;
    CK(h, cudaEventRecord(h->ev_bjoin, h->bst), "event");
    // finished rows may be copied only once the boundary pass has added into them
    if (rc) CK(h, cudaStreamWaitEvent(h->cst, h->ev_bjoin, 0), "stream wait");
    return 0;
  };
  if (bd_concurrent && !fold_clear) {
    const int e = fork_boundary();
    if (e) return e;
  }
  if (h->scatter_mode == GALES_SCATTER_COLOURED) {
    for (int c = 0; c < h->n_colours; ++c) {
      KParams kc = k;
      kc.el_list = h->d_colour_order.p + h->colour_off[c];
      kc.n_list = h->colour_off[c + 1] - h->colour_off[c];
      int rc = run_interior(h, kc, form, want_m, kc.n_list, st);
      if (rc) return rc;
    }
  } else {
    k.el_list = rc ? h->d_sweep_rows.p : h->d_sweep.p;
    k.n_list = h->n_el;
    int e = run_interior(h, k, form, want_m, h->n_el, st, rc, timed,
                         (bd_concurrent && fold_clear) ? &fork_boundary : nullptr);
    if (e) return e;
  }
  if (timed) CK(h, cudaEventRecord(h->evp[2], st), "event");
  if (bd_concurrent) {
    CK(h, cudaStreamWaitEvent(st, h->ev_bjoin, 0), "stream wait");
  } else if (has_bd) {
    LaunchResult r = dispatch_boundary(h, kb, form, kb.n_list, st);
    if (r.err != cudaSuccess) return cuda_fail(h, r.err, "boundary kernel");
    h->launches += r.launches;
  }
  if (timed) CK(h, cudaEventRecord(h->evp[3], st), "event");
  return 0;
}

int finish(gales_asm* h, cudaStream_t st) {
  CK(h, cudaMemcpyAsync(h->h_status, h->d_status.p, sizeof(unsigned int), cudaMemcpyDeviceToHost, st), "status");
  CK(h, cudaMemcpyAsync(h->h_first_bad, h->d_first_bad.p, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st),
     "first_bad");
  CK(h, cudaStreamSynchronize(st), "synchronize");
  h->status = (int)*h->h_status;
  h->first_bad = (*h->h_first_bad == ULLONG_MAX) ? -1 : (int64_t)*h->h_first_bad;
  if (h->status) {
    char buf[160];
    snprintf(buf, sizeof(buf), "kernel status 0x%x at element %lld", h->status, (long long)h->first_bad);
    h->err = buf;
  } else {
    h->err.clear();
  }
  return h->status;
}

int assemble_impl(gales_asm* h, const double* I, const double* P, double dt, int32_t form, double* vals,
                  double* rhs, void* stream) {
  if (!h) return GALES_ERR_BAD_INPUT;
  if (!I || !P || !rhs) return fail(h, GALES_ERR_BAD_INPUT, "null state or rhs pointer");
  if (form != GALES_FORM_FP64 && form != GALES_FORM_MIXED) return fail(h, GALES_ERR_BAD_INPUT, "unknown form");
  if (!(dt > 0.0)) return fail(h, GALES_ERR_BAD_INPUT, "dt must be positive");
  CK(h, cudaSetDevice(h->device), "cudaSetDevice");
  cudaStream_t st = (cudaStream_t)stream;
  const size_t sb = (size_t)h->n_rows * sizeof(double);
  const double* dI = I;
  const double* dP = P;
  double* dvals = vals;
  double* drhs = rhs;
  const bool hI = !is_device_ptr(I), hP = !is_device_ptr(P);
  const bool hV = vals && !is_device_ptr(vals), hR = !is_device_ptr(rhs);
  CK(h, cudaEventRecord(h->ev0, st), "event");
  if (hI) {
    CK(h, h->s_I.alloc(h->n_rows), "staging I");
    CK(h, cudaMemcpyAsync(h->s_I.p, I, sb, cudaMemcpyHostToDevice, st), "copy I");
    dI = h->s_I.p;
  }
  if (hP) {
    CK(h, h->s_P.alloc(h->n_rows), "staging P");
    CK(h, cudaMemcpyAsync(h->s_P.p, P, sb, cudaMemcpyHostToDevice, st), "copy P");
    dP = h->s_P.p;
  }
  if (hV) {
    CK(h, h->s_vals.alloc(h->nnz), "staging vals");
    dvals = h->s_vals.p;
  }
  if (hR) {
    CK(h, h->s_rhs.alloc(h->n_rows), "staging rhs");
    drhs = h->s_rhs.p;
  }
  // host CSR values: copied row prefix by row prefix while the interior pass runs chunk
  // by chunk (mixed form, atomic scatter, page-locked destination), else after the
  // assembly
  const bool pipelined =
      hV && form == GALES_FORM_MIXED && h->scatter_mode == GALES_SCATTER_ATOMIC && is_pinned_host_ptr(vals);
  RowCopy copy{vals, dvals};
  int rc = run_assembly(h, dI, dP, dt, form, dvals, drhs, st, false, pipelined ? &copy : nullptr);
  if (rc) return rc;
  if (pipelined) {
    if (copy.copied_nodes < h->n_nodes) {  // rows not sent during the pass (for instance no chunk)
      CK(h, cudaStreamWaitEvent(h->cst, h->ev_bjoin, 0), "stream wait");
      copy.events = 0;
      CK(h, cudaEventRecord(h->ev_copy[0], st), "event");
      CK(h, cudaStreamWaitEvent(h->cst, h->ev_copy[0], 0), "stream wait");
      const int64_t a = h->node_rp[copy.copied_nodes] * (int64_t)h->nd * h->nd;
      CK(h, cudaMemcpyAsync(vals + a, dvals + a, (size_t)(h->nnz - a) * sizeof(double), cudaMemcpyDeviceToHost,
                            h->cst),
         "copy rows");
    }
    CK(h, cudaEventRecord(h->ev_cjoin, h->cst), "event");
    CK(h, cudaStreamWaitEvent(st, h->ev_cjoin, 0), "stream wait");
  } else if (hV) {
    CK(h, cudaMemcpyAsync(vals, dvals, (size_t)h->nnz * sizeof(double), cudaMemcpyDeviceToHost, st), "copy vals");
  }
  if (hR) CK(h, cudaMemcpyAsync(rhs, drhs, sb, cudaMemcpyDeviceToHost, st), "copy rhs");
  CK(h, cudaEventRecord(h->ev1, st), "event");
  rc = finish(h, st);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, h->ev0, h->ev1);
  h->last_ms = ms;
  return rc;
}

}  // namespace

extern "C" {

int gales_asm_assemble(gales_asm* h, const double* I, const double* P, double dt, int32_t form, double* vals,
                       double* rhs, void* stream) {
  if (h && !vals) return fail(h, GALES_ERR_BAD_INPUT, "null vals pointer (use gales_asm_residual)");
  return assemble_impl(h, I, P, dt, form, vals, rhs, stream);
}

int gales_asm_residual(gales_asm* h, const double* I, const double* P, double dt, int32_t form, double* rhs,
                       void* stream) {
  return assemble_impl(h, I, P, dt, form, nullptr, rhs, stream);
}

int gales_asm_enqueue(gales_asm* h, const double* I, const double* P, double dt, int32_t form, double* vals,
                      double* rhs, void* stream) {
  if (!h) return GALES_ERR_BAD_INPUT;
  if (!I || !P || !rhs) return fail(h, GALES_ERR_BAD_INPUT, "null state or rhs pointer");
  if (form != GALES_FORM_FP64 && form != GALES_FORM_MIXED) return fail(h, GALES_ERR_BAD_INPUT, "unknown form");
  if (!(dt > 0.0)) return fail(h, GALES_ERR_BAD_INPUT, "dt must be positive");
  if (!is_device_ptr(I) || !is_device_ptr(P) || !is_device_ptr(rhs) || (vals && !is_device_ptr(vals)))
    return fail(h, GALES_ERR_BAD_INPUT, "gales_asm_enqueue takes device pointers only");
  CK(h, cudaSetDevice(h->device), "cudaSetDevice");
  return run_assembly(h, I, P, dt, form, vals, rhs, (cudaStream_t)stream, true);
}

int gales_asm_sync(gales_asm* h, void* stream) {
  if (!h) return GALES_ERR_BAD_INPUT;
  CK(h, cudaSetDevice(h->device), "cudaSetDevice");
  cudaStream_t st = (cudaStream_t)stream;
  int rc = finish(h, st);
  CK(h, cudaMemsetAsync(h->d_status.p, 0, sizeof(unsigned int), st), "memset status");
  CK(h, cudaMemsetAsync(h->d_first_bad.p, 0xff, sizeof(unsigned long long), st), "memset first_bad");
  CK(h, cudaStreamSynchronize(st), "synchronize");
  return rc;
}

int gales_asm_element_blocks(gales_asm* h, const double* I, const double* P, double dt, int32_t form,
                             int32_t which, const int32_t* elements, int64_t n, double* m_out, double* r_out,
                             void* stream) {
  if (!h) return GALES_ERR_BAD_INPUT;
  if (!I || !P || !elements || !r_out || n < 0) return fail(h, GALES_ERR_BAD_INPUT, "null argument");
  if (which != 0 && which != 1) return fail(h, GALES_ERR_BAD_INPUT, "which must be 0 or 1");
  if (form != GALES_FORM_FP64 && form != GALES_FORM_MIXED) return fail(h, GALES_ERR_BAD_INPUT, "unknown form");
  if (n == 0) return 0;
  for (int64_t i = 0; i < n; ++i)
    if (elements[i] < 0 || elements[i] >= h->n_el) return fail(h, GALES_ERR_BAD_INPUT, "element out of range");
  CK(h, cudaSetDevice(h->device), "cudaSetDevice");
  cudaStream_t st = (cudaStream_t)stream;
  const int N = h->nen * h->nd;
  const size_t sb = (size_t)h->n_rows * sizeof(double);
  const double* dI = I;
  const double* dP = P;
  if (!is_device_ptr(I)) {
    CK(h, h->s_I.alloc(h->n_rows), "staging I");
    CK(h, cudaMemcpyAsync(h->s_I.p, I, sb, cudaMemcpyHostToDevice, st), "copy I");
    dI = h->s_I.p;
  }
  if (!is_device_ptr(P)) {
    CK(h, h->s_P.alloc(h->n_rows), "staging P");
    CK(h, cudaMemcpyAsync(h->s_P.p, P, sb, cudaMemcpyHostToDevice, st), "copy P");
    dP = h->s_P.p;
  }
  DevBuf<int32_t> d_list;
  DevBuf<int8_t> d_sides;
  DevBuf<double> d_m, d_r;
  CK(h, d_list.alloc(n), "element list");
  CK(h, cudaMemcpy(d_list.p, elements, n * sizeof(int32_t), cudaMemcpyHostToDevice), "copy list");
  const bool hm = m_out && !is_device_ptr(m_out), hr = !is_device_ptr(r_out);
  double* dm = m_out;
  double* dr = r_out;
  if (hm) { CK(h, d_m.alloc((size_t)n * N * N), "m staging"); dm = d_m.p; }
  if (hr) { CK(h, d_r.alloc((size_t)n * N), "r staging"); dr = d_r.p; }
  KParams k = base_params(h, dt);
  k.I = dI;
  k.P = dP;
  k.el_list = d_list.p;
  k.n_list = n;
  k.local_m = dm;
  k.local_r = dr;
  k.vals = dm;
  CK(h, cudaMemsetAsync(h->d_status.p, 0, sizeof(unsigned int), st), "memset status");
  CK(h, cudaMemsetAsync(h->d_first_bad.p, 0xff, sizeof(unsigned long long), st), "memset first_bad");
  if (dm) CK(h, cudaMemsetAsync(dm, 0, (size_t)n * N * N * sizeof(double), st), "memset m");
  CK(h, cudaMemsetAsync(dr, 0, (size_t)n * N * sizeof(double), st), "memset r");
  LaunchResult r;
  if (which == 0) {
    int rc0 = run_interior(h, k, form, dm != nullptr, n, st);
    if (rc0) return rc0;
    r = {cudaSuccess, 0};
  } else {
    std::vector<int8_t> sides((size_t)n * h->ei.nsides);
    for (int64_t i = 0; i < n; ++i)
      for (int s2 = 0; s2 < h->ei.nsides; ++s2)
        sides[i * h->ei.nsides + s2] = h->el_sides[(size_t)elements[i] * h->ei.nsides + s2];
    CK(h, d_sides.alloc(sides.size()), "sides");
    CK(h, cudaMemcpy(d_sides.p, sides.data(), sides.size(), cudaMemcpyHostToDevice), "copy sides");
    k.bd_sides = d_sides.p;
    r = dispatch_boundary(h, k, form, n, st);
  }
  if (r.err != cudaSuccess) return cuda_fail(h, r.err, "element kernel");
  h->launches += r.launches;
  if (hm) CK(h, cudaMemcpyAsync(m_out, dm, (size_t)n * N * N * sizeof(double), cudaMemcpyDeviceToHost, st), "copy m");
  if (hr) CK(h, cudaMemcpyAsync(r_out, dr, (size_t)n * N * sizeof(double), cudaMemcpyDeviceToHost, st), "copy r");
  int rc = finish(h, st);
  d_list.release(); d_sides.release(); d_m.release(); d_r.release();
  return rc;
}

int gales_asm_vjp(gales_asm* h, const double* I, const double* P, double dt, const double* lambda, int32_t mode,
                  double* g_state, double* g_params, void* stream) {
  if (!h) return GALES_ERR_BAD_INPUT;
  if (!I || !P || !lambda || !g_state) return fail(h, GALES_ERR_BAD_INPUT, "null argument");
  if (mode != GALES_VJP_EXACT && mode != GALES_VJP_FROZEN) return fail(h, GALES_ERR_BAD_INPUT, "unknown VJP mode");
  if (!(dt > 0.0)) return fail(h, GALES_ERR_BAD_INPUT, "dt must be positive");
  if (mode == GALES_VJP_EXACT && h->setup.tau != GALES_TAU_NON_DIAG_COMP_2019 && h->setup.tau != GALES_TAU_NONE)
    return fail(h, GALES_ERR_UNSUPPORTED, "the exact VJP is available for tau 2019 and tau none");
  if (mode == GALES_VJP_EXACT && h->mg)
    return fail(h, GALES_ERR_UNSUPPORTED, "the exact VJP differentiates the chemicals' EOS, not magma mixtures");
  CK(h, cudaSetDevice(h->device), "cudaSetDevice");
  cudaStream_t st = (cudaStream_t)stream;
  const size_t sb = (size_t)h->n_rows * sizeof(double);
  const int npar = 3 * h->nc;
  const double* dI = I;
  const double* dP = P;
  const double* dlam = lambda;
  double* dg = g_state;
  double* dth = g_params;
  const bool hI = !is_device_ptr(I), hP = !is_device_ptr(P), hL = !is_device_ptr(lambda);
  const bool hG = !is_device_ptr(g_state), hT = g_params && !is_device_ptr(g_params);
  CK(h, cudaEventRecord(h->ev0, st), "event");
  if (hI) {
    CK(h, h->s_I.alloc(h->n_rows), "staging I");
    CK(h, cudaMemcpyAsync(h->s_I.p, I, sb, cudaMemcpyHostToDevice, st), "copy I");
    dI = h->s_I.p;
  }
  if (hP) {
    CK(h, h->s_P.alloc(h->n_rows), "staging P");
    CK(h, cudaMemcpyAsync(h->s_P.p, P, sb, cudaMemcpyHostToDevice, st), "copy P");
    dP = h->s_P.p;
  }
  if (hL) {
    CK(h, h->s_lam.alloc(h->n_rows), "staging lambda");
    CK(h, cudaMemcpyAsync(h->s_lam.p, lambda, sb, cudaMemcpyHostToDevice, st), "copy lambda");
    dlam = h->s_lam.p;
  }
  if (hG) {
    CK(h, h->s_rhs.alloc(h->n_rows), "staging g_state");
    dg = h->s_rhs.p;
  }
  CK(h, cudaMemsetAsync(h->d_status.p, 0, sizeof(unsigned int), st), "memset status");
  CK(h, cudaMemsetAsync(h->d_first_bad.p, 0xff, sizeof(unsigned long long), st), "memset first_bad");
  CK(h, cudaMemsetAsync(dg, 0, sb, st), "memset g_state");
  const bool want_th = mode == GALES_VJP_EXACT && g_params != nullptr;
  if (want_th) {
    CK(h, h->d_vjp.alloc(kVjpAux), "vjp scratch");
    CK(h, cudaMemsetAsync(h->d_vjp.p, 0, kVjpAux * sizeof(double), st), "memset vjp scratch");
  }
  KParams k = base_params(h, dt);
  k.I = dI;
  k.P = dP;
  k.vjp_lam = dlam;
  k.vjp_g = dg;
  k.vjp_th = want_th ? h->d_vjp.p : nullptr;
  k.scatter_mode = 0;
  k.el_list = h->d_sweep.p;
  k.n_list = h->n_el;
  KParams kb = k;
  kb.el_list = h->d_bd_list.p;
  kb.n_list = (int64_t)h->bd_list.size();
  kb.bd_sides = h->d_bd_sides.p;
  set_boundary_points(h, kb);
  if (mode == GALES_VJP_EXACT) {
    LaunchResult r = dispatch_vjp(h, k, false, h->n_el, st);
    if (r.err != cudaSuccess) return cuda_fail(h, r.err, "vjp interior kernel");
    h->launches += r.launches;
    if (kb.n_list > 0) {
      r = dispatch_vjp(h, kb, true, kb.n_list, st);
      if (r.err != cudaSuccess) return cuda_fail(h, r.err, "vjp boundary kernel");
      h->launches += r.launches;
    }
  } else {
    // the FP64 tangent, contracted with lambda by the matrix and boundary kernels
    int rc = run_interior(h, k, GALES_FORM_FP64, true, h->n_el, st);
    if (rc) return rc;
    if (kb.n_list > 0) {
      LaunchResult r = dispatch_boundary(h, kb, GALES_FORM_FP64, kb.n_list, st);
      if (r.err != cudaSuccess) return cuda_fail(h, r.err, "boundary kernel");
      h->launches += r.launches;
    }
  }
  if (hG) CK(h, cudaMemcpyAsync(g_state, dg, sb, cudaMemcpyDeviceToHost, st), "copy g_state");
  if (want_th) CK(h, cudaMemcpyAsync(h->h_vjp, h->d_vjp.p, kVjpAux * sizeof(double), cudaMemcpyDeviceToHost, st),
                  "copy vjp scratch");
  CK(h, cudaEventRecord(h->ev1, st), "event");
  int rc = finish(h, st);
  if (g_params) {
    // theta cotangents plus the path through u_ref_inv (host arithmetic on nd values)
    double th[3 * GALES_MAX_COMP];
    for (int i = 0; i < npar; ++i) th[i] = want_th ? h->h_vjp[i] : 0.0;
    if (want_th) u_ref_inv_reverse(h, h->h_vjp + npar, th);
    if (hT) {
      memcpy(g_params, th, npar * sizeof(double));
    } else {
      CK(h, cudaMemcpyAsync(dth, th, npar * sizeof(double), cudaMemcpyHostToDevice, st), "copy g_params");
      CK(h, cudaStreamSynchronize(st), "synchronize");
    }
  }
  float ms = 0.f;
  cudaEventElapsedTime(&ms, h->ev0, h->ev1);
  h->last_ms = ms;
  return rc;
}

int gales_asm_norm2(gales_asm* h, const double* rhs, double* out, void* stream) {
  if (!h || !rhs || !out) return GALES_ERR_BAD_INPUT;
  CK(h, cudaSetDevice(h->device), "cudaSetDevice");
  cudaStream_t st = (cudaStream_t)stream;
  const double* d = rhs;
  if (!is_device_ptr(rhs)) {
    CK(h, h->s_aux.alloc(h->n_rows + kNormBlocks + 1), "staging rhs");
    CK(h, cudaMemcpyAsync(h->s_aux.p, rhs, (size_t)h->n_rows * sizeof(double), cudaMemcpyHostToDevice, st),
       "copy rhs");
    d = h->s_aux.p;
  }
  CK(h, h->s_th.alloc(kNormBlocks + 1 > 3 * GALES_MAX_COMP ? kNormBlocks + 1 : 3 * GALES_MAX_COMP), "norm scratch");
  CK(h, launch_norm2(d, h->n_rows, h->s_th.p, st), "norm kernel");
  h->launches += 2;
  double r = 0.0;
  CK(h, cudaMemcpyAsync(h->h_aux, h->s_th.p + kNormBlocks, sizeof(double), cudaMemcpyDeviceToHost, st), "copy norm");
  CK(h, cudaStreamSynchronize(st), "synchronize");
  r = *h->h_aux;
  *out = r;
  return 0;
}

double gales_dt_update(double dt_elem_min, double dt, double dt_min, double dt_max) {
  // set_dt (adaptive_time_step.hpp:380-393): growth bounded by 1% of dt, then clamped
  double d = (dt_elem_min > (1.01 * dt)) ? 1.01 * dt : dt_elem_min;
  d = std::max(std::min(d, dt_max), dt_min);
  return d;
}

int gales_asm_adaptive_dt(gales_asm* h, const double* I, double dt, double cfl, double dt_min, double dt_max,
                          double* dt_el, double* dt_new, void* stream) {
  if (!h) return GALES_ERR_BAD_INPUT;
  if (!I || !dt_new) return fail(h, GALES_ERR_BAD_INPUT, "null state or result pointer");
  if (!(dt > 0.0) || !(cfl > 0.0)) return fail(h, GALES_ERR_BAD_INPUT, "dt and CFL must be positive");
  CK(h, cudaSetDevice(h->device), "cudaSetDevice");
  cudaStream_t st = (cudaStream_t)stream;
  const double* dI = I;
  if (!is_device_ptr(I)) {
    CK(h, h->s_I.alloc(h->n_rows), "staging I");
    CK(h, cudaMemcpyAsync(h->s_I.p, I, (size_t)h->n_rows * sizeof(double), cudaMemcpyHostToDevice, st), "copy I");
    dI = h->s_I.p;
  }
  const bool dev_el = dt_el && is_device_ptr(dt_el);
  double* del = dt_el;
  if (!dev_el) {
    CK(h, h->s_aux.alloc(std::max<int64_t>(h->n_el, 1)), "per-element dt");
    del = h->s_aux.p;
  }
  KParams k = base_params(h, dt);
  k.I = dI;
  if (h->mg) {  // magma lookups report through the status word
    CK(h, cudaMemsetAsync(h->d_status.p, 0, sizeof(unsigned int), st), "memset status");
    CK(h, cudaMemsetAsync(h->d_first_bad.p, 0xff, sizeof(unsigned long long), st), "memset first_bad");
  }
  LaunchResult r = dispatch_adaptive_dt(h, k, cfl, del, h->n_el, st);
  if (r.err != cudaSuccess) return cuda_fail(h, r.err, "adaptive dt kernel");
  h->launches += r.launches;
  CK(h, h->s_th.alloc(std::max(2 * kMinBlocks + 1, 3 * GALES_MAX_COMP)), "min scratch");
  min_partial_kernel<<<kMinBlocks, 256, 0, st>>>(del, h->n_el, h->s_th.p);
  min_final_kernel<<<1, 256, 0, st>>>(h->s_th.p);
  CK(h, cudaGetLastError(), "min kernels");
  h->launches += 2;
  CK(h, cudaMemcpyAsync(h->h_aux, h->s_th.p + 2 * kMinBlocks, sizeof(double), cudaMemcpyDeviceToHost, st),
     "copy min");
  if (dt_el && !dev_el)
    CK(h, cudaMemcpyAsync(dt_el, del, (size_t)h->n_el * sizeof(double), cudaMemcpyDeviceToHost, st), "copy dt");
  int rc = 0;
  if (h->mg) rc = finish(h, st);
  else CK(h, cudaStreamSynchronize(st), "synchronize");
  *dt_new = gales_dt_update(*h->h_aux, dt, dt_min, dt_max);
  return rc;
}

int gales_asm_secondary_dofs(gales_asm* h, const double* I, double* out, void* stream) {
  if (!h) return GALES_ERR_BAD_INPUT;
  if (!I || !out) return fail(h, GALES_ERR_BAD_INPUT, "null state or output pointer");
  CK(h, cudaSetDevice(h->device), "cudaSetDevice");
  cudaStream_t st = (cudaStream_t)stream;
  const double* dI = I;
  if (!is_device_ptr(I)) {
    CK(h, h->s_I.alloc(h->n_rows), "staging I");
    CK(h, cudaMemcpyAsync(h->s_I.p, I, (size_t)h->n_rows * sizeof(double), cudaMemcpyHostToDevice, st), "copy I");
    dI = h->s_I.p;
  }
  const int64_t n = h->n_nodes;
  const bool dev_out = is_device_ptr(out);
  double* dout = out;
  if (!dev_out) {
    CK(h, h->s_aux.alloc(std::max<int64_t>(8 * n, 1)), "staging output");
    dout = h->s_aux.p;
  }
  KParams k = base_params(h, 1.0);
  k.I = dI;
  if (h->mg) {  // magma lookups report through the status word
    CK(h, cudaMemsetAsync(h->d_status.p, 0, sizeof(unsigned int), st), "memset status");
    CK(h, cudaMemsetAsync(h->d_first_bad.p, 0xff, sizeof(unsigned long long), st), "memset first_bad");
  }
  LaunchResult r = h->mg ? h->mops.secondary_dofs(k, h->nc, dout, n, st)
                         : (h->dim == 2 ? secondary_dofs_2d(k, h->nc, dout, n, st)
                                        : secondary_dofs_3d(k, h->nc, dout, n, st));
  if (r.err != cudaSuccess) return cuda_fail(h, r.err, "secondary dofs kernel");
  h->launches += r.launches;
  if (!dev_out)
    CK(h, cudaMemcpyAsync(out, dout, (size_t)(8 * n) * sizeof(double), cudaMemcpyDeviceToHost, st), "copy output");
  if (h->mg) return finish(h, st);
  CK(h, cudaStreamSynchronize(st), "synchronize");
  return 0;
}

int gales_asm_set_magma(gales_asm* h, gales_magma* m) {
  if (!h) return GALES_ERR_BAD_INPUT;
  CK(h, cudaSetDevice(h->device), "cudaSetDevice");
  if (!m) {  // back to the material's chemicals
    h->mg = nullptr;
    h->ops[GALES_FORM_FP64] = h->ops_ch[GALES_FORM_FP64];
    h->ops[GALES_FORM_MIXED] = h->ops_ch[GALES_FORM_MIXED];
    compute_u_ref_inv(h);
    return 0;
  }
  int nc = 0, dev = -1;
  const magma_mix::DevMagma* tab = magma_device_table(m, &nc, &dev);
  if (nc != h->nc)
    return fail(h, GALES_ERR_BAD_INPUT, "the magma material has " + std::to_string(nc) +
                                            " components, the handle " + std::to_string(h->nc));
  if (dev != h->device) return fail(h, GALES_ERR_BAD_INPUT, "the magma material lives on another device");
  MagmaOps mo = h->dim == 2 ? (h->nen == 3 ? magma_ops_tri3() : magma_ops_quad4())
                            : (h->nen == 4 ? magma_ops_tet4() : magma_ops_hex8());
  for (int f = 0; f < 2; ++f) {  // kernel attributes, once, outside any stream capture
    if (mo.interior[f].rec_bytes(h->nc) != h->ops_ch[f].rec_bytes(h->nc))
      return fail(h, GALES_ERR_UNSUPPORTED, "magma point records differ from the chemicals'");
    CK(h, mo.interior[f].prepare(h->nc), "kernel attributes");
    KParams k0;
    memset(&k0, 0, sizeof(k0));
    LaunchResult r = mo.boundary(k0, h->nc, f, -1, 0);
    if (r.err != cudaSuccess) return cuda_fail(h, r.err, "kernel attributes");
  }
  // u_ref_inv from the magma mixture at (p_ref, T_ref, Y_ref = 0.5, shear rate 0)
  // (fluid_2d.hpp:123-135)
  double p = h->setup.p_ref, T = h->setup.T_ref, Y[GALES_MAX_COMP], f[8];
  for (int c = 0; c < nc; ++c) Y[c] = 0.5;
  int rc = gales_magma_properties(m, &p, &T, Y, nullptr, 1, f, nullptr, nullptr);
  if (rc) return fail(h, GALES_ERR_MAGMA, std::string("magma properties at the reference state: ") +
                                              gales_magma_last_error(m));
  h->mops = mo;
  h->mg = tab;
  h->ops[GALES_FORM_FP64] = mo.interior[GALES_FORM_FP64];
  h->ops[GALES_FORM_MIXED] = mo.interior[GALES_FORM_MIXED];
  u_ref_inv_from(h, f[0], f[3]);
  return 0;
}

int gales_asm_magma_fractions(gales_asm* h, const double* I, double* out, void* stream) {
  if (!h) return GALES_ERR_BAD_INPUT;
  if (!I || !out) return fail(h, GALES_ERR_BAD_INPUT, "null state or output pointer");
  if (!h->mg) return fail(h, GALES_ERR_BAD_INPUT, "no magma material attached (gales_asm_set_magma)");
  CK(h, cudaSetDevice(h->device), "cudaSetDevice");
  cudaStream_t st = (cudaStream_t)stream;
  const double* dI = I;
  if (!is_device_ptr(I)) {
    CK(h, h->s_I.alloc(h->n_rows), "staging I");
    CK(h, cudaMemcpyAsync(h->s_I.p, I, (size_t)h->n_rows * sizeof(double), cudaMemcpyHostToDevice, st), "copy I");
    dI = h->s_I.p;
  }
  const int64_t n = h->n_nodes, nf = 2 * h->nc + 6;
  const bool dev_out = is_device_ptr(out);
  double* dout = out;
  if (!dev_out) {
    CK(h, h->s_aux.alloc(std::max<int64_t>(nf * n, 1)), "staging output");
    dout = h->s_aux.p;
  }
  KParams k = base_params(h, 1.0);
  k.I = dI;
  if (h->mg) {  // magma lookups report through the status word
    CK(h, cudaMemsetAsync(h->d_status.p, 0, sizeof(unsigned int), st), "memset status");
    CK(h, cudaMemsetAsync(h->d_first_bad.p, 0xff, sizeof(unsigned long long), st), "memset first_bad");
  }
  LaunchResult r = h->mops.fractions(k, h->nc, dout, n, st);
  if (r.err != cudaSuccess) return cuda_fail(h, r.err, "magma fractions kernel");
  h->launches += r.launches;
  if (!dev_out)
    CK(h, cudaMemcpyAsync(out, dout, (size_t)(nf * n) * sizeof(double), cudaMemcpyDeviceToHost, st), "copy output");
  return finish(h, st);
}

int gales_pressure_profile(const gales_material_desc* mat, double p0, double h, int32_t n_steps, const double* T,
                           const double* T1, const double* Y, const double* Y1, double* p_out) {
  if (!mat || !T || !T1 || !p_out || n_steps < 0) return GALES_ERR_BAD_INPUT;
  const int nc = mat->nb_comp;
  if (nc < 1 || nc > GALES_MAX_COMP) return GALES_ERR_BAD_INPUT;
  if (nc > 1 && (!Y || !Y1)) return GALES_ERR_BAD_INPUT;
  DevChem ch[GALES_MAX_COMP];
  for (int c = 0; c < nc; ++c) fill_chem(mat->comp[c], ch[c]);
  auto full_Y = [&](const double* y, double* out) {  // A[i][nc-1] = 1 - accumulate(A[i][0..nc-2])
    double s = 0.0;
    for (int c = 0; c < nc - 1; ++c) {
      out[c] = y[c];
      s = s + y[c];
    }
    out[nc - 1] = 1.0 - s;
  };
  auto rho = [&](double p, double t, const double* y) {
    switch (nc) {
#define GALES_RHO(N)                        \
  case N: {                                 \
    Props<N> pr;                            \
    mixture<N>(ch, p, t, y, pr);            \
    return pr.rho;                          \
  }
      GALES_RHO(1) GALES_RHO(2) GALES_RHO(3) GALES_RHO(4) GALES_RHO(5) GALES_RHO(6) GALES_RHO(7) GALES_RHO(8)
#undef GALES_RHO
      default: return 0.0;
    }
  };
  double Ya[GALES_MAX_COMP], Yb[GALES_MAX_COMP], Yc[GALES_MAX_COMP];
  p_out[0] = p0;
  for (int32_t i = 0; i < n_steps; ++i) {
    full_Y(Y + (size_t)i * (nc - 1), Ya);
    full_Y(Y1 + (size_t)i * (nc - 1), Yb);
    full_Y(Y + (size_t)(i + 1) * (nc - 1), Yc);
    const double m1 = 9.81 * rho(p_out[i], T[i], Ya);
    const double m2 = 9.81 * rho(p_out[i] + 0.5 * h * m1, T1[i], Yb);
    const double m3 = 9.81 * rho(p_out[i] + 0.5 * h * m2, T1[i], Yb);
    const double m4 = 9.81 * rho(p_out[i] + h * m3, T[i + 1], Yc);
    p_out[i + 1] = p_out[i] + h / 6. * (m1 + 2.0 * (m2 + m3) + m4);
  }
  return 0;
}

int gales_pressure_interpolate(const double* y_col, const double* p_col, int32_t n_col, const double* y, int64_t n,
                               double* p_out) {
  if (!y_col || !p_col || !y || !p_out || n_col < 2 || n < 0) return GALES_ERR_BAD_INPUT;
  const bool ascending = y_col[0] < y_col[n_col - 1];
  for (int64_t k = 0; k < n; ++k) {
    size_t i = ascending ? (size_t)(std::lower_bound(y_col, y_col + n_col, y[k]) - y_col)
                         : (size_t)(std::lower_bound(y_col, y_col + n_col, y[k], std::greater<double>()) - y_col);
    if (i > 0) i--;
    if (i >= (size_t)n_col - 1) return GALES_ERR_BAD_INPUT;  // outside the column (the reference's Error)
    const double f = (y[k] - y_col[i]) / (y_col[i + 1] - y_col[i]);
    p_out[k] = f * p_col[i + 1] + (1.0 - f) * p_col[i];
  }
  return 0;
}

int gales_asm_status(gales_asm* h, int64_t* first_bad_element) {
  if (!h) return GALES_ERR_BAD_INPUT;
  if (first_bad_element) *first_bad_element = h->first_bad;
  return h->status;
}

const char* gales_asm_last_error(gales_asm* h) { return h ? h->err.c_str() : "null handle"; }

double gales_asm_last_ms(gales_asm* h) { return h ? h->last_ms : 0.0; }

double gales_asm_last_phase_ms(gales_asm* h, int32_t phase) {
  if (!h || phase < 0 || phase > 4) return -1.0;
  float ms = -1.f;
  const cudaEvent_t a = phase == 3 ? h->evp[1] : (phase == 4 ? h->evs[0] : h->evp[phase]);
  const cudaEvent_t b = phase == 3 ? h->evs[0] : (phase == 4 ? h->evs[1] : h->evp[phase + 1]);
  if (cudaEventElapsedTime(&ms, a, b) != cudaSuccess) {
    cudaGetLastError();
    return -1.0;
  }
  return ms;
}

int64_t gales_asm_launch_count(gales_asm* h) { return h ? h->launches : 0; }

}  // extern "C"

// ---------------------------------------------------------------------------
// Assembly without any allocation.
//
// Some callers cannot allocate device memory while they assemble: programs whose
// device memory is owned by another allocator (a framework's caching pool, a
// fixed per-process quota) where a raw cudaMalloc would overrun the budget or
// fragment the pool, and time-stepping loops that must keep a fixed memory
// footprint and never meet allocator latency or an out-of-memory failure in the
// middle of a run.  gales_asm_assemble may allocate staging buffers on first use
// (host pointers); the entry point below never does.  Its interior pass runs the
// same point and matrix kernels, with the per-point records in this file-scope
// device array instead of handle-owned buffers.  Every GPU that loads the library
// holds the array until the process exits.
static __device__ __align__(256) unsigned char g_noalloc_scratch[GALES_NOALLOC_SCRATCH_BYTES];

namespace {

// Device address of g_noalloc_scratch per device.  In host code the array's name
// is only a host-side stand-in, so the address is looked up once per device, with
// that device current, by the first gales_asm_assemble_noalloc call on it, and kept
// for the life of the process.  A device reset frees the handles' memory as well and
// would leave this address stale; the header rules out use after a reset.
std::mutex g_noalloc_mu;
void* g_noalloc_ptr[64] = {nullptr};

int noalloc_scratch(gales_asm* h, void** out) {
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (h->device < 0 || h->device >= 64) return fail(h, GALES_ERR_BAD_INPUT, "device index out of range");
  if (!g_noalloc_ptr[h->device]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_fail(h, e, "cudaGetSymbolAddress(g_noalloc_scratch)");
    g_noalloc_ptr[h->device] = p;
  }
  *out = g_noalloc_ptr[h->device];
  return 0;
}

}  // namespace

extern "C" int gales_asm_assemble_noalloc(gales_asm* h, const double* I, const double* P, double dt,
                                          int32_t form, double* vals, double* rhs, void* stream) {
  if (!h) return GALES_ERR_BAD_INPUT;
  if (!I || !P || !vals || !rhs) return fail(h, GALES_ERR_BAD_INPUT, "null state or output pointer");
  if (form != GALES_FORM_FP64 && form != GALES_FORM_MIXED) return fail(h, GALES_ERR_BAD_INPUT, "unknown form");
  if (!(dt > 0.0)) return fail(h, GALES_ERR_BAD_INPUT, "dt must be positive");
  CK(h, cudaSetDevice(h->device), "cudaSetDevice");
  if (!is_device_ptr(I) || !is_device_ptr(P) || !is_device_ptr(vals) || !is_device_ptr(rhs))
    return fail(h, GALES_ERR_BAD_INPUT,
                "gales_asm_assemble_noalloc needs device pointers for I, P, vals and rhs "
                "(host buffers would need staging allocations)");
  const InteriorOps& ops = h->ops[form];
  const size_t rb = ops.rec_bytes(h->nc);
  if (rb == 0) return fail(h, GALES_ERR_UNSUPPORTED, "no interior kernel for this element/component count");
  // point records are written in blocks of a matrix CTA's elements (at most 4), so a
  // chunk is a multiple of 4 elements and its blocks never pass the chunk's bytes
  if (4 * rb > GALES_NOALLOC_SCRATCH_BYTES)
    return fail(h, GALES_ERR_UNSUPPORTED,
                "four elements' point records (" + std::to_string(4 * rb) + " bytes) exceed the " +
                    std::to_string((long long)GALES_NOALLOC_SCRATCH_BYTES) + "-byte no-allocation scratch");
  void* scratch = nullptr;
  int rc = noalloc_scratch(h, &scratch);
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  KParams k = base_params(h, dt);
  k.I = I;
  k.P = P;
  k.vals = vals;
  k.rhs = rhs;
  k.scatter_mode = 0;
  k.el_list = h->d_sweep.p;
  k.n_list = h->n_el;
  CK(h, cudaEventRecord(h->ev0, st), "event");
  CK(h, cudaMemsetAsync(h->d_status.p, 0, sizeof(unsigned int), st), "memset status");
  CK(h, cudaMemsetAsync(h->d_first_bad.p, 0xff, sizeof(unsigned long long), st), "memset first_bad");
  CK(h, cudaMemsetAsync(vals, 0, (size_t)h->nnz * sizeof(double), st), "memset vals");
  CK(h, cudaMemsetAsync(rhs, 0, (size_t)h->n_rows * sizeof(double), st), "memset rhs");
  // The point records of a chunk are written in full by the point kernel before the
  // matrix kernel reads them, so nothing in the scratch has to start at zero.
  const long long chunk = (long long)(GALES_NOALLOC_SCRATCH_BYTES / rb) / 4 * 4;
  for (long long first = 0; first < h->n_el; first += chunk) {
    const long long cnt = std::min(chunk, h->n_el - first);
    LaunchResult r = ops.point(k, h->nc, scratch, first, cnt, st);
    if (r.err != cudaSuccess) return cuda_fail(h, r.err, "point kernel");
    h->launches += r.launches;
    r = ops.matrix(k, h->nc, true, scratch, first, cnt, st);
    if (r.err != cudaSuccess) return cuda_fail(h, r.err, "matrix kernel");
    h->launches += r.launches;
  }
  if (!h->bd_list.empty()) {
    KParams kb = k;
    kb.el_list = h->d_bd_list.p;
    kb.n_list = (int64_t)h->bd_list.size();
    kb.bd_sides = h->d_bd_sides.p;
    set_boundary_points(h, kb);
    LaunchResult r = dispatch_boundary(h, kb, form, kb.n_list, st);
    if (r.err != cudaSuccess) return cuda_fail(h, r.err, "boundary kernel");
    h->launches += r.launches;
  }
  CK(h, cudaEventRecord(h->ev1, st), "event");
  rc = finish(h, st);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, h->ev0, h->ev1);
  h->last_ms = ms;
  return rc;
}
