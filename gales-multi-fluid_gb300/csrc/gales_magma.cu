// Magma mixture properties on the GPU: one thread per (p, T, Y) point evaluates every
// magma component (gales_magma.cuh) and their mixture of sub-mixtures
// (fluid_properties.hpp:171-200); the C ABI of include/gales_asm.h (gales_magma_*).
#include <cuda_runtime.h>

#include <cstring>
#include <string>
#include <vector>

#include "../../include/gales_asm.h"

#include "gales_magma.cuh"

namespace {

using namespace magma_mix;

__global__ void magma_mix_kernel(const DevMagma* __restrict__ mg, int nc, const double* __restrict__ p,
                                 const double* __restrict__ T, const double* __restrict__ Y,
                                 const double* __restrict__ shear, int64_t n, double* __restrict__ out,
                                 double* __restrict__ comp, unsigned* __restrict__ status) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double f[8], cc[GALES_MAX_COMP][4];
  const unsigned st = mix_point(mg, nc, p[i], T[i], Y + i * nc, shear ? shear[i] : 0.0, f, cc);
#pragma unroll
  for (int k = 0; k < 8; ++k) out[k * n + i] = f[k];
  if (comp)
    for (int c = 0; c < nc; ++c)
#pragma unroll
      for (int k = 0; k < 4; ++k) comp[(c * 4 + k) * n + i] = cc[c][k];
  if (st) atomicOr(status, st);
}

bool is_dev(const void* q) {
  if (!q) return false;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, q) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

}  // namespace

struct gales_magma {
  int device = 0;
  int nc = 0;
  DevMagma* d_mg = nullptr;
  std::vector<double*> tables;
  unsigned* d_status = nullptr;
  double* d_scratch = nullptr;
  size_t scratch_n = 0;
  int status = 0;
  std::string err;
};

namespace gales {

const magma_mix::DevMagma* magma_device_table(const gales_magma* m, int* nc, int* device) {
  *nc = m->nc;
  *device = m->device;
  return m->d_mg;
}

}  // namespace gales

extern "C" {

int gales_magma_create(const gales_magma_desc* comps, int32_t nb_comp, gales_magma** out) {
  if (!comps || !out || nb_comp < 1 || nb_comp > GALES_MAX_COMP) return GALES_ERR_BAD_INPUT;
  *out = nullptr;
  for (int c = 0; c < nb_comp; ++c) {
    const gales_magma_desc& d = comps[c];
    if (d.kind == GALES_SUBMIX_CUSTOM) {
      if (!(d.chemical.rho > 0.0)) return GALES_ERR_BAD_INPUT;
      continue;
    }
    if (d.kind == GALES_SUBMIX_CHEMICAL) {
      if (d.chemical.kind == GALES_CH_CUSTOM ? !(d.chemical.rho > 0.0)
                                              : (d.chemical.kind != GALES_CH_IDEAL_GAS || !(d.chemical.R > 0.0)))
        return GALES_ERR_BAD_INPUT;
      continue;
    }
    if (d.kind != GALES_SUBMIX_MAGMA || d.n_p < 2 || d.n_T < 0 || d.n_T == 1 || !d.p_table || !d.wf_l_h2o ||
        !d.wf_l_co2 || (d.n_T > 0 && !d.T_table) || d.gas_on_mu < 0 || d.gas_on_mu > 2 || d.crystal_on_mu < 0 ||
        d.crystal_on_mu > 2)
      return GALES_ERR_BAD_INPUT;
  }
  auto* m = new gales_magma();
  m->nc = nb_comp;
  cudaGetDevice(&m->device);
  std::vector<DevMagma> h(nb_comp);
  auto upload = [&](const double* src, size_t cnt, const double** dst) -> bool {
    double* p = nullptr;
    if (cudaMalloc(&p, cnt * sizeof(double)) != cudaSuccess) return false;
    m->tables.push_back(p);
    if (cudaMemcpy(p, src, cnt * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess) return false;
    *dst = p;
    return true;
  };
  bool ok = true;
  for (int c = 0; c < nb_comp && ok; ++c) {
    const gales_magma_desc& d = comps[c];
    build_constants(d, h[c]);
    h[c].T_tab = nullptr;
    if (d.kind != GALES_SUBMIX_MAGMA) {  // no tables
      h[c].p_tab = h[c].h2o_tab = h[c].co2_tab = nullptr;
      continue;
    }
    const size_t tn = d.n_T > 0 ? (size_t)d.n_T * d.n_p : (size_t)d.n_p;
    ok = upload(d.p_table, d.n_p, &h[c].p_tab) && upload(d.wf_l_h2o, tn, &h[c].h2o_tab) &&
         upload(d.wf_l_co2, tn, &h[c].co2_tab) && (d.n_T == 0 || upload(d.T_table, d.n_T, &h[c].T_tab));
  }
  if (ok) ok = cudaMalloc(&m->d_mg, nb_comp * sizeof(DevMagma)) == cudaSuccess &&
               cudaMemcpy(m->d_mg, h.data(), nb_comp * sizeof(DevMagma), cudaMemcpyHostToDevice) == cudaSuccess &&
               cudaMalloc(&m->d_status, sizeof(unsigned)) == cudaSuccess;
  if (!ok) {
    cudaGetLastError();
    gales_magma_destroy(m);
    return GALES_ERR_NO_MEMORY;
  }
  *out = m;
  return 0;
}

int gales_magma_properties(gales_magma* m, const double* p, const double* T, const double* Y, const double* shear,
                           int64_t n, double* out, double* comp, void* stream) {
  if (!m || !p || !T || !Y || !out || n < 0) return GALES_ERR_BAD_INPUT;
  m->status = 0;
  if (n == 0) return 0;
  cudaSetDevice(m->device);
  cudaStream_t st = (cudaStream_t)stream;
  const int nc = m->nc;
  // stage host arrays in one device scratch: p, T, Y, shear, out, comp
  const size_t n_in = (size_t)n * (2 + nc + (shear ? 1 : 0)), n_out = (size_t)n * (8 + (comp ? 4 * nc : 0));
  const bool dev = is_dev(p) && is_dev(T) && is_dev(Y) && (!shear || is_dev(shear)) && is_dev(out) &&
                   (!comp || is_dev(comp));
  const double *dp = p, *dT = T, *dY = Y, *ds = shear;
  double *dout = out, *dcomp = comp;
  auto fail = [&](cudaError_t e, const char* what) {
    m->err = std::string(what) + ": " + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? GALES_ERR_NO_MEMORY : GALES_ERR_CUDA;
  };
  cudaError_t e;
  if (!dev) {
    if (m->scratch_n < n_in + n_out) {
      if (m->d_scratch) cudaFree(m->d_scratch);
      m->d_scratch = nullptr;
      m->scratch_n = 0;
      if ((e = cudaMalloc(&m->d_scratch, (n_in + n_out) * sizeof(double))) != cudaSuccess) return fail(e, "scratch");
      m->scratch_n = n_in + n_out;
    }
    double* s = m->d_scratch;
    auto put = [&](const double* src, size_t cnt, double*& at) -> cudaError_t {
      double* d = at;
      at += cnt;
      return cudaMemcpyAsync(d, src, cnt * sizeof(double), cudaMemcpyHostToDevice, st);
    };
    double* at = s;
    dp = at;
    if ((e = put(p, n, at)) != cudaSuccess) return fail(e, "copy p");
    dT = at;
    if ((e = put(T, n, at)) != cudaSuccess) return fail(e, "copy T");
    dY = at;
    if ((e = put(Y, (size_t)n * nc, at)) != cudaSuccess) return fail(e, "copy Y");
    if (shear) {
      ds = at;
      if ((e = put(shear, n, at)) != cudaSuccess) return fail(e, "copy shear");
    }
    dout = at;
    at += (size_t)n * 8;
    if (comp) dcomp = at;
  }
  if ((e = cudaMemsetAsync(m->d_status, 0, sizeof(unsigned), st)) != cudaSuccess) return fail(e, "status");
  const int threads = 128;
  magma_mix_kernel<<<(unsigned)((n + threads - 1) / threads), threads, 0, st>>>(m->d_mg, nc, dp, dT, dY, ds, n, dout,
                                                                                 dcomp, m->d_status);
  if ((e = cudaGetLastError()) != cudaSuccess) return fail(e, "magma kernel");
  unsigned hs = 0;
  if ((e = cudaMemcpyAsync(&hs, m->d_status, sizeof(unsigned), cudaMemcpyDeviceToHost, st)) != cudaSuccess)
    return fail(e, "status");
  if (!dev) {
    if ((e = cudaMemcpyAsync(out, dout, (size_t)n * 8 * sizeof(double), cudaMemcpyDeviceToHost, st)) != cudaSuccess)
      return fail(e, "copy out");
    if (comp && (e = cudaMemcpyAsync(comp, dcomp, (size_t)n * 4 * nc * sizeof(double), cudaMemcpyDeviceToHost,
                                     st)) != cudaSuccess)
      return fail(e, "copy comp");
  }
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return fail(e, "synchronize");
  m->status = (int)hs;
  if (hs) {
    m->err = "magma properties: status bits " + std::to_string(hs);
    return GALES_ERR_BAD_INPUT;
  }
  return 0;
}

int gales_magma_status(gales_magma* m) { return m ? m->status : 0; }

const char* gales_magma_last_error(gales_magma* m) { return m ? m->err.c_str() : "null handle"; }

void gales_magma_destroy(gales_magma* m) {
  if (!m) return;
  cudaSetDevice(m->device);
  for (double* p : m->tables) cudaFree(p);
  if (m->d_mg) cudaFree(m->d_mg);
  if (m->d_status) cudaFree(m->d_status);
  if (m->d_scratch) cudaFree(m->d_scratch);
  delete m;
}

}  // extern "C"
