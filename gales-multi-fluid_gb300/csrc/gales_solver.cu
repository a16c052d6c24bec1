// Linear solve of the assembled system on the GPU: flexible GMRES with a right
// ILU(k) preconditioner, the solver the reference runs after every assembly
// (belos_linear_solver::execute, src/fem/ls/belos_linear_solver_factory.hpp:103-218,
// with Ifpack "ILU" and Belos "Flexible GMRES" as sim/fluid_mc/P0/setup.txt:10-16
// selects).  It reads the CSR values the assembly leaves in device memory, so a
// Newton step needs no host copy of the matrix.
//
// Layout.  The assembled matrix has dense nd x nd blocks per pair of connected nodes
// (its scalar rows i*nd+k of node row i hold deg*nd consecutive values, node by
// node).  Scalar ILU(k) on such a pattern is block ILU(k) on the node graph: the
// scalar level of fill of an entry equals the level of its node block (paths through
// the entry's own node add a level-0 step), so the factor is stored as node blocks,
// F[pos][r][c] row-major, with the node rows' blocks sorted by column and the diagonal
// block's position kept.  The factor entries are computed with the same operations in
// the same order as row-oriented scalar elimination, so they equal it bit for bit.
//
// Parallelism.  A node row of the factor and of the forward substitution depends on
// the rows of its lower blocks, a row of the backward substitution on those of its
// upper blocks: rows are grouped by level (longest dependency chain) on the host.  The
// factorisation runs one launch per level with a warp per node row; each substitution
// is one persistent launch in which warps take rows in level order and wait on per-row
// ready flags (see ilu_lower_sweep_kernel).  The preconditioner application is
// captured once into a CUDA graph whose kernels take the Krylov vector's index from
// device memory.  The Arnoldi step (two classical
// Gram-Schmidt passes) uses blocked dot products with fixed partial-sum order, so
// repeated solves are bit-identical.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/gales_asm.h"

namespace {

constexpr int kWarpsPerBlock = 8;   // node rows per CTA in the level kernels
constexpr int kDotThreads = 256;

template <typename T>
struct Dev {
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
  template <typename U>
  cudaError_t upload(const std::vector<U>& v) {
    cudaError_t e = alloc(v.size());
    if (e != cudaSuccess || v.empty()) return e;
    return cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice);
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
};

// ---------------------------------------------------------------------------
// Host: ILU(k) symbolic factorisation of the node graph and the level sets.
// ---------------------------------------------------------------------------

// Ifpack_IlukGraph's level-of-fill rule on node rows: row I starts with its graph
// columns at level 0; for its columns K < I in ascending order, every upper column J of
// row K gets level lev(I,K) + lev(K,J) + 1, kept when <= fill.  A linked list keeps the
// row's columns sorted while fill is inserted.
void iluk_symbolic(int64_t n, const int64_t* rp, const int32_t* col, int fill, std::vector<int64_t>& f_rp,
                   std::vector<int32_t>& f_col, std::vector<int64_t>& f_diag) {
  f_rp.assign(n + 1, 0);
  f_col.clear();
  f_diag.assign(n, -1);
  std::vector<int> f_lev;
  std::vector<int32_t> next(n + 1, -1);  // linked list; index n is the head
  std::vector<int> lev(n, INT32_MAX);
  std::vector<int32_t> touched;
  for (int64_t i = 0; i < n; ++i) {
    touched.clear();
    // graph columns (sorted) plus the diagonal
    int32_t prev = (int32_t)n;
    bool diag_in = false;
    auto push_sorted = [&](int32_t c) {
      next[prev] = c;
      next[c] = -1;
      prev = c;
    };
    next[n] = -1;
    for (int64_t p = rp[i]; p < rp[i + 1]; ++p) {
      const int32_t c = col[p];
      if (!diag_in && c > i) {
        push_sorted((int32_t)i);
        lev[i] = 0;
        touched.push_back((int32_t)i);
        diag_in = true;
      }
      if (c == i) diag_in = true;
      push_sorted(c);
      lev[c] = 0;
      touched.push_back(c);
    }
    if (!diag_in) {
      push_sorted((int32_t)i);
      lev[i] = 0;
      touched.push_back((int32_t)i);
    }
    // eliminate with the rows of the lower columns, in ascending order
    for (int32_t k = next[n]; k >= 0 && k < i; k = next[k]) {
      const int lik = lev[k];
      int32_t at = k;  // insertion cursor: columns after k are > k
      for (int64_t q = f_diag[k] + 1; q < f_rp[k + 1]; ++q) {
        const int l = lik + f_lev[q] + 1;
        if (l > fill) continue;
        const int32_t j = f_col[q];
        if (lev[j] != INT32_MAX) {
          if (l < lev[j]) lev[j] = l;
          continue;
        }
        while (next[at] >= 0 && next[at] < j) at = next[at];
        next[j] = next[at];
        next[at] = j;
        lev[j] = l;
        touched.push_back(j);
      }
    }
    for (int32_t c = next[n]; c >= 0; c = next[c]) {
      if (c == i) f_diag[i] = (int64_t)f_col.size();
      f_col.push_back(c);
      f_lev.push_back(lev[c]);
    }
    f_rp[i + 1] = (int64_t)f_col.size();
    for (int32_t c : touched) lev[c] = INT32_MAX;
  }
}

// Level sets: forward level = 1 + max over lower columns, backward = 1 + max over upper
// columns.  Rows of one level are stored contiguously (ascending) in rows[off[l]..off[l+1]).
void level_sets(int64_t n, const std::vector<int64_t>& f_rp, const std::vector<int32_t>& f_col,
                const std::vector<int64_t>& f_diag, bool forward, std::vector<int32_t>& level,
                std::vector<int64_t>& off, std::vector<int32_t>& rows) {
  level.assign(n, 0);
  int nlev = 0;
  if (forward) {
    for (int64_t i = 0; i < n; ++i) {
      int l = 0;
      for (int64_t p = f_rp[i]; p < f_diag[i]; ++p) l = std::max(l, level[f_col[p]] + 1);
      level[i] = l;
      nlev = std::max(nlev, l + 1);
    }
  } else {
    for (int64_t i = n - 1; i >= 0; --i) {
      int l = 0;
      for (int64_t p = f_diag[i] + 1; p < f_rp[i + 1]; ++p) l = std::max(l, level[f_col[p]] + 1);
      level[i] = l;
      nlev = std::max(nlev, l + 1);
    }
  }
  off.assign(nlev + 1, 0);
  for (int64_t i = 0; i < n; ++i) off[level[i] + 1]++;
  for (int l = 0; l < nlev; ++l) off[l + 1] += off[l];
  rows.assign(n, 0);
  std::vector<int64_t> fillp(off.begin(), off.end() - 1);
  for (int64_t i = 0; i < n; ++i) rows[fillp[level[i]]++] = (int32_t)i;
}

// ---------------------------------------------------------------------------
// Device kernels.
// ---------------------------------------------------------------------------

__device__ __forceinline__ int64_t find_col(const int32_t* __restrict__ c, int64_t lo, int64_t hi, int32_t j) {
  while (lo < hi) {
    const int64_t m = (lo + hi) >> 1;
    const int32_t v = c[m];
    if (v == j) return m;
    if (v < j) lo = m + 1;
    else hi = m;
  }
  return -1;
}

// Scatter the assembled values into the factor blocks (fill blocks stay zero): warp per
// node row, lanes over the row's nd x deg*nd values.
template <int ND, typename T>
__global__ void matrix_to_factor_kernel(const double* __restrict__ vals, const int64_t* __restrict__ node_rp,
                                        const int64_t* __restrict__ a2f, int64_t n_nodes, T* __restrict__ F) {
  const int64_t i = (int64_t)blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
  if (i >= n_nodes) return;
  const int lane = threadIdx.x & 31;
  const int64_t t0 = node_rp[i], deg = node_rp[i + 1] - t0;
  const int64_t base = t0 * ND * ND, len = deg * ND;
  for (int k = 0; k < ND; ++k) {
    for (int64_t e = lane; e < len; e += 32) {
      const int64_t t = t0 + e / ND;
      const int kk = (int)(e % ND);
      F[a2f[t] * (ND * ND) + k * ND + kk] = (T)vals[base + k * len + e];
    }
  }
}

// One level of the numeric factorisation: warp per node row I.  For its lower blocks K
// in ascending order: L_IK = A_IK U_KK^-1 (row-wise substitution, lane r < ND owns row
// r), then A_IJ -= L_IK U_KJ for the upper blocks J of row K present in row I (lanes
// over (J, r)).  Then the row-wise Doolittle step of the diagonal block, applied across
// the whole block row.  Every entry sees the subtractions of the scalar ikj order.
template <int ND, typename T>
__global__ void ilu_factor_level_kernel(T* __restrict__ F, const int64_t* __restrict__ f_rp,
                                        const int32_t* __restrict__ f_col, const int64_t* __restrict__ f_diag,
                                        const int32_t* __restrict__ rows, int64_t count,
                                        unsigned int* __restrict__ status) {
  constexpr int BB = ND * ND;
  const int64_t w = (int64_t)blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
  if (w >= count) return;
  const int lane = threadIdx.x & 31;
  const int32_t I = rows[w];
  const int64_t p0 = f_rp[I], p1 = f_rp[I + 1], pd = f_diag[I];
  for (int64_t p = p0; p < pd; ++p) {
    const int32_t K = f_col[p];
    const int64_t dK = f_diag[K], pK1 = f_rp[K + 1];
    T* B = F + p * BB;
    const T* UK = F + dK * BB;
    if (lane < ND) {
      T row[ND];
#pragma unroll
      for (int c = 0; c < ND; ++c) row[c] = B[lane * ND + c];
#pragma unroll
      for (int c = 0; c < ND; ++c) {
        T s = row[c];
#pragma unroll
        for (int c2 = 0; c2 < c; ++c2) s -= row[c2] * UK[c2 * ND + c];
        row[c] = s / UK[c * ND + c];
      }
#pragma unroll
      for (int c = 0; c < ND; ++c) B[lane * ND + c] = row[c];
    }
    __syncwarp();
    const int64_t items = (pK1 - dK - 1) * ND;
    for (int64_t it = lane; it < items; it += 32) {
      const int64_t q = dK + 1 + it / ND;
      const int r = (int)(it % ND);
      const int64_t pos = find_col(f_col, p + 1, p1, f_col[q]);
      if (pos < 0) continue;
      T l[ND];
#pragma unroll
      for (int m = 0; m < ND; ++m) l[m] = B[r * ND + m];
      const T* U = F + q * BB;
      T* tgt = F + pos * BB + r * ND;
#pragma unroll
      for (int c = 0; c < ND; ++c) {
        T s = tgt[c];
#pragma unroll
        for (int m = 0; m < ND; ++m) s -= l[m] * U[m * ND + c];
        tgt[c] = s;
      }
    }
    __syncwarp();
  }
  // Diagonal block and the upper blocks: rows r in order, pivots c2 < r in order.
  T* D = F + pd * BB;
  const int64_t ncols = (p1 - pd) * ND;  // columns of the block row from the diagonal block on
  for (int r = 1; r < ND; ++r) {
    for (int c2 = 0; c2 < r; ++c2) {
      const T l = D[r * ND + c2] / D[c2 * ND + c2];
      __syncwarp();
      if (lane == 0) D[r * ND + c2] = l;
      for (int64_t e = lane; e < ncols; e += 32) {
        const int64_t b = e / ND;
        const int c = (int)(e % ND);
        if (b == 0 && c <= c2) continue;
        T* Rb = F + (pd + b) * BB;
        Rb[r * ND + c] -= l * Rb[c2 * ND + c];
      }
      __syncwarp();
    }
  }
  if (lane < ND && D[lane * ND + lane] == T(0)) atomicOr(status, (unsigned)GALES_ERR_SINGULAR);
}

// The same factorisation step with the block row I and, for each lower block K, row
// K's diagonal and upper blocks staged in shared memory (one warp per CTA): the row's
// column search, its updates and the diagonal step then run on shared memory, and each
// K costs one coalesced copy.  Same operations in the same order as above.
template <int ND, typename T>
__global__ void ilu_factor_level_smem_kernel(T* __restrict__ F, const int64_t* __restrict__ f_rp,
                                             const int32_t* __restrict__ f_col, const int64_t* __restrict__ f_diag,
                                             const int32_t* __restrict__ rows, int64_t count,
                                             unsigned int* __restrict__ status, int max_row, int max_u) {
  constexpr int BB = ND * ND;
  extern __shared__ __align__(16) unsigned char sm_raw[];
  T* R = reinterpret_cast<T*>(sm_raw);             // [max_row][BB] the block row
  T* UK = R + (size_t)max_row * BB;                // [1 + max_u][BB] row K from its diagonal on
  int32_t* RC = (int32_t*)(UK + (size_t)(1 + max_u) * BB);  // [max_row] the row's columns
  int32_t* UC = RC + max_row;                      // [max_u] row K's upper columns
  const int64_t w = blockIdx.x;
  if (w >= count) return;
  const int lane = threadIdx.x & 31;
  const int32_t I = rows[w];
  const int64_t p0 = f_rp[I], p1 = f_rp[I + 1];
  const int nb = (int)(p1 - p0), bd = (int)(f_diag[I] - p0);
  for (int64_t e = lane; e < (int64_t)nb * BB; e += 32) R[e] = F[p0 * BB + e];
  for (int e = lane; e < nb; e += 32) RC[e] = f_col[p0 + e];
  __syncwarp();
  for (int b = 0; b < bd; ++b) {
    const int32_t K = RC[b];
    const int64_t dK = f_diag[K];
    const int nu = (int)(f_rp[K + 1] - dK - 1);
    for (int64_t e = lane; e < (int64_t)(nu + 1) * BB; e += 32) UK[e] = F[dK * BB + e];
    for (int e = lane; e < nu; e += 32) UC[e] = f_col[dK + 1 + e];
    __syncwarp();
    T* B = R + (size_t)b * BB;
    if (lane < ND) {
      T row[ND];
#pragma unroll
      for (int c = 0; c < ND; ++c) row[c] = B[lane * ND + c];
#pragma unroll
      for (int c = 0; c < ND; ++c) {
        T s = row[c];
#pragma unroll
        for (int c2 = 0; c2 < c; ++c2) s -= row[c2] * UK[c2 * ND + c];
        row[c] = s / UK[c * ND + c];
      }
#pragma unroll
      for (int c = 0; c < ND; ++c) B[lane * ND + c] = row[c];
    }
    __syncwarp();
    const int items = nu * ND;
    for (int it = lane; it < items; it += 32) {
      const int qi = it / ND, r = it - qi * ND;
      const int64_t pos = find_col(RC, b + 1, nb, UC[qi]);
      if (pos < 0) continue;
      T l[ND];
#pragma unroll
      for (int m = 0; m < ND; ++m) l[m] = B[r * ND + m];
      const T* U = UK + (size_t)(1 + qi) * BB;
      T* tgt = R + pos * BB + r * ND;
#pragma unroll
      for (int c = 0; c < ND; ++c) {
        T s = tgt[c];
#pragma unroll
        for (int m = 0; m < ND; ++m) s -= l[m] * U[m * ND + c];
        tgt[c] = s;
      }
    }
    __syncwarp();
  }
  T* D = R + (size_t)bd * BB;
  const int ncols = (nb - bd) * ND;
  for (int r = 1; r < ND; ++r) {
    for (int c2 = 0; c2 < r; ++c2) {
      const T l = D[r * ND + c2] / D[c2 * ND + c2];
      __syncwarp();
      if (lane == 0) D[r * ND + c2] = l;
      for (int e = lane; e < ncols; e += 32) {
        const int bb = e / ND;
        const int c = e - bb * ND;
        if (bb == 0 && c <= c2) continue;
        T* Rb = D + (size_t)bb * BB;
        Rb[r * ND + c] -= l * Rb[c2 * ND + c];
      }
      __syncwarp();
    }
  }
  for (int64_t e = lane; e < (int64_t)nb * BB; e += 32) F[p0 * BB + e] = R[e];
  if (lane < ND && D[lane * ND + lane] == T(0)) atomicOr(status, (unsigned)GALES_ERR_SINGULAR);
}

// Block sums of one node row's lower (upper) blocks: lanes form G = 32 / ND groups of
// ND; lane (g, r) accumulates row r over the blocks g, g + G, ...  The column indices of
// up to 8 blocks per lane are loaded first, so that every block's loads are in flight at
// once (a row's substitution is one dependency level, bound by memory latency).  The
// group partial sums are added in group order (deterministic).
template <int ND, typename T, bool L2Z = false>
__device__ __forceinline__ T block_row_sum(const T* __restrict__ F, const int32_t* __restrict__ f_col, int64_t pa,
                                           int64_t pb, const T* z, T* red) {
  constexpr int BB = ND * ND, G = 32 / ND;
  const int lane = threadIdx.x & 31;
  const int g = lane / ND, r = lane - g * ND;
  T s = 0;
  if (g < G) {
    for (int64_t base = pa + g; base < pb; base += 8 * G) {
      int32_t cidx[8];
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        const int64_t p = base + (int64_t)k * G;
        cidx[k] = p < pb ? f_col[p] : -1;
      }
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        if (cidx[k] < 0) continue;
        const T* B = F + (base + (int64_t)k * G) * BB + r * ND;
        const T* zc = z + (int64_t)cidx[k] * ND;
#pragma unroll
        for (int c = 0; c < ND; ++c) s += B[c] * (L2Z ? __ldcg(zc + c) : zc[c]);
      }
    }
  }
  red[lane] = s;
  __syncwarp();
  T t = 0;
  if (lane < ND)
#pragma unroll
    for (int q = 0; q < G; ++q) t += red[q * ND + lane];
  __syncwarp();
  return t;
}

// y_I = L_II^-1 (v_I - sum_K L_IK y_K), L_II unit lower: warp per node row.  The
// working vector zw is the output column itself for an FP64 factor (zw_follows = 1) or
// a T scratch vector.
template <int ND, typename T>
__global__ void ilu_lower_level_kernel(const T* __restrict__ F, const int64_t* __restrict__ f_rp,
                                       const int32_t* __restrict__ f_col, const int64_t* __restrict__ f_diag,
                                       const int32_t* __restrict__ rows, int64_t count, const double* vbase,
                                       T* zwbase, const int* __restrict__ jidx, int64_t ld, int zw_follows) {
  constexpr int BB = ND * ND;
  __shared__ T red[kWarpsPerBlock][32];
  const int64_t w = (int64_t)blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
  if (w >= count) return;
  const int lane = threadIdx.x & 31;
  const int64_t off = jidx ? (int64_t)(*jidx) * ld : 0;
  const double* v = vbase + off;
  T* zw = zwbase + (zw_follows ? off : 0);
  const int32_t I = rows[w];
  const int64_t p0 = f_rp[I], pd = f_diag[I];
  const int r = lane < ND ? lane : 0;
  const T vi = (T)v[(int64_t)I * ND + r];
  T s = vi - block_row_sum<ND, T>(F, f_col, p0, pd, zw, red[threadIdx.x >> 5]);
  const T* D = F + pd * BB + r * ND;
#pragma unroll
  for (int c = 0; c < ND - 1; ++c) {
    const T zc = __shfl_sync(0xffffffffu, s, c);
    if (lane > c) s -= D[c] * zc;
  }
  if (lane < ND) zw[(int64_t)I * ND + lane] = s;
}

// x_I = U_II^-1 (y_I - sum_J U_IJ x_J), in place on zw; with a scratch zw the row is
// also written to the FP64 output column.
template <int ND, typename T>
__global__ void ilu_upper_level_kernel(const T* __restrict__ F, const int64_t* __restrict__ f_rp,
                                       const int32_t* __restrict__ f_col, const int64_t* __restrict__ f_diag,
                                       const int32_t* __restrict__ rows, int64_t count, T* zwbase,
                                       double* zoutbase, const int* __restrict__ jidx, int64_t ld, int zw_follows) {
  constexpr int BB = ND * ND;
  __shared__ T red[kWarpsPerBlock][32];
  const int64_t w = (int64_t)blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
  if (w >= count) return;
  const int lane = threadIdx.x & 31;
  const int64_t off = jidx ? (int64_t)(*jidx) * ld : 0;
  T* zw = zwbase + (zw_follows ? off : 0);
  double* zout = zoutbase + off;
  const int32_t I = rows[w];
  const int64_t p1 = f_rp[I + 1], pd = f_diag[I];
  const int r = lane < ND ? lane : 0;
  const T yi = zw[(int64_t)I * ND + r];
  T s = yi - block_row_sum<ND, T>(F, f_col, pd + 1, p1, zw, red[threadIdx.x >> 5]);
  const T* D = F + pd * BB + r * ND;
#pragma unroll
  for (int c = ND - 1; c >= 0; --c) {
    const T mine = s / D[c];  // meaningful on lane c only
    const T xc = __shfl_sync(0xffffffffu, mine, c);
    if (lane == c) s = xc;
    else if (lane < c) s -= D[c] * xc;
  }
  if (lane < ND) {
    zw[(int64_t)I * ND + lane] = s;
    if (!zw_follows) zout[(int64_t)I * ND + lane] = (double)s;
  }
}

// Sync-free substitutions: one persistent launch per triangle instead of one launch per
// level.  A warp claims node rows from a ticket counter in level order (rows[] lists
// them level by level), waits until the rows of its row's lower (upper) blocks are
// marked ready, substitutes exactly as the level kernels do, and marks its row ready.
// A warp only ever waits on rows of earlier levels, whose tickets were claimed before
// its own by warps that are running, so the sweep always progresses; every wait is
// still bounded (kSpinMax polls), after which GALES_ERR_TIMEOUT is set in the status
// word and the row is left as it stands.  One lane writes a finished row and releases
// its flag; waiting lanes acquire the flags and then read the rows from L2 (the
// writer's L1 is not this SM's).  The row's factor blocks are prefetched into L1 before
// it waits, so that only the dependent loads remain on the critical path.
constexpr long long kSpinMax = 1ll << 22;

__device__ __forceinline__ int ld_acquire(const int* f) {
  int v;
  asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(f) : "memory");
  return v;
}
__device__ __forceinline__ void st_release(int* f, int v) {
  asm volatile("st.release.gpu.global.b32 [%0], %1;" ::"l"(f), "r"(v) : "memory");
}
__device__ __forceinline__ bool wait_flag(const int* f) {
  for (long long i = 0; i < kSpinMax; ++i) {
    if (ld_acquire(f) != 0) return true;
    __nanosleep(32);
  }
  return false;
}

// Prefetch into L1 the factor blocks rows [pa, pb) that lane (g, r) of block_row_sum
// will read (and their column indices), before the row waits on its dependencies.
template <int ND, typename T>
__device__ __forceinline__ void prefetch_row(const T* __restrict__ F, const int32_t* __restrict__ f_col, int64_t pa,
                                             int64_t pb) {
  constexpr int BB = ND * ND, G = 32 / ND;
  const int lane = threadIdx.x & 31;
  const int g = lane / ND, r = lane - g * ND;
  if (g < G)
    for (int64_t p = pa + g; p < pb; p += G) {
      const T* row = F + p * BB + r * ND;
      asm volatile("prefetch.global.L1 [%0];" ::"l"(row));
      asm volatile("prefetch.global.L1 [%0];" ::"l"(row + ND - 1));
    }
  for (int64_t p = pa + lane; p < pb; p += 32) asm volatile("prefetch.global.L1 [%0];" ::"l"(f_col + p));
}

template <int ND, typename T>
__global__ void __launch_bounds__(32 * kWarpsPerBlock)
    ilu_lower_sweep_kernel(const T* __restrict__ F, const int64_t* __restrict__ f_rp, const int32_t* __restrict__ f_col,
                           const int64_t* __restrict__ f_diag, const int32_t* __restrict__ rows, int64_t n,
                           const double* vbase, T* zwbase, const int* __restrict__ jidx, int64_t ld, int zw_follows,
                           unsigned int* ticket, int* ready, unsigned int* status) {
  constexpr int BB = ND * ND;
  __shared__ T red[kWarpsPerBlock][32];
  const int lane = threadIdx.x & 31;
  const int64_t off = jidx ? (int64_t)(*jidx) * ld : 0;
  const double* v = vbase + off;
  T* zw = zwbase + (zw_follows ? off : 0);
  for (;;) {
    unsigned int t = 0;
    if (lane == 0) t = atomicAdd(ticket, 1u);
    t = __shfl_sync(0xffffffffu, t, 0);
    if ((int64_t)t >= n) break;
    const int32_t I = rows[t];
    const int64_t p0 = f_rp[I], pd = f_diag[I];
    prefetch_row<ND, T>(F, f_col, p0, pd + 1);
    bool ok = true;
    for (int64_t p = p0 + lane; p < pd && ok; p += 32) ok = wait_flag(ready + f_col[p]);
    if (!ok) atomicOr(status, (unsigned)GALES_ERR_TIMEOUT);
    __syncwarp();
    const int r = lane < ND ? lane : 0;
    const T vi = (T)v[(int64_t)I * ND + r];
    T s = vi - block_row_sum<ND, T, true>(F, f_col, p0, pd, zw, red[threadIdx.x >> 5]);
    const T* D = F + pd * BB + r * ND;
#pragma unroll
    for (int c = 0; c < ND - 1; ++c) {
      const T zc = __shfl_sync(0xffffffffu, s, c);
      if (lane > c) s -= D[c] * zc;
    }
    // lane 0 writes the row, then releases its ready flag
    T row[ND];
#pragma unroll
    for (int c = 0; c < ND; ++c) row[c] = __shfl_sync(0xffffffffu, s, c);
    if (lane == 0) {
#pragma unroll
      for (int c = 0; c < ND; ++c) zw[(int64_t)I * ND + c] = row[c];
      st_release(ready + I, 1);
    }
  }
}

template <int ND, typename T>
__global__ void __launch_bounds__(32 * kWarpsPerBlock)
    ilu_upper_sweep_kernel(const T* __restrict__ F, const int64_t* __restrict__ f_rp, const int32_t* __restrict__ f_col,
                           const int64_t* __restrict__ f_diag, const int32_t* __restrict__ rows, int64_t n, T* zwbase,
                           double* zoutbase, const int* __restrict__ jidx, int64_t ld, int zw_follows,
                           unsigned int* ticket, int* ready, unsigned int* status) {
  constexpr int BB = ND * ND;
  __shared__ T red[kWarpsPerBlock][32];
  const int lane = threadIdx.x & 31;
  const int64_t off = jidx ? (int64_t)(*jidx) * ld : 0;
  T* zw = zwbase + (zw_follows ? off : 0);
  double* zout = zoutbase + off;
  for (;;) {
    unsigned int t = 0;
    if (lane == 0) t = atomicAdd(ticket, 1u);
    t = __shfl_sync(0xffffffffu, t, 0);
    if ((int64_t)t >= n) break;
    const int32_t I = rows[t];
    const int64_t p1 = f_rp[I + 1], pd = f_diag[I];
    prefetch_row<ND, T>(F, f_col, pd, p1);
    bool ok = true;
    for (int64_t p = pd + 1 + lane; p < p1 && ok; p += 32) ok = wait_flag(ready + f_col[p]);
    if (!ok) atomicOr(status, (unsigned)GALES_ERR_TIMEOUT);
    __syncwarp();
    const int r = lane < ND ? lane : 0;
    const T yi = __ldcg(zw + (int64_t)I * ND + r);
    T s = yi - block_row_sum<ND, T, true>(F, f_col, pd + 1, p1, zw, red[threadIdx.x >> 5]);
    const T* D = F + pd * BB + r * ND;
#pragma unroll
    for (int c = ND - 1; c >= 0; --c) {
      const T mine = s / D[c];  // meaningful on lane c only
      const T xc = __shfl_sync(0xffffffffu, mine, c);
      if (lane == c) s = xc;
      else if (lane < c) s -= D[c] * xc;
    }
    if (!zw_follows && lane < ND) zout[(int64_t)I * ND + lane] = (double)s;
    // lane 0 writes the row of the working vector, then releases its ready flag
    T row[ND];
#pragma unroll
    for (int c = 0; c < ND; ++c) row[c] = __shfl_sync(0xffffffffu, s, c);
    if (lane == 0) {
#pragma unroll
      for (int c = 0; c < ND; ++c) zw[(int64_t)I * ND + c] = row[c];
      st_release(ready + I, 1);
    }
  }
}

// y = A x (or y = b - A x) on the assembly's CSR values: warp per scalar row.
template <int ND>
__global__ void spmv_kernel(const double* __restrict__ vals, const int64_t* __restrict__ node_rp,
                            const int32_t* __restrict__ node_col, int64_t n_rows, const double* __restrict__ x,
                            const double* __restrict__ b, double* __restrict__ y) {
  const int64_t row = (int64_t)blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
  if (row >= n_rows) return;
  const int lane = threadIdx.x & 31;
  const int64_t i = row / ND;
  const int k = (int)(row % ND);
  const int64_t t0 = node_rp[i], len = (node_rp[i + 1] - t0) * ND;
  const double* a = vals + t0 * ND * ND + k * len;
  double s = 0.0;
  for (int64_t e = lane; e < len; e += 32) s += a[e] * x[(int64_t)node_col[t0 + e / ND] * ND + e % ND];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) y[row] = b ? b[row] - s : s;
}

// Partial dot products of w with the columns V[0..nv) (column stride ld), four columns
// at a time: part[block][c].
__global__ void mdot_kernel(const double* __restrict__ V, int64_t ld, int nv, const double* __restrict__ w,
                            int64_t n, double* __restrict__ part) {
  __shared__ double sh[kDotThreads / 32][4];
  const int64_t per = (n + gridDim.x - 1) / gridDim.x;
  const int64_t lo = (int64_t)blockIdx.x * per, hi = lo + per < n ? lo + per : n;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int c0 = 0; c0 < nv; c0 += 4) {
    double a[4] = {0.0, 0.0, 0.0, 0.0};
    const int m = nv - c0 < 4 ? nv - c0 : 4;
    for (int64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
      const double wi = w[i];
#pragma unroll
      for (int q = 0; q < 4; ++q)
        if (q < m) a[q] += V[(int64_t)(c0 + q) * ld + i] * wi;
    }
#pragma unroll
    for (int q = 0; q < 4; ++q)
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) a[q] += __shfl_xor_sync(0xffffffffu, a[q], o);
    if (lane == 0)
#pragma unroll
      for (int q = 0; q < 4; ++q) sh[wid][q] = a[q];
    __syncthreads();
    if (threadIdx.x < m) {
      double s = 0.0;
      for (int k = 0; k < kDotThreads / 32; ++k) s += sh[k][threadIdx.x];
      part[(int64_t)blockIdx.x * nv + c0 + threadIdx.x] = s;
    }
    __syncthreads();
  }
}

// out[c] (mode 0) = sum_b part[b][c]; mode 1: out[c] += sum; mode 2: out[0] = sqrt(sum).
__global__ void mdot_final_kernel(const double* __restrict__ part, int nb, int nv, double* __restrict__ out,
                                  int mode) {
  for (int c = threadIdx.x; c < nv; c += blockDim.x) {
    double s = 0.0;
    for (int b = 0; b < nb; ++b) s += part[(int64_t)b * nv + c];
    if (mode == 0) out[c] = s;
    else if (mode == 1) out[c] += s;
    else out[c] = sqrt(s);
  }
}

// w -= sum_c V[c] h[c]
__global__ void axpy_multi_kernel(const double* __restrict__ V, int64_t ld, int nv, const double* __restrict__ h,
                                  double* __restrict__ w, int64_t n) {
  extern __shared__ double hs[];
  for (int c = threadIdx.x; c < nv; c += blockDim.x) hs[c] = h[c];
  __syncthreads();
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int c = 0; c < nv; ++c) s += V[(int64_t)c * ld + i] * hs[c];
    w[i] -= s;
  }
}

// x += sum_c Z[c] y[c]
__global__ void update_x_kernel(const double* __restrict__ Z, int64_t ld, int nv, const double* __restrict__ y,
                                double* __restrict__ x, int64_t n) {
  extern __shared__ double ys[];
  for (int c = threadIdx.x; c < nv; c += blockDim.x) ys[c] = y[c];
  __syncthreads();
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int c = 0; c < nv; ++c) s += Z[(int64_t)c * ld + i] * ys[c];
    x[i] += s;
  }
}

// dst = src / *nrm (dst = 0 when the norm is zero)
__global__ void scale_kernel(const double* __restrict__ src, const double* __restrict__ nrm, double* __restrict__ dst,
                             int64_t n) {
  const double d = *nrm;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = d > 0.0 ? src[i] / d : 0.0;
}

__global__ void set_index_kernel(int* __restrict__ p, int v) { *p = v; }

__global__ void copy_kernel(const double* __restrict__ src, double* __restrict__ dst, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = src[i];
}

// fluid_updater::corrector then model::dof_trimmer: I += dx, then the dofs with index
// in [first, last) of every node clamped as max(lo, min(v, hi)).
__global__ void correct_kernel(double* __restrict__ I, const double* __restrict__ dx, int64_t n, int nd, int first,
                               int last, double lo, double hi) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double v = I[i] + dx[i];
    const int k = (int)(i % nd);
    if (k >= first && k < last) v = fmax(lo, fmin(v, hi));
    I[i] = v;
  }
}

}  // namespace

// ---------------------------------------------------------------------------
// Handle and C ABI.
// ---------------------------------------------------------------------------

struct gales_solver {
  int device = 0;
  int nd = 0;
  int sms = 1;
  int64_t n_nodes = 0, n_rows = 0, nnz = 0;
  gales_solver_params prm{};
  std::vector<int64_t> node_rp, f_rp, f_diag, lev_off_f, lev_off_b;
  std::vector<int32_t> node_col, f_col, lev_f, lev_b, rows_f, rows_b;
  Dev<int64_t> d_node_rp, d_f_rp, d_f_diag, d_a2f;
  Dev<int32_t> d_node_col, d_f_col, d_rows_f, d_rows_b;
  Dev<double> d_F, d_V, d_Z, d_w, d_r, d_x, d_part, d_h, d_h2, d_y, d_vals, d_b;
  Dev<float> d_Ff, d_zf;     // FP32 factor and its substitution vector (GALES_PRECOND_ILU_FP32)
  Dev<int> d_j;
  Dev<int> d_sync;           // sweep tickets [2] and ready flags [2][n_nodes] of the substitutions
  Dev<unsigned int> d_status;
  double* h_buf = nullptr;   // pinned: Hessenberg column and the least-squares solution
  int m = 0;                 // Krylov vectors per cycle
  int max_row = 0, max_u = 0;  // longest factor row, longest upper part (blocks)
  int smem_optin = 0;          // opt-in shared memory per CTA
  size_t factor_smem = 0;      // dynamic shared memory of the staged factor kernel (0: not used)
  int dot_blocks = 1;
  cudaGraphExec_t prec_graph = nullptr;
  cudaStream_t cap = nullptr;
  int64_t launches = 0;
  std::string err;
};

namespace {

int sfail(gales_solver* s, int code, const std::string& msg) {
  if (s) s->err = msg;
  return code;
}

#define SCK(s, call, what)                                                                               \
  do {                                                                                                   \
    cudaError_t e__ = (call);                                                                            \
    if (e__ != cudaSuccess)                                                                              \
      return sfail(s, e__ == cudaErrorMemoryAllocation ? GALES_ERR_NO_MEMORY : GALES_ERR_CUDA,            \
                   std::string(what) + ": " + cudaGetErrorString(e__));                                  \
  } while (0)

bool dev_ptr(const void* p) {
  if (!p) return false;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

inline unsigned grid_for(int64_t warps) { return (unsigned)((warps + kWarpsPerBlock - 1) / kWarpsPerBlock); }

template <typename T>
T* factor_ptr(gales_solver* s);
template <>
double* factor_ptr<double>(gales_solver* s) { return s->d_F.p; }
template <>
float* factor_ptr<float>(gales_solver* s) { return s->d_Ff.p; }

// Launch wrappers for nd = ND and a factor stored in T (double: the reference's FP64
// arithmetic; float: FP32 factor and substitutions, scratch vector d_zf).
template <int ND, typename T>
struct Kernels {
  static constexpr bool kF64 = sizeof(T) == sizeof(double);
  static cudaError_t to_factor(gales_solver* s, const double* vals, cudaStream_t st) {
    matrix_to_factor_kernel<ND, T><<<grid_for(s->n_nodes), 32 * kWarpsPerBlock, 0, st>>>(
        vals, s->d_node_rp.p, s->d_a2f.p, s->n_nodes, factor_ptr<T>(s));
    return cudaGetLastError();
  }
  static size_t factor_smem(int max_row, int max_u) {
    return ((size_t)max_row + 1 + max_u) * ND * ND * sizeof(T) + ((size_t)max_row + max_u) * sizeof(int32_t);
  }
  static cudaError_t prepare(gales_solver* s) {
    const size_t bytes = factor_smem(s->max_row, s->max_u);
    s->factor_smem = 0;
    if (bytes > (size_t)s->smem_optin) return cudaSuccess;  // rows too long: the global-memory kernel
    cudaError_t e = cudaFuncSetAttribute(ilu_factor_level_smem_kernel<ND, T>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e == cudaSuccess) s->factor_smem = bytes;
    return e;
  }
  static cudaError_t factor_level(gales_solver* s, int l, cudaStream_t st) {
    const int64_t o = s->lev_off_f[l], c = s->lev_off_f[l + 1] - o;
    if (s->factor_smem)
      ilu_factor_level_smem_kernel<ND, T><<<(unsigned)c, 32, s->factor_smem, st>>>(
          factor_ptr<T>(s), s->d_f_rp.p, s->d_f_col.p, s->d_f_diag.p, s->d_rows_f.p + o, c, s->d_status.p,
          s->max_row, s->max_u);
    else
      ilu_factor_level_kernel<ND, T><<<grid_for(c), 32 * kWarpsPerBlock, 0, st>>>(
          factor_ptr<T>(s), s->d_f_rp.p, s->d_f_col.p, s->d_f_diag.p, s->d_rows_f.p + o, c, s->d_status.p);
    return cudaGetLastError();
  }
  static cudaError_t lower_level(gales_solver* s, int l, const double* v, double* z, const int* j, int64_t ld,
                                 cudaStream_t st) {
    const int64_t o = s->lev_off_f[l], c = s->lev_off_f[l + 1] - o;
    T* zw = kF64 ? reinterpret_cast<T*>(z) : reinterpret_cast<T*>(s->d_zf.p);
    ilu_lower_level_kernel<ND, T><<<grid_for(c), 32 * kWarpsPerBlock, 0, st>>>(
        factor_ptr<T>(s), s->d_f_rp.p, s->d_f_col.p, s->d_f_diag.p, s->d_rows_f.p + o, c, v, zw, j, ld,
        kF64 ? 1 : 0);
    return cudaGetLastError();
  }
  static cudaError_t upper_level(gales_solver* s, int l, double* z, const int* j, int64_t ld, cudaStream_t st) {
    const int64_t o = s->lev_off_b[l], c = s->lev_off_b[l + 1] - o;
    T* zw = kF64 ? reinterpret_cast<T*>(z) : reinterpret_cast<T*>(s->d_zf.p);
    ilu_upper_level_kernel<ND, T><<<grid_for(c), 32 * kWarpsPerBlock, 0, st>>>(
        factor_ptr<T>(s), s->d_f_rp.p, s->d_f_col.p, s->d_f_diag.p, s->d_rows_b.p + o, c, zw, z, j, ld,
        kF64 ? 1 : 0);
    return cudaGetLastError();
  }
  // both substitutions as sync-free sweeps (tickets and ready flags cleared by the caller)
  static cudaError_t sweeps(gales_solver* s, const double* v, double* z, const int* j, int64_t ld, cudaStream_t st) {
    T* zw = kF64 ? reinterpret_cast<T*>(z) : reinterpret_cast<T*>(s->d_zf.p);
    const unsigned g = std::min<unsigned>(grid_for(s->n_nodes), (unsigned)s->sms);
    unsigned int* tk = reinterpret_cast<unsigned int*>(s->d_sync.p);
    int* ready = s->d_sync.p + 2;
    ilu_lower_sweep_kernel<ND, T><<<g, 32 * kWarpsPerBlock, 0, st>>>(
        factor_ptr<T>(s), s->d_f_rp.p, s->d_f_col.p, s->d_f_diag.p, s->d_rows_f.p, s->n_nodes, v, zw, j, ld,
        kF64 ? 1 : 0, tk, ready, s->d_status.p);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    ilu_upper_sweep_kernel<ND, T><<<g, 32 * kWarpsPerBlock, 0, st>>>(
        factor_ptr<T>(s), s->d_f_rp.p, s->d_f_col.p, s->d_f_diag.p, s->d_rows_b.p, s->n_nodes, zw, z, j, ld,
        kF64 ? 1 : 0, tk + 1, ready + s->n_nodes, s->d_status.p);
    return cudaGetLastError();
  }
  static cudaError_t spmv(gales_solver* s, const double* vals, const double* x, const double* b, double* y,
                          cudaStream_t st) {
    spmv_kernel<ND><<<grid_for(s->n_rows), 32 * kWarpsPerBlock, 0, st>>>(vals, s->d_node_rp.p, s->d_node_col.p,
                                                                        s->n_rows, x, b, y);
    return cudaGetLastError();
  }
};

struct Ops {
  cudaError_t (*prepare)(gales_solver*);
  cudaError_t (*to_factor)(gales_solver*, const double*, cudaStream_t);
  cudaError_t (*factor_level)(gales_solver*, int, cudaStream_t);
  cudaError_t (*lower_level)(gales_solver*, int, const double*, double*, const int*, int64_t, cudaStream_t);
  cudaError_t (*upper_level)(gales_solver*, int, double*, const int*, int64_t, cudaStream_t);
  cudaError_t (*sweeps)(gales_solver*, const double*, double*, const int*, int64_t, cudaStream_t);
  cudaError_t (*spmv)(gales_solver*, const double*, const double*, const double*, double*, cudaStream_t);
};

template <int ND, typename T>
Ops ops_for() {
  using K = Kernels<ND, T>;
  return {K::prepare, K::to_factor, K::factor_level, K::lower_level, K::upper_level, K::sweeps, K::spmv};
}

template <typename T>
bool ops_t(int nd, Ops& o) {
  switch (nd) {
    case 4: o = ops_for<4, T>(); return true;
    case 5: o = ops_for<5, T>(); return true;
    case 6: o = ops_for<6, T>(); return true;
    case 7: o = ops_for<7, T>(); return true;
    case 8: o = ops_for<8, T>(); return true;
    case 9: o = ops_for<9, T>(); return true;
    case 10: o = ops_for<10, T>(); return true;
    case 11: o = ops_for<11, T>(); return true;
    case 12: o = ops_for<12, T>(); return true;
    default: return false;
  }
}

bool ops(const gales_solver* s, Ops& o) {
  return s->prm.precond == GALES_PRECOND_ILU_FP32 ? ops_t<float>(s->nd, o) : ops_t<double>(s->nd, o);
}

inline bool has_ilu(const gales_solver* s) {
  return s->prm.precond == GALES_PRECOND_ILU || s->prm.precond == GALES_PRECOND_ILU_FP32;
}

// z = M^-1 v for columns addressed by *j (graph) or plain pointers (j null): the two
// sync-free sweeps after clearing their tickets and ready flags.
int apply_prec(gales_solver* s, const Ops& o, const double* v, double* z, const int* j, int64_t ld, cudaStream_t st) {
  SCK(s, cudaMemsetAsync(s->d_sync.p, 0, s->d_sync.n * sizeof(int), st), "clear sweep flags");
  SCK(s, o.sweeps(s, v, z, j, ld, st), "substitutions");
  s->launches += 2;
  return 0;
}

// norm / dots on device: out[0..nv) = V[0..nv)^T w (mode 0/1) or out[0] = ||w|| (mode 2)
int mdot(gales_solver* s, const double* V, int64_t ld, int nv, const double* w, double* out, int mode,
         cudaStream_t st) {
  mdot_kernel<<<s->dot_blocks, kDotThreads, 0, st>>>(V, ld, nv, w, s->n_rows, s->d_part.p);
  mdot_final_kernel<<<1, 256, 0, st>>>(s->d_part.p, s->dot_blocks, nv, out, mode);
  s->launches += 2;
  SCK(s, cudaGetLastError(), "dot products");
  return 0;
}

unsigned stream_grid(int64_t n, int sms) {
  const int64_t b = (n + 255) / 256;
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(b, (int64_t)sms * 8));
}

int factorize(gales_solver* s, const Ops& o, const double* vals, cudaStream_t st) {
  if (s->prm.precond == GALES_PRECOND_ILU_FP32)
    SCK(s, cudaMemsetAsync(s->d_Ff.p, 0, s->d_Ff.n * sizeof(float), st), "clear factor");
  else
    SCK(s, cudaMemsetAsync(s->d_F.p, 0, s->d_F.n * sizeof(double), st), "clear factor");
  SCK(s, cudaMemsetAsync(s->d_status.p, 0, sizeof(unsigned int), st), "clear status");
  SCK(s, o.to_factor(s, vals, st), "matrix to factor");
  const int nf = (int)s->lev_off_f.size() - 1;
  for (int l = 0; l < nf; ++l) SCK(s, o.factor_level(s, l, st), "factor level");
  s->launches += 1 + nf;
  unsigned int stat = 0;
  SCK(s, cudaMemcpyAsync(&stat, s->d_status.p, sizeof(stat), cudaMemcpyDeviceToHost, st), "status");
  SCK(s, cudaStreamSynchronize(st), "factorisation");
  if (stat) return sfail(s, GALES_ERR_SINGULAR, "zero pivot in the incomplete factorisation");
  return 0;
}

int capture_prec_graph(gales_solver* s, const Ops& o) {
  if (s->prec_graph) return 0;
  SCK(s, cudaStreamCreateWithFlags(&s->cap, cudaStreamNonBlocking), "capture stream");
  SCK(s, cudaStreamBeginCapture(s->cap, cudaStreamCaptureModeThreadLocal), "begin capture");
  const int64_t before = s->launches;
  const int rc = apply_prec(s, o, s->d_V.p, s->d_Z.p, s->d_j.p, s->n_rows, s->cap);
  s->launches = before;
  cudaGraph_t g = nullptr;
  const cudaError_t e = cudaStreamEndCapture(s->cap, &g);
  if (rc) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  SCK(s, e, "end capture");
  const cudaError_t ei = cudaGraphInstantiate(&s->prec_graph, g, 0);
  cudaGraphDestroy(g);
  SCK(s, ei, "instantiate graph");
  return 0;
}

}  // namespace

extern "C" {

void gales_solver_default(gales_solver_params* p) {
  if (!p) return;
  p->rel_res_tol = 1e-9;
  p->maxsubspace = 200;
  p->maxrestarts = 5;
  p->maxiters = -1;
  p->fill = 1;
  p->precond = GALES_PRECOND_ILU;
}

int gales_iluk_pattern(int64_t n, const int64_t* row_ptr, const int32_t* col, int32_t fill, int64_t* nnz,
                       int64_t* f_row_ptr, int32_t* f_col, int32_t* level_fwd, int32_t* level_bwd,
                       int32_t* n_levels) {
  if (n < 0 || !row_ptr || (n > 0 && !col) || fill < 0 || !nnz) return GALES_ERR_BAD_INPUT;
  std::vector<int64_t> rp, diag, off;
  std::vector<int32_t> fc, lev, rows;
  iluk_symbolic(n, row_ptr, col, fill, rp, fc, diag);
  *nnz = (int64_t)fc.size();
  if (f_row_ptr) std::memcpy(f_row_ptr, rp.data(), sizeof(int64_t) * (n + 1));
  if (f_col) std::memcpy(f_col, fc.data(), sizeof(int32_t) * fc.size());
  level_sets(n, rp, fc, diag, true, lev, off, rows);
  if (level_fwd) std::memcpy(level_fwd, lev.data(), sizeof(int32_t) * n);
  if (n_levels) n_levels[0] = (int32_t)off.size() - 1;
  level_sets(n, rp, fc, diag, false, lev, off, rows);
  if (level_bwd) std::memcpy(level_bwd, lev.data(), sizeof(int32_t) * n);
  if (n_levels) n_levels[1] = (int32_t)off.size() - 1;
  return 0;
}

int gales_solver_create(gales_asm* h, const gales_solver_params* prm, gales_solver** out) {
  if (!h || !out) return GALES_ERR_BAD_INPUT;
  *out = nullptr;
  gales_solver_params p;
  gales_solver_default(&p);
  if (prm) p = *prm;
  if (!(p.rel_res_tol >= 0.0) || p.maxsubspace < 1 || p.maxrestarts < 0 || p.fill < 0 ||
      (p.precond != GALES_PRECOND_ILU && p.precond != GALES_PRECOND_ILU_FP32 && p.precond != GALES_PRECOND_NONE))
    return GALES_ERR_BAD_INPUT;
  int64_t n_nodes = 0, nnz_nodes = 0, n_rows = 0, nnz = 0;
  const int64_t* nrp = nullptr;
  const int32_t* ncol = nullptr;
  int rc = gales_asm_node_graph(h, &n_nodes, &nnz_nodes, &nrp, &ncol);
  if (rc) return rc;
  rc = gales_asm_pattern(h, &n_rows, &nnz, nullptr, nullptr);
  if (rc) return rc;
  if (n_nodes <= 0 || n_rows % n_nodes) return GALES_ERR_BAD_INPUT;
  auto* s = new gales_solver();
  s->prm = p;
  s->nd = (int)(n_rows / n_nodes);
  s->n_nodes = n_nodes;
  s->n_rows = n_rows;
  s->nnz = nnz;
  s->m = p.maxsubspace;
  Ops o;
  if (!ops(s, o)) {
    delete s;
    return GALES_ERR_UNSUPPORTED;
  }
  s->node_rp.assign(nrp, nrp + n_nodes + 1);
  s->node_col.assign(ncol, ncol + nnz_nodes);
  auto bail = [&](int code) {
    gales_solver_destroy(s);
    return code;
  };
  cudaGetDevice(&s->device);
  cudaDeviceGetAttribute(&s->sms, cudaDevAttrMultiProcessorCount, s->device);
  s->dot_blocks = std::max(1, 2 * s->sms);
  std::vector<int64_t> a2f;
  if (has_ilu(s)) {
    iluk_symbolic(n_nodes, s->node_rp.data(), s->node_col.data(), p.fill, s->f_rp, s->f_col, s->f_diag);
    level_sets(n_nodes, s->f_rp, s->f_col, s->f_diag, true, s->lev_f, s->lev_off_f, s->rows_f);
    level_sets(n_nodes, s->f_rp, s->f_col, s->f_diag, false, s->lev_b, s->lev_off_b, s->rows_b);
    for (int64_t i = 0; i < n_nodes; ++i) {
      s->max_row = std::max(s->max_row, (int)(s->f_rp[i + 1] - s->f_rp[i]));
      s->max_u = std::max(s->max_u, (int)(s->f_rp[i + 1] - s->f_diag[i] - 1));
    }
    a2f.resize(nnz_nodes);
    for (int64_t i = 0; i < n_nodes; ++i) {
      int64_t q = s->f_rp[i];
      for (int64_t t = s->node_rp[i]; t < s->node_rp[i + 1]; ++t) {
        while (s->f_col[q] != s->node_col[t]) ++q;
        a2f[t] = q;
      }
    }
  }
  const size_t bb = (size_t)s->nd * s->nd;
  if (s->d_node_rp.upload(s->node_rp) || s->d_node_col.upload(s->node_col) || s->d_f_rp.upload(s->f_rp) ||
      s->d_f_col.upload(s->f_col) || s->d_f_diag.upload(s->f_diag) || s->d_a2f.upload(a2f) ||
      s->d_rows_f.upload(s->rows_f) || s->d_rows_b.upload(s->rows_b) || (p.precond == GALES_PRECOND_ILU ? s->d_F.alloc(s->f_col.size() * bb)
                                       : s->d_Ff.alloc(s->f_col.size() * bb)) ||
      (p.precond == GALES_PRECOND_ILU_FP32 ? s->d_zf.alloc(n_rows) : cudaSuccess) ||
      s->d_V.alloc((size_t)(s->m + 1) * n_rows) || s->d_Z.alloc((size_t)s->m * n_rows) || s->d_w.alloc(n_rows) ||
      s->d_r.alloc(n_rows) || s->d_x.alloc(n_rows) || s->d_part.alloc((size_t)s->dot_blocks * (s->m + 2)) ||
      s->d_h.alloc(s->m + 2) || s->d_h2.alloc(s->m + 2) || s->d_y.alloc(s->m + 2) || s->d_j.alloc(1) ||
      s->d_sync.alloc(2 + 2 * (size_t)n_nodes) || s->d_status.alloc(1)) {
    cudaGetLastError();
    return bail(GALES_ERR_NO_MEMORY);
  }
  if (cudaMallocHost(&s->h_buf, sizeof(double) * 2 * (s->m + 2)) != cudaSuccess) {
    cudaGetLastError();
    return bail(GALES_ERR_NO_MEMORY);
  }
  if (has_ilu(s)) {
    cudaDeviceGetAttribute(&s->smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, s->device);
    if (o.prepare(s) != cudaSuccess) {
      cudaGetLastError();
      s->factor_smem = 0;
    }
    rc = capture_prec_graph(s, o);
    if (rc) {
      // plain launches remain available
      cudaGetLastError();
      s->prec_graph = nullptr;
    }
  }
  *out = s;
  return 0;
}

int gales_solver_factorize(gales_solver* s, const double* vals, void* stream) {
  if (!s || !vals) return GALES_ERR_BAD_INPUT;
  if (!has_ilu(s)) return 0;
  SCK(s, cudaSetDevice(s->device), "cudaSetDevice");
  cudaStream_t st = (cudaStream_t)stream;
  const double* dv = vals;
  if (!dev_ptr(vals)) {
    SCK(s, s->d_vals.alloc(s->nnz), "staging values");
    SCK(s, cudaMemcpyAsync(s->d_vals.p, vals, s->nnz * sizeof(double), cudaMemcpyHostToDevice, st), "copy values");
    dv = s->d_vals.p;
  }
  Ops o;
  ops(s, o);
  return factorize(s, o, dv, st);
}

int gales_solver_apply(gales_solver* s, const double* v, double* z, void* stream) {
  if (!s || !v || !z || !dev_ptr(v) || !dev_ptr(z)) return GALES_ERR_BAD_INPUT;
  SCK(s, cudaSetDevice(s->device), "cudaSetDevice");
  cudaStream_t st = (cudaStream_t)stream;
  if (!has_ilu(s)) {
    copy_kernel<<<stream_grid(s->n_rows, s->sms), 256, 0, st>>>(v, z, s->n_rows);
    SCK(s, cudaGetLastError(), "copy");
    return 0;
  }
  Ops o;
  ops(s, o);
  return apply_prec(s, o, v, z, nullptr, 0, st);
}

int gales_solver_factor(gales_solver* s, int64_t* n_block_rows, int64_t* nnz_blocks, const int64_t** row_ptr,
                        const int32_t** col, double* vals) {
  if (!s) return GALES_ERR_BAD_INPUT;
  if (n_block_rows) *n_block_rows = s->n_nodes;
  if (nnz_blocks) *nnz_blocks = (int64_t)s->f_col.size();
  if (row_ptr) *row_ptr = s->f_rp.data();
  if (col) *col = s->f_col.data();
  if (vals && !s->f_col.empty()) {
    SCK(s, cudaSetDevice(s->device), "cudaSetDevice");
    SCK(s, cudaDeviceSynchronize(), "synchronize");
    const size_t cnt = s->f_col.size() * s->nd * s->nd;
    if (s->prm.precond == GALES_PRECOND_ILU_FP32) {
      std::vector<float> tmp(cnt);
      SCK(s, cudaMemcpy(tmp.data(), s->d_Ff.p, cnt * sizeof(float), cudaMemcpyDeviceToHost), "copy factor");
      for (size_t i = 0; i < cnt; ++i) vals[i] = tmp[i];
    } else {
      SCK(s, cudaMemcpy(vals, s->d_F.p, cnt * sizeof(double), cudaMemcpyDeviceToHost), "copy factor");
    }
  }
  return 0;
}

int gales_solver_levels(gales_solver* s, int32_t* n_levels_fwd, int32_t* n_levels_bwd) {
  if (!s) return GALES_ERR_BAD_INPUT;
  if (n_levels_fwd) *n_levels_fwd = s->lev_off_f.empty() ? 0 : (int32_t)s->lev_off_f.size() - 1;
  if (n_levels_bwd) *n_levels_bwd = s->lev_off_b.empty() ? 0 : (int32_t)s->lev_off_b.size() - 1;
  return 0;
}

int gales_solver_solve(gales_solver* s, const double* vals, const double* rhs, double* x, gales_solver_result* res,
                       void* stream) {
  if (!s || !vals || !rhs || !x) return GALES_ERR_BAD_INPUT;
  const auto t_start = std::chrono::steady_clock::now();
  SCK(s, cudaSetDevice(s->device), "cudaSetDevice");
  cudaStream_t st = (cudaStream_t)stream;
  const int64_t n = s->n_rows;
  const int m = s->m;
  const gales_solver_params& p = s->prm;
  const int64_t maxiters = p.maxiters < 0 ? n - 1 : p.maxiters;
  Ops o;
  ops(s, o);
  const double* dA = vals;
  if (!dev_ptr(vals)) {
    SCK(s, s->d_vals.alloc(s->nnz), "staging values");
    SCK(s, cudaMemcpyAsync(s->d_vals.p, vals, s->nnz * sizeof(double), cudaMemcpyHostToDevice, st), "copy values");
    dA = s->d_vals.p;
  }
  const double* db = rhs;
  if (!dev_ptr(rhs)) {
    SCK(s, s->d_b.alloc(n), "staging rhs");
    SCK(s, cudaMemcpyAsync(s->d_b.p, rhs, n * sizeof(double), cudaMemcpyHostToDevice, st), "copy rhs");
    db = s->d_b.p;
  }
  const bool x_dev = dev_ptr(x);
  double* dx = x_dev ? x : s->d_x.p;
  const bool prec = has_ilu(s);
  if (prec) {
    const int rc = factorize(s, o, dA, st);
    if (rc) return rc;
  }
  SCK(s, cudaMemsetAsync(dx, 0, n * sizeof(double), st), "clear x");
  const unsigned sg = stream_grid(n, s->sms);
  double* V = s->d_V.p;
  double* Z = s->d_Z.p;
  double* hb = s->h_buf;
  std::vector<double> H((size_t)(m + 1) * m), cs(m), sn(m), g(m + 1), y(m), h(m + 2);
  // ||b||; r = b (x0 = 0)
  int rc = mdot(s, db, 0, 1, db, s->d_h.p + m + 1, 2, st);
  if (rc) return rc;
  SCK(s, cudaMemcpyAsync(hb, s->d_h.p + m + 1, sizeof(double), cudaMemcpyDeviceToHost, st), "norm");
  SCK(s, cudaStreamSynchronize(st), "norm");
  const double bnorm = hb[0];
  double beta = bnorm;
  const double* r = db;
  int64_t iters = 0;
  int cycles = 0;
  bool converged = bnorm == 0.0;
  while (!converged && cycles <= p.maxrestarts && iters < maxiters && beta > 0.0) {
    ++cycles;
    // V0 = r / beta (beta on the device in d_h[m+1])
    scale_kernel<<<sg, 256, 0, st>>>(r, s->d_h.p + m + 1, V, n);
    ++s->launches;
    std::fill(g.begin(), g.end(), 0.0);
    g[0] = beta;
    int j = 0;
    bool est_conv = false;
    for (; j < m && iters < maxiters; ++j) {
      double* vj = V + (int64_t)j * n;
      double* zj = Z + (int64_t)j * n;
      if (prec) {
        if (s->prec_graph) {
          set_index_kernel<<<1, 1, 0, st>>>(s->d_j.p, j);
          SCK(s, cudaGraphLaunch(s->prec_graph, st), "preconditioner graph");
          s->launches += 3;
        } else {
          rc = apply_prec(s, o, vj, zj, nullptr, 0, st);
          if (rc) return rc;
        }
      } else {
        copy_kernel<<<sg, 256, 0, st>>>(vj, zj, n);
        ++s->launches;
      }
      SCK(s, o.spmv(s, dA, zj, nullptr, s->d_w.p, st), "spmv");
      ++s->launches;
      // two classical Gram-Schmidt passes: h = V^T w, w -= V h (twice; h summed)
      rc = mdot(s, V, n, j + 1, s->d_w.p, s->d_h.p, 0, st);
      if (rc) return rc;
      axpy_multi_kernel<<<sg, 256, (j + 1) * sizeof(double), st>>>(V, n, j + 1, s->d_h.p, s->d_w.p, n);
      rc = mdot(s, V, n, j + 1, s->d_w.p, s->d_h2.p, 0, st);
      if (rc) return rc;
      axpy_multi_kernel<<<sg, 256, (j + 1) * sizeof(double), st>>>(V, n, j + 1, s->d_h2.p, s->d_w.p, n);
      mdot_final_kernel<<<1, 256, 0, st>>>(s->d_h2.p, 1, j + 1, s->d_h.p, 1);  // h += h2
      rc = mdot(s, s->d_w.p, 0, 1, s->d_w.p, s->d_h.p + j + 1, 2, st);
      if (rc) return rc;
      scale_kernel<<<sg, 256, 0, st>>>(s->d_w.p, s->d_h.p + j + 1, V + (int64_t)(j + 1) * n, n);
      s->launches += 4;
      SCK(s, cudaGetLastError(), "Arnoldi step");
      SCK(s, cudaMemcpyAsync(hb, s->d_h.p, (j + 2) * sizeof(double), cudaMemcpyDeviceToHost, st), "Hessenberg");
      SCK(s, cudaStreamSynchronize(st), "Arnoldi step");
      for (int c = 0; c <= j + 1; ++c) h[c] = hb[c];
      const double hn = h[j + 1];
      for (int c = 0; c < j; ++c) {
        const double t = cs[c] * h[c] + sn[c] * h[c + 1];
        h[c + 1] = -sn[c] * h[c] + cs[c] * h[c + 1];
        h[c] = t;
      }
      const double d = std::hypot(h[j], h[j + 1]);
      cs[j] = d > 0.0 ? h[j] / d : 1.0;
      sn[j] = d > 0.0 ? h[j + 1] / d : 0.0;
      h[j] = d;
      h[j + 1] = 0.0;
      g[j + 1] = -sn[j] * g[j];
      g[j] = cs[j] * g[j];
      for (int c = 0; c <= j; ++c) H[(size_t)c * m + j] = h[c];
      ++iters;
      if (std::fabs(g[j + 1]) <= p.rel_res_tol * bnorm || hn == 0.0) {
        est_conv = true;
        ++j;
        break;
      }
    }
    for (int c = j - 1; c >= 0; --c) {
      double sum = g[c];
      for (int t = c + 1; t < j; ++t) sum -= H[(size_t)c * m + t] * y[t];
      y[c] = sum / H[(size_t)c * m + c];
    }
    for (int c = 0; c < j; ++c) hb[m + 2 + c] = y[c];
    SCK(s, cudaMemcpyAsync(s->d_y.p, hb + m + 2, j * sizeof(double), cudaMemcpyHostToDevice, st), "solution");
    update_x_kernel<<<sg, 256, j * sizeof(double), st>>>(Z, n, j, s->d_y.p, dx, n);
    // r = b - A x, beta = ||r||
    SCK(s, o.spmv(s, dA, dx, db, s->d_r.p, st), "residual");
    s->launches += 2;
    rc = mdot(s, s->d_r.p, 0, 1, s->d_r.p, s->d_h.p + m + 1, 2, st);
    if (rc) return rc;
    SCK(s, cudaMemcpyAsync(hb, s->d_h.p + m + 1, sizeof(double), cudaMemcpyDeviceToHost, st), "residual norm");
    SCK(s, cudaStreamSynchronize(st), "residual");
    beta = hb[0];
    r = s->d_r.p;
    if (est_conv && beta <= p.rel_res_tol * bnorm) converged = true;
  }
  if (!x_dev) {
    SCK(s, cudaMemcpyAsync(x, dx, n * sizeof(double), cudaMemcpyDeviceToHost, st), "copy x");
    SCK(s, cudaStreamSynchronize(st), "copy x");
  }
  if (prec) {  // a substitution wait that ran out (not expected on a working device)
    unsigned int stat = 0;
    SCK(s, cudaMemcpyAsync(&stat, s->d_status.p, sizeof(stat), cudaMemcpyDeviceToHost, st), "status");
    SCK(s, cudaStreamSynchronize(st), "status");
    if (stat & GALES_ERR_TIMEOUT) return sfail(s, GALES_ERR_TIMEOUT, "a substitution wait ran out");
  }
  if (res) {
    res->iterations = iters;
    res->abs_res = beta;
    res->rel_res = bnorm > 0.0 ? beta / bnorm : 0.0;
    res->converged = converged ? 1 : 0;
    res->cycles = cycles;
    res->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
  }
  return 0;
}

int gales_solver_correct(gales_solver* s, double* I, const double* dx, int32_t trim_first, int32_t trim_last,
                         double lo, double hi, void* stream) {
  if (!s || !I || !dx || !dev_ptr(I) || !dev_ptr(dx)) return GALES_ERR_BAD_INPUT;
  SCK(s, cudaSetDevice(s->device), "cudaSetDevice");
  cudaStream_t st = (cudaStream_t)stream;
  correct_kernel<<<stream_grid(s->n_rows, s->sms), 256, 0, st>>>(I, dx, s->n_rows, s->nd, trim_first, trim_last, lo,
                                                                  hi);
  ++s->launches;
  SCK(s, cudaGetLastError(), "correct");
  return 0;
}

int64_t gales_solver_launches(gales_solver* s) { return s ? s->launches : 0; }

const char* gales_solver_last_error(gales_solver* s) { return s ? s->err.c_str() : "null handle"; }

void gales_solver_destroy(gales_solver* s) {
  if (!s) return;
  cudaSetDevice(s->device);
  if (s->prec_graph) cudaGraphExecDestroy(s->prec_graph);
  if (s->cap) cudaStreamDestroy(s->cap);
  if (s->h_buf) cudaFreeHost(s->h_buf);
  for (auto* b : {&s->d_node_rp, &s->d_f_rp, &s->d_f_diag, &s->d_a2f}) b->release();
  for (auto* b : {&s->d_node_col, &s->d_f_col, &s->d_rows_f, &s->d_rows_b}) b->release();
  s->d_Ff.release();
  s->d_zf.release();
  for (auto* b : {&s->d_F, &s->d_V, &s->d_Z, &s->d_w, &s->d_r, &s->d_x, &s->d_part, &s->d_h, &s->d_h2, &s->d_y,
                  &s->d_vals, &s->d_b})
    b->release();
  s->d_j.release();
  s->d_status.release();
  delete s;
}

}  // extern "C"
