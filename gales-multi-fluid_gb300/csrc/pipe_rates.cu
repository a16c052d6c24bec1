// Arithmetic pipe rates of the device, for the compute side of the assembly's roofline:
// FP64 fused multiply-add, FP64 multiply, FP32 fused multiply-add (thread operations
// per SM per clock, independent chains, every SM busy), and whether FP64 and FP32
// work in different warps of one SM overlap: half the warps run the FP64 chain, half
// an FP32 chain sized to take as long alone; the time of both together over the
// longer one alone is 1 if they overlap and 2 if they share one pipe.
//
//   pipe_rates  ->  one JSON line on stdout
//
// Every store is to out[block * blockDim + thread] of a buffer sized for the grid.
#include <cuda_runtime.h>

#include <cstdio>

namespace {

constexpr int kChains = 8;

__global__ void dfma_chains(double* out, int iters, double a, double b) {
  double x[kChains];
#pragma unroll
  for (int i = 0; i < kChains; ++i) x[i] = threadIdx.x * 1e-3 + i;
  for (int it = 0; it < iters; ++it)
#pragma unroll
    for (int i = 0; i < kChains; ++i) x[i] = fma(x[i], a, b);
  double s = 0.0;
#pragma unroll
  for (int i = 0; i < kChains; ++i) s += x[i];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void dmul_chains(double* out, int iters, double a) {
  double x[kChains];
#pragma unroll
  for (int i = 0; i < kChains; ++i) x[i] = threadIdx.x * 1e-3 + i + 1.0;
  for (int it = 0; it < iters; ++it)
#pragma unroll
    for (int i = 0; i < kChains; ++i) x[i] = x[i] * a;
  double s = 0.0;
#pragma unroll
  for (int i = 0; i < kChains; ++i) s += x[i];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void ffma_chains(double* out, int iters, float a, float b) {
  float x[kChains];
#pragma unroll
  for (int i = 0; i < kChains; ++i) x[i] = threadIdx.x * 1e-3f + i;
  for (int it = 0; it < iters; ++it)
#pragma unroll
    for (int i = 0; i < kChains; ++i) x[i] = fmaf(x[i], a, b);
  float s = 0.f;
#pragma unroll
  for (int i = 0; i < kChains; ++i) s += x[i];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

// even warps: dfma chains for diters; odd warps: ffma chains for fiters (either may be 0)
__global__ void split_chains(double* out, int diters, int fiters, double a, double b) {
  const bool f64 = ((threadIdx.x >> 5) & 1) == 0;
  double r = 0.0;
  if (f64) {
    double x[kChains];
#pragma unroll
    for (int i = 0; i < kChains; ++i) x[i] = threadIdx.x * 1e-3 + i;
    for (int it = 0; it < diters; ++it)
#pragma unroll
      for (int i = 0; i < kChains; ++i) x[i] = fma(x[i], a, b);
#pragma unroll
    for (int i = 0; i < kChains; ++i) r += x[i];
  } else {
    float x[kChains];
#pragma unroll
    for (int i = 0; i < kChains; ++i) x[i] = threadIdx.x * 1e-3f + i;
    for (int it = 0; it < fiters; ++it)
#pragma unroll
      for (int i = 0; i < kChains; ++i) x[i] = fmaf(x[i], (float)a, (float)b);
    float s = 0.f;
#pragma unroll
    for (int i = 0; i < kChains; ++i) s += x[i];
    r = s;
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = r;
}

}  // namespace

int main() {
  int sms = 0, clk_khz = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0) != cudaSuccess ||
      cudaDeviceGetAttribute(&clk_khz, cudaDevAttrClockRate, 0) != cudaSuccess) {
    printf("{\"error\": \"no device\"}\n");
    return 1;
  }
  const int threads = 256, blocks = sms * 4;
  double* out = nullptr;
  if (cudaMalloc(&out, sizeof(double) * blocks * threads) != cudaSuccess) {
    printf("{\"error\": \"allocation\"}\n");
    return 1;
  }
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  auto ms_of = [&](auto launch) {
    launch();
    cudaDeviceSynchronize();
    cudaEventRecord(e0);
    launch();
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    return (double)ms;
  };
  const double cycles_per_ms = clk_khz * 1.0;  // kHz = cycles per ms
  const int it = 2048;
  const double per_launch = (double)kChains * it * blocks * threads;
  const double t_dfma = ms_of([&] { dfma_chains<<<blocks, threads>>>(out, it, 1.0000001, 1e-9); });
  const double t_dmul = ms_of([&] { dmul_chains<<<blocks, threads>>>(out, it, 1.0000001); });
  const double t_ffma = ms_of([&] { ffma_chains<<<blocks, threads>>>(out, it * 32, 1.0000001f, 1e-9f); });
  const double dfma = per_launch / (t_dfma * cycles_per_ms) / sms;
  const double dmul = per_launch / (t_dmul * cycles_per_ms) / sms;
  const double ffma = per_launch * 32 / (t_ffma * cycles_per_ms) / sms;
  // FP32 iterations that take as long as `it` FP64 iterations in half the warps
  const int fit = (int)(it * ffma / dfma);
  const double t_d = ms_of([&] { split_chains<<<blocks, threads>>>(out, it, 0, 1.0000001, 1e-9); });
  const double t_f = ms_of([&] { split_chains<<<blocks, threads>>>(out, 0, fit, 1.0000001, 1e-9); });
  const double t_both = ms_of([&] { split_chains<<<blocks, threads>>>(out, it, fit, 1.0000001, 1e-9); });
  const cudaError_t err = cudaDeviceSynchronize();
  cudaFree(out);
  if (err != cudaSuccess) {
    printf("{\"error\": \"%s\"}\n", cudaGetErrorString(err));
    return 1;
  }
  printf("{\"sm_count\": %d, \"clock_mhz\": %.0f, \"dfma_per_clk_sm\": %.4f, \"dmul_per_clk_sm\": %.4f, "
         "\"ffma_per_clk_sm\": %.3f, \"fp64_fp32_overlap\": {\"fp64_alone_ms\": %.4f, \"fp32_alone_ms\": %.4f, "
         "\"both_ms\": %.4f, \"both_over_longer\": %.3f}}\n",
         sms, clk_khz / 1000.0, dfma, dmul, ffma, t_d, t_f, t_both, t_both / (t_d > t_f ? t_d : t_f));
  return 0;
}
