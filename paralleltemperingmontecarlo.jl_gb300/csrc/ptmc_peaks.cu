// ptmc_peaks.cu — in-situ arithmetic peaks of the current GPU, used as the
// roofline denominators of the replica-cycle kernels (which are bound by the
// FP32/FP64 FMA pipes and the MUFU unit, not by HBM or tensor cores).
//
// Each probe runs independent dependency chains (8 per thread) over a grid of
// 8 CTAs per SM so every pipe is saturated; the result is the best of 3 timed
// launches.  FFMA/DFMA count 2 flops, MUFU ex2 counts 1 op.
#include <cuda_runtime.h>

#include "../../include/ptmc_gb300.h"

namespace {
constexpr int ITERS = 4096;

__global__ void k_ffma(float* out, float a, float b) {
  float x[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) x[k] = threadIdx.x * 1e-3f + k;
  for (int i = 0; i < ITERS; ++i)
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = fmaf(x[k], a, b);
  float s = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += x[k];
  if (s == 12345.678f) out[0] = s;
}
__global__ void k_dfma(double* out, double a, double b) {
  double x[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) x[k] = threadIdx.x * 1e-3 + k;
  for (int i = 0; i < ITERS / 16; ++i)
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = fma(x[k], a, b);
  double s = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += x[k];
  if (s == 12345.678) out[0] = s;
}
__global__ void k_mufu(float* out, float a) {
  float x[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) x[k] = threadIdx.x * 1e-6f + k * 1e-3f;
  for (int i = 0; i < ITERS / 4; ++i)
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      float y;
      asm volatile("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x[k]));
      x[k] = y * a;
    }
  float s = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += x[k];
  if (s == 12345.678f) out[0] = s;
}

template <typename F>
float best_ms(F launch) {
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  launch();  // warm-up
  float best = 1e30f;
  for (int r = 0; r < 3; ++r) {
    cudaEventRecord(e0);
    launch();
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) best = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return best;
}
}  // namespace

extern "C" int ptmc_measure_peaks(int device, double* fp32_tflops, double* fp64_tflops,
                                  double* mufu_tops) {
  if (cudaSetDevice(device) != cudaSuccess) return PTMC_ERR_CUDA;
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return PTMC_ERR_CUDA;
  int grid = prop.multiProcessorCount * 8, block = 256;
  float* df = nullptr;
  double* dd = nullptr;
  if (cudaMalloc(&df, 16) != cudaSuccess || cudaMalloc(&dd, 16) != cudaSuccess) return PTMC_ERR_CUDA;
  double threads = (double)grid * block;
  float ms = best_ms([&] { k_ffma<<<grid, block>>>(df, 1.0000001f, 1e-7f); });
  if (fp32_tflops) *fp32_tflops = threads * ITERS * 8 * 2 / (ms * 1e-3) / 1e12;
  ms = best_ms([&] { k_dfma<<<grid, block>>>(dd, 1.0000000001, 1e-10); });
  if (fp64_tflops) *fp64_tflops = threads * (ITERS / 16) * 8 * 2 / (ms * 1e-3) / 1e12;
  ms = best_ms([&] { k_mufu<<<grid, block>>>(df, 0.999f); });
  if (mufu_tops) *mufu_tops = threads * (ITERS / 4) * 8 / (ms * 1e-3) / 1e12;
  cudaError_t e = cudaGetLastError();
  cudaFree(df);
  cudaFree(dd);
  return e == cudaSuccess ? PTMC_OK : PTMC_ERR_CUDA;
}
