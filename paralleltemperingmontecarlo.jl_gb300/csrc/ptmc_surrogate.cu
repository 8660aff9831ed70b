// ptmc_surrogate.cu — evaluation and training of the delayed-acceptance pair
// surrogate on the GPU (no counterpart in the reference; the model and the
// tile forward pass are in ptmc_surrogate.cuh).
//
// Kernels (one record = one move = one 128-row tile, one CTA of 128 threads):
//   k_sur_eval   dE_s of n records (tensor-core forward, block sum),
//   k_sur_grad   Huber loss of (dE_s - dE)/escale over a minibatch of
//                records drawn with Philox, and its gradient: tensor-core
//                forward; backward on the CUDA cores in FP32 (dh1 = W2 dz2 per
//                row, then the weight gradients as column sums over the 128
//                rows, each thread owning ~13 parameters in registers across
//                the records it processes, one atomicAdd per parameter per CTA),
//   k_sur_adam   Adam step on the FP32 master parameters; clears the gradient.
// The BF16 rounding of the forward operands is treated as the identity in the
// backward pass (the gradient of the function the tensor cores computed, with
// the rounded operands).
#include <cuda_runtime.h>

#include "ptmc_device.cuh"
#include "ptmc_surrogate.cuh"

namespace ptmc {

namespace {

constexpr int SUR_THREADS = 128;
constexpr int DZ_LD = 33;  // padded row length of the per-row backward vectors

struct GradSmem {
  float* dz1;   // [128][33]
  float* dz2;   // [128][33]
  float* h2d;   // [128][33]  dphi * h2
  float* dphi;  // [128]
  float* red;   // [8]
};

__device__ __forceinline__ float block_sum128(float v, float* red) {
  v = warp_sum(v);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  float t = red[0] + red[1] + red[2] + red[3];
  __syncthreads();
  return t;
}

__device__ void sur_prologue(SurSmem& s, unsigned char* smem, const float* P, uint32_t& tbase) {
  sur_carve(s, smem);
  sur_stage(s, P);
  if (threadIdx.x < 32) tmem_alloc(smem_u32(s.tslot), SUR_TMEM_COLS);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  tbase = *s.tslot;
}

__device__ void sur_epilogue(const SurSmem& s, uint32_t tbase, int* err_flag) {
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (threadIdx.x < 32) tmem_dealloc(tbase, SUR_TMEM_COLS);
  if (threadIdx.x == 0 && *s.err) atomicOr(err_flag, 1);
}

}  // namespace

__global__ void __launch_bounds__(SUR_THREADS) k_sur_eval(SurCfgDev c, const float* __restrict__ P,
                                                          const float* __restrict__ rows, int n,
                                                          double* __restrict__ out, int* err_flag) {
  extern __shared__ __align__(128) unsigned char smem[];
  SurSmem s;
  uint32_t tbase;
  sur_prologue(s, smem, P, tbase);
  float* red = s.vec + 100;
  uint32_t phase = 0;
  for (int b = blockIdx.x; b < n; b += gridDim.x) {
    const float r = rows[(size_t)b * SUR_ROWS + threadIdx.x];
    float phi = 0.f;
    if (!sur_tile_forward(s, c, tbase, phase, r, phi, nullptr, nullptr)) {
      if (threadIdx.x == 0) *s.err = 1;
      break;
    }
    float v = r >= 0.f ? (threadIdx.x < SUR_ROWS / 2 ? phi : -phi) : 0.f;
    float e = block_sum128(v, red);
    if (threadIdx.x == 0) out[b] = (double)e;
  }
  sur_epilogue(s, tbase, err_flag);
}

// phi at the SUR_TAB_N grid distances, 128 per tile (accurate forward)
__global__ void __launch_bounds__(SUR_THREADS) k_sur_table(SurCfgDev c, const float* __restrict__ P,
                                                           float* __restrict__ tab, int* err_flag) {
  extern __shared__ __align__(128) unsigned char smem[];
  SurSmem s;
  uint32_t tbase;
  sur_prologue(s, smem, P, tbase);
  uint32_t phase = 0;
  const float h = c.r_cut / (float)(SUR_TAB_N - 1);
  for (int b = blockIdx.x; b * SUR_ROWS < SUR_TAB_N; b += gridDim.x) {
    const int k = b * SUR_ROWS + (int)threadIdx.x;
    const float r = k < SUR_TAB_N ? (float)k * h : -1.f;
    float phi = 0.f;
    if (!sur_tile_forward(s, c, tbase, phase, r, phi, nullptr, nullptr)) {
      if (threadIdx.x == 0) *s.err = 1;
      break;
    }
    if (k < SUR_TAB_N) tab[k] = phi;
  }
  sur_epilogue(s, tbase, err_flag);
}

// one parameter's column sum over the 128 rows of the current tile
__device__ __forceinline__ float sur_param_grad(int p, const SurSmem& s, const GradSmem& g) {
  float acc = 0.f;
  if (p < SUR_B1) {  // W1[f][n]: g_f * dz1_n
    const int f = p / SUR_H, n = p % SUR_H;
    for (int q = 0; q < SUR_ROWS; ++q)
      acc += __bfloat162float(*(const __nv_bfloat16*)(s.A1 + umma_off(q, f, SUR_LBO, SUR_SBO_K16))) *
             g.dz1[q * DZ_LD + n];
  } else if (p < SUR_W2) {  // b1[n]
    const int n = p - SUR_B1;
    for (int q = 0; q < SUR_ROWS; ++q) acc += g.dz1[q * DZ_LD + n];
  } else if (p < SUR_B2) {  // W2[k][m]: bf16(h1_k) * dz2_m
    const int k = (p - SUR_W2) / SUR_H, m = (p - SUR_W2) % SUR_H;
    for (int q = 0; q < SUR_ROWS; ++q)
      acc += __bfloat162float(*(const __nv_bfloat16*)(s.A2 + umma_off(q, k, SUR_LBO, SUR_SBO_K32))) *
             g.dz2[q * DZ_LD + m];
  } else if (p < SUR_W3) {  // b2[m]
    const int m = p - SUR_B2;
    for (int q = 0; q < SUR_ROWS; ++q) acc += g.dz2[q * DZ_LD + m];
  } else if (p < SUR_B3) {  // w3[m]: dphi * h2_m
    const int m = p - SUR_W3;
    for (int q = 0; q < SUR_ROWS; ++q) acc += g.h2d[q * DZ_LD + m];
  } else {  // b3
    for (int q = 0; q < SUR_ROWS; ++q) acc += g.dphi[q];
  }
  return acc;
}

constexpr int SUR_PER_THREAD = (SUR_NP + SUR_THREADS - 1) / SUR_THREADS;  // 13

// Minibatch loss and gradient.  Record b of the minibatch is record
// idx[b] when idx != NULL, else floor(u * n_rec) with u the Philox draw
// (seed, step, b).  grad (SUR_NP floats) and loss (one double) accumulate.
__global__ void __launch_bounds__(SUR_THREADS) k_sur_grad(SurCfgDev c, const float* __restrict__ P,
                                                          const float* __restrict__ rows,
                                                          const float* __restrict__ y, int n_rec,
                                                          const int* __restrict__ idx, int batch,
                                                          unsigned long long seed, int step,
                                                          float* __restrict__ grad,
                                                          double* __restrict__ loss, int* err_flag) {
  extern __shared__ __align__(128) unsigned char smem[];
  SurSmem s;
  uint32_t tbase;
  sur_prologue(s, smem, P, tbase);
  GradSmem g;
  float* base = (float*)(smem + SUR_SMEM_BYTES);
  g.dz1 = base;
  g.dz2 = g.dz1 + SUR_ROWS * DZ_LD;
  g.h2d = g.dz2 + SUR_ROWS * DZ_LD;
  g.dphi = g.h2d + SUR_ROWS * DZ_LD;
  g.red = g.dphi + SUR_ROWS;
  const int tid = threadIdx.x;
  const float w3s = c.escale;
  float own[SUR_PER_THREAD];
#pragma unroll
  for (int j = 0; j < SUR_PER_THREAD; ++j) own[j] = 0.f;
  double lsum = 0.0;
  uint32_t phase = 0;
  const float inv_b = 1.0f / (float)batch;
  for (int b = blockIdx.x; b < batch; b += gridDim.x) {
    int rec;
    if (idx) {
      rec = idx[b];
    } else {
      double u = philox_u01(seed, 0xFFFFFFF0u, (uint32_t)step, (unsigned long long)b);
      rec = (int)(u * n_rec);
      if (rec >= n_rec) rec = n_rec - 1;
    }
    const float r = rows[(size_t)rec * SUR_ROWS + tid];
    float phi = 0.f, h1[SUR_H], h2[SUR_H];
    if (!sur_tile_forward(s, c, tbase, phase, r, phi, h1, h2)) {
      if (tid == 0) *s.err = 1;
      break;
    }
    const float sgn = r >= 0.f ? (tid < SUR_ROWS / 2 ? 1.f : -1.f) : 0.f;
    const float e = block_sum128(sgn * phi, g.red);
    const float res = (e - y[rec]) / c.escale;
    const float a = fabsf(res);
    if (tid == 0) lsum += a <= 1.f ? 0.5 * (double)res * res : (double)a - 0.5;
    const float G = fminf(fmaxf(res, -1.f), 1.f) * inv_b / c.escale;  // dL / d dE_s
    // per-row backward (thread = row)
    const float dphi = sgn * G * w3s;
    float dz2[SUR_H];
#pragma unroll
    for (int m = 0; m < SUR_H; ++m) {
      dz2[m] = dphi * s.vec[2 * SUR_H + m] * (1.f - h2[m] * h2[m]);
      g.dz2[tid * DZ_LD + m] = dz2[m];
      g.h2d[tid * DZ_LD + m] = dphi * h2[m];
    }
    g.dphi[tid] = dphi;
#pragma unroll 4
    for (int k = 0; k < SUR_H; ++k) {  // dh1_k = sum_m bf16(W2[k][m]) dz2_m
      float dh = 0.f;
#pragma unroll
      for (int m = 0; m < SUR_H; ++m)
        dh += __bfloat162float(*(const __nv_bfloat16*)(s.B2 + umma_off(m, k, SUR_LBO, SUR_SBO_K32))) *
              dz2[m];
      g.dz1[tid * DZ_LD + k] = dh * (1.f - h1[k] * h1[k]);
    }
    __syncthreads();
    // column sums: thread owns parameters tid, tid + 128, ...
#pragma unroll
    for (int j = 0; j < SUR_PER_THREAD; ++j) {
      const int p = tid + SUR_THREADS * j;
      if (p < SUR_NP) own[j] += sur_param_grad(p, s, g);
    }
    __syncthreads();
  }
#pragma unroll
  for (int j = 0; j < SUR_PER_THREAD; ++j) {
    const int p = tid + SUR_THREADS * j;
    if (p < SUR_NP && own[j] != 0.f) atomicAdd(grad + p, own[j]);
  }
  if (tid == 0 && lsum != 0.0) atomicAdd(loss, lsum / batch);
  sur_epilogue(s, tbase, err_flag);
}

// Adam (Kingma & Ba 2015) on the FP32 master parameters; the gradient is
// cleared for the next minibatch.  One thread per parameter.
__global__ void k_sur_adam(float* __restrict__ P, float* __restrict__ grad, float* __restrict__ m,
                           float* __restrict__ v, int t, float lr, float b1, float b2, float eps) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= SUR_NP) return;
  const float gr = grad[p];
  grad[p] = 0.f;
  const float mm = b1 * m[p] + (1.f - b1) * gr;
  const float vv = b2 * v[p] + (1.f - b2) * gr * gr;
  m[p] = mm;
  v[p] = vv;
  const float mh = mm / (1.f - powf(b1, (float)t));
  const float vh = vv / (1.f - powf(b2, (float)t));
  P[p] -= lr * mh / (sqrtf(vh) + eps);
}

// ---------------------------------------------------------------- launchers
static int sur_smem_opt_in(const void* kern, size_t bytes) {
  if (bytes <= 48 * 1024) return 0;
  return (int)cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

size_t sur_grad_smem_bytes() {
  return SUR_SMEM_BYTES + sizeof(float) * (3 * SUR_ROWS * DZ_LD + SUR_ROWS + 8);
}

int sur_launch_eval(const SurCfgDev& c, const float* P, const float* rows, int n, double* out,
                    int* err_flag, int grid, void* stream) {
  if (n <= 0) return 0;
  if (grid <= 0 || grid > n) grid = n;
  k_sur_eval<<<grid, SUR_THREADS, SUR_SMEM_BYTES, (cudaStream_t)stream>>>(c, P, rows, n, out,
                                                                         err_flag);
  return (int)cudaGetLastError();
}

int sur_launch_table(const SurCfgDev& c, const float* P, float* tab, int* err_flag, void* stream) {
  const int grid = (SUR_TAB_N + SUR_ROWS - 1) / SUR_ROWS;
  k_sur_table<<<grid, SUR_THREADS, SUR_SMEM_BYTES, (cudaStream_t)stream>>>(c, P, tab, err_flag);
  return (int)cudaGetLastError();
}

int sur_launch_grad(const SurCfgDev& c, const float* P, const float* rows, const float* y,
                    int n_rec, const int* idx, int batch, unsigned long long seed, int step,
                    float* grad, double* loss, int* err_flag, int grid, void* stream) {
  if (batch <= 0) return 0;
  size_t sm = sur_grad_smem_bytes();
  int e = sur_smem_opt_in((const void*)k_sur_grad, sm);
  if (e) return e;
  if (grid <= 0 || grid > batch) grid = batch;
  k_sur_grad<<<grid, SUR_THREADS, sm, (cudaStream_t)stream>>>(c, P, rows, y, n_rec, idx, batch, seed,
                                                              step, grad, loss, err_flag);
  return (int)cudaGetLastError();
}

int sur_launch_adam(float* P, float* grad, float* m, float* v, int t, float lr, void* stream) {
  k_sur_adam<<<(SUR_NP + 255) / 256, 256, 0, (cudaStream_t)stream>>>(P, grad, m, v, t, lr, 0.9f,
                                                                     0.999f, 1e-8f);
  return (int)cudaGetLastError();
}

}  // namespace ptmc
