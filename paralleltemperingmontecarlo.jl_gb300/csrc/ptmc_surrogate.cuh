// ptmc_surrogate.cuh — the learned pair surrogate of delayed-acceptance
// moves (no counterpart in the reference): device parameters, shared-memory
// tiles and the 128-row tensor-core forward pass shared by the NN cycle
// kernel (ptmc_nn.cu) and the training kernels (ptmc_surrogate.cu).
//
// Model (16 Gaussian radial features -> 32 -> 32 -> 1, tanh hidden units):
//   g_k(r) = fc(r) exp(-gamma (r - mu_k)^2),  mu_k = r_lo + k (r_hi - r_lo)/15,
//   fc(r)  = (cos(pi r / r_cut) + 1)/2 for r < r_cut, else 0,
//   h1 = tanh(W1^T g + b1),  h2 = tanh(W2^T h1 + b2),  phi = escale (w3 . h2 + b3).
// E_s(x) = sum over pairs phi(r_ij).  A move of atom i from x_i to t is one
// 128-row tile: rows 0..63 are the new distances |t - x_j|, rows 64..127 the
// old distances |x_i - x_j| (j < N, j != i; other rows carry no pair), so
//   dE_s = sum_{rows < 64} phi - sum_{rows >= 64} phi
// is an exact difference of the state function E_s, which keeps the
// delayed-acceptance chain exact (Christen & Fox 2005).
//
// The two matrix products per tile (128x16 * 16x32 and 128x32 * 32x32) run on
// the tensor cores: BF16 operands in shared memory (canonical no-swizzle
// K-major layout, ptmc_umma.cuh), FP32 accumulators in 32 columns of tensor
// memory, read back by warps 0-3 (one row per thread).
#pragma once
#include <cuda_bf16.h>

#include "ptmc_umma.cuh"

namespace ptmc {

constexpr int SUR_F = 16, SUR_H = 32, SUR_ROWS = 128;
// parameter vector layout: W1[16][32] (input-major), b1[32], W2[32][32], b2[32], w3[32], b3
constexpr int SUR_B1 = SUR_F * SUR_H;
constexpr int SUR_W2 = SUR_B1 + SUR_H;
constexpr int SUR_B2 = SUR_W2 + SUR_H * SUR_H;
constexpr int SUR_W3 = SUR_B2 + SUR_H;
constexpr int SUR_B3 = SUR_W3 + SUR_H;
constexpr int SUR_NP = SUR_B3 + 1;  // 1633
constexpr int SUR_TMEM_COLS = 32;

// core-matrix strides (bytes) of the staged operands: K direction / row direction
constexpr uint32_t SUR_LBO = 128;
constexpr uint32_t SUR_SBO_K16 = 256;  // operands with K = 16 (A1, B1)
constexpr uint32_t SUR_SBO_K32 = 512;  // operands with K = 32 (A2, B2)

struct SurCfgDev {
  float r_lo, dmu, gamma, r_cut, escale;
};

// shared-memory tiles of one CTA (byte sizes; every tile 128-byte aligned)
struct SurSmem {
  unsigned char* A1;  // 128 x 16 BF16 features          4096 B
  unsigned char* A2;  // 128 x 32 BF16 first hidden layer 8192 B
  unsigned char* B1;  // W1^T: 32 x 16 BF16               1024 B
  unsigned char* B2;  // W2^T: 32 x 32 BF16               2048 B
  float* vec;         // b1[32], b2[32], w3[32], b3, partial sums [4]
  unsigned long long* mbar;
  uint32_t* tslot;
  int* err;
};

constexpr size_t SUR_SMEM_BYTES = 4096 + 8192 + 1024 + 2048 + 128 * 4 + 16 + 16 + 16;

__device__ __forceinline__ size_t sur_carve(SurSmem& s, unsigned char* base) {
  s.A1 = base;
  s.A2 = base + 4096;
  s.B1 = base + 12288;
  s.B2 = base + 13312;
  s.vec = (float*)(base + 15360);
  s.mbar = (unsigned long long*)(base + 15360 + 512);
  s.tslot = (uint32_t*)(base + 15360 + 528);
  s.err = (int*)(base + 15360 + 544);
  return SUR_SMEM_BYTES;
}

// W1/W2 -> BF16 operand tiles (B[n][k] = W[k][n], K-major), biases and w3 ->
// FP32; mbarrier initialised; called by every thread of the CTA, followed by
// a __syncthreads() of the caller
__device__ __forceinline__ void sur_stage(const SurSmem& s, const float* __restrict__ P) {
  for (int e = threadIdx.x; e < SUR_F * SUR_H; e += blockDim.x) {
    int k = e / SUR_H, n = e % SUR_H;
    *(__nv_bfloat16*)(s.B1 + umma_off(n, k, SUR_LBO, SUR_SBO_K16)) = __float2bfloat16_rn(P[e]);
  }
  for (int e = threadIdx.x; e < SUR_H * SUR_H; e += blockDim.x) {
    int k = e / SUR_H, n = e % SUR_H;
    *(__nv_bfloat16*)(s.B2 + umma_off(n, k, SUR_LBO, SUR_SBO_K32)) =
        __float2bfloat16_rn(P[SUR_W2 + e]);
  }
  for (int e = threadIdx.x; e < 3 * SUR_H + 1; e += blockDim.x) {
    int src = e < SUR_H ? SUR_B1 + e : e < 2 * SUR_H ? SUR_B2 + (e - SUR_H) : SUR_W3 + (e - 2 * SUR_H);
    s.vec[e] = P[src];  // the last one (e = 96) is b3 = P[SUR_W3 + 32]
  }
  if (threadIdx.x == 0) {
    mbar_init(smem_u32(s.mbar), 1);
    *s.err = 0;
  }
  fence_async_smem();
}

__device__ __forceinline__ float tanh_fast(float x) {
  float y;
  asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
template <bool FAST>
__device__ __forceinline__ float sur_tanh(float x) {
  return FAST ? tanh_fast(x) : tanhf(x);
}

// 16 features of one distance (r < 0: no pair -> zeros).  FAST uses the MUFU
// approximations (first stage of a move); training and evaluation use the
// accurate functions the oracle restates.
template <bool FAST>
__device__ __forceinline__ void sur_features(const SurCfgDev& c, float r, float (&g)[SUR_F]) {
  float fc = 0.f;
  if (r >= 0.f && r < c.r_cut)
    fc = 0.5f * ((FAST ? __cosf(3.14159265358979f * (r / c.r_cut))
                       : cosf(3.14159265358979f * (r / c.r_cut))) + 1.f);
#pragma unroll
  for (int k = 0; k < SUR_F; ++k) {
    float d = r - (c.r_lo + (float)k * c.dmu);
    g[k] = fc * (FAST ? __expf(-c.gamma * (d * d)) : expf(-c.gamma * (d * d)));
  }
}

// Forward pass of one 128-row tile, called by every thread of the CTA
// (blockDim >= 128).  FAST: MUFU tanh/exp/cos (the first stage of a move: any
// deterministic pair function keeps dE_s an exact difference of a state
// function, so the chain stays exact); otherwise the accurate functions.  Threads 0..127 pass their row's distance in `r` and get
// phi back (garbage for rows with r < 0, which the caller masks); with
// `keep` they also get h1 (FP32, before BF16 rounding) and h2.  `phase` is the
// mbarrier parity, flipped twice per call.  Returns false (every thread) if a
// tensor-core completion wait ran out; the caller must then stop issuing.
template <bool FAST = false>
__device__ __forceinline__ bool sur_tile_forward(const SurSmem& s, const SurCfgDev& c,
                                                 uint32_t tbase, uint32_t& phase, float r,
                                                 float& phi, float* h1keep, float* h2keep) {
  const int tid = threadIdx.x;
  const uint32_t idesc = umma_idesc_bf16(128, 32);
  const uint32_t mb = smem_u32(s.mbar);
  const uint32_t lane_addr = tbase + ((uint32_t)(32 * (tid >> 5)) << 16);
  if (tid < SUR_ROWS) {
    float g[SUR_F];
    sur_features<FAST>(c, r, g);
#pragma unroll
    for (int k = 0; k < SUR_F; k += 2) {
      __nv_bfloat162 v = __floats2bfloat162_rn(g[k], g[k + 1]);
      *(__nv_bfloat162*)(s.A1 + umma_off(tid, k, SUR_LBO, SUR_SBO_K16)) = v;
    }
  }
  fence_async_smem();
  tc_fence_before();
  __syncthreads();
  if (tid == 0) {
    tc_fence_after();
    umma_bf16(tbase, umma_sdesc(smem_u32(s.A1), SUR_LBO, SUR_SBO_K16),
              umma_sdesc(smem_u32(s.B1), SUR_LBO, SUR_SBO_K16), idesc, 0);
    umma_commit(mb);
  }
  int bad = 0;
  float acc[32];
  if (tid < SUR_ROWS) {
    if (!mbar_wait(mb, phase)) bad = 1;
    tc_fence_after();
    tmem_ld32(lane_addr, acc);
#pragma unroll
    for (int n = 0; n < SUR_H; n += 2) {
      float a = sur_tanh<FAST>(acc[n] + s.vec[n]), b = sur_tanh<FAST>(acc[n + 1] + s.vec[n + 1]);
      if (h1keep) {
        h1keep[n] = a;
        h1keep[n + 1] = b;
      }
      *(__nv_bfloat162*)(s.A2 + umma_off(tid, n, SUR_LBO, SUR_SBO_K32)) =
          __floats2bfloat162_rn(a, b);
    }
  }
  phase ^= 1u;
  fence_async_smem();
  tc_fence_before();
  if (__syncthreads_or(bad)) return false;
  if (tid == 0) {
    tc_fence_after();
    const uint32_t a2 = smem_u32(s.A2), b2 = smem_u32(s.B2);
    umma_bf16(tbase, umma_sdesc(a2, SUR_LBO, SUR_SBO_K32), umma_sdesc(b2, SUR_LBO, SUR_SBO_K32),
              idesc, 0);
    umma_bf16(tbase, umma_sdesc(a2 + 2 * SUR_LBO, SUR_LBO, SUR_SBO_K32),
              umma_sdesc(b2 + 2 * SUR_LBO, SUR_LBO, SUR_SBO_K32), idesc, 1);
    umma_commit(mb);
  }
  if (tid < SUR_ROWS) {
    if (!mbar_wait(mb, phase)) bad = 1;
    tc_fence_after();
    tmem_ld32(lane_addr, acc);
    float e = 0.f;
#pragma unroll
    for (int n = 0; n < SUR_H; ++n) {
      float h = sur_tanh<FAST>(acc[n] + s.vec[SUR_H + n]);
      if (h2keep) h2keep[n] = h;
      e += s.vec[2 * SUR_H + n] * h;
    }
    phi = c.escale * (e + s.vec[3 * SUR_H]);
  }
  phase ^= 1u;
  tc_fence_before();
  return !__syncthreads_or(bad);
}

// The frozen surrogate of a screening chain as a table: phi at the n grid
// distances r_k = k r_cut / (n - 1) from the accurate tile forward (the
// function training, evaluation and calibration use); beyond r_cut every
// feature is zero and phi is the constant phi(r_cut).  The first stage of a
// move interpolates linearly between grid points: a fixed pair function of
// the distance, so dE_s stays an exact difference of a state function.
constexpr int SUR_TAB_N = 4097;
__device__ __forceinline__ float sur_tab_phi(const float* __restrict__ tab, float inv_h, float r) {
  const float x = fminf(r * inv_h, (float)(SUR_TAB_N - 1));
  const int k = min((int)x, SUR_TAB_N - 2);
  const float a = __ldg(tab + k), b = __ldg(tab + k + 1);
  return fmaf(x - (float)k, b - a, a);
}

// launchers (ptmc_surrogate.cu); every pointer is device memory
int sur_launch_table(const SurCfgDev& c, const float* P, float* tab, int* err_flag, void* stream);
size_t sur_grad_smem_bytes();
int sur_launch_eval(const SurCfgDev& c, const float* P, const float* rows, int n, double* out,
                    int* err_flag, int grid, void* stream);
int sur_launch_grad(const SurCfgDev& c, const float* P, const float* rows, const float* y,
                    int n_rec, const int* idx, int batch, unsigned long long seed, int step,
                    float* grad, double* loss, int* err_flag, int grid, void* stream);
int sur_launch_adam(float* P, float* grad, float* m, float* v, int t, float lr, void* stream);

}  // namespace ptmc
