// ptmc_fp32.cuh — device helpers of the FP32_RESYNC form, shared by its two
// cycle kernels (ptmc_cycles32.cu: 16 or 32 lanes per walker; ptmc_cycles32n.cu:
// 4 or 8 lanes per walker): FP32 pair terms, float-float position arithmetic,
// bit-assembled uniforms, segmented warp sums, the FP64 resync energy and the
// exchange acceptance.
#pragma once
#include <cuda_runtime.h>

#include "ptmc_device.cuh"
#include "ptmc_engine.cuh"

namespace ptmc {
namespace f32k {

// ELJ pair energy in FP32: sum_k c_k x^k times r^-6, x = 1/r (ELJPotential)
// or 1/r^2 (ELJPotentialEven), with the coefficients read as kernel-parameter
// (constant bank) operands and the Horner recurrence unrolled for the
// coefficient count KK: no shared-memory loads and no loop overhead per pair
// term (a runtime-K loop over shared-memory coefficients costs ~5
// instructions per term).
template <int KK>
__device__ __forceinline__ float horner_p(const KParams& P, float x) {
  float v = P.cf[KK - 1];
#pragma unroll
  for (int k = KK - 2; k >= 0; --k) v = fmaf(v, x, P.cf[k]);
  return v;
}
template <int POT>
__device__ __forceinline__ float v32p(const KParams& P, const float* c, int K, float r2) {
  float x, s;
  if (POT == POT_ELJ) {
    const float ir = rsqrtf(r2);
    const float inv = ir * ir;
    x = ir;
    s = inv * inv * inv;
  } else {
    const float inv = rcpf(r2);
    x = inv;
    s = inv * inv * inv;
  }
  float v;
  switch (K) {  // uniform across the grid
    case 4: v = horner_p<4>(P, x); break;
    case 5: v = horner_p<5>(P, x); break;
    case 6: v = horner_p<6>(P, x); break;
    case 7: v = horner_p<7>(P, x); break;
    case 8: v = horner_p<8>(P, x); break;
    case 10: v = horner_p<10>(P, x); break;
    default:
      v = c[K - 1];
      for (int k = K - 2; k >= 0; --k) v = fmaf(v, x, c[k]);
  }
  // rounded as written: a pair term is the same float in every kernel of
  // the form (no contraction into the caller's difference)
  return __fmul_rn(v, s);
}
__device__ __forceinline__ double v_even64(const double* c, int K, double r2) {
  double inv = 1.0 / r2;
  double v = c[K - 1];
  for (int k = K - 2; k >= 0; --k) v = fma(v, inv, c[k]);
  return v * (inv * inv * inv);
}
__device__ __forceinline__ double v_all64(const double* c, int K, double r2) {
  double ir = 1.0 / sqrt(r2);
  double inv = ir * ir;
  double v = c[K - 1];
  for (int k = K - 2; k >= 0; --k) v = fma(v, ir, c[k]);
  return v * (inv * inv * inv);
}
template <int POT>
__device__ __forceinline__ double v64(const double* c, int K, double r2) {
  return POT == POT_ELJ ? v_all64(c, K, r2) : v_even64(c, K, r2);
}
__device__ __forceinline__ double lrc64(int N, double rc2, const double* c, int K) {
  if (rc2 <= 50) return 0.0;
  double rcs = sqrt(rc2);
  double rc3 = rc2 * rcs;
  double e = 0.0;
  for (int i = 1; i <= K; ++i) {
    e += c[i - 1] / rc3 / (2 * i + 1);
    rc3 *= rc2;
  }
  e *= 3.141592653589793 * (double)(N * N) / 4 / (rcs * rcs * rcs);
  return e;
}

// lrc64 in FP32 (the correction is ~1e-2 of the energy, its FP32 rounding far
// below the FP32 pair sum's): pi N^2 / 4 rc^-6 sum_i c_i rc^(-2i) / (2i + 3),
// zero for r_c^2 <= 50 as in the FP64 form
__device__ __forceinline__ float lrc32(int N, double rc2, const float* c, int K) {
  if (rc2 <= 50) return 0.f;
  const float ir2 = 1.f / (float)rc2;
  float e = 0.f;
  for (int i = K - 1; i >= 0; --i) e = fmaf(e, ir2, c[i] / (float)(2 * i + 3));
  return e * (ir2 * ir2 * ir2) * (3.14159265f * (float)(N * N) * 0.25f);
}

// min(1, exp((beta_k - beta_k+1) (H_1 - H_2))), H = E + p L^3 (p = 0: NVT),
// every operation rounded as written: both cycle-end forms of k_cycles32
// evaluate it alike, whatever the compiler contracts elsewhere
__device__ __forceinline__ double exch_acc(double bk, double bk1, double e1, double e2, double L1,
                                           double L2, double p) {
  if (p != 0.0) {
    e1 = __dadd_rn(e1, __dmul_rn(p, __dmul_rn(__dmul_rn(L1, L1), L1)));
    e2 = __dadd_rn(e2, __dmul_rn(p, __dmul_rn(__dmul_rn(L2, L2), L2)));
  }
  const double a = exp(__dmul_rn(__dadd_rn(bk, -bk1), __dadd_rn(e1, -e2)));
  return a > 1.0 ? 1.0 : a;
}

template <int BC>
__device__ __forceinline__ float pf2(float4 a, float4 b, float L, float iL) {
  float dx = a.x - b.x, dy = a.y - b.y, dz = a.z - b.z;
  if (BC == BC_CUB) return f2_cub(dx, dy, dz, L, iL);
  return fmaf(dx, dx, fmaf(dy, dy, dz * dz));
}

// (hi, lo) += d for a step d much smaller than the coordinate: Dekker's
// fast two-sum (exact when |hi| >= |d|; for the rare coordinate inside one
// step of zero the sum is still correct to the float rounding of d), then
// renormalisation
__device__ __forceinline__ void ff_add(float& hi, float& lo, float d) {
  float s = hi + d;
  float err = d - (s - hi);
  float l = lo + err;
  hi = s + l;
  lo = l - (hi - s);
}
// (hi, lo) *= s: the exact product hi s (its rounding error by FMA) plus lo s,
// renormalised by a fast two-sum (|hi s| >= |lo s + err|)
__device__ __forceinline__ void ff_scale(float& hi, float& lo, float s) {
  const float p = hi * s;
  const float q = fmaf(lo, s, fmaf(hi, s, -p));
  hi = p + q;
  lo = q - (hi - p);
}
// uniform in [0, 1) from the top 23 bits of a Philox word
__device__ __forceinline__ float u01f(uint32_t w) {
  return __uint_as_float(0x3F800000u | (w >> 9)) - 1.0f;
}
// a step of the symmetric uniform (-md/2, md/2): md ((k + 1/2) 2^-23 - 1/2)
// for the 23-bit k of the word, one FMA with mdc = md (3/2 - 2^-24) per slot
__device__ __forceinline__ float stepf(uint32_t w, float md, float mdc) {
  return fmaf(__uint_as_float(0x3F800000u | (w >> 9)), md, -mdc);
}

// sum over the LPR lanes of one walker (xor partners stay inside the group)
template <int LPR, typename T>
__device__ __forceinline__ T seg_sum(T v, unsigned mask) {
#pragma unroll
  for (int o = LPR / 2; o > 0; o >>= 1) v += __shfl_xor_sync(mask, v, o);
  return v;
}

// FP64 energy of one walker from its float-float positions (resync); the
// walker's LPR lanes share the work (lane = lane within the walker's group).
// EAM: the recomputed densities are staged in rho_tmp[a * rho_stride] and go
// into the w lanes of Xh once every lane has read the positions; sqrt(rho)
// into sq32.
template <int POT, int BC, int ENS, int LPR>
__device__ double energy64(float4* Xh, const float4* Xl, int N, double L, double rc2,
                           const double* c, int K, double hn, double hm, double ean,
                           double ecam, float* rho_tmp, float* sq32, int lane, unsigned gmask,
                           int rho_stride = 1) {
  auto P = [&](int a, double& x, double& y, double& z) {
    float4 h = Xh[a], l = Xl[a];
    x = (double)h.x + (double)l.x;
    y = (double)h.y + (double)l.y;
    z = (double)h.z + (double)l.z;
  };
  double e = 0.0;
  if constexpr (POT == POT_EAM) {
    for (int a = lane; a < N; a += LPR) {
      double xa, ya, za, A = 0.0, B = 0.0;
      P(a, xa, ya, za);
      for (int j = 0; j < N; ++j) {
        if (j == a) continue;
        double xj, yj, zj;
        P(j, xj, yj, zj);
        double r2 = BC == BC_CUB ? d2_cub(xa, ya, za, xj, yj, zj, L) : d2_sph(xa, ya, za, xj, yj, zj);
        double lg = log(r2);
        A += exp(hn * lg);
        B += exp(hm * lg);
      }
      if (rho_tmp) rho_tmp[a * rho_stride] = (float)B;
      if (sq32) sq32[a] = (float)sqrt(B);
      e += ean * A - ecam * sqrt(B);
    }
    // the electron density goes into the w lane of the position after every
    // lane has read the positions
    __syncwarp(gmask);
    if (rho_tmp)
      for (int a = lane; a < N; a += LPR) Xh[a].w = rho_tmp[a * rho_stride];
    __syncwarp(gmask);
    return seg_sum<LPR>(e, gmask);
  } else {
    for (int i = 0; i < N; ++i) {
      double xi, yi, zi;
      P(i, xi, yi, zi);
      for (int j = i + 1 + lane; j < N; j += LPR) {
        double xj, yj, zj;
        P(j, xj, yj, zj);
        double r2 = BC == BC_CUB ? d2_cub(xi, yi, zi, xj, yj, zj, L) : d2_sph(xi, yi, zi, xj, yj, zj);
        if (ENS == ENS_NPT && !(r2 <= rc2)) continue;
        e += v64<POT>(c, K, r2);
      }
    }
    e = seg_sum<LPR>(e, gmask);
    if (ENS == ENS_NPT) e += lrc64(N, rc2, c, K);
    return e;
  }
}

}  // namespace f32k
}  // namespace ptmc
