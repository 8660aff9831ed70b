// ptmc_device.cuh — device helpers shared by the engine kernels.
//
// Draw streams: Philox4x32-10 (Salmon et al., SC'11).  Draw k of a stream is
// half (k & 1) of Philox block k >> 1 with counter {block lo, block hi, stream,
// run} and key = seed; half 0 takes 53 bits from words (0,1), half 1 from
// words (2,3).  Walker streams use stream = walker index in the run; the
// run-level stream (exchange draws) uses stream = 0xFFFFFFFF.
#pragma once
#include <cstdint>

namespace ptmc {

__device__ __forceinline__ void philox4x32_10(uint32_t c[4], uint32_t k0,
                                              uint32_t k1) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
  const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    if (r > 0) {
      k0 += W0;
      k1 += W1;
    }
    uint32_t lo0 = M0 * c[0], hi0 = __umulhi(M0, c[0]);
    uint32_t lo1 = M1 * c[2], hi1 = __umulhi(M1, c[2]);
    uint32_t n0 = hi1 ^ c[1] ^ k0;
    uint32_t n2 = hi0 ^ c[3] ^ k1;
    c[0] = n0;
    c[1] = lo1;
    c[2] = n2;
    c[3] = lo0;
  }
}

// both halves of block `blk`
__device__ __forceinline__ void philox_pair(uint64_t seed, uint32_t stream,
                                            uint32_t run, uint64_t blk,
                                            double& u0, double& u1) {
  uint32_t c[4] = {(uint32_t)blk, (uint32_t)(blk >> 32), stream, run};
  philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
  uint64_t b0 = ((uint64_t)c[0] << 21) | (uint64_t)(c[1] >> 11);
  uint64_t b1 = ((uint64_t)c[2] << 21) | (uint64_t)(c[3] >> 11);
  u0 = (double)b0 * 0x1.0p-53;
  u1 = (double)b1 * 0x1.0p-53;
}

// single draw k of a stream (thread-local use: the run-level stream)
__device__ __forceinline__ double philox_u01(uint64_t seed, uint32_t stream,
                                             uint32_t run, uint64_t k) {
  double u0, u1;
  philox_pair(seed, stream, run, k >> 1, u0, u1);
  return (k & 1) ? u1 : u0;
}

// rand(1:n), 0-based: floor(u*n), clamped to n-1
__device__ __forceinline__ int randint(double u, int n) {
  int k = (int)(u * (double)n);
  return k >= n ? n - 1 : k;
}

// IEEE round-to-nearest operations that nvcc never contracts into an FMA;
// proposals and squared distances use them so that they are bit-identical to
// the reference's (x*x + y*y) + z*z evaluation.
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double ddiv(double a, double b) { return __ddiv_rn(a, b); }

__device__ __forceinline__ double dot3(double x, double y, double z) {
  return dadd(dadd(dmul(x, x), dmul(y, y)), dmul(z, z));
}
// distance2 (src/Configurations.jl:101)
__device__ __forceinline__ double d2_sph(double ax, double ay, double az,
                                         double bx, double by, double bz) {
  return dot3(dsub(ax, bx), dsub(ay, by), dsub(az, bz));
}
// distance2 with CubicBC minimum image (src/Configurations.jl:103-109)
__device__ __forceinline__ double d2_cub(double ax, double ay, double az,
                                         double bx, double by, double bz,
                                         double L) {
  double ix = dadd(bx, dmul(L, rint(ddiv(dsub(ax, bx), L))));
  double iy = dadd(by, dmul(L, rint(ddiv(dsub(ay, by), L))));
  double iz = dadd(bz, dmul(L, rint(ddiv(dsub(az, bz), L))));
  return dot3(dsub(ax, ix), dsub(ay, iy), dsub(az, iz));
}

// RectangularBC minimum image, side L in x and y, height H in z
// (src/Configurations.jl:121-126)
__device__ __forceinline__ double d2_rect(double ax, double ay, double az,
                                          double bx, double by, double bz,
                                          double L, double H) {
  double ix = dadd(bx, dmul(L, rint(ddiv(dsub(ax, bx), L))));
  double iy = dadd(by, dmul(L, rint(ddiv(dsub(ay, by), L))));
  double iz = dadd(bz, dmul(H, rint(ddiv(dsub(az, bz), H))));
  return dot3(dsub(ax, ix), dsub(ay, iy), dsub(az, iz));
}
// sqrt(3) as a double (the value of 3^0.5 in the reference)
constexpr double SQRT3 = 1.7320508075688772;
// RhombicBC minimum image (src/Configurations.jl:110-120): y on the rhombus
// height sqrt(3)/2 L, x along the sheared axis, z on the height H
__device__ __forceinline__ double d2_rhb(double ax, double ay, double az,
                                         double bx, double by, double bz,
                                         double L, double H) {
  const double hy = dmul(SQRT3 / 2, L), is3 = 1.0 / SQRT3;
  double iy = dadd(by, dmul(hy, rint(ddiv(dsub(ay, by), hy))));
  double q = ddiv(dsub(dsub(ax, bx), dmul(is3, dsub(ay, by))), L);
  double ix = dadd(dadd(dsub(bx, ddiv(by, SQRT3)), dmul(L, rint(q))), dmul(is3, iy));
  double iz = dadd(bz, dmul(H, rint(ddiv(dsub(az, bz), H))));
  return dot3(dsub(ax, ix), dsub(ay, iy), dsub(az, iz));
}

// rintf(x * y) for |x * y| < 2^22 on the FMA pipes: adding and subtracting
// 1.5 * 2^23 rounds to the nearest integer, ties to even (the spacing of
// floats in [2^23, 2^24) is 1), as rintf does; the product is rounded first,
// as in rintf(x * y), and the _rn forms keep the three steps from being
// contracted.  rintf is an XU-pipe instruction whose result waits on the
// short scoreboard.
__device__ __forceinline__ float rint_mul(float x, float y) {
  constexpr float M = 12582912.f;  // 1.5 * 2^23
  return __fadd_rn(__fadd_rn(__fmul_rn(x, y), M), -M);
}
// FP32 minimum image for the FP32 form (coordinate differences within 2^22
// box lengths)
__device__ __forceinline__ float f2_cub(float dx, float dy, float dz, float L,
                                        float iL) {
  dx -= L * rint_mul(dx, iL);
  dy -= L * rint_mul(dy, iL);
  dz -= L * rint_mul(dz, iL);
  return fmaf(dx, dx, fmaf(dy, dy, dz * dz));
}

// MUFU approximations (PTX lg2.approx / ex2.approx)
__device__ __forceinline__ float lg2f(float x) {
  float y;
  asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float ex2f(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float rcpf(float x) {
  float y;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float sqrtf_approx(float x) {
  float y;
  asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

}  // namespace ptmc
