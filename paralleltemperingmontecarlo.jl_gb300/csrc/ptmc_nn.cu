// ptmc_nn.cu — RuNNer (Behler-Parrinello) neural-network potential path.
//
// RuNNerPotential (src/EnergyEvaluation.jl:1182-1275): per-atom symmetry
// functions G (radial G2 and angular G4, MachineLearningPotential/SymmFunc.jl
// :184-312, min/max scaled), updated incrementally when one atom moves
// (MachineLearningPotential/DeltaMatrix.jl:794-975), fed to a per-atom MLP
// (ForwardPass.jl:23-84, linear/tanh/.../linear).  Only the active symmetry
// functions of one element (radial type 11, angular type 111; the others are
// identically zero, SymmFunc.jl:261,281) are stored; their MLP input rows are
// gathered on the host.
//
// Execution: one CTA of 256 threads per walker (a move is ~10^5 FLOP, far too
// much for one warp), one launch per MC cycle (N moves per walker), then a
// per-run epilogue kernel does the exchange, step adaptation and sampling of
// the cycle.  The host captures [cycle, epilogue] x C in one CUDA graph.  The
// FP32 form fits two walker CTAs per SM (98 KB at N = 55).
//
// Per move:
//   1. warp 0 draws the proposal (walker stream, reference draw order),
//   2. threads over j: new/old distance rows, cut-off rows, hard-core test
//      (with delayed acceptance the first stage follows: the frozen surrogate's
//      tabulated pair function of the new and old distances),
//   3. radial deltas: threads over (sf, j),
//   4. angular deltas.  FP32, table-specialised (a compiled pattern of eta
//      groups, lambda signs and zeta powers, NN_PAT_CU55 for scripts/cu55.jl):
//      lanes over the atoms j != i, chunks over cyclic offsets d of k; a
//      triangle costs one exponential per eta group for its new and old shape
//      and shared powers (1 +- cos)^(2^e), every function one FMA.  Otherwise
//      (generic tables, FP64): threads over (j, k-chunk), each ordered pair
//      (j, k) evaluates the old and new triangle once and adds the centre-j
//      term, one of (j, k) and (k, j) also the centre-i term; FP64:
//      exponentials shared by the functions with equal eta, powers by repeated
//      squaring; FP32: one ex2(zeta lg2(1 + lambda cos) + lg2(tpz) - eta
//      log2(e) s) per function and term,
//   5. the MLP on every atom (every column of G changes): FP32 on the tensor
//      cores (two 3xTF32 tcgen05 GEMMs, rows = atoms, activations on all 8
//      warps), FP64 on the CUDA cores, threads over (atom, hidden unit),
//   6. Metropolis on warp 0; on acceptance warp 0 moves the atom and goes on
//      to the next proposal while warps 1-7 commit the distance and cut-off
//      rows and G += dG.
#include <cuda_runtime.h>

#include "ptmc_device.cuh"
#include "ptmc_engine.cuh"
#include "ptmc_nn.cuh"
#include "ptmc_nn2.cuh"

namespace ptmc {

namespace {

constexpr int NN_THREADS = 256;
constexpr int NCH = 4;  // k chunks of the angular work items

template <typename Real>
__device__ __forceinline__ Real rexp(Real x);
template <>
__device__ __forceinline__ double rexp<double>(double x) { return exp(x); }
template <>
__device__ __forceinline__ float rexp<float>(float x) { return __expf(x); }

template <typename Real>
__device__ __forceinline__ Real rtanh(Real x);
template <>
__device__ __forceinline__ double rtanh<double>(double x) { return tanh(x); }

// cutoff_function (MachineLearningPotential/Cutoff.jl:79-90)
template <typename Real>
__device__ __forceinline__ Real cutoff(Real r, Real rc) {
  return r < rc ? Real(0.5) * (cos(Real(3.141592653589793) * (r / rc)) + Real(1)) : Real(0);
}

// (1 + lam*c)^zeta for zeta in {1,2,4,8,16}, general zeta via pow
template <typename Real>
__device__ __forceinline__ Real tpow(Real b, int zc, Real zeta) {
  if (zc == 0) return pow(b, zeta);
  Real p = b;
  if (zc >= 2) p = p * p;
  if (zc >= 3) p = p * p;
  if (zc >= 4) p = p * p;
  if (zc >= 5) p = p * p;
  return p;
}
// same with the code stored as a real: > 0 code, <= 0 minus a general zeta
template <typename Real>
__device__ __forceinline__ Real tpowc(Real b, Real code) {
  if (code <= Real(0)) return pow(b, -code);
  Real p = b;
  if (code >= Real(2)) p = p * p;
  if (code >= Real(3)) p = p * p;
  if (code >= Real(4)) p = p * p;
  if (code >= Real(5)) p = p * p;
  return p;
}

template <typename Real>
struct NNSmem {
  double* Xd;  // [N][3] positions (FP64 master: proposals and commits)
  Real* X;     // [N][3] positions in the arithmetic type
  Real* D2;    // [N][ld]
  Real* F;     // [N][ld]
  Real* G;     // [S][N]
  Real* dG;    // [S][N]
  Real* part;  // [NCH][SA][64]
  Real* rows;  // d2n, fn, rn, d2o, fo, ro, 1/rn, 1/ro [8][64]
  Real* vn;    // [64][3] t - x_j
  Real* vo;    // [64][3] x_i - x_j
  Real* W;     // MLP parameters (gathered layout)
  Real* h1;    // [N][H1]
  Real* h2;    // [N][H2]
  Real* red;   // block-reduction scratch [NN_THREADS/32 + 8]
  Real* dGi;   // [S] centre-i deltas
  Real* sfp;   // [SA][4] angular parameters: FP64 eta, lambda, tpz, zeta code;
               // FP32 -eta*log2(e), zeta, log2(tpz), lambda
  double* drw; // draw buffer [16]
  double* tpos;// trial position [3]
  int* flags;  // [4]
  int ld;      // row stride of D2 and F: N rounded up to even, so that lanes
               // reading (j, j + d) pairs (stride ld + 1) hit distinct banks
  // FP32 form: per-move rows packed for the table-specialised angular loop
  float4* pr4;  // [64] {d2n, fn, d2o, fo}
  float4* vn4;  // [64] {t - x_j, 1 / r_new}
  float4* vo4;  // [64] {x_i - x_j, 1 / r_old}
  float* tpzf;  // [MAX_NN_ANG] tpz of the angular functions
};

template <typename Real>
__device__ size_t nn_carve(NNSmem<Real>& s, unsigned char* base, int N, int S, int SA, int H1,
                           int H2, int nW) {
  size_t off = 0;
  auto take = [&](size_t bytes) {
    unsigned char* p = base + off;
    off += (bytes + 15) / 16 * 16;
    return p;
  };
  s.Xd = (double*)take(sizeof(double) * N * 3);
  s.X = (Real*)take(sizeof(Real) * N * 3);
  s.ld = N + (N & 1);
  s.D2 = (Real*)take(sizeof(Real) * N * s.ld);
  s.F = (Real*)take(sizeof(Real) * N * s.ld);
  s.G = (Real*)take(sizeof(Real) * S * N);
  s.dG = (Real*)take(sizeof(Real) * S * N);
  // the FP32 form runs the MLP on the tensor cores (weights staged straight
  // from global memory into its tiles) and keeps the angular partial sums in
  // the MLP input tile, which is free until the MLP phase of the move: only
  // the FP64 form carves the weights, hidden activations and partial sums
  s.part = s.W = s.h1 = s.h2 = nullptr;
  if constexpr (sizeof(Real) == 8) s.part = (Real*)take(sizeof(Real) * NCH * (SA > 0 ? SA : 1) * 64);
  s.rows = (Real*)take(sizeof(Real) * 8 * 64);
  s.vn = (Real*)take(sizeof(Real) * 64 * 3);
  s.vo = (Real*)take(sizeof(Real) * 64 * 3);
  if constexpr (sizeof(Real) == 8) {
    s.W = (Real*)take(sizeof(Real) * nW);
    s.h1 = (Real*)take(sizeof(Real) * N * H1);
    s.h2 = (Real*)take(sizeof(Real) * N * H2);
  }
  s.red = (Real*)take(sizeof(Real) * 64);
  s.dGi = (Real*)take(sizeof(Real) * (S > 0 ? S : 1));
  s.sfp = (Real*)take(sizeof(Real) * 4 * MAX_NN_ANG);
  s.drw = (double*)take(sizeof(double) * DRAW_BUF);
  s.tpos = (double*)take(sizeof(double) * 4);
  s.flags = (int*)take(sizeof(int) * 4);
  s.pr4 = s.vn4 = s.vo4 = nullptr;
  s.tpzf = nullptr;
  if constexpr (sizeof(Real) == 4) {
    s.pr4 = (float4*)take(sizeof(float4) * 64);
    s.vn4 = (float4*)take(sizeof(float4) * 64);
    s.vo4 = (float4*)take(sizeof(float4) * 64);
    s.tpzf = (float*)take(sizeof(float) * MAX_NN_ANG);
  }
  return off;
}

template <typename Real>
__device__ Real block_sum(Real v, Real* red) {
  v = warp_sum(v);
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __syncthreads();
  if (lane == 0) red[w] = v;
  __syncthreads();
  Real t = 0;
  if (threadIdx.x < 32) {
    t = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : Real(0);
    t = warp_sum(t);
    if (threadIdx.x == 0) red[32] = t;
  }
  __syncthreads();
  t = red[32];
  __syncthreads();
  return t;
}

// E = sum_a MLP(G[:, a] + (dG ? dG[:, a] : 0))
template <typename Real>
__device__ Real mlp_energy(const NNParams& Q, NNSmem<Real>& s, int N, bool with_delta) {
  const int S = Q.S, H1 = Q.H1, H2 = Q.H2;
  const Real* W1 = s.W;               // [S][H1]
  const Real* B1 = W1 + S * H1;       // [H1]
  const Real* W2 = B1 + H1;           // [H1][H2]
  const Real* B2 = W2 + H1 * H2;      // [H2]
  const Real* W3 = B2 + H2;           // [H2]
  const Real b3 = W3[H2];
  for (int t = threadIdx.x; t < N * H1; t += blockDim.x) {
    int a = t / H1, h = t % H1;
    Real z = 0;
    for (int q = 0; q < S; ++q) {
      Real g = s.G[q * N + a];
      if (with_delta) g += s.dG[q * N + a];
      z += g * W1[q * H1 + h];
    }
    s.h1[a * H1 + h] = rtanh<Real>(z + B1[h]);
  }
  __syncthreads();
  for (int t = threadIdx.x; t < N * H2; t += blockDim.x) {
    int a = t / H2, h = t % H2;
    Real z = 0;
    for (int q = 0; q < H1; ++q) z += s.h1[a * H1 + q] * W2[q * H2 + h];
    s.h2[a * H2 + h] = rtanh<Real>(z + B2[h]);
  }
  __syncthreads();
  Real e = 0;
  for (int a = threadIdx.x; a < N; a += blockDim.x) {
    Real z = 0;
    for (int q = 0; q < H2; ++q) z += s.h2[a * H2 + q] * W3[q];
    e += z + b3;
  }
  return block_sum(e, s.red);
}

template <typename Real>
__device__ void load_walker(const NNParams& Q, NNSmem<Real>& s, const double* X, const double* Gg,
                            int N) {
  for (int k = threadIdx.x; k < 3 * N; k += blockDim.x) {
    s.Xd[k] = X[k];
    s.X[k] = (Real)X[k];
  }
  if (s.W)
    for (int k = threadIdx.x; k < Q.nW; k += blockDim.x) s.W[k] = (Real)Q.W[k];
  for (int q = threadIdx.x; q < Q.SA; q += blockDim.x) {
    const NNSF& f = Q.sf[Q.SR + q];
    if constexpr (sizeof(Real) == 4) {  // exponent form of the FP32 path
      s.tpzf[q] = (float)f.tpz;
      s.sfp[4 * q] = (Real)(-f.eta * 1.4426950408889634);
      s.sfp[4 * q + 1] = (Real)f.zeta;
      s.sfp[4 * q + 2] = (Real)log2(f.tpz);
      s.sfp[4 * q + 3] = (Real)f.lambda;
    } else {
      s.sfp[4 * q] = (Real)f.eta;
      s.sfp[4 * q + 1] = (Real)f.lambda;
      s.sfp[4 * q + 2] = (Real)f.tpz;
      s.sfp[4 * q + 3] = (Real)(f.zc == 0 ? -f.zeta : (double)f.zc);  // >0: code, <=0: -zeta
    }
  }
  if (Gg)
    for (int k = threadIdx.x; k < Q.S * N; k += blockDim.x) s.G[k] = (Real)Gg[k];
  __syncthreads();
  for (int t = threadIdx.x; t < N * N; t += blockDim.x) {
    int a = t / N, b = t % N;
    Real dx = s.X[3 * a] - s.X[3 * b], dy = s.X[3 * a + 1] - s.X[3 * b + 1],
         dz = s.X[3 * a + 2] - s.X[3 * b + 2];
    Real d2 = (dx * dx + dy * dy) + dz * dz;
    if (a == b) d2 = Real(0);
    s.D2[a * s.ld + b] = d2;
    s.F[a * s.ld + b] = cutoff<Real>(sqrt(d2), (Real)Q.rcut);
  }
  __syncthreads();
}

// ---------------------------------------------------------------- tensor-core MLP
// FP32 form: the per-atom MLP (ForwardPass.jl:23-84) of all N <= 64 atoms as
// two tcgen05 GEMMs, rows = atoms (M = 128, rows >= N zero), K = 32 (active
// symmetry functions, then the first hidden layer, zero-padded), N = 32
// (hidden units, zero-padded).  Operands are split into TF32 hi + lo parts
// (hi = x with the low 13 mantissa bits cleared, lo = x - hi) and each product
// is hi*hi + hi*lo + lo*hi (3xTF32, ~1e-6 relative like an FP32 GEMM); accumulators in 32 TMEM columns, read back by warps 0-1 (one
// atom per thread), tanh and the output layer on the CUDA cores.  The FP64
// form keeps the CUDA-core MLP.
constexpr uint32_t MLP_LBO = 128, MLP_SBO = 1024;  // K = 32 TF32: 8 core matrices per row group
constexpr size_t MLP_TC_BYTES = 2 * 16384 + 4 * 4096 + 512 + 16;
static_assert(NCH * MAX_NN_ANG * 64 * sizeof(float) <= 2 * 16384,
              "angular partial sums must fit the MLP input tile");

struct MlpSmem {
  unsigned char *Ah, *Al;              // 128 x 32 TF32 inputs (hi, lo)
  unsigned char *B1h, *B1l, *B2h, *B2l;  // W1^T, W2^T: 32 x 32 TF32 (hi, lo)
  float* vec;                          // b1[32], b2[32], w3[32], b3
  unsigned long long* mbar;
  uint32_t* tslot;
};

__device__ __forceinline__ void mlp_carve(MlpSmem& m, unsigned char* base) {
  m.Ah = base;
  m.Al = base + 16384;
  m.B1h = base + 32768;
  m.B1l = base + 36864;
  m.B2h = base + 40960;
  m.B2l = base + 45056;
  m.vec = (float*)(base + 49152);
  m.mbar = (unsigned long long*)(base + 49152 + 512);
  m.tslot = (uint32_t*)(base + 49152 + 520);
}

// W: gathered parameters W1[S][H1], b1, W2[H1][H2], b2, w3[H2], b3 (global
// memory, rounded to FP32 here)
__device__ void mlp_stage(const MlpSmem& m, const double* W, int S, int H1, int H2) {
  const double* W2 = W + S * H1 + H1;
  for (int e = threadIdx.x; e < 2 * 16384 / 4; e += blockDim.x) ((float*)m.Ah)[e] = 0.f;
  for (int e = threadIdx.x; e < 32 * 32; e += blockDim.x) {
    const int n = e / 32, k = e % 32;
    const float x1 = (k < S && n < H1) ? (float)W[k * H1 + n] : 0.f;
    const float x2 = (k < H1 && n < H2) ? (float)W2[k * H2 + n] : 0.f;
    const uint32_t o = umma_off32(n, k, MLP_LBO, MLP_SBO);
    const float h1 = tf32_hi(x1), h2 = tf32_hi(x2);
    *(float*)(m.B1h + o) = h1;
    *(float*)(m.B1l + o) = x1 - h1;
    *(float*)(m.B2h + o) = h2;
    *(float*)(m.B2l + o) = x2 - h2;
  }
  for (int n = threadIdx.x; n < 32; n += blockDim.x) {
    m.vec[n] = n < H1 ? (float)W[S * H1 + n] : 0.f;
    m.vec[32 + n] = n < H2 ? (float)W2[H1 * H2 + n] : 0.f;
    m.vec[64 + n] = n < H2 ? (float)W2[H1 * H2 + H2 + n] : 0.f;
  }
  if (threadIdx.x == 0) {
    m.vec[96] = (float)W2[H1 * H2 + 2 * H2];
    mbar_init(smem_u32(m.mbar), 1);
  }
  fence_async_smem();
}

// three TF32 products per K = 8 step: hi*hi, hi*lo, lo*hi
__device__ __forceinline__ void mlp_issue(uint32_t tbase, const unsigned char* Ah,
                                          const unsigned char* Al, const unsigned char* Bh,
                                          const unsigned char* Bl) {
  const uint32_t id = umma_idesc_tf32(128, 32);
  const uint32_t ah = smem_u32(Ah), al = smem_u32(Al), bh = smem_u32(Bh), bl = smem_u32(Bl);
#pragma unroll
  for (int ks = 0; ks < 4; ++ks) {
    const uint32_t o = 2u * MLP_LBO * ks;
    umma_tf32(tbase, umma_sdesc(ah + o, MLP_LBO, MLP_SBO), umma_sdesc(bh + o, MLP_LBO, MLP_SBO), id,
              ks > 0);
    umma_tf32(tbase, umma_sdesc(ah + o, MLP_LBO, MLP_SBO), umma_sdesc(bl + o, MLP_LBO, MLP_SBO), id, 1);
    umma_tf32(tbase, umma_sdesc(al + o, MLP_LBO, MLP_SBO), umma_sdesc(bh + o, MLP_LBO, MLP_SBO), id, 1);
  }
}

// E = sum_a MLP(G[:, a] (+ dG[:, a])); every thread calls it.  `ph` is the
// mbarrier parity (flipped twice); *bad is set (uniformly) when a
// tensor-core wait ran out.
// tanh(x) = 1 - 2 / (1 + 2^(2 log2(e) x)) with MUFU ex2 and rcp: absolute
// error ~3e-7 (the FP32 form's MLP; saturates to +-1 without overflow)
__device__ __forceinline__ float tanh_mufu(float x) {
  return 1.f - __fdividef(2.f, 1.f + ex2f(x * 2.8853900817779268f));
}

__device__ float mlp_energy_tc(const NNSmem<float>& s, const MlpSmem& m, int N, int S, int H1,
                               int H2, bool with_delta, uint32_t tbase, uint32_t& ph, int* bad) {
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t mb = smem_u32(m.mbar);
  {  // inputs: thread (atom a = tid % 64, columns q = tid / 64, + 4, ...), columns S..31 zero
    const int a = tid & 63;
    if (a < N) {
      const uint32_t ob = umma_off32(a, 0, MLP_LBO, MLP_SBO);
      for (int q = tid >> 6; q < 32; q += NN_THREADS / 64) {
        float x = 0.f;
        if (q < S) {
          x = s.G[q * N + a];
          if (with_delta) x += s.dG[q * N + a];
        }
        const uint32_t o = ob + (uint32_t)(q >> 2) * MLP_LBO + (uint32_t)(q & 3) * 4u;
        const float h = tf32_hi(x);
        *(float*)(m.Ah + o) = h;
        *(float*)(m.Al + o) = x - h;
      }
    }
  }
  fence_async_smem();
  tc_fence_before();
  __syncthreads();
  if (tid == 0) {
    tc_fence_after();
    mlp_issue(tbase, m.Ah, m.Al, m.B1h, m.B1l);
    umma_commit(mb);
  }
  // accumulator rows = atoms 0..63 live in TMEM lanes 0-63, readable by warps
  // 0, 1 and 4, 5 (a warp reads the lane quarter warp % 4), columns 16 (warp / 4)
  // .. +15; they are staged column-major in the upper half of the A hi tile
  // (rows 64-127, whose products are never read back), and all 8 warps apply
  // the activations: thread (atom a = tid % 64, columns 8 (tid / 64) .. +7)
  float* stg = (float*)(m.Ah + 8192);
  const bool tw = (warp & 3) < 2;
  const int ta = 32 * (warp & 1) + lane, half = warp >> 2;
  const uint32_t taddr = tbase + ((uint32_t)(32 * (warp & 3)) << 16) + 16u * (uint32_t)half;
  int b = 0;
  auto stage = [&]() {
    if (tw) {
      if (!mbar_wait(mb, ph)) b = 1;
      tc_fence_after();
      float acc[16];
      tmem_ld16(taddr, acc);
#pragma unroll
      for (int c = 0; c < 16; ++c) stg[(16 * half + c) * 64 + ta] = acc[c];
    }
    ph ^= 1u;
    tc_fence_before();
  };
  const int a = tid & 63, c0 = 8 * (tid >> 6);
  stage();
  if (__syncthreads_or(b)) {
    *bad = 1;
    return 0.f;
  }
  if (a < N) {  // first hidden layer -> second GEMM's input (hi, lo)
    const uint32_t ob = umma_off32(a, 0, MLP_LBO, MLP_SBO);
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      const int n = c0 + c;
      const float h = n < H1 ? tanh_mufu(stg[n * 64 + a] + m.vec[n]) : 0.f;
      const uint32_t o = ob + (uint32_t)(n >> 2) * MLP_LBO + (uint32_t)(n & 3) * 4u;
      const float hh = tf32_hi(h);
      *(float*)(m.Ah + o) = hh;
      *(float*)(m.Al + o) = h - hh;
    }
  }
  fence_async_smem();
  tc_fence_before();
  __syncthreads();
  if (tid == 0) {
    tc_fence_after();
    mlp_issue(tbase, m.Ah, m.Al, m.B2h, m.B2l);
    umma_commit(mb);
  }
  stage();
  if (__syncthreads_or(b)) {
    *bad = 1;
    return 0.f;
  }
  float e = 0.f;
  if (a < N) {
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      const int n = c0 + c;
      if (n < H2) e += m.vec[64 + n] * tanh_mufu(stg[n * 64 + a] + m.vec[32 + n]);
    }
    if (c0 == 0) e += m.vec[96];
  }
  e = warp_sum(e);
  if (lane == 0) s.red[warp] = e;
  __syncthreads();
  return ((s.red[0] + s.red[1]) + (s.red[2] + s.red[3])) +
         ((s.red[4] + s.red[5]) + (s.red[6] + s.red[7]));
}

// tensor-core state of a walker CTA (FP32 form): the MLP tiles and one
// 32-column TMEM allocation; the FP64 form has none
template <typename Real>
struct TcState {
  MlpSmem m{};
  uint32_t tbase = 0, mph = 0;
  bool on = false;
};

template <typename Real>
__device__ void tc_setup(TcState<Real>& t, unsigned char* smem_raw, size_t off, const NNParams& Q) {
  if constexpr (sizeof(Real) == 4) {
    const uint32_t a = smem_u32(smem_raw) + (uint32_t)off;
    off += (128u - (a & 127u)) & 127u;
    mlp_carve(t.m, smem_raw + off);
    mlp_stage(t.m, Q.W, Q.S, Q.H1, Q.H2);
    t.on = true;
    if ((threadIdx.x >> 5) == 0) tmem_alloc(smem_u32(t.m.tslot), 32);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    t.tbase = *t.m.tslot;
  }
}

template <typename Real>
__device__ void tc_teardown(const TcState<Real>& t) {
  if (!t.on) return;
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if ((threadIdx.x >> 5) == 0) tmem_dealloc(t.tbase, 32);
}

// acc[q] += E_g (1 + lambda cos_new)^zeta - E'_g (1 + lambda cos_old)^zeta for
// every function q of pattern PAT (mapping fixed at compile time; powers 2^e of
// both signs by repeated squaring, the unused ones are never formed)
template <int PAT>
__device__ __forceinline__ void pat_accumulate(float* acc, const float* En, const float* Eo,
                                               float cn, float co) {
  float pn[2][5], po[2][5];
  pn[0][0] = 1.f + cn;
  pn[1][0] = 1.f - cn;
  po[0][0] = 1.f + co;
  po[1][0] = 1.f - co;
#pragma unroll
  for (int e = 1; e < 5; ++e)
#pragma unroll
    for (int sg = 0; sg < 2; ++sg) {
      pn[sg][e] = pn[sg][e - 1] * pn[sg][e - 1];
      po[sg][e] = po[sg][e - 1] * po[sg][e - 1];
    }
#pragma unroll
  for (int q = 0; q < nn_pat_sa(PAT); ++q) {
    const int t = nn_pat_term(PAT, q);
    const int g = t & 15, sg = (t >> 4) & 1, e = t >> 5;
    acc[q] = fmaf(En[g], pn[sg][e], acc[q]);
    acc[q] = fmaf(-Eo[g], po[sg][e], acc[q]);
  }
}

}  // namespace

// --------------------------------------------------------------- init kernel
// set_variables + initialise_energy (src/EnergyEvaluation.jl:1812-1822,
// 1737-1747; total_symm_calc, SymmFunc.jl:494-510, with every angular row).
template <typename Real>
__global__ void __launch_bounds__(NN_THREADS) k_nn_init(KParams P, NNParams Q) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int gw = blockIdx.x;  // global walker
  const int run = Q.run_of_walker[gw];
  const RunDesc* rd = P.runs + run;
  const int N = rd->N, w = gw - rd->wk;
  NNSmem<Real> s;
  const size_t nn_off = nn_carve(s, smem_raw, N, Q.S, Q.SA, Q.H1, Q.H2, Q.nW);
  const double* X = P.pos + rd->pos_off + (size_t)w * N * 3;
  load_walker(Q, s, X, nullptr, N);
  TcState<Real> tc;
  tc_setup(tc, smem_raw, nn_off, Q);
  const int S = Q.S, SR = Q.SR, ld = s.ld;
  for (int t = threadIdx.x; t < S * N; t += blockDim.x) s.G[t] = 0;
  __syncthreads();
  // radial: G_s[a] = sum_b gnorm f_ab exp(-eta r2_ab) (fc != 0, 1 excluded, SymmFunc.jl:234)
  for (int t = threadIdx.x; t < SR * N; t += blockDim.x) {
    int q = t / N, a = t % N;
    const NNSF& f = Q.sf[q];
    Real g = 0;
    for (int b = 0; b < N; ++b) {
      if (b == a) continue;
      Real fc = s.F[a * ld + b];
      if (fc != Real(0) && fc != Real(1))
        g += fc * rexp<Real>(-(Real)f.eta * s.D2[a * ld + b]) * (Real)f.gnorm;
    }
    s.G[q * N + a] = g + (Real)f.goffset;
  }
  // angular: centre a, pairs b < c
  for (int t = threadIdx.x; t < (S - SR) * N; t += blockDim.x) {
    int q = SR + t / N, a = t % N;
    const NNSF& f = Q.sf[q];
    Real g = 0;
    for (int b = 0; b < N; ++b) {
      if (b == a) continue;
      for (int c = b + 1; c < N; ++c) {
        if (c == a) continue;
        Real rab = s.D2[a * ld + b], rac = s.D2[a * ld + c], rbc = s.D2[b * ld + c];
        Real ex = rexp<Real>(-(Real)f.eta * (rab + rac + rbc)) * s.F[a * ld + b] * s.F[a * ld + c] *
                  s.F[b * ld + c];
        if (ex == Real(0)) continue;
        Real abx = s.X[3 * a] - s.X[3 * b], aby = s.X[3 * a + 1] - s.X[3 * b + 1],
             abz = s.X[3 * a + 2] - s.X[3 * b + 2];
        Real acx = s.X[3 * a] - s.X[3 * c], acy = s.X[3 * a + 1] - s.X[3 * c + 1],
             acz = s.X[3 * a + 2] - s.X[3 * c + 2];
        Real cs = ((abx * acx + aby * acy) + abz * acz) / (sqrt(rab) * sqrt(rac));
        g += ex * tpow<Real>(Real(1) + (Real)f.lambda * cs, f.zc, (Real)f.zeta) * (Real)f.tpz;
      }
    }
    s.G[q * N + a] = g + (Real)f.goffset;
  }
  __syncthreads();
  Real e;
  int bad = 0;
  if constexpr (sizeof(Real) == 4)
    e = mlp_energy_tc(s, tc.m, N, S, Q.H1, Q.H2, false, tc.tbase, tc.mph, &bad);
  else
    e = mlp_energy<Real>(Q, s, N, false);
  double* Gg = Q.G + (size_t)gw * S * Q.Nmax;
  for (int t = threadIdx.x; t < S * N; t += blockDim.x) Gg[t] = (double)s.G[t];
  if (threadIdx.x == 0) {
    P.en[rd->wk + w] = (double)e;
    P.status[rd->wk + w] = bad ? ST_TIMEOUT : ST_OK;
    P.drift[rd->wk + w] = 0.0;
  }
  tc_teardown(tc);
}

// --------------------------------------------------------------- cycle kernel
template <typename Real, int PAT>
__global__ void __launch_bounds__(NN_THREADS, sizeof(Real) == 4 ? 2 : 1)
    k_nn_cycle(KParams P, NNParams Q, int phase) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int gw = blockIdx.x;
  const int run = Q.run_of_walker[gw];
  const RunDesc* rd = P.runs + run;
  const int N = rd->N, w = gw - rd->wk, g = rd->wk + w;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int S = Q.S, SR = Q.SR, SA = Q.SA;
  NNSmem<Real> s;
  const size_t nn_off = nn_carve(s, smem_raw, N, S, SA, Q.H1, Q.H2, Q.nW);
  const int ld = s.ld;
  double* Xg = P.pos + rd->pos_off + (size_t)w * N * 3;
  double* Gg = Q.G + (size_t)gw * S * Q.Nmax;
  load_walker(Q, s, Xg, Gg, N);
  if (P.status[g] != ST_OK) return;
  // tensor-core tiles after the walker state: MLP (FP32 form), surrogate (delayed acceptance)
  TcState<Real> tc;
  tc_setup(tc, smem_raw, nn_off, Q);
  // FP32: angular partial sums in the MLP input tile (Ah, Al: 32 KB >= NCH x
  // MAX_NN_ANG x 64 floats); rows of that tile beyond N are then not zero, but
  // each row of an MMA product depends on its own row only and rows >= N are
  // never read back
  if constexpr (sizeof(Real) == 4) s.part = (Real*)tc.m.Ah;
  const uint32_t tbase = tc.tbase;
  long long n_rej1 = 0, n_exact = 0;
  const int slot = Q.sow[g];
  const int gs = rd->wk + slot;
  const float kap = Q.da ? Q.da_kappa[gs] : 0.f;
  const double beta = P.beta[gs];
  const double md = P.maxd[2 * gs];
  double en = P.en[g];
  unsigned long long ctr = P.ctr[g];
  unsigned long long base = ctr + DRAW_BUF;
  int status = ST_OK;
  long long acc = 0;
  const Real rc = (Real)Q.rcut;
  const float pirc = (float)(3.141592653589793 / Q.rcut);
  const uint32_t run_word = (uint32_t)rd->run_id;
  const double R2 = P.box[g] * P.box[g];

  auto draw = [&]() -> double {  // warp 0 only, lanes in lockstep
    if (ctr - base >= (unsigned long long)DRAW_BUF) {
      __syncwarp();
      base = ctr & ~1ull;
      if (lane < DRAW_BUF / 2) {
        double u0, u1;
        philox_pair(P.seed, (uint32_t)w, run_word, (base >> 1) + lane, u0, u1);
        s.drw[2 * lane] = u0;
        s.drw[2 * lane + 1] = u1;
      }
      __syncwarp();
    }
    double u = s.drw[ctr - base];
    ++ctr;
    return u;
  };

  for (int step = 0; step < N; ++step) {
    // ---- 1. proposal (atom_displacement, src/MCMoves.jl:33-48, 115-143)
    if (warp == 0) {
      int i = randint(draw(), N);
      double xi = s.Xd[3 * i], yi = s.Xd[3 * i + 1], zi = s.Xd[3 * i + 2];
      double tx, ty, tz;
      auto propose = [&]() {
        double ux = draw(), uy = draw(), uz = draw();
        tx = dadd(xi, dmul(dsub(ux, 0.5), md));
        ty = dadd(yi, dmul(dsub(uy, 0.5), md));
        tz = dadd(zi, dmul(dsub(uz, 0.5), md));
      };
      propose();
      int count = 0, err = 0, rec = 0;
      while (dot3(tx, ty, tz) > R2) {
        ++count;
        if (count == 50) {
          rec = 1;  // recentre handled by the whole CTA below (rare path)
          break;
        }
        propose();
        if (count == 100) {
          err = 1;
          break;
        }
      }
      if (lane == 0) {
        s.tpos[0] = tx;
        s.tpos[1] = ty;
        s.tpos[2] = tz;
        s.flags[0] = i;
        s.flags[1] = err;
        s.flags[2] = rec;
      }
    }
    __syncthreads();
    if (s.flags[2]) {
      // recentre! at the 50th retry (src/MCMoves.jl:126-128): the rare path
      // shifts the configuration and the move continues with fresh proposals
      if (tid == 0) {  // mean of the positions, in order (src/Configurations.jl:64-85)
        double cx = 0, cy = 0, cz = 0;
        for (int a = 0; a < N; ++a) {
          cx += s.Xd[3 * a];
          cy += s.Xd[3 * a + 1];
          cz += s.Xd[3 * a + 2];
        }
        cx /= N;
        cy /= N;
        cz /= N;
        for (int a = 0; a < N; ++a) {
          s.Xd[3 * a] -= cx;
          s.Xd[3 * a + 1] -= cy;
          s.Xd[3 * a + 2] -= cz;
          s.X[3 * a] = (Real)s.Xd[3 * a];
          s.X[3 * a + 1] = (Real)s.Xd[3 * a + 1];
          s.X[3 * a + 2] = (Real)s.Xd[3 * a + 2];
        }
      }
      __syncthreads();
      if (warp == 0) {
        int i = s.flags[0];
        double xi = s.Xd[3 * i], yi = s.Xd[3 * i + 1], zi = s.Xd[3 * i + 2];
        double tx = 0, ty = 0, tz = 0;
        int err = 1;
        for (int count = 51; count <= 100; ++count) {
          double ux = draw(), uy = draw(), uz = draw();
          tx = dadd(xi, dmul(dsub(ux, 0.5), md));
          ty = dadd(yi, dmul(dsub(uy, 0.5), md));
          tz = dadd(zi, dmul(dsub(uz, 0.5), md));
          if (count == 100) break;
          if (!(dot3(tx, ty, tz) > R2)) {
            err = 0;
            break;
          }
        }
        if (lane == 0) {
          s.tpos[0] = tx;
          s.tpos[1] = ty;
          s.tpos[2] = tz;
          s.flags[1] = err;
        }
      }
      __syncthreads();
    }
    if (s.flags[1]) {
      status = ST_SPHERE;
      break;
    }
    const int i = s.flags[0];
    const Real tx = (Real)s.tpos[0], ty = (Real)s.tpos[1], tz = (Real)s.tpos[2];
    Real* d2n = s.rows;
    Real* fn = s.rows + 64;
    Real* rn = s.rows + 128;
    Real* d2o = s.rows + 192;
    Real* fo = s.rows + 256;
    Real* ro = s.rows + 320;
    Real* rin = s.rows + 384;
    Real* rio = s.rows + 448;
    // ---- 2. rows and hard core (energy_update! RuNNer, src/EnergyEvaluation.jl:1593-1606)
    int hard = 0;
    for (int j = tid; j < N; j += blockDim.x) {
      Real vx = tx - s.X[3 * j], vy = ty - s.X[3 * j + 1], vz = tz - s.X[3 * j + 2];
      Real d = (vx * vx + vy * vy) + vz * vz;
      if (j == i) d = 0;
      d2n[j] = d;
      if constexpr (sizeof(Real) == 4) {  // MUFU rsqrt and cos (argument in [0, pi])
        rin[j] = j == i ? 0.f : rsqrtf(d);
        rn[j] = d * rin[j];
        fn[j] = rn[j] < rc ? 0.5f * (__cosf(rn[j] * pirc) + 1.f) : 0.f;
      } else {
        rn[j] = sqrt(d);
        fn[j] = cutoff<Real>(rn[j], rc);
      }
      s.vn[3 * j] = vx;
      s.vn[3 * j + 1] = vy;
      s.vn[3 * j + 2] = vz;
      Real ox = s.X[3 * i] - s.X[3 * j], oy = s.X[3 * i + 1] - s.X[3 * j + 1],
           oz = s.X[3 * i + 2] - s.X[3 * j + 2];
      s.vo[3 * j] = ox;
      s.vo[3 * j + 1] = oy;
      s.vo[3 * j + 2] = oz;
      d2o[j] = s.D2[i * ld + j];
      if constexpr (sizeof(Real) == 4) {
        rio[j] = j == i ? 0.f : rsqrtf(d2o[j]);
        ro[j] = d2o[j] * rio[j];
      } else {
        ro[j] = sqrt(d2o[j]);
        rin[j] = Real(1) / rn[j];
        rio[j] = Real(1) / ro[j];
      }
      fo[j] = s.F[i * ld + j];
      if constexpr (sizeof(Real) == 4) {
        s.pr4[j] = make_float4(d, fn[j], d2o[j], fo[j]);
        s.vn4[j] = make_float4(vx, vy, vz, rin[j]);
        s.vo4[j] = make_float4(ox, oy, oz, rio[j]);
      }
      if (j != i && d < (Real)Q.boundary2) hard = 1;
    }
    hard = __syncthreads_or(hard);
    // ---- delayed acceptance, stage 1 (Christen & Fox 2005): the surrogate
    // dE_s screens the proposal with its own draw; a rejection here costs no
    // exact evaluation
    double dEs = 0.0;
    if (kap > 0.f) {
      // dE_s = sum_j phi(|t - x_j|) - phi(|x_i - x_j|), phi from the frozen
      // surrogate's table (threads j < N <= 64: warps 0 and 1)
      float v = 0.f;
      if (tid < N && tid != i)
        v = sur_tab_phi(Q.sur_tab, Q.sur_tab_inv_h, (float)rn[tid]) -
            sur_tab_phi(Q.sur_tab, Q.sur_tab_inv_h, (float)ro[tid]);
      v = warp_sum(v);
      if (lane == 0 && warp < 2) s.red[16 + warp] = v;
      __syncthreads();
      // screening strength kappa: stage 1 on exp(-kappa beta dE_s), stage 2 on
      // exp(-beta (dE - kappa dE_s)); exact for any fixed kappa
      dEs = (double)(kap * (float)(s.red[16] + s.red[17]));
      int pass = 0;
      if (warp == 0) {
        double p1;
        if constexpr (sizeof(Real) == 4) {  // MUFU exp, min(1, exp(x)) = 2^(min(x, 0) log2 e)
          p1 = (double)ex2f(fminf((float)(-dEs * beta), 0.f) * 1.4426950408889634f);
        } else {
          p1 = exp(-dEs * beta);
          if (p1 > 1) p1 = 1.0;
        }
        pass = p1 >= draw();
      }
      if (!__syncthreads_or(warp == 0 && lane == 0 && pass)) {
        ++n_rej1;
        continue;
      }
      ++n_exact;
    } else if (Q.da) {
      ++n_exact;  // an unscreened slot: every move is evaluated exactly
    }
    Real new_en;
    if (hard) {
      new_en = Real(100.0);
    } else {
      for (int q = tid; q < S; q += blockDim.x) s.dGi[q] = 0;
      __syncthreads();
      // ---- 3. radial deltas (radial_symmetry_calculation!, DeltaMatrix.jl:794-822)
      for (int t = tid; t < SR * N; t += blockDim.x) {
        int q = t / N, j = t % N;
        Real d = 0;
        if (j != i) {
          const NNSF& f = Q.sf[q];
          Real eta = (Real)f.eta, gn = (Real)f.gnorm;
          d = rexp<Real>(-eta * d2n[j]) * (fn[j] * gn) - rexp<Real>(-eta * d2o[j]) * (fo[j] * gn);
        }
        s.dG[q * N + j] = d;
      }
      // ---- 4. angular deltas (angular_symmetry_calculation!, DeltaMatrix.jl:827-871)
      if constexpr (sizeof(Real) == 4 && PAT != NN_PAT_GENERIC) {
        // Table-specialised FP32 form.  Every function q is (eta group g,
        // lambda sign, zeta = 2^e) with the mapping known at compile time, so a
        // triangle costs one exponential per eta group for its new and its old
        // shape, E_g = f_ij f_ik f_jk 2^(-eta_g log2(e) s), and the powers
        // (1 +- cos)^(2^e) by repeated squaring, shared by all functions; each
        // function adds E_g P to its accumulator with one FMA, and tpz scales
        // the sums.  Lanes jj = 0 .. N-2 of a 64-lane group run over the atoms
        // j != i, chunk c over the cyclic offsets d = c+1, c+1+NCH, ... < N-1 of
        // k = jj + d (mod N-1).  The centre-i term of an unordered pair {j, k}
        // is taken at 2d < N-1 (and at 2d = N-1 by the lower index): the same
        // for every lane of a warp at a given d.
        constexpr int SAp = nn_pat_sa(PAT), NGp = nn_pat_ng(PAT);
        static_assert(SAp <= MAX_NN_ANG && NGp <= 8, "pattern sizes");
        const int Np = N - 1, jj = tid & 63, c = tid >> 6;
        float accj[SAp], acci[SAp];
#pragma unroll
        for (int q = 0; q < SAp; ++q) {
          accj[q] = 0.f;
          acci[q] = 0.f;
        }
        int j = -1;
        if (jj < Np) {
          j = jj + (jj >= i);
          const float4 vj = s.vn4[j], wj = s.vo4[j], pj = s.pr4[j];
          const float* D2j = s.D2 + j * ld;
          const float* Fj = s.F + j * ld;
          int kk = jj + c + 1;
          if (kk >= Np) kk -= Np;
          for (int d = c + 1; d < Np; d += NCH) {
            const int k = kk + (kk >= i);
            const bool ci = 2 * d < Np || (2 * d == Np && jj < kk);
            kk += NCH;
            if (kk >= Np) kk -= Np;
            const float rjk2 = D2j[k], fjk = Fj[k];
            const float4 pk = s.pr4[k], vk = s.vn4[k];
            // f products folded into the exponent (lg2 0 = -inf gives E = 0)
            const float lfn = lg2f((pj.y * pk.y) * fjk), lfo = lg2f((pj.w * pk.w) * fjk);
            const float sn = (pj.x + pk.x) + rjk2, so = (pj.z + pk.z) + rjk2;
            float En[NGp], Eo[NGp];
#pragma unroll
            for (int g = 0; g < NGp; ++g) {
              En[g] = ex2f(fmaf(Q.ang_nle[g], sn, lfn));
              Eo[g] = ex2f(fmaf(Q.ang_nle[g], so, lfo));
            }
            const float rjki = rsqrtf(rjk2);
            const float ux = vj.x - vk.x, uy = vj.y - vk.y, uz = vj.z - vk.z;  // x_k - x_j
            // angle at j: (t - x_j).(x_k - x_j) / (r_new,j r_jk), old: (x_i - x_j)
            const float cjn = ((vj.x * ux + vj.y * uy) + vj.z * uz) * (vj.w * rjki);
            const float cjo = ((wj.x * ux + wj.y * uy) + wj.z * uz) * (wj.w * rjki);
            pat_accumulate<PAT>(accj, En, Eo, cjn, cjo);
            if (ci) {  // angle at the moved atom: (x_j - t).(x_k - t) / (r_j r_k)
              const float4 wk = s.vo4[k];
              const float cin = ((vj.x * vk.x + vj.y * vk.y) + vj.z * vk.z) * (vj.w * vk.w);
              const float cio = ((wj.x * wk.x + wj.y * wk.y) + wj.z * wk.z) * (wj.w * wk.w);
              pat_accumulate<PAT>(acci, En, Eo, cin, cio);
            }
          }
        }
#pragma unroll
        for (int q = 0; q < SAp; ++q) {
          const float tz = s.tpzf[q];
          if (j >= 0) s.part[(c * SAp + q) * 64 + j] = accj[q] * tz;
          const float v = warp_sum(acci[q]);
          if (lane == 0 && v != 0.f) atomicAdd(&s.dGi[SR + q], v * tz);
        }
      } else {
        const int j = tid % 64, c = tid / 64;
        Real accj[MAX_NN_ANG], acci[MAX_NN_ANG];
#pragma unroll
        for (int q = 0; q < MAX_NN_ANG; ++q) {
          accj[q] = 0;
          acci[q] = 0;
        }
        if (j < N && j != i) {
          const int k0 = (c * N) / NCH, k1 = ((c + 1) * N) / NCH;
          const Real vnx = s.vn[3 * j], vny = s.vn[3 * j + 1], vnz = s.vn[3 * j + 2];
          const Real vox = s.vo[3 * j], voy = s.vo[3 * j + 1], voz = s.vo[3 * j + 2];
          const Real rnj = rn[j], roj = ro[j], fnj = fn[j], foj = fo[j];
          if constexpr (sizeof(Real) == 4) {
            // FP32: every term is one ex2 of zeta*lg2(1 + lambda cos) + lg2(tpz) -
            // eta*log2(e)*s (no per-function branches); the centre-i term of an
            // unordered pair {j, k} is taken by exactly one of (j, k) and (k, j),
            // chosen by the parity of j + k so that the threads share it evenly
            const float rnji = rin[j], roji = rio[j], d2nj = d2n[j], d2oj = d2o[j];
            const float4* sf4 = reinterpret_cast<const float4*>(s.sfp);
            for (int k = k0; k < k1; ++k) {
              if (k == i || k == j) continue;
              const float rjk2 = s.D2[j * ld + k], fjk = s.F[j * ld + k];
              const float fpn = fnj * fn[k] * fjk, fpo = foj * fo[k] * fjk;
              if (fpn == 0.f && fpo == 0.f) continue;
              const float rjki = rsqrtf(rjk2);
              const float ux = s.X[3 * k] - s.X[3 * j], uy = s.X[3 * k + 1] - s.X[3 * j + 1],
                          uz = s.X[3 * k + 2] - s.X[3 * j + 2];
              const float cjn = ((vnx * ux + vny * uy) + vnz * uz) * (rnji * rjki);
              const float cjo = ((vox * ux + voy * uy) + voz * uz) * (roji * rjki);
              const float sn = (d2nj + d2n[k]) + rjk2, so = (d2oj + d2o[k]) + rjk2;
              const bool ci_on = (j < k) == (((j + k) & 1) != 0);
              const float ljn_p = lg2f(fmaxf(1.f + cjn, 0.f)), ljn_m = lg2f(fmaxf(1.f - cjn, 0.f));
              const float ljo_p = lg2f(fmaxf(1.f + cjo, 0.f)), ljo_m = lg2f(fmaxf(1.f - cjo, 0.f));
              float lin_p = 0.f, lin_m = 0.f, lio_p = 0.f, lio_m = 0.f;
              if (ci_on) {
                const float cin = ((vnx * s.vn[3 * k] + vny * s.vn[3 * k + 1]) + vnz * s.vn[3 * k + 2]) *
                                  (rnji * rin[k]);
                const float cio = ((vox * s.vo[3 * k] + voy * s.vo[3 * k + 1]) + voz * s.vo[3 * k + 2]) *
                                  (roji * rio[k]);
                lin_p = lg2f(fmaxf(1.f + cin, 0.f));
                lin_m = lg2f(fmaxf(1.f - cin, 0.f));
                lio_p = lg2f(fmaxf(1.f + cio, 0.f));
                lio_m = lg2f(fmaxf(1.f - cio, 0.f));
              }
#pragma unroll
              for (int q = 0; q < MAX_NN_ANG; ++q) {
                if (q < SA) {
                  const float4 pr = sf4[q];  // -eta*log2e, zeta, lg2(tpz), lambda
                  const float tn = fmaf(pr.x, sn, pr.z), to = fmaf(pr.x, so, pr.z);
                  const bool lp = pr.w > 0.f;
                  accj[q] = fmaf(fpn, ex2f(fmaf(pr.y, lp ? ljn_p : ljn_m, tn)), accj[q]);
                  accj[q] = fmaf(-fpo, ex2f(fmaf(pr.y, lp ? ljo_p : ljo_m, to)), accj[q]);
                  if (ci_on) {
                    acci[q] = fmaf(fpn, ex2f(fmaf(pr.y, lp ? lin_p : lin_m, tn)), acci[q]);
                    acci[q] = fmaf(-fpo, ex2f(fmaf(pr.y, lp ? lio_p : lio_m, to)), acci[q]);
                  }
                }
              }
            }
          } else
          for (int k = k0; k < k1; ++k) {
            if (k == i || k == j) continue;
            const Real rjk2 = s.D2[j * ld + k], fjk = s.F[j * ld + k];
            const Real fpn = fnj * fn[k] * fjk, fpo = foj * fo[k] * fjk;
            if (fpn == Real(0) && fpo == Real(0)) continue;
            const Real rjk = sqrt(rjk2);
            // x_k - x_j
            const Real ux = s.X[3 * k] - s.X[3 * j], uy = s.X[3 * k + 1] - s.X[3 * j + 1],
                       uz = s.X[3 * k + 2] - s.X[3 * j + 2];
            // angle at j: (t - x_j).(x_k - x_j) / (|t - x_j| |x_k - x_j|)
            const Real cjn = ((vnx * ux + vny * uy) + vnz * uz) / (rnj * rjk);
            const Real cjo = ((vox * ux + voy * uy) + voz * uz) / (roj * rjk);
            const Real sn = (d2n[j] + d2n[k]) + rjk2, so = (d2o[j] + d2o[k]) + rjk2;
            const bool ci_on = j < k;
            Real cin = 0, cio = 0;
            if (ci_on) {  // angle at the moved atom: (x_j - t).(x_k - t) / (r_j r_k)
              cin = ((vnx * s.vn[3 * k] + vny * s.vn[3 * k + 1]) + vnz * s.vn[3 * k + 2]) / (rnj * rn[k]);
              cio = ((vox * s.vo[3 * k] + voy * s.vo[3 * k + 1]) + voz * s.vo[3 * k + 2]) / (roj * ro[k]);
            }
            Real en_e = 0, eo_e = 0, last_eta = -1;
#pragma unroll
            for (int q = 0; q < MAX_NN_ANG; ++q) {  // unrolled: accumulators stay in registers
              if (q < SA) {
                const Real eta = s.sfp[4 * q], lam = s.sfp[4 * q + 1], tpz = s.sfp[4 * q + 2],
                           zc = s.sfp[4 * q + 3];
                if (eta != last_eta) {  // sorted by eta: one exp pair per distinct eta
                  en_e = rexp<Real>(-eta * sn) * fpn;
                  eo_e = rexp<Real>(-eta * so) * fpo;
                  last_eta = eta;
                }
                accj[q] += (en_e * tpowc<Real>(Real(1) + lam * cjn, zc) -
                            eo_e * tpowc<Real>(Real(1) + lam * cjo, zc)) * tpz;
                if (ci_on)
                  acci[q] += (en_e * tpowc<Real>(Real(1) + lam * cin, zc) -
                              eo_e * tpowc<Real>(Real(1) + lam * cio, zc)) * tpz;
              }
            }
          }
        }
#pragma unroll
        for (int q = 0; q < MAX_NN_ANG; ++q) {
          if (q < SA) {
            s.part[(c * SA + q) * 64 + j] = accj[q];
            Real v = warp_sum(acci[q]);
            if (lane == 0 && v != Real(0)) atomicAdd(&s.dGi[SR + q], v);
          }
        }
      }
      __syncthreads();
      {  // thread: atom j = tid % 64, functions q = tid / 64, + 4, ...
        const int j = tid & 63;
        if (j < N)
          for (int q = tid >> 6; q < SA; q += NN_THREADS / 64) {
            Real v = 0;
            if (j != i)
              for (int c = 0; c < NCH; ++c) v += s.part[(c * SA + q) * 64 + j];
            s.dG[(SR + q) * N + j] = v;
          }
      }
      for (int q = warp; q < SR; q += NN_THREADS / 32) {  // centre-i radial deltas
        Real v = 0;
        for (int j = lane; j < N; j += 32) v += s.dG[q * N + j];
        v = warp_sum(v);
        if (lane == 0) s.dGi[q] = v;
      }
      __syncthreads();
      for (int q = tid; q < S; q += blockDim.x) s.dG[q * N + i] = s.dGi[q];
      __syncthreads();
      // ---- 5. MLP on every atom (calc_new_runner_energy!, src/EnergyEvaluation.jl:1269-1275)
      if constexpr (sizeof(Real) == 4) {
        int bad = 0;
        new_en = mlp_energy_tc(s, tc.m, N, S, Q.H1, Q.H2, true, tbase, tc.mph, &bad);
        if (bad) {
          status = ST_TIMEOUT;
          break;
        }
      } else {
        new_en = mlp_energy<Real>(Q, s, N, true);
      }
    }
    // ---- training record of this exact move (proposal rows and exact dE)
    if (Q.rec_rows && !hard) {
      const long long m = (rd->cyc[phase]) * (long long)N + step;
      if (m % Q.rec_every == 0) {
        if (tid == 0) s.flags[2] = (int)(atomicAdd(Q.rec_n, 1ull) % (unsigned long long)Q.rec_cap);
        __syncthreads();
        const size_t at = (size_t)s.flags[2];
        if (tid < SUR_ROWS) {
          const int j = tid & (SUR_ROWS / 2 - 1);
          float r = -1.f;
          if (j < N && j != i) r = (float)(tid < SUR_ROWS / 2 ? rn[j] : ro[j]);
          Q.rec_rows[at * SUR_ROWS + tid] = r;
        }
        if (tid == 0) {
          Q.rec_y[at] = (float)((double)new_en - en);
          Q.rec_slot[at] = slot;
        }
      }
    }
    // ---- 6. Metropolis (src/MCRun.jl:122-132) and commit (swap_vars!, swap_config.jl:213-221);
    // with delayed acceptance this is the second stage, exp(-beta (dE - dE_s))
    if (warp == 0) {
      const double x = -(((double)new_en - en) - dEs) * beta;
      double prob;
      if constexpr (sizeof(Real) == 4) {  // FP32 form: MUFU exp, as the pair kernels
        prob = (double)ex2f(fminf((float)x, 0.f) * 1.4426950408889634f);
      } else {
        prob = exp(x);
        if (prob > 1) prob = 1.0;
      }
      double u = draw();
      if (lane == 0) s.flags[3] = (prob >= u) ? 1 : 0;
    }
    __syncthreads();
    // commit on acceptance: warp 0 moves the atom and goes on to the next
    // proposal (which reads positions only) while warps 1-7 update the distance
    // and cut-off rows and G; the next proposal's barrier orders both before
    // any use.  flags[3] is written only here, by the Metropolis step.
    if (s.flags[3]) {
      if (warp == 0) {
        if (lane == 0)
          for (int k = 0; k < 3; ++k) {
            s.Xd[3 * i + k] = s.tpos[k];
            s.X[3 * i + k] = (Real)s.tpos[k];
          }
        __syncwarp();
      } else {
        const int ct = tid - 32, cn = NN_THREADS - 32;
        for (int j = ct; j < N; j += cn) {
          Real d = d2n[j];
          s.D2[i * ld + j] = d;
          s.D2[j * ld + i] = d;
          if (!hard) {  // the hard-core branch computes no new cut-off row or G
            Real f = fn[j];
            s.F[i * ld + j] = f;
            s.F[j * ld + i] = f;
          }
        }
        if (!hard)
          for (int t = ct; t < S * N; t += cn) s.G[t] += s.dG[t];
      }
      en = (double)new_en;
      ++acc;
    }
  }
  __syncthreads();
  // store back
  for (int k = tid; k < 3 * N; k += blockDim.x) Xg[k] = s.Xd[k];
  for (int t = tid; t < S * N; t += blockDim.x) Gg[t] = (double)s.G[t];
  if (tid == 0) {
    P.en[g] = en;
    P.status[g] = status;
    P.cnt[6 * (size_t)gs + 0] += acc;
    P.cnt[6 * (size_t)gs + 1] += acc;
    if (Q.da) {
      Q.da_cnt[2 * (size_t)g] += n_rej1;
      Q.da_cnt[2 * (size_t)g + 1] += n_exact;
    }
  }
  if (warp == 0 && lane == 0) P.ctr[g] = ctr;
  tc_teardown(tc);  // free the tensor memory (every path out of the move loop comes here)
}

// --------------------------------------------------------------- run epilogue
// After every walker finished its cycle: exchange (src/Exchange.jl:132-154),
// step adaptation (src/Exchange.jl:250-257) and sampling (src/Sampling.jl:330-371)
// of one run, on global slot tables.  One CTA per run, one thread per slot.
__global__ void k_run_epilogue(KParams P, NNParams Q, int run0, int phase) {
  RunDesc* rd = P.runs + run0 + blockIdx.x;
  const int R = rd->R, N = rd->N, wk = rd->wk, s = threadIdx.x;
  const long long idx = rd->cyc[phase];
  const uint32_t run_word = (uint32_t)rd->run_id;
  if (s == 0 && R > 1) {
    unsigned long long rc = rd->run_ctr;
    double u = philox_u01(P.seed, 0xFFFFFFFFu, run_word, rc++);
    if (u < P.exch_prob) {
      int k = randint(philox_u01(P.seed, 0xFFFFFFFFu, run_word, rc++), R - 1);
      P.cnt[6 * (size_t)(wk + k) + 4] += 1;
      P.cnt[6 * (size_t)(wk + k + 1) + 4] += 1;
      int w1 = P.wos[wk + k], w2 = P.wos[wk + k + 1];
      double e1 = P.en[wk + w1], e2 = P.en[wk + w2];
      double a = exp((P.beta[wk + k] - P.beta[wk + k + 1]) * (e1 - e2));
      if (a > 1.0) a = 1.0;
      if (a > philox_u01(P.seed, 0xFFFFFFFFu, run_word, rc++)) {
        P.cnt[6 * (size_t)(wk + k) + 5] += 1;
        P.cnt[6 * (size_t)(wk + k + 1) + 5] += 1;
        P.wos[wk + k] = w2;
        P.wos[wk + k + 1] = w1;
        Q.sow[wk + w2] = k;
        Q.sow[wk + w1] = k + 1;
      }
    }
    rd->run_ctr = rc;
  }
  __syncthreads();
  if (s < R) {
    const int gs = wk + s;
    if (idx % P.n_adjust == 0) {
      double acc = (double)P.cnt[6 * (size_t)gs + 1] / (double)((long long)P.n_adjust * N);
      if (acc < P.min_acc) P.maxd[2 * gs] *= 0.9;
      else if (acc > P.max_acc) P.maxd[2 * gs] *= 1.1;
      P.cnt[6 * (size_t)gs + 1] = 0;
    }
    if (phase == PHASE_PROD && idx % P.mc_sample == 0) {
      const double e = P.en[wk + P.wos[gs]];
      P.ham[2 * gs] += e;
      P.ham[2 * gs + 1] = dadd(P.ham[2 * gs + 1], dmul(e, e));
      const int nb = P.n_bin;
      double h = (e - rd->en_min) / rd->dE + 1;
      int ie = !(h >= 1) ? 1 : (h > nb ? nb + 2 : (int)floor(h) + 1);
      atomicAdd(P.hist + rd->hist_off + (size_t)s * rd->hist_stride + (ie - 1), 1u);
    }
  }
  __syncthreads();
  if (P.rdf && phase == PHASE_PROD && idx % P.mc_sample == 0 && idx % RDF_EVERY == 0) {
    // update_rdf! (src/Sampling.jl:301-316): every slot's walker, pairs k < i
    for (int sl = 0; sl < R; ++sl) {
      const double* X = P.pos + rd->pos_off + (size_t)P.wos[wk + sl] * N * 3;
      unsigned int* row = P.rdf + (size_t)(wk + sl) * 5 * P.n_bin;
      for (int p = threadIdx.x; p < N * N; p += blockDim.x) {
        const int i = p / N, k = p % N;
        if (k >= i) continue;
        rdf_add(row, 5 * P.n_bin,
                d2_sph(X[3 * i], X[3 * i + 1], X[3 * i + 2], X[3 * k], X[3 * k + 1], X[3 * k + 2]),
                rd->dr2);
      }
    }
  }
  __syncthreads();
  if (s == 0) rd->cyc[phase] = idx + 1;
}

// --------------------------------------------------------------- launchers
size_t nn_smem_bytes(const NNParams& Q, int N, bool f64) {
  size_t es = f64 ? 8 : 4;
  auto al = [](size_t b) { return (b + 15) / 16 * 16; };
  size_t b = 0;
  const size_t ld = (size_t)N + (N & 1);
  b += al(8 * N * 3) + al(es * N * 3) + 2 * al(es * N * ld) + 2 * al(es * Q.S * N);
  if (f64) b += al(es * NCH * (Q.SA > 0 ? Q.SA : 1) * 64);
  b += al(es * 8 * 64) + 2 * al(es * 64 * 3);
  if (f64) b += al(es * Q.nW) + al(es * N * Q.H1) + al(es * N * Q.H2);
  b += al(es * 64) + al(es * (Q.S > 0 ? Q.S : 1));
  b += al(es * 4 * MAX_NN_ANG);
  b += al(8 * DRAW_BUF) + al(8 * 4) + al(4 * 4);
  if (!f64) b += 3 * al(16 * 64) + al(4 * MAX_NN_ANG);  // packed rows, tpz
  b += 128;                                 // alignment of the tensor-core tiles
  if (!f64) b += MLP_TC_BYTES;              // FP32 form: tensor-core MLP tiles
  return b;
}

template <typename K>
static int set_smem(K kern, size_t smem) {
  if (smem <= 48 * 1024) return 0;
  int dev = 0, optin = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  cudaFuncAttributes fa;
  cudaError_t e = cudaFuncGetAttributes(&fa, kern);
  if (e != cudaSuccess) return (int)e;
  if ((long long)smem + (long long)fa.sharedSizeBytes > optin) return (int)cudaErrorInvalidValue;
  return (int)cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

int nn_launch_init(const KParams& P, const NNParams& Q, int n_walkers, int maxN, bool f64,
                   void* stream) {
  size_t smem = nn_smem_bytes(Q, maxN, f64);
  cudaStream_t st = (cudaStream_t)stream;
  int e;
  if (f64) {
    if ((e = set_smem(k_nn_init<double>, smem))) return e;
    k_nn_init<double><<<n_walkers, NN_THREADS, smem, st>>>(P, Q);
  } else {
    if ((e = set_smem(k_nn_init<float>, smem))) return e;
    k_nn_init<float><<<n_walkers, NN_THREADS, smem, st>>>(P, Q);
  }
  return (int)cudaGetLastError();
}

int nn_launch_cycle(const KParams& P, const NNParams& Q, int n_walkers, int n_runs, int R,
                    int maxN, bool f64, int phase, void* stream) {
  size_t smem = nn_smem_bytes(Q, maxN, f64);
  cudaStream_t st = (cudaStream_t)stream;
  int e;
  if (f64) {
    if ((e = set_smem(k_nn_cycle<double, NN_PAT_GENERIC>, smem))) return e;
    k_nn_cycle<double, NN_PAT_GENERIC><<<n_walkers, NN_THREADS, smem, st>>>(P, Q, phase);
  } else {
    if (Q.ang_pat == NN_PAT_CU55) {
      if ((e = set_smem(k_nn_cycle<float, NN_PAT_CU55>, smem))) return e;
      k_nn_cycle<float, NN_PAT_CU55><<<n_walkers, NN_THREADS, smem, st>>>(P, Q, phase);
    } else {
      if ((e = set_smem(k_nn_cycle<float, NN_PAT_GENERIC>, smem))) return e;
      k_nn_cycle<float, NN_PAT_GENERIC><<<n_walkers, NN_THREADS, smem, st>>>(P, Q, phase);
    }
  }
  if ((e = (int)cudaGetLastError())) return e;
  k_run_epilogue<<<n_runs, ((R + 31) / 32) * 32, 0, st>>>(P, Q, 0, phase);
  return (int)cudaGetLastError();
}

int nn_launch_epilogue(const KParams& P, const NNParams& Q, int n_runs, int R, int phase,
                       void* stream) {
  k_run_epilogue<<<n_runs, ((R + 31) / 32) * 32, 0, (cudaStream_t)stream>>>(P, Q, 0, phase);
  return (int)cudaGetLastError();
}

}  // namespace ptmc
