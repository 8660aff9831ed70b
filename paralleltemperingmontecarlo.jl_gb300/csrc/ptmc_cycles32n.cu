// ptmc_cycles32n.cu — replica-cycle kernel of the FP32_RESYNC form with 4 or
// 8 lanes per walker (NVT: the pair potentials and EAM, sphere or cube).
//
// The arithmetic of a move is the FP32_RESYNC form's (ptmc_cycles32.cu):
// float-float positions, FP32 pair terms on hi, MUFU Metropolis, the FP64
// running total absorbing the FP32 dE once per cycle, an FP64 recompute every
// `resync_every` cycles.  What changes is how a warp is spent:
//
//  * A warp holds 32 / LPR walkers.  The N - 1 pair terms of a move are spread
//    over the walker's LPR lanes (Cu55: 14 per lane at LPR = 4), so the scalar
//    work of a move — slot draw, proposal, float-float steps, Metropolis,
//    commit — is issued once for 8 (or 4) walkers instead of once per walker,
//    and the pair sums need 2 (3) shuffle levels instead of 5.  The walkers of
//    a warp make their moves in lockstep (same N, same step count); they
//    diverge only on accept vs reject and on the rare spherical retry.
//  * The pair and commit loops are unrolled (at most JPL terms per lane,
//    N <= 64) in chunks of NARROW_CH terms under one warp-uniform test each;
//    inside a chunk the terms carry no branch, so the compiler overlaps their
//    MUFU and shared-memory chains, and the EAM density deltas stay in
//    registers.
//  * Shared memory per walker is small, so more walkers share an SM: FP32 hi
//    positions (float4, the EAM density rho in w; padded with far-away
//    sentinel atoms to whole chunks) and 32 buffered draw words.  sqrt(rho_j)
//    of the embedding term is taken per pair (one MUFU op) rather than kept
//    per atom: at Cu55 the 8.7 KB it took per 32 walkers decided between 4
//    and 5 CTAs per SM.  The lo halves of the float-float positions are touched only by
//    the moved atom's proposal and commit, so they live in HBM (L2): one
//    16-byte load per move, issued one move ahead.
//  * Draw words are refilled for the whole warp at once (when any walker needs
//    words at the start of a step): a refill re-creates a walker's buffer from
//    its stream index, so an early refill changes no draw.
//  * One CTA per run (R * LPR threads); the cycle end (exchange, step
//    adaptation, sampling) is the barrier form of ptmc_cycles32.cu.
//
// The walker draw streams are those of the FP32 form (word k of walker w of
// the run), so a chain differs from the 16/32-lane form only by the order in
// which FP32 pair terms are added.
#include <cuda_runtime.h>

#include <type_traits>

#include "ptmc_device.cuh"
#include "ptmc_engine.cuh"
#include "ptmc_fp32.cuh"

namespace ptmc {

namespace {
using namespace f32k;

// draw words buffered per walker (a refill is DRWN / 4 Philox blocks)
constexpr uint32_t DRWN = 32;
// pair terms per unrolled chunk
constexpr int CH = NARROW_CH;
// a position no atom comes near: a pair with it has r^2 ~ 3e36, whose FP32
// ELJ and EAM terms (r^-6 and beyond; r^-n, r^-m) underflow to exactly zero
constexpr float FAR = 1.0e18f;

// JPL: pair terms per lane at most (N <= JPL * LPR = 64).
// At most 32 walkers (R * LPR threads).  The register cap keeps, for 32
// walkers per CTA, 4 CTAs per SM with EAM at LPR = 4 (128 registers; its
// shared memory allows no more) and 3 at LPR = 8 (80 registers), and 8 / 4
// CTAs (64 registers) with the pair potentials, whose small-N runs need
// little shared memory and gain from more resident warps.
template <int POT, int BC, int LPR, int JPL>
__global__ void __launch_bounds__(32 * LPR, POT == POT_EAM ? (LPR == 4 ? 5 : 3) : (LPR == 4 ? 7 : 4))
    k_cycles32n(KParams P, int run0, int ncycles, int phase) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ double s_c[MAX_COEFF];
  __shared__ float s_cf[MAX_COEFF];
  const RunDesc* rdp = P.runs + run0 + blockIdx.x;
  const int N = rdp->N, R = rdp->R;
  const int Ns = narrow_stride(N, LPR);
  const int tid = threadIdx.x, lane = tid & (LPR - 1);
  const int w = tid / LPR;  // walker within the run
  const unsigned gmask = ((1u << LPR) - 1u) << ((tid & 31) & ~(LPR - 1));
  const int nthr = blockDim.x;
  const int K = P.K;

  unsigned char* sp = smem_raw;
  auto carve = [&](long long bytes) {
    unsigned char* p = sp;
    sp += (bytes + 15) / 16 * 16;
    return p;
  };
  // order and sizes as in cycles32n_smem_bytes
  float4* s_xh = (float4*)carve((long long)R * Ns * 16);
  uint32_t* s_drw = (uint32_t*)carve((long long)R * DRWN * 4);
  double* s_beta = (double*)carve((long long)R * 8);
  double* s_en = (double*)carve((long long)R * 8);
  double* s_ham = (double*)carve((long long)R * 16);
  double* s_maxd = (double*)carve((long long)R * 16);
  long long* s_cnt = (long long*)carve((long long)R * 48);
  int* s_wos = (int*)carve((long long)R * 4);
  int* s_sow = (int*)carve((long long)R * 4);
  float* s_bl2e = (float*)carve((long long)R * 4);  // beta * log2(e) per slot
  float* s_mdf = (float*)carve((long long)R * 4);   // atom step size per slot
  float* s_mdc = (float*)carve((long long)R * 4);   // its step offset md (3/2 - 2^-24)
  int* s_acc = (int*)carve((long long)R * 4);       // this cycle's accepted moves per walker

  if (tid < K) {
    s_c[tid] = P.c[tid];
    s_cf[tid] = (float)P.c[tid];
  }
  const double* gpos = P.pos + rdp->pos_off;
  float4* glo = (float4*)P.lo + rdp->pos_off / 3;  // lo halves, walker-major, N per walker
  for (int k = tid; k < R * N; k += nthr) {
    const int v = k / N, a = k - v * N;
    const double x = gpos[3 * k], y = gpos[3 * k + 1], z = gpos[3 * k + 2];
    const float4 h = make_float4((float)x, (float)y, (float)z, 0.f);
    s_xh[v * Ns + a] = h;
    glo[k] = make_float4((float)(x - (double)h.x), (float)(y - (double)h.y),
                         (float)(z - (double)h.z), 0.f);
  }
  // the pad atoms N .. Ns - 1 of every walker are far-away sentinels (their
  // pair terms are zero; EAM density and its root 1 keep the embedding term
  // of a zero delta finite)
  for (int k = tid; k < R * (Ns - N); k += nthr) {
    const int v = k / (Ns - N), a = N + (k - v * (Ns - N));
    s_xh[v * Ns + a] = make_float4(FAR, FAR, FAR, 1.f);
  }
  if (POT == POT_EAM) {
    const double* gc = P.comp + rdp->comp_off;
    __syncthreads();
    for (int k = tid; k < R * N; k += nthr) {  // rho in the w lane of the position
      const int v = k / N, a = k - v * N;
      s_xh[v * Ns + a].w = (float)gc[2 * k + 1];
    }
  }
  const int wk0 = rdp->wk;
  for (int s = tid; s < R; s += nthr) {
    const int g = wk0 + s;
    s_beta[s] = P.beta[g];
    s_ham[2 * s] = P.ham[2 * g];
    s_ham[2 * s + 1] = P.ham[2 * g + 1];
    s_maxd[2 * s] = P.maxd[2 * g];
    s_maxd[2 * s + 1] = P.maxd[2 * g + 1];
    for (int k = 0; k < 6; ++k) s_cnt[6 * s + k] = P.cnt[6 * (size_t)g + k];
    s_wos[s] = P.wos[g];
    s_bl2e[s] = (float)(P.beta[g] * 1.4426950408889634);
    s_mdf[s] = (float)P.maxd[2 * g];
    s_mdc[s] = (float)(P.maxd[2 * g] * (1.5 - 0x1.0p-24));
  }
  __syncthreads();
  for (int s = tid; s < R; s += nthr) s_sow[s_wos[s]] = s;
  __syncthreads();

  const int g = wk0 + w;
  double en = P.en[g];
  double L = P.box[g];
  const double rc2 = P.rc2[g];
  // draw words: drw[k] is word `base + k` of this walker's stream; `off` is
  // the next one (>= DRWN: refill from the 4-aligned word at base + off)
  unsigned long long base = (P.ctr[g] & ~3ull) - DRWN;
  uint32_t off = DRWN + (uint32_t)(P.ctr[g] & 3ull);
  int status = P.status[g];
  double drift = P.drift[g];
  float4* Xh = s_xh + (size_t)w * Ns;
  float4* Xl = glo + (size_t)w * N;
  uint32_t* drw = s_drw + w * DRWN;
  const double hn = -0.5 * P.eam_n, hm = -0.5 * P.eam_m;
  const float hnf = P.f_hn, hmf = P.f_hm, ecamf = P.f_ecam;
  const float ean2f = 2.f * P.f_ean, necamf = -P.f_ecam;
  const uint32_t run_word = (uint32_t)rdp->run_id;
  const float Lf = (float)L, Llo = (float)(L - (double)Lf), iLf = __frcp_rn(Lf);
  // pair-term chunks per lane: warp-uniform
  const int qmax = (N + LPR - 1) / LPR;

  // refill of this walker's buffer by its own lanes (spherical retries)
  auto refill = [&]() {
    __syncwarp(gmask);
    base += off & ~3u;
    off &= 3u;
    for (int bl = lane; bl < (int)DRWN / 4; bl += LPR) {
      const uint64_t blk = (base >> 2) + bl;
      uint32_t c4[4] = {(uint32_t)blk, (uint32_t)(blk >> 32), (uint32_t)w, run_word};
      philox4x32_10(c4, (uint32_t)P.seed, (uint32_t)(P.seed >> 32));
      *(uint4*)(drw + 4 * bl) = make_uint4(c4[0], c4[1], c4[2], c4[3]);
    }
    __syncwarp(gmask);
  };
  auto word = [&]() -> uint32_t {
    if (off >= DRWN) refill();
    return drw[off++];
  };
  auto ensure = [&](uint32_t n) {
    if (off > DRWN - n) refill();
  };
  auto word_nc = [&]() -> uint32_t { return drw[off++]; };

  // ---------------------------------------------------------- atom move
  // l0: the lo half of atom i (from the prefetch register or a load)
  int kpre = -1;  // atom whose lo half is in lpre (-1: none)
  float4 lpre = make_float4(0.f, 0.f, 0.f, 0.f);
  auto atom_move = [&](int i, float4 l0, float beta_l2e, float mdf, float mdc,
                       float& de_acc) -> int {
    float4 h0 = Xh[i];
    float th[3], tl[3];
    auto propose = [&]() {  // the first attempt's words are ensured by the caller
      const float d0 = stepf(word_nc(), mdf, mdc), d1 = stepf(word_nc(), mdf, mdc),
                  d2 = stepf(word_nc(), mdf, mdc);
      th[0] = h0.x; tl[0] = l0.x; ff_add(th[0], tl[0], d0);
      th[1] = h0.y; tl[1] = l0.y; ff_add(th[1], tl[1], d1);
      th[2] = h0.z; tl[2] = l0.z; ff_add(th[2], tl[2], d2);
    };
    propose();
    if (BC == BC_SPH) {
      const float R2 = Lf * Lf;
      int count = 0;
      while (fmaf(th[0], th[0], fmaf(th[1], th[1], th[2] * th[2])) > R2) {
        ++count;
        if (count == 50) {  // recentre! (src/Configurations.jl:79-85), in FP64
          double sx = 0, sy = 0, sz = 0;
          for (int a = lane; a < N; a += LPR) {
            const float4 h = Xh[a], l = Xl[a];
            sx += (double)h.x + l.x;
            sy += (double)h.y + l.y;
            sz += (double)h.z + l.z;
          }
          sx = seg_sum<LPR>(sx, gmask) / N;
          sy = seg_sum<LPR>(sy, gmask) / N;
          sz = seg_sum<LPR>(sz, gmask) / N;
          __syncwarp(gmask);
          for (int a = lane; a < N; a += LPR) {
            const float4 hh = Xh[a], ll = Xl[a];
            const double x = (double)hh.x + ll.x - sx, y = (double)hh.y + ll.y - sy,
                         z = (double)hh.z + ll.z - sz;
            const float4 h = make_float4((float)x, (float)y, (float)z, hh.w);
            Xh[a] = h;
            Xl[a] = make_float4((float)(x - h.x), (float)(y - h.y), (float)(z - h.z), 0.f);
          }
          __syncwarp(gmask);
          h0 = Xh[i];
          l0 = Xl[i];
          kpre = -1;  // every lo half moved
        } else {
          ensure(3);
          propose();
          if (count == 100) {
            status = ST_SPHERE;
            return 0;
          }
        }
      }
    } else {  // periodic wrap t -= L * round(t / L)
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const float m = rint_mul(th[k], iLf);
        if (m != 0.f) {
          ff_add(th[k], tl[k], -m * Lf);
          ff_add(th[k], tl[k], -m * Llo);
        }
      }
    }
    const float4 tf = make_float4(th[0], th[1], th[2], 0.f);
    const float4 x4 = h0;
    // Spherical container: during the pair loop atom i itself is a far-away
    // sentinel, so its pair term, like the pad atoms', is exactly zero and no
    // term needs a mask.  A periodic box would fold the sentinel back into the
    // box by the minimum image, so the cube masks the self pair and the pads.
    constexpr bool SENT = BC == BC_SPH;
    const int own = i & (LPR - 1);  // the lane that holds atom i in the loops
    if (SENT) {
      __syncwarp(gmask);  // every lane has read atom i
      if (lane == own) Xh[i] = make_float4(FAR, FAR, FAR, 1.f);
      __syncwarp(gmask);
    }
    float de = 0.f, sbf = 0.f;
    float dreg[POT == POT_EAM ? JPL : 1];  // this lane's density deltas db_j
    if (POT == POT_EAM) {
      // the phi part of dE is 2 ean sum_j da (the pair changes phi_i and phi_j
      // alike); rho_j is the w lane of atom j's position
      auto term = [&](int c, int u) {
        const int j = lane + (c + u) * LPR;
        const float4 b = Xh[j];
        const float ln_ = lg2f(pf2<BC>(tf, b, Lf, iLf));
        const float lo_ = lg2f(pf2<BC>(x4, b, Lf, iLf));
        float da = ex2f(hnf * ln_) - ex2f(hnf * lo_);
        float db = ex2f(hmf * ln_) - ex2f(hmf * lo_);
        if (!SENT) {  // the self pair (zero old distance) and the pads
          const bool skip = j == i || j >= N;
          da = skip ? 0.f : da;
          db = skip ? 0.f : db;
        }
        dreg[c + u] = db;
        sbf += db;
        // sqrt(rho + db) - sqrt(rho) in the cancellation-free form
        de = fmaf(ean2f, da, de);
        de = fmaf(necamf * db, rcpf(sqrtf_approx(b.w) + sqrtf_approx(b.w + db)), de);
      };
      // whole chunks without a test per term; the last, partial chunk tests
      // each term against qmax (the same for every lane of the warp), so the
      // pad terms beyond it (exactly zero) are not evaluated
#pragma unroll
      for (int c = 0; c < JPL; c += CH) {
        if (c + CH <= qmax) {
#pragma unroll
          for (int u = 0; u < CH; ++u) term(c, u);
        } else if (c < qmax) {
#pragma unroll
          for (int u = 0; u < CH; ++u)
            if (c + u < qmax) term(c, u);
        }
      }
      sbf = seg_sum<LPR>(sbf, gmask);
      de = seg_sum<LPR>(de, gmask);
      de -= ecamf * sbf * rcpf(sqrtf_approx(x4.w) + sqrtf_approx(x4.w + sbf));
    } else {
      // ELJ pair terms with the coefficient count as a compile-time constant
      // (the neon coefficients have 6) or a runtime loop
      auto rows = [&](auto kk) {
        constexpr int KK = decltype(kk)::value;
        auto v = [&](float r2) -> float {
          float x, s3;
          if (POT == POT_ELJ) {
            const float ir = rsqrtf(r2);
            const float inv = ir * ir;
            x = ir;
            s3 = inv * inv * inv;
          } else {
            const float inv = rcpf(r2);
            x = inv;
            s3 = inv * inv * inv;
          }
          float p;
          if constexpr (KK > 0) {
            p = horner_p<KK>(P, x);
          } else {
            p = s_cf[K - 1];
            for (int k = K - 2; k >= 0; --k) p = fmaf(p, x, s_cf[k]);
          }
          return __fmul_rn(p, s3);  // rounded as in v32p of the 16/32-lane kernel
        };
        // whole chunks only (a partial last chunk, as in the EAM loop, made the
        // Ne13 kernel slower: its 13 atoms fill one chunk of 4 terms per lane)
#pragma unroll
        for (int c = 0; c < JPL; c += CH) {
          if (c < qmax) {
#pragma unroll
            for (int u = 0; u < CH; ++u) {
              const int j = lane + (c + u) * LPR;
              const float4 b = Xh[j];
              const float t = __fsub_rn(v(pf2<BC>(tf, b, Lf, iLf)), v(pf2<BC>(x4, b, Lf, iLf)));
              if (SENT) de += t;
              else de += (j == i || j >= N) ? 0.f : t;
            }
          }
        }
      };
      if (K == 6) rows(std::integral_constant<int, 6>{});
      else rows(std::integral_constant<int, 0>{});
      de = seg_sum<LPR>(de, gmask);
    }
    const float u = u01f(word());
    if (!(ex2f(-beta_l2e * de) >= u)) {
      if (SENT && lane == own) Xh[i] = h0;  // rejected: atom i back in place
      return 0;
    }
    __syncwarp(gmask);
    if (POT == POT_EAM) {
      // density deltas of every slot up to the lane's term count, without a
      // test per slot: the pads and atom i itself (a sentinel during the pair
      // loop, or masked in the cube) carry an exact zero, and atom i's record
      // is written after a warp barrier
#pragma unroll
      for (int c = 0; c < JPL; c += CH) {
        if (c + CH <= qmax) {
#pragma unroll
          for (int u = 0; u < CH; ++u) Xh[lane + (c + u) * LPR].w += dreg[c + u];
        } else if (c < qmax) {
#pragma unroll
          for (int u = 0; u < CH; ++u)
            if (c + u < qmax) Xh[lane + (c + u) * LPR].w += dreg[c + u];
        }
      }
      __syncwarp(gmask);
    }
    if (lane == 0) {
      const float rho_i = POT == POT_EAM ? x4.w + sbf : 0.f;
      Xh[i] = make_float4(tf.x, tf.y, tf.z, rho_i);
      Xl[i] = make_float4(tl[0], tl[1], tl[2], 0.f);
    }
    de_acc += de;
    __syncwarp(gmask);
    return 1;
  };

  // ---------------------------------------------------------- cycle end
  // update_max_stepsize! and sampling_step! of slot s, whose walker ended the
  // cycle with energy e (one thread per slot)
  auto slot_epilogue = [&](int s, long long idx, double e) {
    if (idx % P.n_adjust == 0) {  // update_max_stepsize! (src/Exchange.jl:250-257)
      const double acc = (double)s_cnt[6 * s + 1] / (double)((long long)P.n_adjust * N);
      if (acc < P.min_acc) s_maxd[2 * s] *= 0.9;
      else if (acc > P.max_acc) s_maxd[2 * s] *= 1.1;
      s_mdf[s] = (float)s_maxd[2 * s];
      s_mdc[s] = (float)(s_maxd[2 * s] * (1.5 - 0x1.0p-24));
      s_cnt[6 * s + 1] = 0;
    }
    if (phase == PHASE_PROD && idx % P.mc_sample == 0) {  // sampling_step! (src/Sampling.jl:330-371)
      const int nb = P.n_bin;
      unsigned int* hrow = P.hist + rdp->hist_off + (size_t)s * rdp->hist_stride;
      s_ham[2 * s] += e;
      s_ham[2 * s + 1] += e * e;
      const double h = (e - rdp->en_min) / rdp->dE + 1;
      const int ie = !(h >= 1) ? 1 : h > nb ? nb + 2 : (int)floor(h) + 1;
      atomicAdd(hrow + (ie - 1), 1u);
    }
  };

  // ---------------------------------------------------------- cycles
  const long long first = rdp->cyc[phase];
  unsigned long long run_ctr = rdp->run_ctr;
  for (int cyc = 0; cyc < ncycles; ++cyc) {
    const long long idx = first + cyc;
    const int slot = s_sow[w];
    const float beta_l2e = s_bl2e[slot];
    const float mdf = s_mdf[slot], mdc = s_mdc[slot];
    int acc_a = 0;
    float de_acc = 0.f;
    kpre = -1;
    for (int st = 0; st < N; ++st) {
      // every walker of the warp is at the same step: one refill decision for
      // the warp (slot draw, three displacements, acceptance: 5 words)
      __syncwarp();
      if (__any_sync(0xffffffffu, off > DRWN - 5)) {
        base += off & ~3u;
        off &= 3u;
        for (int bl = lane; bl < (int)DRWN / 4; bl += LPR) {
          const uint64_t blk = (base >> 2) + bl;
          uint32_t c4[4] = {(uint32_t)blk, (uint32_t)(blk >> 32), (uint32_t)w, run_word};
          philox4x32_10(c4, (uint32_t)P.seed, (uint32_t)(P.seed >> 32));
          *(uint4*)(drw + 4 * bl) = make_uint4(c4[0], c4[1], c4[2], c4[3]);
        }
        __syncwarp();
      }
      if (status == ST_OK) {
        const int k = (int)__umulhi(word_nc(), (uint32_t)N);  // rand(1:N)
        const float4 l0 = k == kpre ? lpre : Xl[k];
        // The lo halves live in L2: the load for the next move's atom is
        // issued now, from the slot word that follows this move's three
        // displacements and acceptance draw (the next slot word unless a
        // spherical retry draws more; a refill re-creates the same word).
        kpre = -1;
        if (off + 4 < DRWN) {
          kpre = (int)__umulhi(drw[off + 4], (uint32_t)N);
          lpre = Xl[kpre];
        }
        const int a = atom_move(k, l0, beta_l2e, mdf, mdc, de_acc);
        if (a && kpre == k) kpre = -1;  // the prefetched lo half was just replaced
        acc_a += a;
      }
    }
    en += (double)de_acc;
    if (status == ST_OK && P.resync_every > 0 && idx % P.resync_every == 0) {
      // EAM: the recomputed densities are staged in the w lanes of the lo
      // halves (unused otherwise)
      const double e64 = energy64<POT, BC, ENS_NVT, LPR>(
          Xh, Xl, N, L, rc2, s_c, K, hn, hm, P.eam_ean, P.eam_ecam,
          POT == POT_EAM ? &Xl[0].w : nullptr, nullptr, lane, gmask, 4);
      drift = fmax(drift, fabs(en - e64));
      en = e64;
      __syncwarp(gmask);
    }
    // barrier form of the cycle end: counters of the slot each walker
    // occupied, then the exchange (thread 0), then the slots' epilogues
    if (lane == 0) {
      s_en[w] = en;
      s_acc[w] = acc_a;
    }
    __syncthreads();
    for (int v = tid; v < R; v += nthr) {
      const int sl = s_sow[v];
      s_cnt[6 * sl + 0] += s_acc[v];
      s_cnt[6 * sl + 1] += s_acc[v];
    }
    __syncthreads();
    if (tid == 0 && R > 1) {  // parallel_tempering_exchange! (src/Exchange.jl:132-154)
      const double u = philox_u01(P.seed, 0xFFFFFFFFu, run_word, run_ctr++);
      if (u < P.exch_prob) {
        const int k = randint(philox_u01(P.seed, 0xFFFFFFFFu, run_word, run_ctr++), R - 1);
        s_cnt[6 * k + 4] += 1;
        s_cnt[6 * (k + 1) + 4] += 1;
        const int w1 = s_wos[k], w2 = s_wos[k + 1];
        const double acc = exch_acc(s_beta[k], s_beta[k + 1], s_en[w1], s_en[w2], 0.0, 0.0, 0.0);
        if (acc > philox_u01(P.seed, 0xFFFFFFFFu, run_word, run_ctr++)) {
          s_cnt[6 * k + 5] += 1;
          s_cnt[6 * (k + 1) + 5] += 1;
          s_wos[k] = w2;
          s_wos[k + 1] = w1;
          s_sow[w2] = k;
          s_sow[w1] = k + 1;
        }
      }
    }
    __syncthreads();
    if (tid < R) slot_epilogue(tid, idx, s_en[s_wos[tid]]);
    __syncthreads();
    if (P.rdf && phase == PHASE_PROD && idx % P.mc_sample == 0 && idx % RDF_EVERY == 0) {
      // update_rdf! (src/Sampling.jl:301-316) from the FP32 positions
      unsigned int* row = P.rdf + (size_t)(wk0 + s_sow[w]) * 5 * P.n_bin;
      for (int i = 1; i < N; ++i)
        for (int k = lane; k < i; k += LPR)
          rdf_add(row, 5 * P.n_bin, (double)pf2<BC>(Xh[i], Xh[k], Lf, iLf), rdp->dr2);
    }
  }

  double* gpos_w = P.pos + rdp->pos_off;
  for (int k = tid; k < R * N; k += nthr) {
    const int v = k / N, a = k - v * N;
    const float4 h = s_xh[v * Ns + a], l = glo[k];
    gpos_w[3 * k] = (double)h.x + (double)l.x;
    gpos_w[3 * k + 1] = (double)h.y + (double)l.y;
    gpos_w[3 * k + 2] = (double)h.z + (double)l.z;
  }
  if (POT == POT_EAM) {
    double* gc = P.comp + rdp->comp_off;
    for (int k = tid; k < R * N; k += nthr) {
      const int v = k / N, a = k - v * N;
      gc[2 * k + 1] = s_xh[v * Ns + a].w;  // rho; the FP32 form keeps no phi
    }
  }
  if (lane == 0) {
    P.en[g] = en;
    P.ctr[g] = base + off;
    P.status[g] = status;
    P.drift[g] = drift;
  }
  for (int s = tid; s < R; s += nthr) {
    const int gs = wk0 + s;
    P.ham[2 * gs] = s_ham[2 * s];
    P.ham[2 * gs + 1] = s_ham[2 * s + 1];
    P.maxd[2 * gs] = s_maxd[2 * s];
    P.maxd[2 * gs + 1] = s_maxd[2 * s + 1];
    for (int k = 0; k < 6; ++k) P.cnt[6 * (size_t)gs + k] = s_cnt[6 * s + k];
    P.wos[gs] = s_wos[s];
  }
  __syncthreads();  // every thread has read the run descriptor
  if (tid == 0) {
    P.runs[run0 + blockIdx.x].cyc[phase] = first + ncycles;
    P.runs[run0 + blockIdx.x].run_ctr = run_ctr;
  }
}

// shared-memory opt-in, per instantiation and per device; only ever raised
template <int POT, int BC, int LPR, int JPL>
int opt_in_n(long long smem) {
  static long long attr_set[MAX_DEVICES] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return (int)e;
  if (dev < 0 || dev >= MAX_DEVICES) return (int)cudaErrorInvalidDevice;
  if (smem > 48 * 1024 && smem > attr_set[dev]) {
    int optin = 0;
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaFuncAttributes fa;
    e = cudaFuncGetAttributes(&fa, k_cycles32n<POT, BC, LPR, JPL>);
    if (e != cudaSuccess) return (int)e;
    if (smem + (long long)fa.sharedSizeBytes > optin) return (int)cudaErrorInvalidValue;
    e = cudaFuncSetAttribute(k_cycles32n<POT, BC, LPR, JPL>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return (int)e;
    attr_set[dev] = smem;
  }
  return 0;
}

// what = 0: launch; what = 1: resident CTAs per SM into *occ
template <int POT, int BC, int LPR, int JPL>
int launch_n(int what, const KParams& P, int run0, int nruns, int R, int maxN, int ncycles,
             int phase, cudaStream_t st, int* occ) {
  if ((R * LPR) % 32 != 0 || R > 32 || maxN > JPL * LPR) return (int)cudaErrorInvalidValue;
  const long long smem = cycles32n_smem_bytes(POT, R, maxN, LPR);
  int e = opt_in_n<POT, BC, LPR, JPL>(smem);
  if (e) return e;
  if (what == 1)
    return (int)cudaOccupancyMaxActiveBlocksPerMultiprocessor(occ, k_cycles32n<POT, BC, LPR, JPL>,
                                                              R * LPR, (size_t)smem);
  k_cycles32n<POT, BC, LPR, JPL><<<nruns, (unsigned)(R * LPR), (size_t)smem, st>>>(P, run0, ncycles,
                                                                                   phase);
  return (int)cudaGetLastError();
}

// N <= 64 atoms: 16 pair terms per lane at 4 lanes, 8 at 8 lanes
template <int POT, int BC>
int launch_nl(int what, const KParams& P, int run0, int nruns, int R, int maxN, int ncycles,
              int phase, int lpr, cudaStream_t st, int* occ) {
  // pair-potential runs of at most 16 atoms (Ne13): one chunk of 4 terms per
  // lane, without the tests of the three chunks such runs never reach
  if (POT != POT_EAM && lpr == 4 && maxN <= 16)
    return launch_n<POT, BC, 4, 4>(what, P, run0, nruns, R, maxN, ncycles, phase, st, occ);
  if (lpr == 4) return launch_n<POT, BC, 4, 16>(what, P, run0, nruns, R, maxN, ncycles, phase, st, occ);
  if (lpr == 8) return launch_n<POT, BC, 8, 8>(what, P, run0, nruns, R, maxN, ncycles, phase, st, occ);
  return (int)cudaErrorInvalidValue;
}

int dispatch_n(int what, int pot, int bc, const KParams& P, int run0, int nruns, int R, int maxN,
               int ncycles, int phase, int lpr, cudaStream_t st, int* occ) {
#define PT32N(PO, B) \
  if (pot == PO && bc == B) return launch_nl<PO, B>(what, P, run0, nruns, R, maxN, ncycles, phase, lpr, st, occ);
  PT32N(POT_ELJ, BC_SPH)
  PT32N(POT_ELJEVEN, BC_SPH)
  PT32N(POT_EAM, BC_SPH)
  PT32N(POT_ELJ, BC_CUB)
  PT32N(POT_ELJEVEN, BC_CUB)
  PT32N(POT_EAM, BC_CUB)
#undef PT32N
  return -1;
}

}  // namespace

long long cycles32n_smem_bytes(int pot, int R, int N, int lpr) {
  auto al = [](long long b) { return (b + 15) / 16 * 16; };
  const long long Ns = narrow_stride(N, lpr);
  long long b = al(R * Ns * 16);                           // float4 hi positions (+ rho)
  b += al(R * (long long)DRWN * 4);                        // draw words
  b += 2 * al(R * 8LL) + 2 * al(R * 16LL) + al(R * 48LL);  // beta, en, ham, maxd, counters
  b += 6 * al(R * 4LL);                                    // wos, sow, bl2e, mdf, mdc, acc
  return b;
}

int launch_cycles32n(int pot, int bc, const KParams& P, int run0, int nruns, int R, int maxN,
                     int ncycles, int phase, int lpr, void* stream) {
  return dispatch_n(0, pot, bc, P, run0, nruns, R, maxN, ncycles, phase, lpr, (cudaStream_t)stream,
                    nullptr);
}

int occupancy_cycles32n(int pot, int bc, int R, int N, int lpr, int* ctas_per_sm) {
  KParams P{};
  return dispatch_n(1, pot, bc, P, 0, 0, R, N, 0, 0, lpr, nullptr, ctas_per_sm);
}

}  // namespace ptmc
