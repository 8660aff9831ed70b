// ptmc_cycles32.cu — replica-cycle kernel of the FP32_RESYNC form.
//
// Same execution model as ptmc_cycles.cu (one CTA per PT run, one warp per
// walker, exchange by slot permutation), but the per-move path issues no FP64
// instruction: on GB300 the FP64 pipe runs at ~1/70 of the FP32 rate, and a
// warp-wide FP64 instruction costs the same pipe time whether 1 or 32 lanes are
// active, so every FP64 operation of the scalar move logic (proposal,
// Metropolis exp) would cost as much as the whole FP32 pair loop.
//
//  * Positions are float-float pairs (hi + lo, ~48 significant bits).  A
//    proposal adds an FP32 displacement d to (hi, lo) with an error-free
//    two-sum, so x' - x = d to ~2^-48 relative and the proposal stays
//    symmetric; the pair terms read hi only.  No int<->float conversion
//    appears in the move path: on GB300 conversions issue to the FP64 pipe.
//  * Draws are 32-bit Philox words (word k of a walker stream = word k & 3 of
//    Philox block k >> 2).  Uniforms are built by bit assembly,
//    u = float(1.m23) - 1, displacements use the symmetric grid
//    u - 1/2 + 2^-24, and rand(1:n) = mulhi(w, n).
//  * Metropolis: accept iff ex2(-beta * log2(e) * dE) >= u, dE in FP32.
//  * The FP64 running total absorbs the FP32 dE sum once per cycle; every
//    `resync_every` cycles each walker recomputes its energy (and EAM
//    components) in FP64 from hi + lo and records the drift
//    |E_running - E_fp64|.
//  * NPT volume moves (one step in N+1) are FP32 too: ln(V_new/V_old) as
//    drawn, FP32 pair terms with Kahan-compensated lane sums reduced as
//    float-float, FP32 tail correction and pV, the energy total in FP64, and an
//    exact-product float-float rescale of accepted positions.
//  * With one CTA per run and a warp per walker there is no CTA barrier per
//    cycle: every walker draws the run's exchange decisions, and only the two
//    walkers of the drawn pair wait for each other (bounded handshake through
//    per-slot records in shared memory); results equal the barrier form's bit
//    for bit.
//  * A run may be split over a thread-block cluster of C CTAs (C SMs): CTA
//    rank q holds walkers q*R/C .. (q+1)*R/C - 1.  After the moves of a cycle
//    every CTA gathers all walkers' energies, boxes and acceptance counts
//    through distributed shared memory (cluster barrier, DSMEM reads, cluster
//    barrier) and then runs the exchange, step adaptation and sampling on its
//    own full copy of the slot tables; the inputs and the run-level draws are
//    the same in every CTA, so the copies stay identical and rank 0 alone
//    writes them back.  Walker arithmetic and draw streams do not depend on C:
//    results are bit-identical for every C.  C is chosen per atom count by
//    ptmc_autotune (C = 1: a plain CTA launch, no cluster barrier).
//  * LPR lanes per walker (32 or 16): with 16, the two halves of a warp hold two
//    walkers; pair loops stride by LPR, reductions are segmented shuffles under
//    the walker's lane mask, and every warp-level barrier takes that mask, so
//    the halves may diverge (accept vs reject, refills) without waiting on each
//    other.  Small N wastes fewer lanes and shares the per-move fixed work.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include "ptmc_device.cuh"
#include "ptmc_engine.cuh"
#include "ptmc_fp32.cuh"

namespace ptmc {

// draw words buffered per walker (a refill is DRW32 / 4 Philox blocks)
constexpr uint32_t DRW32 = 128;

namespace {
using namespace f32k;

// waits until *f >= v (a flag in shared memory written by another warp of the
// CTA); false after `limit` clocks (2^33 unless a test shortens it), or at once
// when another walker of the CTA gave up (which then ends every other wait)
__device__ bool wait_flag(const int* f, int v, int* abort_flag, long long limit) {
  const long long t0 = clock64();
  while (*(const volatile int*)f < v) {
    if (*(volatile int*)abort_flag) return false;
    if (clock64() - t0 > limit) {
      *(volatile int*)abort_flag = 1;
      return false;
    }
    __nanosleep(64);
  }
  return true;
}
}  // namespace

// shared memory bytes of one run CTA (FP32 form) holding Rl = R / C walkers
long long cycles32_smem_bytes(int pot, int R, int N, int C) {
  auto al = [](long long b) { return (b + 15) / 16 * 16; };
  const long long Rl = R / C;
  long long b = 0;
  b += al(Rl * N * 16);  // float4 hi positions
  b += al(Rl * N * 16);  // float4 lo positions
  if (pot == POT_EAM) b += al(Rl * N * 4);  // density deltas
  b += al(Rl * DRW32 * 4);                                       // draw words
  b += al((long long)R * 8) * 6 + al((long long)R * 16) + al((long long)R * 48) + al((long long)R * 4) * 5;
  b += al((long long)R * 8);                                     // per-walker accepted counts
  return b;
}

template <int POT, int BC, int ENS, bool SPLIT, int LPR>
__global__ void __launch_bounds__(1024)
    k_cycles32(KParams P, int run0, int ncycles, int phase, int ncta) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ double s_c[MAX_COEFF];
  __shared__ float s_cf[MAX_COEFF];
  namespace cg = cooperative_groups;
  const int CL = SPLIT ? ncta : 1;          // CTAs of this run (cluster size)
  const int q = SPLIT ? (int)cg::this_cluster().block_rank() : 0;
  const int run_local = blockIdx.x / CL;
  const RunDesc* rdp = P.runs + run0 + run_local;  // fields read on demand
  const int N = rdp->N, R = rdp->R;
  const int Rl = R / CL;                    // walkers held by this CTA
  // LPR lanes per walker, 32 / LPR walkers per warp; gmask = the walker's lanes
  constexpr int WPW = 32 / LPR;
  const int tid = threadIdx.x, lane = tid & (LPR - 1);
  const int wl = (tid >> 5) * WPW + (tid & 31) / LPR;  // walker within this CTA
  const unsigned gmask = LPR == 32 ? 0xffffffffu : (((1u << LPR) - 1u) << ((tid & 31) & ~(LPR - 1)));
  const int w = q * Rl + wl;                // walker index within the run
  const int nthr = blockDim.x;
  const int K = P.K;
  const int n_steps = ENS == ENS_NPT ? N + 1 : N;

  unsigned char* sp = smem_raw;
  auto carve = [&](long long bytes) {
    unsigned char* p = sp;
    sp += (bytes + 15) / 16 * 16;
    return p;
  };
  float4* s_xh = (float4*)carve((long long)Rl * N * 16);
  float4* s_xl = (float4*)carve((long long)Rl * N * 16);
  float* s_d32 = nullptr;
  if (POT == POT_EAM) s_d32 = (float*)carve((long long)Rl * N * 4);
  uint32_t* s_drw = (uint32_t*)carve((long long)Rl * DRW32 * 4);
  double* s_beta = (double*)carve((long long)R * 8);
  double* s_maxbox = (double*)carve((long long)R * 8);
  double* s_en = (double*)carve((long long)R * 8);
  double* s_box = (double*)carve((long long)R * 8);
  double* s_ham = (double*)carve((long long)R * 16);
  double* s_maxd = (double*)carve((long long)R * 16);
  long long* s_cnt = (long long*)carve((long long)R * 48);
  int* s_wos = (int*)carve((long long)R * 4);
  int* s_sow = (int*)carve((long long)R * 4);
  float* s_bl2e = (float*)carve((long long)R * 4);  // beta * log2(e) per slot
  float* s_mdf = (float*)carve((long long)R * 4);   // atom step size per slot
  float* s_mdc = (float*)carve((long long)R * 4);   // its step offset md (3/2 - 2^-24)
  int2* s_acc = (int2*)carve((long long)R * 8);     // this cycle's accepted atom/volume moves per walker

  if (tid < K) {
    s_c[tid] = P.c[tid];
    s_cf[tid] = (float)P.c[tid];
  }
  const double* gpos = P.pos + rdp->pos_off + (size_t)q * Rl * N * 3;
  for (int k = tid; k < Rl * N; k += nthr) {
    double x = gpos[3 * k], y = gpos[3 * k + 1], z = gpos[3 * k + 2];
    float4 h = make_float4((float)x, (float)y, (float)z, 0.f);
    s_xh[k] = h;
    s_xl[k] = make_float4((float)(x - (double)h.x), (float)(y - (double)h.y),
                          (float)(z - (double)h.z), 0.f);
  }
  if (POT == POT_EAM) {
    const double* gc = P.comp + rdp->comp_off + (size_t)q * Rl * N * 2;
    for (int k = tid; k < Rl * N; k += nthr) {  // rho in the w lane of the position
      s_xh[k].w = (float)gc[2 * k + 1];
    }
  }
  const int wk0 = rdp->wk;
  for (int s = tid; s < R; s += nthr) {
    int g = wk0 + s;
    s_beta[s] = P.beta[g];
    s_maxbox[s] = P.maxbox[g];
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
  double rc2 = P.rc2[g];
  // draw words: drw[k] is word `base + k` of this walker's stream; `off` is
  // the next one (>= DRW32: refill from the 4-aligned word at base + off,
  // DRW32 / 4 Philox blocks spread over the walker's lanes)
  unsigned long long base = (P.ctr[g] & ~3ull) - DRW32;
  uint32_t off = DRW32 + (uint32_t)(P.ctr[g] & 3ull);
  int status = P.status[g];
  double drift = P.drift[g];
  float4* Xh = s_xh + (size_t)wl * N;
  float4* Xl = s_xl + (size_t)wl * N;
  uint32_t* drw = s_drw + wl * DRW32;
  const double hn = -0.5 * P.eam_n, hm = -0.5 * P.eam_m;
  const float hnf = P.f_hn, hmf = P.f_hm, ecamf = P.f_ecam;
  const float ean2f = 2.f * P.f_ean, necamf = -P.f_ecam;
  const uint32_t run_word = (uint32_t)rdp->run_id;
  const float pressf = (float)P.pressure;
  float Lf, iLf, Llo, rcf = (float)rc2;
  // the FP32 box: nearest float, its remainder, correctly rounded reciprocal
  auto set_box = [&](double Lnew) {
    L = Lnew;
    Lf = (float)L;
    Llo = (float)(L - (double)Lf);
    iLf = __frcp_rn(Lf);
  };
  set_box(L);

  auto refill = [&]() {
    __syncwarp(gmask);
    base += off & ~3u;
    off &= 3u;
    for (int bl = lane; bl < DRW32 / 4; bl += LPR) {
      uint64_t blk = (base >> 2) + bl;
      uint32_t c4[4] = {(uint32_t)blk, (uint32_t)(blk >> 32), (uint32_t)w, run_word};
      philox4x32_10(c4, (uint32_t)P.seed, (uint32_t)(P.seed >> 32));
      *(uint4*)(drw + 4 * bl) = make_uint4(c4[0], c4[1], c4[2], c4[3]);
    }
    __syncwarp(gmask);
  };
  auto word = [&]() -> uint32_t {
    if (off >= DRW32) refill();
    return drw[off++];
  };
  // the next n words are buffered (one check for a whole atom move; a refill
  // re-creates the unread words from their stream index)
  auto ensure = [&](uint32_t n) {
    if (off > DRW32 - n) refill();
  };
  auto word_nc = [&]() -> uint32_t { return drw[off++]; };

  // ---------------------------------------------------------- atom move
  auto atom_move = [&](int i, float beta_l2e, float mdf, float mdc, float& de_acc) -> int {
    float4 h0 = Xh[i], l0 = Xl[i];
    float th[3], tl[3];
    auto propose = [&]() {  // the first attempt's words are ensured by the caller
      float d0 = stepf(word_nc(), mdf, mdc), d1 = stepf(word_nc(), mdf, mdc),
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
            sx += (double)Xh[a].x + Xl[a].x;
            sy += (double)Xh[a].y + Xl[a].y;
            sz += (double)Xh[a].z + Xl[a].z;
          }
          sx = seg_sum<LPR>(sx, gmask) / N;
          sy = seg_sum<LPR>(sy, gmask) / N;
          sz = seg_sum<LPR>(sz, gmask) / N;
          __syncwarp(gmask);
          for (int a = lane; a < N; a += LPR) {
            double x = (double)Xh[a].x + Xl[a].x - sx, y = (double)Xh[a].y + Xl[a].y - sy,
                   z = (double)Xh[a].z + Xl[a].z - sz;
            float4 h = make_float4((float)x, (float)y, (float)z, Xh[a].w);
            Xh[a] = h;
            Xl[a] = make_float4((float)(x - h.x), (float)(y - h.y), (float)(z - h.z), 0.f);
          }
          __syncwarp(gmask);
          h0 = Xh[i];
          l0 = Xl[i];
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
        float m = rint_mul(th[k], iLf);
        if (m != 0.f) {
          ff_add(th[k], tl[k], -m * Lf);
          ff_add(th[k], tl[k], -m * Llo);
        }
      }
    }
    const float4 tf = make_float4(th[0], th[1], th[2], 0.f);
    const float4 x4 = h0;
    float de = 0.f, sbf = 0.f;
    if (POT == POT_EAM) {
      // The phi sums enter the energy linearly: the pair (i, j) changes phi_j
      // and phi_i by the same da, so the phi part of dE is 2 ean sum_j da and
      // no phi is kept.  rho_j is the w lane of atom j's position.
      float* D = s_d32 + (size_t)wl * N;
      for (int j = lane; j < N; j += LPR) {
        // the self pair (j == i: zero old distance) is masked, not branched
        const bool self = j == i;
        float4 b = Xh[j];
        float ln_ = lg2f(pf2<BC>(tf, b, Lf, iLf));
        float lo_ = lg2f(pf2<BC>(x4, b, Lf, iLf));
        float da = ex2f(hnf * ln_) - ex2f(hnf * lo_);
        float db = ex2f(hmf * ln_) - ex2f(hmf * lo_);
        da = self ? 0.f : da;
        db = self ? 0.f : db;
        D[j] = db;
        sbf += db;
        // sqrt(rho + db) - sqrt(rho) in the cancellation-free form
        de = fmaf(ean2f, da, de);
        de = fmaf(necamf * db, rcpf(sqrtf_approx(b.w) + sqrtf_approx(b.w + db)), de);
      }
      sbf = seg_sum<LPR>(sbf, gmask);
      de = seg_sum<LPR>(de, gmask);
      de -= ecamf * sbf * rcpf(sqrtf_approx(x4.w) + sqrtf_approx(x4.w + sbf));
    } else {
      for (int j = lane; j < N; j += LPR) {
        const bool self = j == i;  // masked, not branched (its old distance is 0)
        float4 b = Xh[j];
        float dn = pf2<BC>(tf, b, Lf, iLf);
        float dol = pf2<BC>(x4, b, Lf, iLf);
        if (ENS == ENS_NPT) {  // the cutoff as selects, not branches
          const float vn = v32p<POT>(P, s_cf, K, dn), vo = v32p<POT>(P, s_cf, K, dol);
          const float t = (dn <= rcf ? vn : 0.f) - (dol <= rcf ? vo : 0.f);
          de += self ? 0.f : t;
        } else {
          const float t = __fsub_rn(v32p<POT>(P, s_cf, K, dn), v32p<POT>(P, s_cf, K, dol));
          de += self ? 0.f : t;
        }
      }
      de = seg_sum<LPR>(de, gmask);
    }
    float u = u01f(word());
    if (!(ex2f(-beta_l2e * de) >= u)) return 0;
    __syncwarp(gmask);
    if (lane == 0) {
      float rho_i = 0.f;
      if (POT == POT_EAM) {
        rho_i = x4.w + sbf;
      }
      Xh[i] = make_float4(tf.x, tf.y, tf.z, rho_i);
      Xl[i] = make_float4(tl[0], tl[1], tl[2], 0.f);
    }
    if (POT == POT_EAM) {
      const float* D = s_d32 + (size_t)wl * N;
      for (int k = lane; k < N; k += LPR) {
        if (k == i) continue;
        Xh[k].w += D[k];
      }
    }
    de_acc += de;
    __syncwarp(gmask);
    return 1;
  };

  // ---------------------------------------------------------- volume move
  // volume_change (src/MCMoves.jl), every step but the box length and the
  // energy total in FP32: the drawn ln(V_new / V_old) = (u - 1/2) max_vchange
  // enters the acceptance as is (N log(V_new / V_old) needs no log), the scale
  // is its cube root, the pair sum is FP32 with Kahan compensation reduced as
  // float-float, and the accepted rescale of the float-float positions is an
  // exact-product step.  GB300 runs FP64 at ~1/70 of the FP32 rate, and a
  // walker's volume moves (Binomial(N + 1, 1 / (N + 1)) of them in a cycle)
  // would otherwise hold the whole CTA at the end-of-cycle barrier.
  auto volume_move = [&](float beta_l2e, float mdvf, double maxbox) -> int {
    float lnv = (u01f(word()) - 0.5f) * mdvf;  // ln(V_new / V_old)
    float scale = expf(lnv * (1.f / 3.f));
    if (L >= maxbox && scale > 1.f) {
      scale = 1.f;
      lnv = 0.f;
    }
    const double Ln = L * (double)scale;
    const double rcn = Ln * Ln * 0.25;
    const float s2 = scale * scale, rcnf = (float)rcn;
    float acc = 0.f, comp = 0.f;  // Kahan-compensated lane sum
    for (int i = 0; i < N; ++i) {
      float4 a = Xh[i];
      for (int j = i + 1 + lane; j < N; j += LPR) {
        const float x = pf2<BC>(a, Xh[j], Lf, iLf) * s2;
        const float v = v32p<POT>(P, s_cf, K, x);
        const float y = (x <= rcnf ? v : 0.f) - comp;
        const float tt = acc + y;
        comp = (tt - acc) - y;
        acc = tt;
      }
    }
    float hi = acc, lo = -comp;
#pragma unroll
    for (int o = LPR / 2; o > 0; o >>= 1) {  // float-float sum; every lane ends with the same pair
      const float oh = __shfl_xor_sync(gmask, hi, o), ol = __shfl_xor_sync(gmask, lo, o);
      const float s = hi + oh, bb = s - hi;
      const float err = (hi - (s - bb)) + (oh - bb);  // two-sum: exact in either operand order
      lo = (lo + ol) + err;
      hi = s + lo;
      lo = lo - (hi - s);
    }
    const double e = ((double)hi + (double)lo) + (double)lrc32(N, rcn, s_cf, K);
    const float vof = Lf * Lf * Lf;
    const float dh = (float)(e - en) + pressf * vof * expm1f(lnv);
    const float ua = u01f(word());
    if (!(ex2f(fmaf(-dh, beta_l2e, (float)N * lnv * 1.4426950408889634f)) >= ua)) return 0;
    __syncwarp(gmask);
    for (int a = lane; a < N; a += LPR) {
      float4 h = Xh[a], l = Xl[a];
      ff_scale(h.x, l.x, scale);
      ff_scale(h.y, l.y, scale);
      ff_scale(h.z, l.z, scale);
      Xh[a] = h;
      Xl[a] = make_float4(l.x, l.y, l.z, 0.f);
    }
    set_box(Ln);
    rc2 = rcn;
    rcf = rcnf;
    en = e;
    __syncwarp(gmask);
    return 1;
  };

  // ---------------------------------------------------------- cycle end
  // update_max_stepsize! and sampling_step! of slot s, whose walker ended the
  // cycle with energy e in a box of length Lw (one thread per slot)
  auto slot_epilogue = [&](int s, long long idx, double e, double Lw) {
    if (idx % P.n_adjust == 0) {  // update_max_stepsize!
      double acc = (double)s_cnt[6 * s + 1] / (double)((long long)P.n_adjust * N);
      if (acc < P.min_acc) s_maxd[2 * s] *= 0.9;
      else if (acc > P.max_acc) s_maxd[2 * s] *= 1.1;
      s_mdf[s] = (float)s_maxd[2 * s];
      s_mdc[s] = (float)(s_maxd[2 * s] * (1.5 - 0x1.0p-24));
      s_cnt[6 * s + 1] = 0;
      if (ENS == ENS_NPT) {
        double av = (double)s_cnt[6 * s + 3] / (double)(P.n_adjust * 1);
        if (av < P.min_acc) s_maxd[2 * s + 1] *= 0.9;
        else if (av > P.max_acc) s_maxd[2 * s + 1] *= 1.1;
        s_cnt[6 * s + 3] = 0;
      }
    }
    if (phase == PHASE_PROD && idx % P.mc_sample == 0) {  // sampling_step!
      const int nb = P.n_bin;
      unsigned int* hrow = P.hist + rdp->hist_off + (size_t)s * rdp->hist_stride;
      auto hidx = [&](double h) -> int {
        if (!(h >= 1)) return 1;
        if (h > nb) return nb + 2;
        return (int)floor(h) + 1;
      };
      if (ENS == ENS_NPT) {
        double V = Lw * Lw * Lw;
        double H = e + P.pressure * V;
        s_ham[2 * s] += H;
        s_ham[2 * s + 1] += H * H;
        int ie = hidx(floor((e - rdp->en_min) / rdp->dE) + 1);
        int iv = hidx(floor((V - rdp->v_min) / rdp->dV) + 1);
        if (q == 0) atomicAdd(hrow + (size_t)(ie - 1) * (nb + 2) + (iv - 1), 1u);
      } else {
        s_ham[2 * s] += e;
        s_ham[2 * s + 1] += e * e;
        int ie = hidx((e - rdp->en_min) / rdp->dE + 1);
        if (q == 0) atomicAdd(hrow + (ie - 1), 1u);
      }
    }
  };

  // Handshake form (one CTA per run, a warp per walker): no CTA barrier per
  // cycle.  The exchange draws do not depend on the walkers, so every walker
  // draws them; only the two walkers of the drawn pair (k, k + 1) wait for
  // each other, through per-slot records (energy, box, a flag = 2 cyc + 1 when
  // written, 2 cyc + 2 once the partner's record has been read).  Slot s's
  // counters, step sizes and sums are only touched by the walker holding s or
  // by its partner in the exchange that hands s over, in cycle order, so the
  // results are those of the barrier form bit for bit.
  constexpr bool HANDSHAKE = !SPLIT && LPR == 32;
  double* s_xen = s_en;              // slot records (the barrier form's per-walker arrays)
  double* s_xbox = s_box;
  int* s_xflag = (int*)s_acc;
  __shared__ int s_abort;            // a partner wait ran out: the others stop waiting
  if (HANDSHAKE) {
    for (int s = tid; s < R; s += nthr) s_xflag[s] = 0;
    if (tid == 0) s_abort = 0;
    __syncthreads();
  }
  int myslot = s_sow[w];

  // ---------------------------------------------------------- cycles
  const long long first = rdp->cyc[phase];
  unsigned long long run_ctr = rdp->run_ctr;
  for (int cyc = 0; cyc < ncycles; ++cyc) {
    const long long idx = first + cyc;
    const int slot = HANDSHAKE ? myslot : s_sow[w];
    const float mdvf = (float)s_maxd[2 * slot + 1];
    const double maxbox = s_maxbox[slot];
    const float beta_l2e = s_bl2e[slot];
    const float mdf = s_mdf[slot], mdc = s_mdc[slot];
    long long acc_a = 0, acc_v = 0;
    if (status == ST_OK) {
      float de_acc = 0.f;
      for (int st = 0; st < n_steps; ++st) {
        ensure(5);  // slot draw, three displacements, acceptance
        int k = (int)__umulhi(word_nc(), (uint32_t)n_steps);  // rand(1:n_steps)
        if (ENS == ENS_NVT || k < N) {  // NVT: every step is an atom move
          acc_a += atom_move(k, beta_l2e, mdf, mdc, de_acc);
        } else {
          en += (double)de_acc;  // fold the FP32 sum before the FP64 enthalpy
          de_acc = 0.f;
          acc_v += volume_move(beta_l2e, mdvf, maxbox);
        }
        if (status != ST_OK) break;
      }
      en += (double)de_acc;
      if (P.resync_every > 0 && idx % P.resync_every == 0) {
        double e64 = energy64<POT, BC, ENS, LPR>(Xh, Xl, N, L, rc2, s_c, K, hn, hm, P.eam_ean,
                                            P.eam_ecam, POT == POT_EAM ? s_d32 + (size_t)wl * N : nullptr,
                                            nullptr, lane, gmask);
        drift = fmax(drift, fabs(en - e64));
        en = e64;
        __syncwarp(gmask);
      }
    }
    if constexpr (HANDSHAKE) {
      if (lane == 0) {  // this cycle's moves were made in slot myslot
        s_cnt[6 * myslot + 0] += acc_a;
        s_cnt[6 * myslot + 1] += acc_a;
        s_cnt[6 * myslot + 2] += acc_v;
        s_cnt[6 * myslot + 3] += acc_v;
      }
      int k = -1;  // parallel_tempering_exchange! (src/Exchange.jl:132-180): the pair (k, k + 1)
      double ux = 0.0;
      if (R > 1) {
        double u = philox_u01(P.seed, 0xFFFFFFFFu, run_word, run_ctr++);
        if (u < P.exch_prob) {
          k = randint(philox_u01(P.seed, 0xFFFFFFFFu, run_word, run_ctr++), R - 1);
          ux = philox_u01(P.seed, 0xFFFFFFFFu, run_word, run_ctr++);
        }
      }
      if (k >= 0 && (myslot == k || myslot == k + 1)) {
        const int other = myslot == k ? k + 1 : k;
        const int tag = 2 * cyc + 1;
        // a test of the failure path waits for a flag value no walker writes
        const int want = P.xwait_never ? tag + (1 << 30) : tag;
        if (lane == 0) {
          s_xen[myslot] = en;
          s_xbox[myslot] = L;
          __threadfence_block();
          *(volatile int*)(s_xflag + myslot) = tag;
        }
        __syncwarp();
        bool ok = wait_flag(s_xflag + other, want, &s_abort, P.xwait_clocks);
        __threadfence_block();
        const double eo = *(volatile double*)(s_xen + other), Lo = *(volatile double*)(s_xbox + other);
        __syncwarp();  // every lane has read the partner's record
        // the second flag goes up only after a successful first wait, so the
        // partner's second wait succeeds only when this walker got its record:
        // both sides swap, or neither does
        if (ok) {
          if (lane == 0) *(volatile int*)(s_xflag + myslot) = tag + 1;
          ok = wait_flag(s_xflag + other, want + 1, &s_abort, P.xwait_clocks);
        }
        if (!ok) {
          // the walker stops (status), keeps its slot and counts no exchange;
          // the host reports the error and the context must be rebuilt
          status = ST_XWAIT;
        } else {
          const bool lo_side = myslot == k;
          const double p = exch_acc(s_beta[k], s_beta[k + 1], lo_side ? en : eo, lo_side ? eo : en,
                                    lo_side ? L : Lo, lo_side ? Lo : L, ENS == ENS_NPT ? P.pressure : 0.0);
          const bool swap = p > ux;
          if (swap) myslot = other;
          if (lane == 0) {
            s_cnt[6 * myslot + 4] += 1;
            if (swap) s_cnt[6 * myslot + 5] += 1;
          }
        }
      }
      if (lane == 0) {
        s_sow[w] = myslot;
        s_wos[myslot] = w;
        slot_epilogue(myslot, idx, en, L);
      }
      __syncwarp();
    } else {
      if (lane == 0) {
        s_en[w] = en;
        s_box[w] = L;
        s_acc[w] = make_int2((int)acc_a, (int)acc_v);
      }
      if constexpr (SPLIT) {  // gather the other CTAs' walkers through distributed shared memory
        cg::cluster_group cl = cg::this_cluster();
        cl.sync();
        for (int v = tid; v < R; v += nthr) {
          const int owner = v / Rl;
          if (owner != q) {
            s_en[v] = *cl.map_shared_rank(s_en + v, owner);
            s_box[v] = *cl.map_shared_rank(s_box + v, owner);
            s_acc[v] = *cl.map_shared_rank(s_acc + v, owner);
          }
        }
        cl.sync();  // every remote read is done before any CTA writes its next results
      } else {
        __syncthreads();
      }
      for (int v = tid; v < R; v += nthr) {  // counters of the slot each walker occupied
        const int sl = s_sow[v];
        const int2 a = s_acc[v];
        s_cnt[6 * sl + 0] += a.x;
        s_cnt[6 * sl + 1] += a.x;
        s_cnt[6 * sl + 2] += a.y;
        s_cnt[6 * sl + 3] += a.y;
      }
      __syncthreads();
      if (tid == 0 && R > 1) {  // parallel_tempering_exchange! (src/Exchange.jl:132-180)
        double u = philox_u01(P.seed, 0xFFFFFFFFu, run_word, run_ctr++);
        if (u < P.exch_prob) {
          int k = randint(philox_u01(P.seed, 0xFFFFFFFFu, run_word, run_ctr++), R - 1);
          s_cnt[6 * k + 4] += 1;
          s_cnt[6 * (k + 1) + 4] += 1;
          int w1 = s_wos[k], w2 = s_wos[k + 1];
          double acc = exch_acc(s_beta[k], s_beta[k + 1], s_en[w1], s_en[w2], s_box[w1], s_box[w2],
                                ENS == ENS_NPT ? P.pressure : 0.0);
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
      if (tid < R) {
        const int wk = s_wos[tid];
        slot_epilogue(tid, idx, s_en[wk], s_box[wk]);
      }
      __syncthreads();
    }
    if (P.rdf && phase == PHASE_PROD && idx % P.mc_sample == 0 && idx % RDF_EVERY == 0) {
      // update_rdf! (src/Sampling.jl:301-316) from the FP32 positions
      unsigned int* row = P.rdf + (size_t)(wk0 + (HANDSHAKE ? myslot : s_sow[w])) * 5 * P.n_bin;
      for (int i = 1; i < N; ++i)
        for (int k = lane; k < i; k += LPR)
          rdf_add(row, 5 * P.n_bin, (double)pf2<BC>(Xh[i], Xh[k], Lf, iLf), rdp->dr2);
    }
  }
  if (HANDSHAKE) __syncthreads();  // every walker has finished its cycles and slot updates

  double* gpos_w = P.pos + rdp->pos_off + (size_t)q * Rl * N * 3;
  for (int k = tid; k < Rl * N; k += nthr) {
    float4 h = s_xh[k], l = s_xl[k];
    gpos_w[3 * k] = (double)h.x + (double)l.x;
    gpos_w[3 * k + 1] = (double)h.y + (double)l.y;
    gpos_w[3 * k + 2] = (double)h.z + (double)l.z;
  }
  if (POT == POT_EAM) {
    double* gc = P.comp + rdp->comp_off + (size_t)q * Rl * N * 2;
    for (int k = tid; k < Rl * N; k += nthr) {
      gc[2 * k + 1] = s_xh[k].w;  // rho; the FP32 form keeps no phi
    }
  }
  if (lane == 0) {
    P.en[g] = en;
    P.box[g] = L;
    P.rc2[g] = rc2;
    P.ctr[g] = base + off;
    P.status[g] = status;
    P.drift[g] = drift;
  }
  for (int s = tid; s < R && q == 0; s += nthr) {  // slot tables: identical in every CTA
    int gs = wk0 + s;
    P.ham[2 * gs] = s_ham[2 * s];
    P.ham[2 * gs + 1] = s_ham[2 * s + 1];
    P.maxd[2 * gs] = s_maxd[2 * s];
    P.maxd[2 * gs + 1] = s_maxd[2 * s + 1];
    for (int k = 0; k < 6; ++k) P.cnt[6 * (size_t)gs + k] = s_cnt[6 * s + k];
    P.wos[gs] = s_wos[s];
  }
  __syncthreads();  // every thread has read the run descriptor
  if (tid == 0 && q == 0) {
    P.runs[run0 + run_local].cyc[phase] = first + ncycles;
    P.runs[run0 + run_local].run_ctr = run_ctr;
  }
}

template <int POT, int BC, int ENS, int LPR>
static int set_smem32(long long smem) {
  // per instantiation and per device: the attribute belongs to the current
  // device's context
  static long long attr_set[MAX_DEVICES] = {};
  int dev = 0, optin = 0;
  cudaError_t ge = cudaGetDevice(&dev);
  if (ge != cudaSuccess) return (int)ge;
  if (dev < 0 || dev >= MAX_DEVICES) return (int)cudaErrorInvalidDevice;
  if (smem <= 48 * 1024 || smem <= attr_set[dev]) return 0;
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  cudaFuncAttributes fa;
  cudaError_t e = cudaFuncGetAttributes(&fa, k_cycles32<POT, BC, ENS, false, LPR>);
  if (e != cudaSuccess) return (int)e;
  if (smem + (long long)fa.sharedSizeBytes > optin) return (int)cudaErrorInvalidValue;
  e = cudaFuncSetAttribute(k_cycles32<POT, BC, ENS, false, LPR>,
                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return (int)e;
  e = cudaFuncSetAttribute(k_cycles32<POT, BC, ENS, true, LPR>,
                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return (int)e;
  attr_set[dev] = smem;
  return 0;
}

template <int POT, int BC, int ENS, int LPR>
static int launch32l(const KParams& P, int run0, int nruns, int R, int maxN, int ncycles,
                     int phase, int ncta, cudaStream_t st, int* occ = nullptr) {
  constexpr int WPW = 32 / LPR;
  if (ncta < 1 || ncta > 8 || R % ncta != 0 || (R / ncta) % WPW != 0)
    return (int)cudaErrorInvalidValue;
  long long smem = cycles32_smem_bytes(POT, R, maxN, ncta);
  int e = set_smem32<POT, BC, ENS, LPR>(smem);
  if (e) return e;
  const unsigned threads = (unsigned)(R / ncta * LPR);
  if (occ) {  // resident CTAs per SM (a cluster's CTAs count one each)
    if (ncta == 1)
      return (int)cudaOccupancyMaxActiveBlocksPerMultiprocessor(
          occ, k_cycles32<POT, BC, ENS, false, LPR>, (int)threads, (size_t)smem);
    return (int)cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        occ, k_cycles32<POT, BC, ENS, true, LPR>, (int)threads, (size_t)smem);
  }
  if (ncta == 1) {
    k_cycles32<POT, BC, ENS, false, LPR><<<nruns, threads, (size_t)smem, st>>>(P, run0, ncycles,
                                                                               phase, 1);
    return (int)cudaGetLastError();
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)(nruns * ncta), 1, 1);
  cfg.blockDim = dim3(threads, 1, 1);
  cfg.dynamicSmemBytes = (size_t)smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = (unsigned)ncta;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cudaError_t ce =
      cudaLaunchKernelEx(&cfg, k_cycles32<POT, BC, ENS, true, LPR>, P, run0, ncycles, phase, ncta);
  if (ce != cudaSuccess) return (int)ce;
  return (int)cudaGetLastError();
}

template <int POT, int BC, int ENS>
static int launch32(const KParams& P, int run0, int nruns, int R, int maxN, int ncycles,
                    int phase, int ncta, int lpr, cudaStream_t st, int* occ = nullptr) {
  if (lpr == 16)
    return launch32l<POT, BC, ENS, 16>(P, run0, nruns, R, maxN, ncycles, phase, ncta, st, occ);
  if (lpr == 32)
    return launch32l<POT, BC, ENS, 32>(P, run0, nruns, R, maxN, ncycles, phase, ncta, st, occ);
  return (int)cudaErrorInvalidValue;
}

int launch_cycles32(int pot, int bc, int ens, const KParams& P, int run0, int nruns, int R,
                    int maxN, int ncycles, int phase, int ncta, int lpr, void* stream) {
  cudaStream_t st = (cudaStream_t)stream;
  if (lpr == 4 || lpr == 8) {  // a few lanes per walker: ptmc_cycles32n.cu (NVT, one CTA per run)
    if (ncta != 1 || ens != ENS_NVT) return (int)cudaErrorInvalidValue;
    return launch_cycles32n(pot, bc, P, run0, nruns, R, maxN, ncycles, phase, lpr, stream);
  }
#define PT32(PO, B, E) \
  if (pot == PO && bc == B && ens == E) return launch32<PO, B, E>(P, run0, nruns, R, maxN, ncycles, phase, ncta, lpr, st);
  PT32(POT_ELJ, BC_SPH, ENS_NVT)
  PT32(POT_ELJEVEN, BC_SPH, ENS_NVT)
  PT32(POT_EAM, BC_SPH, ENS_NVT)
  PT32(POT_ELJ, BC_CUB, ENS_NVT)
  PT32(POT_ELJEVEN, BC_CUB, ENS_NVT)
  PT32(POT_EAM, BC_CUB, ENS_NVT)
  PT32(POT_ELJEVEN, BC_CUB, ENS_NPT)
#undef PT32
  return -1;
}

int occupancy_cycles32(int pot, int bc, int ens, int R, int N, int ncta, int lpr, int* ctas_per_sm) {
  if (lpr == 4 || lpr == 8) {
    if (ncta != 1 || ens != ENS_NVT) return (int)cudaErrorInvalidValue;
    return occupancy_cycles32n(pot, bc, R, N, lpr, ctas_per_sm);
  }
  KParams P{};
#define OC32(PO, B, E) \
  if (pot == PO && bc == B && ens == E) return launch32<PO, B, E>(P, 0, 0, R, N, 0, 0, ncta, lpr, nullptr, ctas_per_sm);
  OC32(POT_ELJ, BC_SPH, ENS_NVT)
  OC32(POT_ELJEVEN, BC_SPH, ENS_NVT)
  OC32(POT_EAM, BC_SPH, ENS_NVT)
  OC32(POT_ELJ, BC_CUB, ENS_NVT)
  OC32(POT_ELJEVEN, BC_CUB, ENS_NVT)
  OC32(POT_EAM, BC_CUB, ENS_NVT)
  OC32(POT_ELJEVEN, BC_CUB, ENS_NPT)
#undef OC32
  return -1;
}

}  // namespace ptmc
