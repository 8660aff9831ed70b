// ptmc_cycles.cu — replica-cycle kernels of the GB300 PT-MC engine.
//
// Execution model.  One CTA runs one PT run; one warp owns one walker.  A
// walker is the configuration-bound part of an MCState (positions, distance
// matrix, energy, potential variables, box, draw stream); a slot is the
// temperature-bound part (beta, max_displ, counters, E/E^2 sums, histogram
// row).  The reference swaps whole configurations between temperature slots on
// an accepted exchange (src/Exchange.jl:115-124); here the exchange swaps the
// walker<->slot index, which is the same transition and moves no data.
//
// Per cycle (mc_cycle!, src/MCRun.jl:192-253): every warp makes n_steps moves
// of its walker (mc_step!/mc_move!, src/MCRun.jl:142-182) with positions and
// per-atom potential variables in shared memory and the move's pair terms
// spread over the 32 lanes (warp-shuffle reductions give dE); then, after a
// CTA barrier, thread 0 makes the exchange draw (parallel_tempering_exchange!,
// src/Exchange.jl:132-180), threads 0..R-1 adapt step sizes
// (update_max_stepsize!, src/Exchange.jl:198-257) and sample
// (sampling_step!, src/Sampling.jl:330-371).  The loop runs `ncycles` cycles
// per launch; there are no spin-waits and no inter-CTA communication.
//
// Draw order per move (both forms, identical to the CPU oracle): slot index
// (rand(1:n_steps)), 3 displacement draws (+3 per spherical retry), the
// acceptance draw; volume move: scale draw, acceptance draw.
//
// This file holds the plain FP64 form: every quantity in FP64; proposals and
// squared distances use non-contracted IEEE operations, so they are
// bit-identical to the reference's; pair energies use FMA Horner forms (agree
// to ~1e-16 relative).  The FP32_RESYNC form's cycle kernel is in
// ptmc_cycles32.cu; k_init and k_resync here serve both forms.
//
// Pair cache.  The reference keeps each state's squared-distance matrix and
// recomputes the old pair energies of a moved atom from it
// (dimer_energy_update!, src/EnergyEvaluation.jl:804-821; EAM
// calc_components, :1105-1148).  In NVT the plain form keeps the pair energies
// themselves in HBM (ELJ: V(r_ij); EAM: (r_ij^-n, r_ij^-m)), one N x N matrix
// per walker, so a move evaluates only its N - 1 trial pairs and reads the old
// row; an accepted move writes the row and the column.  A cached value is the
// value computed from the distance the reference stores for the pair, so the
// chain is the reference's arithmetic.  NPT and the angle-dependent
// potentials keep the squared-distance matrix (volume moves rescale it) and
// evaluate the old pair energies from it, as the reference does.
#include <cuda_runtime.h>

#include "ptmc_device.cuh"
#include "ptmc_engine.cuh"

namespace ptmc {

// ------------------------------------------------------------ pair energies
// ELJPotentialEven (src/EnergyEvaluation.jl:934-942): sum_k c_k r^-(6+2k)
__device__ __forceinline__ double v_even64(const double* c, int K, double r2) {
  double inv = 1.0 / r2;
  double v = c[K - 1];
  for (int k = K - 2; k >= 0; --k) v = fma(v, inv, c[k]);
  return v * (inv * inv * inv);
}
// ELJPotential (src/EnergyEvaluation.jl:923-932): sum_k c_k r^-(6+k)
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
// lrc (src/EnergyEvaluation.jl:968-982); rc2 is the squared cut-off
__device__ double lrc64(int N, double rc2, const double* c, int K) {
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
// long-range correction of dimer_energy_config for the box
// (src/EnergyEvaluation.jl:419, 444, 469-472): lrc assumes a cube, the other
// boxes rescale it
template <int BC>
__device__ double lrc_box(int N, double rc2, const double* c, int K, double L, double H) {
  const double l = lrc64(N, rc2, c, K);
  if (BC == BC_RHB) return l * 3 / 4 * L / H;
  if (BC == BC_RECT) return L < H ? l * L / H : l * (H * H) / (L * L);
  return l;
}
// invrexp (src/EnergyEvaluation.jl:1088-1095): (r^-n, r^-m) from r^2
__device__ __forceinline__ void invrexp64(double r2, double hn, double hm,
                                          double& a, double& b) {
  if (r2 != 0.0) {
    double lg = log(r2);
    a = exp(hn * lg);
    b = exp(hm * lg);
  } else {
    a = 0.0;
    b = 0.0;
  }
}

template <int BC>
__device__ __forceinline__ double pd2(double ax, double ay, double az,
                                      const double* b, double L, double H) {
  if (BC == BC_CUB) return d2_cub(ax, ay, az, b[0], b[1], b[2], L);
  if (BC == BC_RECT) return d2_rect(ax, ay, az, b[0], b[1], b[2], L, H);
  if (BC == BC_RHB) return d2_rhb(ax, ay, az, b[0], b[1], b[2], L, H);
  return d2_sph(ax, ay, az, b[0], b[1], b[2]);
}
// boxes with a separate height (RectangularBC, RhombicBC)
template <int BC>
__host__ __device__ constexpr bool has_height() { return BC == BC_RECT || BC == BC_RHB; }
// get_r_cut (src/Ensembles.jl:118-155)
template <int BC>
__device__ __forceinline__ double box_rcut(double L, double H) {
  if (BC == BC_RHB) return fmin(L * L * 3 / 16, H * H / 4);
  if (BC == BC_RECT) return fmin(L * L / 4, H * H / 4);
  return L * L / 4;
}
// get_volume (src/Configurations.jl:246-256)
template <int BC>
__device__ __forceinline__ double box_volume(double L, double H) {
  if (BC == BC_RHB) return L * L * H * SQRT3 / 2;
  if (BC == BC_RECT) return dmul(dmul(L, L), H);
  return dmul(dmul(L, L), L);
}
// the volume the NPT histogram index is taken from (src/Sampling.jl:64-130):
// the box volume, except that the rhombic branch computes L^2 * 3 H^0.5 / 2
template <int BC>
__device__ __forceinline__ double hist_volume(double L, double H) {
  if (BC == BC_RHB) return dmul(dmul(L, L), dmul(3.0, sqrt(H))) / 2;
  return box_volume<BC>(L, H);
}

// ---- ELJPotentialB and LookupTablePotential: pair energies that depend on
// |tan| of the angle between the pair vector and z
// get_tan (src/Configurations.jl:181-215) with the minimum image of the box
template <int BC>
__device__ __forceinline__ double ptan(double ax, double ay, double az, const double* b,
                                       double L, double H) {
  double bx = b[0], by = b[1], bz = b[2];
  if (BC == BC_CUB || BC == BC_RECT) {
    const double Hz = BC == BC_RECT ? H : L;
    bx = dadd(b[0], dmul(L, rint(ddiv(dsub(ax, b[0]), L))));
    by = dadd(b[1], dmul(L, rint(ddiv(dsub(ay, b[1]), L))));
    bz = dadd(b[2], dmul(Hz, rint(ddiv(dsub(az, b[2]), Hz))));
  } else if (BC == BC_RHB) {
    const double hy = dmul(SQRT3 / 2, L), is3 = 1.0 / SQRT3;
    by = dadd(b[1], dmul(hy, rint(ddiv(dsub(ay, b[1]), hy))));
    double q = ddiv(dsub(dsub(ax, b[0]), dmul(is3, dsub(ay, b[1]))), L);
    bx = dadd(dadd(dsub(b[0], ddiv(b[1], SQRT3)), dmul(L, rint(q))), dmul(is3, by));
    bz = dadd(b[2], dmul(H, rint(ddiv(dsub(az, b[2]), H))));
  }
  const double dx = dsub(ax, bx), dy = dsub(ay, by);
  return fabs(ddiv(sqrt(dadd(dmul(dx, dx), dmul(dy, dy))), dsub(az, bz)));
}
// dimer_energy ELJPotentialB (src/EnergyEvaluation.jl:943-958)
__device__ __forceinline__ double v_eljb(const double* a, const double* b, const double* c, int K,
                                         double r2, double tn) {
  if (!(r2 >= 5.30)) return 0.1;
  double r6inv = 1.0 / (r2 * r2 * r2);
  const double t2 = 2.0 / (tn * tn + 1.0) - 1.0;  // cos(2 theta)
  const double t4 = 2.0 * (t2 * t2) - 1.0;
  double s = c[0] * r6inv * (1.0 + a[0] * t2 + b[0] * t4);
  r6inv /= r2;
  const double r = sqrt(r2);
  for (int i = 1; i < K; ++i) {
    s += c[i] * r6inv * (1.0 + a[i] * t2 + b[i] * t4);
    r6inv /= r;
  }
  return s;
}
// dimer_energy LookupTablePotential (src/EnergyEvaluation.jl:277-298): angle
// index from atan(|tan|) in table steps, distance index from sqrt(r2), the c6
// tail beyond the table; Julia's round is half-to-even (rint), the indices are
// kept inside the table
__device__ __forceinline__ double v_lut(const KParams& P, double r2, double tn) {
  int ia = 1;
  const double at = fabs(tn);
  if (at > 0.00872687153 && at <= 114.592845357)
    ia = (int)rint(atan(at) / P.lut_da * 180.0 / 3.141592653589793 + 1.0);
  else if (at > 114.592845357)
    ia = 91;
  ia = min(max(ia, 1), P.lut_na);
  const double r0 = P.lut_start + 0.5 * P.lut_dd, r1 = P.lut_start + P.lut_nd * P.lut_dd;
  if (r2 <= r0 * r0) return __ldg(P.lut + (ia - 1));
  if (r2 <= r1 * r1) {
    int id = (int)rint((sqrt(r2) - P.lut_start) / P.lut_dd);
    id = min(max(id, 1), P.lut_nd);
    return __ldg(P.lut + (size_t)(id - 1) * P.lut_na + (ia - 1));
  }
  return P.lut_c6 / (r2 * r2 * r2);
}
template <int POT>
__device__ __forceinline__ double vb(const KParams& P, const double* a, const double* b,
                                     const double* c, int K, double r2, double tn) {
  return POT == POT_ELJB ? v_eljb(a, b, c, K, r2, tn) : v_lut(P, r2, tn);
}
// lrc of the B potentials (src/EnergyEvaluation.jl:983-1009) with the box
// factor of dimer_energy_config
template <int POT, int BC>
__device__ double lrc_b(const KParams& P, int N, double rc2, double L, double H) {
  double l;
  const double rcs = sqrt(rc2);
  if (POT == POT_ELJB) {
    const double cf[4] = {-0.1279111890228638, -1.328138539967966, 12.260941135261255,
                          41.12212408251662};
    if (rc2 <= 16) {
      l = 0.0;
    } else {
      double rc3 = rc2 * rcs;
      l = 0.0;
      for (int i = 1; i <= 4; ++i) {
        l += cf[i - 1] / rc3 / (2 * i + 1);
        rc3 *= rc2;
      }
      l *= 3.141592653589793 * (double)(N * N) / 4 / (rcs * rcs * rcs);
    }
  } else {
    if (rc2 <= 10) {
      l = 1.0;
    } else {
      l = P.lut_c6 / (rc2 * rcs) / 3;
      l *= 3.141592653589793 * (double)(N * N) / 4 / (rcs * rcs * rcs);
    }
  }
  if (BC == BC_RHB) return l * 3 / 4 * L / H;
  if (BC == BC_RECT) return L < H ? l * L / H : l * (H * H) / (L * L);
  return l;
}
// FP64 energy of one walker for the B potentials: fills the distance and
// tangent matrices (get_distance2_mat, get_tantheta_mat) and sums
// dimer_energy_config (src/EnergyEvaluation.jl:476-780)
template <int POT, int BC, int ENS>
__device__ double walker_energy_b(const KParams& P, const double* X, int N, double L, double H,
                                  double rc2, const double* a, const double* b, const double* c,
                                  int K, double* M, double* T, int lane) {
  double e = 0.0;
  for (int i = 0; i < N; ++i) {
    const double xi = X[3 * i], yi = X[3 * i + 1], zi = X[3 * i + 2];
    for (int j = i + 1 + lane; j < N; j += 32) {
      const double x = pd2<BC>(xi, yi, zi, X + 3 * j, L, H);
      const double t = ptan<BC>(xi, yi, zi, X + 3 * j, L, H);
      M[(size_t)i * N + j] = x;
      M[(size_t)j * N + i] = x;
      T[(size_t)i * N + j] = t;
      T[(size_t)j * N + i] = t;
      if (ENS == ENS_NPT && !(x <= rc2)) continue;
      e += vb<POT>(P, a, b, c, K, x, t);
    }
    if (lane == 0) {
      M[(size_t)i * N + i] = 0.0;
      T[(size_t)i * N + i] = 0.0;
    }
  }
  e = warp_sum(e);
  if (ENS == ENS_NPT) e = e + lrc_b<POT, BC>(P, N, rc2, L, H);
  return e;
}

// ------------------------------------------------------------ FP64 energy of
// one walker from positions (init and resync).  ELJ: dimer_energy_config
// (src/EnergyEvaluation.jl:378-420); EAM: set_variables + energy
// (src/EnergyEvaluation.jl:1800-1810, 1156-1162).  Writes the NPT distance
// matrix, the EAM components and the NVT pair cache (PE: ELJ V(r_ij) as N x N
// doubles, EAM (r_ij^-n, r_ij^-m) as N x N double pairs, zero diagonal) when
// the pointers are given.
template <int POT, int BC, int ENS>
__device__ double walker_energy64(const double* X, int N, double L, double H, double rc2,
                                  const double* c, int K, double hn, double hm,
                                  double ean, double ecam, double* M,
                                  double* comp64, double* PE, int lane) {
  double e = 0.0;
  if constexpr (POT == POT_EAM) {
    double2* PE2 = (double2*)PE;
    for (int k = lane; k < N; k += 32) {
      double a = 0.0, b = 0.0;
      for (int j = 0; j < N; ++j) {
        if (j == k) {
          if (PE2) PE2[(size_t)k * N + k] = make_double2(0.0, 0.0);
          continue;
        }
        double x = pd2<BC>(X[3 * k], X[3 * k + 1], X[3 * k + 2], X + 3 * j, L, H);
        double pa, pb;
        invrexp64(x, hn, hm, pa, pb);
        if (PE2) PE2[(size_t)k * N + j] = make_double2(pa, pb);
        a += pa;
        b += pb;
      }
      if (comp64) {
        comp64[2 * k] = a;
        comp64[2 * k + 1] = b;
      }
      e += ean * a - ecam * sqrt(b);
    }
    return warp_sum(e);
  } else {
    for (int i = 0; i < N; ++i) {
      double xi = X[3 * i], yi = X[3 * i + 1], zi = X[3 * i + 2];
      for (int j = i + 1 + lane; j < N; j += 32) {
        double x = pd2<BC>(xi, yi, zi, X + 3 * j, L, H);
        if (M) {
          M[(size_t)i * N + j] = x;
          M[(size_t)j * N + i] = x;
        }
        if (ENS == ENS_NPT && !(x <= rc2)) continue;
        const double v = v64<POT>(c, K, x);
        if (PE) {
          PE[(size_t)i * N + j] = v;
          PE[(size_t)j * N + i] = v;
        }
        e += v;
      }
      if (M && lane == 0) M[(size_t)i * N + i] = 0.0;
      if (PE && lane == 0) PE[(size_t)i * N + i] = 0.0;
    }
    e = warp_sum(e);
    if (ENS == ENS_NPT) e = e + lrc_box<BC>(N, rc2, c, K, L, H);
    return e;
  }
}

// FP64 energy (and EAM components) of one configuration with every thread of
// the CTA, for a run whose replicas all start from one configuration: thread
// (row k, group g) sums the pair terms of row k over j = g, g + G, ... (the
// pair potentials: j > k only), the groups of a row are added in order and
// the rows by a fixed tree, so the result does not depend on the timing.
// Needs blockDim.x >= N.
template <int POT, int BC, int ENS>
__device__ double start_energy_cta(const KParams& P, const double* X, int N, double L, double H,
                                   double rc2, double* comp64) {
  __shared__ double s_pa[1024], s_pb[1024];
  const int T = blockDim.x, t = threadIdx.x;
  const int G = T / N;
  double a = 0.0, b = 0.0;
  if (t < G * N) {
    const int k = t % N, g = t / N;
    const double xk = X[3 * k], yk = X[3 * k + 1], zk = X[3 * k + 2];
    if constexpr (POT == POT_EAM) {
      for (int j = g; j < N; j += G) {
        if (j == k) continue;
        double pa, pb;
        invrexp64(pd2<BC>(xk, yk, zk, X + 3 * j, L, H), -0.5 * P.eam_n, -0.5 * P.eam_m, pa, pb);
        a += pa;
        b += pb;
      }
    } else {
      for (int j = k + 1 + g; j < N; j += G) {
        const double x = pd2<BC>(xk, yk, zk, X + 3 * j, L, H);
        if (ENS == ENS_NPT && !(x <= rc2)) continue;
        a += v64<POT>(P.c, P.K, x);
      }
    }
  }
  s_pa[t] = a;
  s_pb[t] = b;
  __syncthreads();
  double e = 0.0;
  if (t < N) {
    double ra = 0.0, rb = 0.0;
    for (int g = 0; g < G; ++g) {
      ra += s_pa[g * N + t];
      rb += s_pb[g * N + t];
    }
    if constexpr (POT == POT_EAM) {
      if (comp64) {
        comp64[2 * t] = ra;
        comp64[2 * t + 1] = rb;
      }
      e = P.eam_ean * ra - P.eam_ecam * sqrt(rb);
    } else {
      e = ra;
    }
  }
  __syncthreads();
  s_pa[t] = e;
  __syncthreads();
  int p2 = 1;  // the largest power of two <= T: fold the rest onto it, then a tree
  while (2 * p2 <= T) p2 *= 2;
  if (t >= p2) s_pa[t - p2] += s_pa[t];
  __syncthreads();
  for (int h = p2 >> 1; h > 0; h >>= 1) {
    if (t < h) s_pa[t] += s_pa[t + h];
    __syncthreads();
  }
  e = s_pa[0];
  __syncthreads();
  if constexpr (ENS == ENS_NPT && POT != POT_EAM) e = e + lrc_box<BC>(N, rc2, P.c, P.K, L, H);
  return e;
}

// ------------------------------------------------------------ init kernel
// MCState constructor (src/MCStates.jl:137-162): distance matrix, potential
// variables and initial energy of every walker, in FP64, from HBM positions.
template <int POT, int BC, int ENS, bool F32>
__global__ void __launch_bounds__(1024) k_init(KParams P, int run0) {
  // walkers w >= n_start start from the configuration of walker w mod n_start
  // (src/Initialization.jl:88-96): only the distinct starts are evaluated, the
  // other walkers copy their energy and variables
  // a warp per walker; with more than 32 walkers (R > blockDim / 32) each
  // warp takes every nw-th walker
  const RunDesc rd = P.runs[run0 + blockIdx.x];
  const int N = rd.N, warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  const int ns = rd.n_start > 0 && rd.n_start < rd.R ? rd.n_start : rd.R;
  const bool keep_m = (ENS == ENS_NPT || pot_b(POT)) && !F32;
  constexpr bool keep_pe = pair_cache(POT, ENS) && !F32;  // plain form's NVT pair cache
  constexpr int pe_w = POT == POT_EAM ? 2 : 1;            // doubles per cached pair
  auto mat = [&](int v) { return P.mat + rd.mat_off + (size_t)v * N * N; };
  auto cmp = [&](int v) { return P.comp + rd.comp_off + (size_t)v * N * 2; };
  auto pe = [&](int v) { return P.pe + rd.pe_off + (size_t)v * N * N * pe_w; };
  // FP32 form, one start for every replica: the whole CTA evaluates it (a
  // single warp would leave the SM's FP64 pipes mostly idle)
  const bool cta = F32 && !pot_b(POT) && ns == 1 && N <= (int)blockDim.x;
  if constexpr (F32 && !pot_b(POT)) {
    if (cta) {
      const int g = rd.wk;
      const double e = start_energy_cta<POT, BC, ENS>(
          P, P.pos + rd.pos_off, N, P.box[g], P.boxh[g], P.rc2[g], POT == POT_EAM ? cmp(0) : nullptr);
      if (threadIdx.x == 0) {
        P.en[g] = e;
        P.status[g] = ST_OK;
        P.drift[g] = 0.0;
      }
    }
  }
  for (int w = cta ? ns : warp; w < ns; w += nw) {
    const int g = rd.wk + w;
    const double* X = P.pos + rd.pos_off + (size_t)w * N * 3;
    double* M = keep_m ? mat(w) : nullptr;
    double* comp = POT == POT_EAM ? cmp(w) : nullptr;
    double e;
    if constexpr (pot_b(POT))
      e = walker_energy_b<POT, BC, ENS>(P, X, N, P.box[g], P.boxh[g], P.rc2[g], P.ca, P.cb, P.c,
                                        P.K, M, P.tan + rd.mat_off + (size_t)w * N * N, lane);
    else
      e = walker_energy64<POT, BC, ENS>(X, N, P.box[g], P.boxh[g], P.rc2[g], P.c, P.K,
                                        -0.5 * P.eam_n, -0.5 * P.eam_m,
                                        P.eam_ean, P.eam_ecam, M, comp,
                                        keep_pe ? pe(w) : nullptr, lane);
    if (lane == 0) {
      P.en[g] = e;
      P.status[g] = ST_OK;
      P.drift[g] = 0.0;
    }
  }
  __syncthreads();
  for (int w = ns + warp; w < rd.R; w += nw) {
    const int g = rd.wk + w, src = w % ns;
    if (POT == POT_EAM)
      for (int k = lane; k < 2 * N; k += 32) cmp(w)[k] = cmp(src)[k];
    if (keep_m)
      for (int k = lane; k < N * N; k += 32) mat(w)[k] = mat(src)[k];
    if (keep_pe)
      for (int k = lane; k < N * N * pe_w; k += 32) pe(w)[k] = pe(src)[k];
    if (pot_b(POT))
      for (int k = lane; k < N * N; k += 32)
        P.tan[rd.mat_off + (size_t)w * N * N + k] = P.tan[rd.mat_off + (size_t)src * N * N + k];
    if (lane == 0) {
      P.en[g] = P.en[rd.wk + src];
      P.status[g] = ST_OK;
      P.drift[g] = 0.0;
    }
  }
}

// ------------------------------------------------------------ cycle kernel
template <int POT, int BC, int ENS>
__global__ void __launch_bounds__(1024)
    k_cycles(KParams P, int run0, int ncycles, int phase) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ double s_c[MAX_COEFF];
  __shared__ double s_ca[pot_b(POT) ? MAX_COEFF : 1], s_cb[pot_b(POT) ? MAX_COEFF : 1];
  constexpr bool BPOT = pot_b(POT);
  constexpr bool KEEP_M = ENS == ENS_NPT || BPOT;  // stored distance matrix
  constexpr bool PEC = pair_cache(POT, ENS);        // NVT pair cache in HBM
  const RunDesc rd = P.runs[run0 + blockIdx.x];
  const int N = rd.N, R = rd.R;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int nthr = blockDim.x, nw = nthr >> 5;
  // a warp per walker; with more walkers than warps (R > 32) each warp makes
  // the moves of every nw-th walker in turn, its state parked in shared memory
  const bool multi = R > nw;
  const int K = P.K;
  const int n_steps = ENS == ENS_NPT ? N + 1 : N;

  // ---- carve shared memory (order matches cycles_smem_bytes) ----
  unsigned char* sp = smem_raw;
  auto carve = [&](long long bytes) {
    unsigned char* p = sp;
    sp += (bytes + 15) / 16 * 16;
    return p;
  };
  // Per-atom state (positions, EAM components, trial rows) sits in shared
  // memory, or, when a run's replicas do not fit a CTA (P.glob), in HBM:
  // the positions and components in place, the trial rows in the per-walker
  // scratch P.scr (L1/L2 serve the rows a move touches).
  const bool glob = P.glob != 0;
  const long long NA = glob ? 0 : N;  // atoms held in shared memory per walker
  double* s_pos = (double*)carve((long long)R * NA * 3 * 8);
  double2* s_c64 = nullptr;
  double2* s_t64 = nullptr;  // EAM: the trial row's (r^-n, r^-m)
  if (POT == POT_EAM) {
    s_c64 = (double2*)carve((long long)R * NA * 16);
    s_t64 = (double2*)carve((long long)R * NA * 16);
  }
  // trial row: squared distances (NPT, B potentials) or pair energies (NVT ELJ)
  double* s_row = (KEEP_M || POT != POT_EAM) ? (double*)carve((long long)R * NA * 8) : nullptr;
  double* s_trow = BPOT ? (double*)carve((long long)R * NA * 8) : nullptr;
  double* s_drw = (double*)carve((long long)R * DRAW_BUF * 8);
  double* s_beta = (double*)carve((long long)R * 8);
  double* s_maxbox = (double*)carve((long long)R * 8);
  double* s_en = (double*)carve((long long)R * 8);
  double* s_box = (double*)carve((long long)R * 8);
  double* s_ham = (double*)carve((long long)R * 16);
  double* s_maxd = (double*)carve((long long)R * 16);
  long long* s_cnt = (long long*)carve((long long)R * 48);
  int* s_wos = (int*)carve((long long)R * 4);
  int* s_sow = (int*)carve((long long)R * 4);
  double* s_boxh = (double*)carve((long long)R * 8);
  double* s_maxboxh = (double*)carve((long long)R * 8);
  double* s_maxd_sep = (double*)carve((long long)R * 16);
  long long* s_cnt_sep = (long long*)carve((long long)R * 32);
  // walker state besides en / box / box height (s_en, s_box, s_boxh)
  double* s_wrc2 = (double*)carve((long long)R * 8);
  double* s_wdrift = (double*)carve((long long)R * 8);
  unsigned long long* s_wctr = (unsigned long long*)carve((long long)R * 8);
  unsigned long long* s_wbase = (unsigned long long*)carve((long long)R * 8);
  int* s_wst = (int*)carve((long long)R * 4);

  // ---- load the run into shared memory ----
  if (tid < K) {
    s_c[tid] = P.c[tid];
    if (BPOT) {
      s_ca[tid] = P.ca[tid];
      s_cb[tid] = P.cb[tid];
    }
  }
  const double* gpos = P.pos + rd.pos_off;
  if (!glob) for (int k = tid; k < R * N * 3; k += nthr) s_pos[k] = gpos[k];
  if (POT == POT_EAM && !glob) {
    const double* gc = P.comp + rd.comp_off;
    for (int k = tid; k < R * N; k += nthr) s_c64[k] = make_double2(gc[2 * k], gc[2 * k + 1]);
  }
  for (int s = tid; s < R; s += nthr) {
    int g = rd.wk + s;
    s_beta[s] = P.beta[g];
    s_maxbox[s] = P.maxbox[g];
    s_ham[2 * s] = P.ham[2 * g];
    s_ham[2 * s + 1] = P.ham[2 * g + 1];
    s_maxd[2 * s] = P.maxd[2 * g];
    s_maxd[2 * s + 1] = P.maxd[2 * g + 1];
    for (int q = 0; q < 6; ++q) s_cnt[6 * s + q] = P.cnt[6 * (size_t)g + q];
    s_wos[s] = P.wos[g];
    // walker s's state
    s_en[s] = P.en[g];
    s_box[s] = P.box[g];
    s_boxh[s] = has_height<BC>() ? P.boxh[g] : P.box[g];
    s_wrc2[s] = P.rc2[g];
    s_wdrift[s] = P.drift[g];
    s_wctr[s] = P.ctr[g];
    s_wbase[s] = P.ctr[g] + DRAW_BUF;  // forces a refill on the first draw
    s_wst[s] = P.status[g];
    if (has_height<BC>()) {
      s_maxboxh[s] = P.maxboxh[g];
      s_maxd_sep[2 * s] = P.maxd_sep[2 * g];
      s_maxd_sep[2 * s + 1] = P.maxd_sep[2 * g + 1];
      for (int q = 0; q < 4; ++q) s_cnt_sep[4 * s + q] = P.cnt_sep[4 * (size_t)g + q];
    }
  }
  __syncthreads();
  for (int s = tid; s < R; s += nthr) s_sow[s_wos[s]] = s;
  __syncthreads();

  // ---- the current walker's registers (warp-uniform) ----
  int w = warp;  // walker within the run
  double en, L, H, rc2, drift;  // H: box height (RectangularBC, RhombicBC)
  unsigned long long ctr, base;
  int status;
  double *X, *drw, *M, *PE, *TM, *row, *trow;
  double2 *C2 = nullptr, *T2w = nullptr;  // EAM components and trial terms of the walker
  auto bind = [&](int v) {  // pointers of walker v
    w = v;
    X = glob ? P.pos + rd.pos_off + (size_t)v * N * 3 : s_pos + (size_t)v * N * 3;
    drw = s_drw + v * DRAW_BUF;
    M = KEEP_M ? P.mat + rd.mat_off + (size_t)v * N * N : nullptr;
    // NVT pair cache of this walker: ELJ V(r_ij), EAM (r_ij^-n, r_ij^-m)
    PE = PEC ? P.pe + rd.pe_off + (size_t)v * N * N * (POT == POT_EAM ? 2 : 1) : nullptr;
    TM = BPOT ? P.tan + rd.mat_off + (size_t)v * N * N : nullptr;  // tangent matrix
    // HBM scratch of walker v: trial row [N], tangent row [N], EAM trial terms [2N]
    double* scr = glob ? P.scr + (size_t)(rd.wk + v) * P.scr_stride : nullptr;
    if (KEEP_M || POT != POT_EAM) row = glob ? scr : s_row + (size_t)v * N;
    else row = nullptr;
    trow = BPOT ? (glob ? scr + N : s_trow + (size_t)v * N) : nullptr;
    if (POT == POT_EAM) {
      C2 = glob ? (double2*)(P.comp + rd.comp_off) + (size_t)v * N : s_c64 + (size_t)v * N;
      T2w = glob ? (double2*)(scr + 2 * (size_t)N) : s_t64 + (size_t)v * N;
    }
  };
  auto load = [&](int v) {  // walker v's state from shared memory
    bind(v);
    en = s_en[v];
    L = s_box[v];
    H = s_boxh[v];
    rc2 = s_wrc2[v];
    drift = s_wdrift[v];
    ctr = s_wctr[v];
    base = s_wbase[v];
    status = s_wst[v];
  };
  auto save = [&]() {  // the current walker's state to shared memory (lane 0)
    if (lane == 0) {
      s_en[w] = en;
      s_box[w] = L;
      s_boxh[w] = H;
      s_wrc2[w] = rc2;
      s_wdrift[w] = drift;
      s_wctr[w] = ctr;
      s_wbase[w] = base;
      s_wst[w] = status;
    }
    __syncwarp();
  };
  if (warp < R) load(warp);
  const double hn = -0.5 * P.eam_n, hm = -0.5 * P.eam_m;
  const double ean = P.eam_ean, ecam = P.eam_ecam;
  const uint32_t run_word = (uint32_t)rd.run_id;

  // draw from this walker's stream (all lanes in lockstep)
  auto draw = [&]() -> double {
    if (ctr - base >= (unsigned long long)DRAW_BUF) {
      __syncwarp();
      base = ctr & ~1ull;
      if (lane < DRAW_BUF / 2) {
        double u0, u1;
        philox_pair(P.seed, (uint32_t)w, run_word, (base >> 1) + lane, u0, u1);
        drw[2 * lane] = u0;
        drw[2 * lane + 1] = u1;
      }
      __syncwarp();
    }
    double u = drw[ctr - base];
    ++ctr;
    return u;
  };

  // ---------------------------------------------------------- atom move
  // mc_move! with an "atommove" slot (src/MCRun.jl:142-162)
  auto atom_move = [&](int i, double beta, double md) -> int {
    double xi = X[3 * i], yi = X[3 * i + 1], zi = X[3 * i + 2];
    double tx, ty, tz;
    auto propose = [&]() {  // atom_displacement (src/MCMoves.jl:33-64)
      double ux = draw(), uy = draw(), uz = draw();
      tx = dadd(xi, dmul(dsub(ux, 0.5), md));
      ty = dadd(yi, dmul(dsub(uy, 0.5), md));
      tz = dadd(zi, dmul(dsub(uz, 0.5), md));
    };
    propose();
    if (BC == BC_SPH) {  // spherical retry loop (src/MCMoves.jl:117-136)
      const double R2 = dmul(L, L);
      int count = 0;
      while (dot3(tx, ty, tz) > R2) {
        ++count;
        if (count == 50) {  // recentre! (src/Configurations.jl:79-85)
          double sx = 0, sy = 0, sz = 0;
          for (int a = lane; a < N; a += 32) {
            sx += X[3 * a];
            sy += X[3 * a + 1];
            sz += X[3 * a + 2];
          }
          sx = warp_sum(sx) / N;
          sy = warp_sum(sy) / N;
          sz = warp_sum(sz) / N;
          __syncwarp();
          for (int a = lane; a < N; a += 32) {
            X[3 * a] -= sx;
            X[3 * a + 1] -= sy;
            X[3 * a + 2] -= sz;
          }
          __syncwarp();
          xi = X[3 * i];
          yi = X[3 * i + 1];
          zi = X[3 * i + 2];
        } else {
          propose();
          if (count == 100) {
            status = ST_SPHERE;
            return 0;
          }
        }
      }
    } else if (BC == BC_RHB) {  // rhombic wrap (src/MCMoves.jl:66-83)
      const double ky = rint(ddiv(dsub(ty, ddiv(dmul(L, SQRT3), 4.0)), ddiv(dmul(L, SQRT3), 2.0)));
      const double sx = dadd(dmul(L, rint(ddiv(dsub(dsub(tx, ddiv(ty, SQRT3)), ddiv(L, 2.0)), L))),
                             dmul(ddiv(L, 2.0), ky));
      const double sy = dmul(ddiv(dmul(L, SQRT3), 2.0), ky);
      const double sz = dmul(H, rint(ddiv(dsub(tz, ddiv(H, 2.0)), H)));
      tx = dsub(tx, sx);
      ty = dsub(ty, sy);
      tz = dsub(tz, sz);
    } else {  // periodic wrap (src/MCMoves.jl:50-64, 85-98)
      tx = dsub(tx, dmul(L, rint(ddiv(tx, L))));
      ty = dsub(ty, dmul(L, rint(ddiv(ty, L))));
      tz = dsub(tz, dmul(H, rint(ddiv(tz, H))));
    }

    double new_en;
    double sa = 0.0, sb = 0.0;  // EAM: sum of component deltas of atom i
    if (BPOT) {  // energy_update! for the B potentials (src/EnergyEvaluation.jl:1508-1564)
      double e_n = 0.0, e_o = 0.0;
      const double* Mi = M + (size_t)i * N;
      const double* Ti = TM + (size_t)i * N;
      for (int j = lane; j < N; j += 32) {
        if (j == i) {
          row[j] = 0.0;
          trow[j] = 0.0;
          continue;
        }
        const double dn = pd2<BC>(tx, ty, tz, X + 3 * j, L, H);
        const double tn = ptan<BC>(tx, ty, tz, X + 3 * j, L, H);
        row[j] = dn;
        trow[j] = tn;
        const double dol = Mi[j], tol = Ti[j];
        if (ENS != ENS_NPT || dn <= rc2) e_n += vb<POT>(P, s_ca, s_cb, s_c, K, dn, tn);
        if (ENS != ENS_NPT || dol <= rc2) e_o += vb<POT>(P, s_ca, s_cb, s_c, K, dol, tol);
      }
      e_n = warp_sum(e_n);
      e_o = warp_sum(e_o);
      new_en = (e_n - e_o) + en;
    } else if (POT == POT_ELJ || POT == POT_ELJEVEN) {
      // dimer_energy_update! (src/EnergyEvaluation.jl:804-821)
      double e_n = 0.0, e_o = 0.0;
      const double* Mi = M ? M + (size_t)i * N : nullptr;
      const double* Ei = PE ? PE + (size_t)i * N : nullptr;
      for (int j = lane; j < N; j += 32) {
        if (j == i) {
          row[j] = 0.0;
          continue;
        }
        const double dn = pd2<BC>(tx, ty, tz, X + 3 * j, L, H);
        if (ENS == ENS_NPT) {
          const double dol = Mi[j];
          row[j] = dn;
          if (dn <= rc2) e_n += v64<POT>(s_c, K, dn);
          if (dol <= rc2) e_o += v64<POT>(s_c, K, dol);
        } else if (PEC) {  // trial pair energies; the old ones from the cache
          const double vn = v64<POT>(s_c, K, dn);
          row[j] = vn;
          e_n += vn;
          e_o += Ei[j];
        } else {  // RectangularBC / RhombicBC in NVT: old distances from positions
          e_n += v64<POT>(s_c, K, dn);
          e_o += v64<POT>(s_c, K, pd2<BC>(xi, yi, zi, X + 3 * j, L, H));
        }
      }
      e_n = warp_sum(e_n);
      e_o = warp_sum(e_o);
      new_en = (e_n - e_o) + en;
    } else {  // EAM energy_update! (src/EnergyEvaluation.jl:1567-1591)
      // calc_components (:1105-1148): the trial row's (r^-n, r^-m); the old
      // ones from the pair cache
      double2* C = C2;
      double2* T2 = T2w;
      const double2* Ei = (const double2*)PE + (size_t)i * N;
      for (int j = lane; j < N; j += 32) {
        if (j == i) {
          T2[j] = make_double2(0.0, 0.0);
          continue;
        }
        double dn = pd2<BC>(tx, ty, tz, X + 3 * j, L, H);
        double a1, b1;
        invrexp64(dn, hn, hm, a1, b1);
        const double2 o = Ei[j];
        T2[j] = make_double2(a1, b1);
        sa += a1 - o.x;
        sb += b1 - o.y;
      }
      sa = warp_sum(sa);
      sb = warp_sum(sb);
      double e = 0.0;  // calc_energies_from_components (:1156-1162)
      for (int k = lane; k < N; k += 32) {  // lane k reads only what lane k wrote
        double2 c = C[k];
        double2 d = make_double2(sa, sb);
        if (k != i) {
          const double2 t = T2[k], o = Ei[k];
          d = make_double2(t.x - o.x, t.y - o.y);
        }
        e += ean * (c.x + d.x) - ecam * sqrt(c.y + d.y);
      }
      new_en = warp_sum(e);
    }

    // acc_test! / metropolis_condition (src/MCRun.jl:122-132, Exchange.jl:53-57)
    double prob = exp(-(new_en - en) * beta);
    if (prob > 1) prob = 1.0;
    double u = draw();
    if (!(prob >= u)) return 0;
    // swap_atom_config! (src/swap_config.jl:40-51)
    __syncwarp();
    if (lane == 0) {
      X[3 * i] = tx;
      X[3 * i + 1] = ty;
      X[3 * i + 2] = tz;
    }
    if (M) {
      for (int j = lane; j < N; j += 32) {
        double v = row[j];
        M[(size_t)i * N + j] = v;
        M[(size_t)j * N + i] = v;
        if (BPOT) {  // swap_vars! B potentials (src/swap_config.jl:198-206)
          TM[(size_t)i * N + j] = trow[j];
          TM[(size_t)j * N + i] = trow[j];
        }
      }
    }
    if (POT == POT_EAM) {  // swap_vars! EAM (src/swap_config.jl:208-211)
      double2* C = C2;
      const double2* T2 = T2w;
      double2* PE2 = (double2*)PE;
      for (int k = lane; k < N; k += 32) {
        double2 c = C[k];
        if (k == i) {
          C[k] = make_double2(c.x + sa, c.y + sb);
          continue;
        }
        // each lane reads its old cache entries before it overwrites them
        const double2 t = T2[k], o = PE2[(size_t)i * N + k];
        C[k] = make_double2(c.x + (t.x - o.x), c.y + (t.y - o.y));
        PE2[(size_t)i * N + k] = t;  // pair cache: row and column of atom i
        PE2[(size_t)k * N + i] = t;
      }
    } else if (PEC) {
      for (int j = lane; j < N; j += 32) {
        if (j == i) continue;
        const double v = row[j];
        PE[(size_t)i * N + j] = v;
        PE[(size_t)j * N + i] = v;
      }
    }
    en = new_en;
    __syncwarp();
    return 1;
  };

  // ---------------------------------------------------------- volume move
  // volume_change (src/MCMoves.jl:350-356), NPT energy (src/MCRun.jl:76-85),
  // metropolis_condition NPT (src/Exchange.jl:58-70), swap_config_v!
  // (src/swap_config.jl:113-141).  Always FP64.  Uniform moves
  // (volume_change_uniform, :277-287) scale the distance matrix by scale^2;
  // separated moves (volume_change_separated, :298-343; RectangularBC and
  // RhombicBC) draw rand(1:6) for z (1), xy (2-3) or all directions (4-6) and
  // evaluate the trial energy from the scaled positions; the distance matrix is
  // rebuilt from the new positions when the move is accepted.  Returns the
  // accepted kind + 1 (1 all directions, 2 xy, 3 z), 0 when rejected.
  auto volume_move = [&](double beta, int slot, double mdv, double maxbox) -> int {
    int kind = 0;
    double fx = 1.0, fz = 1.0, Ln = L, Hn = H;
    auto change_xyz = [&]() {  // volume_change_xyz (src/MCMoves.jl:169-177)
      double u = draw();
      double scale = pow(exp((u - 0.5) * mdv), 1.0 / 3.0);
      if (L >= maxbox && scale > 1.0) scale = 1.0;
      fx = fz = scale;
      Ln = scale * L;
      Hn = has_height<BC>() ? scale * H : Ln;
    };
    const bool sep = has_height<BC>() && P.sep_vol;
    if (sep) {
      const double maxboxh = s_maxboxh[slot];
      const double lh = maxbox / maxboxh;  // lh_ratio (src/MCStates.jl:103)
      const double ratio = L / H;
      const int ra = randint(draw(), 6) + 1;
      if (ra == 1) {  // volume_change_z (src/MCMoves.jl:257-271)
        kind = 2;
        double u = draw();
        double scale = exp((u - 0.5) * s_maxd_sep[2 * slot + 1]);
        if (ratio <= lh * 1.1 && scale > 1.0) scale = 1 / scale;
        else if (ratio >= lh * 0.909 && scale < 1.0) scale = 1 / scale;
        if (H >= maxboxh && scale > 1.0) scale = 1 / scale;
        fz = scale;
        Hn = H * scale;
      } else if (ra <= 3) {  // volume_change_xy (src/MCMoves.jl:231-247)
        kind = 1;
        double u = draw();
        double scale = pow(exp((u - 0.5) * s_maxd_sep[2 * slot]), 0.5);
        if (ratio >= lh * 1.1 && scale > 1.0) scale = 1 / scale;
        else if (ratio <= lh * 0.909 && scale < 1.0) scale = 1 / scale;
        if (L >= maxbox && scale > 1.0) scale = 1 / scale;
        fx = scale;
        Ln = L * scale;
      } else {
        change_xyz();
      }
    } else {
      change_xyz();
    }
    const double rcn = box_rcut<BC>(Ln, Hn);
    const double s2 = fx * fx;
    // the pair energy of a trial pair: B potentials take the tangent of the
    // trial (separated z / xy moves, get_tantheta_mat!) or the current one
    auto pair_e = [&](double x, int i, int j, const double* a3, const double* b3) -> double {
      if constexpr (BPOT) {
        const double t = (sep && kind != 0) ? ptan<BC>(a3[0], a3[1], a3[2], b3, Ln, Hn)
                                            : TM[(size_t)i * N + j];
        return vb<POT>(P, s_ca, s_cb, s_c, K, x, t);
      } else {
        return v64<POT>(s_c, K, x);
      }
    };
    double e = 0.0;
    if (!sep) {
      for (int i = 0; i < N; ++i)
        for (int j = i + 1 + lane; j < N; j += 32) {
          double x = M[(size_t)i * N + j] * s2;
          if (x <= rcn) e += pair_e(x, i, j, nullptr, nullptr);
        }
    } else {
      for (int i = 0; i < N; ++i) {
        const double a3[3] = {X[3 * i] * fx, X[3 * i + 1] * fx, X[3 * i + 2] * fz};
        for (int j = i + 1 + lane; j < N; j += 32) {
          const double b[3] = {X[3 * j] * fx, X[3 * j + 1] * fx, X[3 * j + 2] * fz};
          double x = pd2<BC>(a3[0], a3[1], a3[2], b, Ln, Hn);
          if (x <= rcn) e += pair_e(x, i, j, a3, b);
        }
      }
    }
    if constexpr (BPOT)
      e = warp_sum(e) + lrc_b<POT, BC>(P, N, rcn, Ln, Hn);
    else
      e = warp_sum(e) + lrc_box<BC>(N, rcn, s_c, K, Ln, Hn);
    const double Vn = box_volume<BC>(Ln, Hn), Vo = box_volume<BC>(L, H);
    double dh = dadd(dsub(e, en), dmul(P.pressure, dsub(Vn, Vo)));
    double prob = exp(dadd(dmul(-dh, beta), dmul((double)N, log(Vn / Vo))));
    if (prob > 1) prob = 1.0;
    double ua = draw();
    if (!(prob >= ua)) return 0;
    __syncwarp();
    for (int a = lane; a < N; a += 32) {
      X[3 * a] = X[3 * a] * fx;
      X[3 * a + 1] = X[3 * a + 1] * fx;
      X[3 * a + 2] = X[3 * a + 2] * fz;
    }
    __syncwarp();
    if (sep) {  // get_distance2_mat! of the accepted configuration
      for (int i = 0; i < N; ++i) {
        for (int j = i + 1 + lane; j < N; j += 32) {
          double x = pd2<BC>(X[3 * i], X[3 * i + 1], X[3 * i + 2], X + 3 * j, Ln, Hn);
          M[(size_t)i * N + j] = x;
          M[(size_t)j * N + i] = x;
          if (BPOT && kind != 0) {  // tangents of z / xy moves
            double t = ptan<BC>(X[3 * i], X[3 * i + 1], X[3 * i + 2], X + 3 * j, Ln, Hn);
            TM[(size_t)i * N + j] = t;
            TM[(size_t)j * N + i] = t;
          }
        }
        if (lane == 0) M[(size_t)i * N + i] = 0.0;
      }
    } else {
      for (int k = lane; k < N * N; k += 32) M[k] = M[k] * s2;
    }
    __syncwarp();
    L = Ln;
    H = Hn;
    rc2 = rcn;
    en = e;
    __syncwarp();
    return kind + 1;
  };

  // ---------------------------------------------------------- cycles
  const long long first = rd.cyc[phase];
  unsigned long long run_ctr = rd.run_ctr;
  for (int cyc = 0; cyc < ncycles; ++cyc) {
    const long long idx = first + cyc;
    for (int wv = warp; wv < R; wv += nw) {  // this warp's walkers (one unless R > 32)
      if (multi) load(wv);
      const int slot = s_sow[w];
      const double beta = s_beta[slot];
      const double md = s_maxd[2 * slot], mdv = s_maxd[2 * slot + 1];
      const double maxbox = s_maxbox[slot];
      long long acc_a = 0, acc_v = 0, acc_xy = 0, acc_z = 0;
      if (status == ST_OK) {
        for (int st = 0; st < n_steps; ++st) {
          int k = randint(draw(), n_steps);
          if (k < N) {
            acc_a += atom_move(k, beta, md);
          } else {
            const int v = volume_move(beta, slot, mdv, maxbox);
            acc_v += v == 1;
            acc_xy += v == 2;
            acc_z += v == 3;
          }
          if (status != ST_OK) break;
        }
      }
      if (lane == 0) {
        s_en[w] = en;
        s_box[w] = L;
        s_boxh[w] = H;
        s_cnt[6 * slot + 0] += acc_a;
        s_cnt[6 * slot + 1] += acc_a;
        s_cnt[6 * slot + 2] += acc_v;
        s_cnt[6 * slot + 3] += acc_v;
        if (has_height<BC>()) {  // count_vol_xy, count_vol_z
          s_cnt_sep[4 * slot + 0] += acc_xy;
          s_cnt_sep[4 * slot + 1] += acc_xy;
          s_cnt_sep[4 * slot + 2] += acc_z;
          s_cnt_sep[4 * slot + 3] += acc_z;
        }
      }
      if (multi) save();
    }
    __syncthreads();
    if (tid == 0 && R > 1) {  // parallel_tempering_exchange! (src/Exchange.jl:132-180)
      double u = philox_u01(P.seed, 0xFFFFFFFFu, run_word, run_ctr++);
      if (u < P.exch_prob) {
        int k = randint(philox_u01(P.seed, 0xFFFFFFFFu, run_word, run_ctr++), R - 1);
        s_cnt[6 * k + 4] += 1;
        s_cnt[6 * (k + 1) + 4] += 1;
        int w1 = s_wos[k], w2 = s_wos[k + 1];
        double e1 = s_en[w1], e2 = s_en[w2];
        if (ENS == ENS_NPT) {  // enthalpies with get_volume (src/Exchange.jl:166-176)
          e1 = dadd(e1, dmul(P.pressure, box_volume<BC>(s_box[w1], s_boxh[w1])));
          e2 = dadd(e2, dmul(P.pressure, box_volume<BC>(s_box[w2], s_boxh[w2])));
        }
        double acc = exp((s_beta[k] - s_beta[k + 1]) * (e1 - e2));
        if (acc > 1.0) acc = 1.0;
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
      const int s = tid;
      if (idx % P.n_adjust == 0) {  // update_max_stepsize!
        double acc = (double)s_cnt[6 * s + 1] / (double)((long long)P.n_adjust * N);
        if (acc < P.min_acc) s_maxd[2 * s] *= 0.9;
        else if (acc > P.max_acc) s_maxd[2 * s] *= 1.1;
        s_cnt[6 * s + 1] = 0;
        if (ENS == ENS_NPT && !(has_height<BC>() && P.sep_vol)) {
          double av = (double)s_cnt[6 * s + 3] / (double)(P.n_adjust * 1);
          if (av < P.min_acc) s_maxd[2 * s + 1] *= 0.9;
          else if (av > P.max_acc) s_maxd[2 * s + 1] *= 1.1;
          s_cnt[6 * s + 3] = 0;
        } else if (ENS == ENS_NPT) {  // separated: all, xy, z (src/Exchange.jl:221-244)
          const double nu = (double)(P.n_adjust * 1);
          auto adapt = [&](long long& c, double& mdx, double den) {
            double av = (double)c / den;
            if (av < P.min_acc) mdx *= 0.9;
            else if (av > P.max_acc) mdx *= 1.1;
            c = 0;
          };
          adapt(s_cnt[6 * s + 3], s_maxd[2 * s + 1], nu * 1 / 2);
          adapt(s_cnt_sep[4 * s + 1], s_maxd_sep[2 * s], nu * 1 / 3);
          adapt(s_cnt_sep[4 * s + 3], s_maxd_sep[2 * s + 1], nu / 6);
        }
      }
      if (phase == PHASE_PROD && idx % P.mc_sample == 0) {  // sampling_step!
        const int wk = s_wos[s];
        const double e = s_en[wk];
        const int nb = P.n_bin;
        unsigned int* hrow = P.hist + rd.hist_off + (size_t)s * rd.hist_stride;
        auto hidx = [&](double h) -> int {  // find_hist_index (Sampling.jl:53-62)
          if (!(h >= 1)) return 1;          // also catches NaN (the reference throws)
          if (h > nb) return nb + 2;
          return (int)floor(h) + 1;
        };
        if (ENS == ENS_NPT) {
          const double Lw = s_box[wk], Hw = s_boxh[wk];
          double V = box_volume<BC>(Lw, Hw);
          double Hs = dadd(e, dmul(P.pressure, V));
          s_ham[2 * s] += Hs;
          s_ham[2 * s + 1] = dadd(s_ham[2 * s + 1], dmul(Hs, Hs));
          int ie = hidx(floor((e - rd.en_min) / rd.dE) + 1);
          int iv = hidx(floor((hist_volume<BC>(Lw, Hw) - rd.v_min) / rd.dV) + 1);
          atomicAdd(hrow + (size_t)(ie - 1) * (nb + 2) + (iv - 1), 1u);
        } else {
          s_ham[2 * s] += e;
          s_ham[2 * s + 1] = dadd(s_ham[2 * s + 1], dmul(e, e));
          int ie = hidx((e - rd.en_min) / rd.dE + 1);
          atomicAdd(hrow + (ie - 1), 1u);
        }
      }
    }
    __syncthreads();
    if (P.rdf && phase == PHASE_PROD && idx % P.mc_sample == 0 && idx % RDF_EVERY == 0) {
      // update_rdf!: pairs k < i of each walker into the row of its slot; NPT
      // reads the distance matrix (scaled on volume moves, as the reference's)
      for (int wv = warp; wv < R; wv += nw) {
        if (multi) load(wv);
        unsigned int* hrow = P.rdf + (size_t)(rd.wk + s_sow[w]) * 5 * P.n_bin;
        for (int i = 1; i < N; ++i)
          for (int k = lane; k < i; k += 32) {
            double r2;
            if (M) r2 = M[(size_t)i * N + k];
            else
              r2 = pd2<BC>(X[3 * i], X[3 * i + 1], X[3 * i + 2], X + 3 * k, L, H);
            rdf_add(hrow, 5 * P.n_bin, r2, rd.dr2);
          }
      }
    }
  }

  // ---- store the run back to HBM ----
  if (!multi) save();  // the warps' walker registers to shared memory
  __syncthreads();
  double* gpos_w = P.pos + rd.pos_off;
  if (!glob) for (int k = tid; k < R * N * 3; k += nthr) gpos_w[k] = s_pos[k];
  if (POT == POT_EAM && !glob) {
    double* gc = P.comp + rd.comp_off;
    for (int k = tid; k < R * N; k += nthr) {
      gc[2 * k] = s_c64[k].x;
      gc[2 * k + 1] = s_c64[k].y;
    }
  }
  for (int s = tid; s < R; s += nthr) {  // walker s's state
    const int gw = rd.wk + s;
    P.en[gw] = s_en[s];
    P.box[gw] = s_box[s];
    if (has_height<BC>()) P.boxh[gw] = s_boxh[s];
    P.rc2[gw] = s_wrc2[s];
    P.ctr[gw] = s_wctr[s];
    P.status[gw] = s_wst[s];
    P.drift[gw] = s_wdrift[s];
  }
  for (int s = tid; s < R; s += nthr) {
    int gs = rd.wk + s;
    P.ham[2 * gs] = s_ham[2 * s];
    P.ham[2 * gs + 1] = s_ham[2 * s + 1];
    P.maxd[2 * gs] = s_maxd[2 * s];
    P.maxd[2 * gs + 1] = s_maxd[2 * s + 1];
    for (int q = 0; q < 6; ++q) P.cnt[6 * (size_t)gs + q] = s_cnt[6 * s + q];
    P.wos[gs] = s_wos[s];
    if (has_height<BC>()) {
      P.maxd_sep[2 * gs] = s_maxd_sep[2 * s];
      P.maxd_sep[2 * gs + 1] = s_maxd_sep[2 * s + 1];
      for (int q = 0; q < 4; ++q) P.cnt_sep[4 * (size_t)gs + q] = s_cnt_sep[4 * s + q];
    }
  }
  if (tid == 0) {
    P.runs[run0 + blockIdx.x].cyc[phase] = first + ncycles;
    P.runs[run0 + blockIdx.x].run_ctr = run_ctr;
  }
}

// FP32 form: explicit FP64 recompute of every walker (ptmc_resync)
template <int POT, int BC, int ENS, bool F32>
__global__ void __launch_bounds__(1024) k_resync(KParams P, int run0) {
  const RunDesc rd = P.runs[run0 + blockIdx.x];
  const int N = rd.N, warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  for (int w = warp; w < rd.R; w += nw) {  // every nw-th walker
    const int g = rd.wk + w;
    const double* X = P.pos + rd.pos_off + (size_t)w * N * 3;
    double* comp = POT == POT_EAM ? P.comp + rd.comp_off + (size_t)w * N * 2 : nullptr;
    double e;
    if constexpr (pot_b(POT))
      e = walker_energy_b<POT, BC, ENS>(P, X, N, P.box[g], P.boxh[g], P.rc2[g], P.ca, P.cb, P.c,
                                        P.K, P.mat + rd.mat_off + (size_t)w * N * N,
                                        P.tan + rd.mat_off + (size_t)w * N * N, lane);
    else
      e = walker_energy64<POT, BC, ENS>(X, N, P.box[g], P.boxh[g], P.rc2[g], P.c, P.K,
                                        -0.5 * P.eam_n, -0.5 * P.eam_m,
                                        P.eam_ean, P.eam_ecam, nullptr, comp,
                                        nullptr, lane);
    if (lane == 0) {
      P.drift[g] = fmax(P.drift[g], fabs(P.en[g] - e));
      P.en[g] = e;
    }
  }
}

// ------------------------------------------------------------ dispatch
// opt in to more than 48 KB of dynamic shared memory when needed, within the
// device limit minus the kernel's static shared memory; the attribute belongs
// to the current device's context, so it is recorded per device, and it is
// only ever raised (a later launch with more shared memory raises it again)
template <int POT, int BC, int ENS>
static int opt_in64(long long smem) {
  static long long attr_set[MAX_DEVICES] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return (int)e;
  if (dev < 0 || dev >= MAX_DEVICES) return (int)cudaErrorInvalidDevice;
  if (smem <= 48 * 1024 || smem <= attr_set[dev]) return 0;
  int optin = 0;
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  cudaFuncAttributes fa;
  e = cudaFuncGetAttributes(&fa, k_cycles<POT, BC, ENS>);
  if (e != cudaSuccess) return (int)e;
  if (smem + (long long)fa.sharedSizeBytes > optin) return (int)cudaErrorInvalidValue;
  e = cudaFuncSetAttribute(k_cycles<POT, BC, ENS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)smem);
  if (e != cudaSuccess) return (int)e;
  attr_set[dev] = smem;
  return 0;
}

// what: 0 cycle kernel launch, 1 k_init, 2 k_resync, 3 occupancy query of the
// cycle kernel (resident CTAs per SM into *occ)
template <int POT, int BC, int ENS, bool F32>
static int run_instance(int what, const KParams& P, int run0, int nruns, int R,
                        int maxN, int ncycles, int phase, cudaStream_t st, int* occ) {
  // a warp per walker, at most 32 warps (a warp then serves several walkers)
  dim3 grid(nruns), block((R < 32 ? R : 32) * 32);
  if constexpr (F32) {
    if (what == 0 || what == 3) return (int)cudaErrorInvalidValue;  // FP32 form: ptmc_cycles32.cu
  } else if (what == 0 || what == 3) {
    // with the per-atom state in HBM (P.glob) only the slot and walker tables
    // are in shared memory
    const long long smem = cycles_smem_bytes(POT, ENS, false, R, P.glob ? 0 : maxN);
    const int e = opt_in64<POT, BC, ENS>(smem);
    if (e) return e;
    if (what == 3)
      return (int)cudaOccupancyMaxActiveBlocksPerMultiprocessor(occ, k_cycles<POT, BC, ENS>,
                                                                (int)block.x, (size_t)smem);
    k_cycles<POT, BC, ENS><<<grid, block, (size_t)smem, st>>>(P, run0, ncycles, phase);
    return (int)cudaGetLastError();
  }
  if (what == 1) {
    k_init<POT, BC, ENS, F32><<<grid, block, 0, st>>>(P, run0);
  } else {
    k_resync<POT, BC, ENS, F32><<<grid, block, 0, st>>>(P, run0);
  }
  return (int)cudaGetLastError();
}

template <int POT, int BC, int ENS>
static int run_prec(bool f32, int what, const KParams& P, int run0, int nruns,
                    int R, int maxN, int ncycles, int phase, cudaStream_t st, int* occ) {
  return f32 ? run_instance<POT, BC, ENS, true>(what, P, run0, nruns, R, maxN, ncycles, phase, st, occ)
             : run_instance<POT, BC, ENS, false>(what, P, run0, nruns, R, maxN, ncycles, phase, st, occ);
}

static int dispatch(int pot, int bc, int ens, bool f32, int what,
                    const KParams& P, int run0, int nruns, int R, int maxN,
                    int ncycles, int phase, void* stream, int* occ = nullptr) {
  cudaStream_t st = (cudaStream_t)stream;
#define PT_CASE(PO, B, E)                                                  \
  if (pot == PO && bc == B && ens == E)                                    \
    return run_prec<PO, B, E>(f32, what, P, run0, nruns, R, maxN, ncycles, \
                              phase, st, occ);
  PT_CASE(POT_ELJ, BC_SPH, ENS_NVT)
  PT_CASE(POT_ELJEVEN, BC_SPH, ENS_NVT)
  PT_CASE(POT_EAM, BC_SPH, ENS_NVT)
  PT_CASE(POT_ELJ, BC_CUB, ENS_NVT)
  PT_CASE(POT_ELJEVEN, BC_CUB, ENS_NVT)
  PT_CASE(POT_EAM, BC_CUB, ENS_NVT)
  PT_CASE(POT_ELJEVEN, BC_CUB, ENS_NPT)
#undef PT_CASE
  // RectangularBC / RhombicBC: plain FP64 form only
#define PT_CASE64(PO, B, E)                                                              \
  if (pot == PO && bc == B && ens == E)                                                  \
    return f32 ? (int)cudaErrorInvalidValue                                              \
               : run_instance<PO, B, E, false>(what, P, run0, nruns, R, maxN, ncycles,   \
                                               phase, st, occ);
  PT_CASE64(POT_ELJ, BC_RECT, ENS_NVT)
  PT_CASE64(POT_ELJEVEN, BC_RECT, ENS_NVT)
  PT_CASE64(POT_ELJ, BC_RHB, ENS_NVT)
  PT_CASE64(POT_ELJEVEN, BC_RHB, ENS_NVT)
  PT_CASE64(POT_ELJEVEN, BC_RECT, ENS_NPT)
  PT_CASE64(POT_ELJEVEN, BC_RHB, ENS_NPT)
  // ELJPotentialB and LookupTablePotential: plain FP64 form
  PT_CASE64(POT_ELJB, BC_SPH, ENS_NVT)
  PT_CASE64(POT_ELJB, BC_CUB, ENS_NVT)
  PT_CASE64(POT_ELJB, BC_CUB, ENS_NPT)
  PT_CASE64(POT_ELJB, BC_RECT, ENS_NPT)
  PT_CASE64(POT_ELJB, BC_RHB, ENS_NPT)
  PT_CASE64(POT_LUT, BC_SPH, ENS_NVT)
  PT_CASE64(POT_LUT, BC_CUB, ENS_NVT)
  PT_CASE64(POT_LUT, BC_CUB, ENS_NPT)
  PT_CASE64(POT_LUT, BC_RECT, ENS_NPT)
  PT_CASE64(POT_LUT, BC_RHB, ENS_NPT)
#undef PT_CASE64
  return -1;
}

int launch_cycles(int pot, int bc, int ens, bool f32, const KParams& P,
                  int run0, int nruns, int R, int maxN, int ncycles, int phase,
                  void* stream, int ncta, int lpr) {
  if (f32) return launch_cycles32(pot, bc, ens, P, run0, nruns, R, maxN, ncycles, phase, ncta, lpr, stream);
  return dispatch(pot, bc, ens, false, 0, P, run0, nruns, R, maxN, ncycles, phase, stream);
}
int launch_init(int pot, int bc, int ens, bool f32, const KParams& P, int run0,
                int nruns, int R, void* stream) {
  return dispatch(pot, bc, ens, f32, 1, P, run0, nruns, R, 0, 0, 0, stream);
}
int launch_resync(int pot, int bc, int ens, bool f32, const KParams& P,
                  int run0, int nruns, int R, void* stream) {
  return dispatch(pot, bc, ens, f32, 2, P, run0, nruns, R, 0, 0, 0, stream);
}
int occupancy_cycles(int pot, int bc, int ens, int R, int N, int* ctas_per_sm) {
  KParams P{};
  return dispatch(pot, bc, ens, false, 3, P, 0, 0, R, N, 0, 0, nullptr, ctas_per_sm);
}

}  // namespace ptmc
