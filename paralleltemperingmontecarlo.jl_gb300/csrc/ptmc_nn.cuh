// ptmc_nn.cuh — parameters of the neural-network potential path (ptmc_nn.cu).
#pragma once
#include "ptmc_engine.cuh"
#include "ptmc_surrogate.cuh"

namespace ptmc {

constexpr int MAX_NN_ANG = 32;   // active angular symmetry functions
constexpr int MAX_NN_ATOMS = 64; // atoms per configuration on the NN path

// one active symmetry function, scaled as RadialType2 / AngularType3 with
// G_vals = [max, min] (MachineLearningPotential/SymmFunc.jl:37-44, 104-112)
struct NNSF {
  double eta, lambda, zeta;
  double gnorm, goffset, tpz;  // 1/(max-min), -min*gnorm, 2^(1-zeta)*gnorm
  int zc;                      // zeta code: 1,2,3,4,5 = zeta 1,2,4,8,16; 0 = general
  int pad;
};

// Angular function sets with a compiled cycle kernel.  Active angular
// functions are ordered by (eta, lambda, zeta); a set whose structure matches
// one below runs the table-specialised FP32 kernel: term q of a set is
// (eta group g, lambda sign, zeta = 2^e), packed as g | (lambda < 0) << 4 | e << 5.
// NN_PAT_CU55: the 26 type-111 functions of scripts/cu55.jl, eta groups
// 1e-4, 3e-3, 8e-3, 0.015, 0.025, 0.045, 0.08.
constexpr int NN_PAT_GENERIC = 0, NN_PAT_CU55 = 1;
__host__ __device__ constexpr int nn_pat_sa(int pat) { return pat == NN_PAT_CU55 ? 26 : 0; }
__host__ __device__ constexpr int nn_pat_ng(int pat) { return pat == NN_PAT_CU55 ? 7 : 0; }
__host__ __device__ constexpr int nn_pat_term(int pat, int q) {
#define T(g, neg, e) ((g) | ((neg) << 4) | ((e) << 5))
  constexpr int cu55[26] = {
      T(0, 1, 1), T(0, 0, 0),                                      // eta 1e-4
      T(1, 1, 0), T(1, 1, 1),                                      // 3e-3
      T(2, 1, 0), T(2, 1, 1), T(2, 0, 1),                          // 8e-3
      T(3, 1, 1), T(3, 1, 2), T(3, 1, 4), T(3, 0, 0),              // 0.015
      T(4, 1, 0), T(4, 1, 2), T(4, 1, 4), T(4, 0, 0), T(4, 0, 1), T(4, 0, 4),  // 0.025
      T(5, 1, 1), T(5, 1, 2), T(5, 0, 0), T(5, 0, 2), T(5, 0, 4),  // 0.045
      T(6, 1, 1), T(6, 1, 2), T(6, 0, 0), T(6, 0, 2)};             // 0.08
#undef T
  return pat == NN_PAT_CU55 && q >= 0 && q < 26 ? cu55[q] : -1;
}

struct NNParams {
  int S, SR, SA;      // active functions: all, radial (first), angular (sorted by eta)
  int H1, H2;         // hidden layer widths
  int nW;             // gathered MLP parameters: W1[S][H1], b1, W2[H1][H2], b2, w3[H2], b3
  int Nmax;           // G stride per walker
  double rcut, boundary2;
  const NNSF* sf;     // [S]
  const double* W;    // [nW]
  double* G;          // [walkers][S][Nmax]
  const int* run_of_walker;
  int* sow;           // slot of walker (global walker index -> slot within its run)
  // delayed acceptance (two-stage moves screened by the pair surrogate)
  int da;             // 1: on
  SurCfgDev sc;
  const float* surP;  // [SUR_NP] surrogate parameters
  const float* sur_tab;  // [SUR_TAB_N] phi on the grid (first stage of a move)
  float sur_tab_inv_h;   // (SUR_TAB_N - 1) / r_cut
  long long* da_cnt;  // [walkers][2]: first-stage rejections, exact evaluations
  const float* da_kappa;  // [slots] screening strength per temperature slot (0 = no screening)
  // training-record capture (exact moves only): move m of a walker in cycle c
  // is recorded when (c * N + m) % rec_every == 0, into a ring of rec_cap
  float* rec_rows;    // [rec_cap][128] distances (ptmc_surrogate.cuh row layout), NULL = off
  float* rec_y;       // [rec_cap] exact dE
  int* rec_slot;      // [rec_cap] temperature slot (within its run) of the move
  unsigned long long* rec_n;  // records written so far
  int rec_cap, rec_every;
  // table-specialised angular kernel (FP32 form): pattern, -eta*log2(e) per eta group
  int ang_pat;
  float ang_nle[8];
};

size_t nn_smem_bytes(const NNParams& Q, int N, bool f64);
int nn_launch_init(const KParams& P, const NNParams& Q, int n_walkers, int maxN, bool f64,
                   void* stream);
int nn_launch_cycle(const KParams& P, const NNParams& Q, int n_walkers, int n_runs, int R,
                    int maxN, bool f64, int phase, void* stream);

}  // namespace ptmc
