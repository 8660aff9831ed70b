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
  long long* da_cnt;  // [walkers][2]: first-stage rejections, exact evaluations
  const float* da_kappa;  // [slots] screening strength per temperature slot (0 = no screening)
  // training-record capture (exact moves only): move m of a walker in cycle c
  // is recorded when (c * N + m) % rec_every == 0, into a ring of rec_cap
  float* rec_rows;    // [rec_cap][128] distances (ptmc_surrogate.cuh row layout), NULL = off
  float* rec_y;       // [rec_cap] exact dE
  int* rec_slot;      // [rec_cap] temperature slot (within its run) of the move
  unsigned long long* rec_n;  // records written so far
  int rec_cap, rec_every;
};

size_t nn_smem_bytes(const NNParams& Q, int N, bool f64);
int nn_launch_init(const KParams& P, const NNParams& Q, int n_walkers, int maxN, bool f64,
                   void* stream);
int nn_launch_cycle(const KParams& P, const NNParams& Q, int n_walkers, int n_runs, int R,
                    int maxN, bool f64, int phase, void* stream);

}  // namespace ptmc
