// ptmc_nn2.cuh — parameters of the two-species RuNNer potential path
// (ptmc_nn2.cu), the NNVT ensemble with atom swaps.
#pragma once
#include "ptmc_engine.cuh"
#include "ptmc_nn.cuh"

namespace ptmc {

constexpr int MAX_NN2_ATOMS = 64;   // atoms per configuration
constexpr int MAX_NN2_HIDDEN = 64;  // units per hidden layer

struct NN2Params {
  int n1;             // species-1 atoms (indices 0..n1-1)
  int nrad, nang;     // radial and angular functions (2 nrad + 3 nang rows of G)
  int H1, H2;         // hidden layer widths (nodes = [2 nrad + 3 nang, H1, H2, 1])
  int n_swaps;        // atom swaps per cycle (NNVT.n_atom_swaps)
  double rcut;        // cutoff of the cutoff function (the first radial function's)
  const double* rad;  // [nrad][10]: eta, r_cut, G_offset[4], G_norm[4]
  const double* ang;  // [nang][16]: eta, lambda, zeta, r_cut, tpz[6], G_offset[6]
  const double* W1;   // species-1 network: W1[Ng][H1], b1, W2[H1][H2], b2, w3[H2], b3
  const double* W2;   // species-2 network, same layout
  const int* run_of_walker;
  const int* sow;     // slot of walker (global walker index -> slot within its run)
  long long* swaps_acc;  // [walkers] accepted swaps
};

size_t nn2_smem_bytes(const NN2Params& Q, int N);
int nn2_launch_init(const KParams& P, const NN2Params& Q, int n_walkers, int maxN, void* stream);
int nn2_launch_cycle(const KParams& P, const NN2Params& Q, const NNParams& Q1, int n_walkers,
                     int n_runs, int R, int maxN, int phase, void* stream);
// exchange, step adaptation and sampling of every run after a cycle (ptmc_nn.cu)
int nn_launch_epilogue(const KParams& P, const NNParams& Q, int n_runs, int R, int phase,
                       void* stream);

}  // namespace ptmc
