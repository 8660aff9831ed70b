/*
 * ptmc_oracle.h — CPU ORACLE for the parallel-tempering Monte Carlo hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is a plain FP64 C++17 restatement of
 * ParallelTemperingMonteCarlo.jl's replica cycle (moves, energies, Metropolis,
 * exchange, step adaptation, sampling, multihistogram).  It is the checker the
 * GPU engine is compared against; it is never linked into, loaded by or called
 * from the product library.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline leg of bench.py may load it.
 *
 * Pinning: the deterministic known-answer tests of the reference
 * (test/test_potentials.jl, test/runtests.jl, test/configurations.jl,
 * test/test_runner_forward.jl) and the multihistogram golden vectors embedded in
 * test/multihist_test.jl are checked against this library in tests/.  The
 * reference's RNG-seeded pins (test/test_states.jl) need Julia's Xoshiro stream
 * and cannot be reproduced; instead oracle and engine share one Philox4x32-10
 * draw stream (same draw order as the reference, see src/MCRun.jl:142-162).
 *
 * All functions return 0 on success and a negative code on error;
 * orc_last_error() gives the message.
 */
#ifndef PTMC_ORACLE_H
#define PTMC_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_run orc_run;

/* potential kinds (src/EnergyEvaluation.jl) */
#define ORC_POT_ELJ 0      /* ELJPotential      :923 */
#define ORC_POT_ELJEVEN 1  /* ELJPotentialEven  :934 */
#define ORC_POT_EAM 2      /* EmbeddedAtomPotential :1059 */
#define ORC_POT_NN 3       /* RuNNerPotential   :1182 */
#define ORC_POT_ELJB 4     /* ELJPotentialB     :161 */
#define ORC_POT_LUT 5      /* LookupTablePotential :210 */
#define ORC_POT_NN2 6      /* RuNNerPotential2Atom :1287 */
/* boundary kinds (src/BoundaryConditions.jl) */
#define ORC_BC_SPHERE 0
#define ORC_BC_CUBIC 1
#define ORC_BC_RECT 2      /* RectangularBC :89 */
#define ORC_BC_RHOMBIC 3   /* RhombicBC     :110 */
/* ensembles (src/Ensembles.jl) */
#define ORC_NVT 0
#define ORC_NPT 1
#define ORC_NNVT 2         /* NNVT :138 (two species, atom swaps) */

/* One PT run of R replicas of N atoms.  xyz holds R start configurations
 * (walker w starts from xyz[w*N*3 ...]); T holds the R temperatures (K);
 * max_displ holds 2 values per slot (atom, volume).  bc_param is the sphere
 * radius or the cubic side length.  run_index selects the Philox stream. */
orc_run* orc_create(int N, int R, int ensemble, double pressure, int bc_kind,
                    double bc_param, const double* xyz, const double* T,
                    const double* max_displ, int n_bin, int n_adjust,
                    int mc_sample, double min_acc, double max_acc,
                    double exch_prob, uint64_t seed, int run_index);
void orc_destroy(orc_run* r);
/* RectangularBC / RhombicBC (bc_param of orc_create is box_length): box
 * height, NPT separated volume moves and the initial max_displ[3:4] (2 per
 * slot: xy, z; NULL = 0.1).  Before orc_init. */
int orc_set_box(orc_run* r, double height, int separated, const double* max_displ_sep);
/* walker box heights [R]; slot max_displ[3:4] [2R]; count_vol_xy, count_vol_z [2R] */
int orc_get_box(orc_run* r, double* height, double* max_displ_sep, long* count_xy,
                long* count_z);
const char* orc_last_error(void);

int orc_set_pot_elj(orc_run* r, const double* c, int K, int even);
int orc_set_pot_eam(orc_run* r, double n, double m, double ean, double ecam);
/* RuNNerPotential2Atom (EnergyEvaluation.jl:1287-1314) for the NNVT ensemble:
 * n1 atoms of species 1 (indices 0..n1-1), the rest species 2; rad: nrad rows
 * {eta, r_cut, G_offset[4], G_norm[4]} (RadialType2a, SymmFunc.jl:54-85);
 * ang: nang rows {eta, lambda, zeta, r_cut, tpz[6], G_offset[6]}
 * (AngularType3a, :114-175); w1 / w2: the two species' MLP weights (our
 * layout), nodes[0] == 2 nrad + 3 nang; n_swaps atom swaps per cycle. */
int orc_set_pot_nn2(orc_run* r, const double* rad, int nrad, const double* ang, int nang,
                    const double* w1, const double* w2, int nw, const int* nodes, int n_layers,
                    int n1, int n_swaps);
/* ELJPotentialB(a, b, c) (EnergyEvaluation.jl:161-183) */
int orc_set_pot_eljb(orc_run* r, const double* a, const double* b, const double* c, int K);
/* LookupTablePotential (EnergyEvaluation.jl:210-260); table is Julia's
 * Matrix(l_angle, l_dist), column-major: entry (angle a, distance d) at
 * (d-1)*l_angle + (a-1) */
int orc_set_pot_lut(orc_run* r, const double* table, int l_angle, int l_dist, double start_dist,
                    double start_angle, double d_dist, double d_angle, double c6);
/* sf: nsf rows of 8 doubles {kind(0 radial,1 angular), type, eta, lambda,
 * zeta, rcut, gmin, gmax}; weights: our layout (per layer: W[n_in][n_out]
 * input-major, then b[n_out]); nodes: n_layers node counts; boundary: hard-core
 * distance (bohr) below which E = 100 (EnergyEvaluation.jl:1602). */
int orc_set_pot_nn(orc_run* r, const double* sf, int nsf, const double* weights,
                   int nw, const int* nodes, int n_layers, double boundary);
int orc_init(orc_run* r);

/* equilibration_cycle! (MCRun.jl:282): eq_cycles/2 cycles, ebounds, counters
 * reset, histogram initialisation (Sampling.jl:141). */
int orc_equilibrate(orc_run* r, int eq_cycles);
/* production cycles i = first .. first+n-1 (MCRun.jl:397, mc_cycle! :215) */
int orc_production(orc_run* r, long first, long n);
/* plain cycles without sampling (mc_cycle! :192) */
int orc_cycles(orc_run* r, long first, long n);

/* walker-bound state (config order = walker order) */
int orc_get_walkers(orc_run* r, double* xyz, double* en_tot, double* box);
/* slot-bound state (slot = temperature index) */
int orc_get_slots(orc_run* r, int* walker_of_slot, double* max_displ,
                  long* count_atom, long* count_vol, long* count_exc,
                  double* ham);
/* histogram state: NVT en_hist R*(n_bin+2), NPT ev_hist R*(n_bin+2)^2
 * (row-major [slot][e][v]); hp = {en_min, en_max, v_min, v_max, dE, dV} */
int orc_get_hist(orc_run* r, double* en_hist, double* ev_hist, double* hp);
/* finalise_results (Sampling.jl:377) */
int orc_finalise(orc_run* r, long mc_cycles, int mc_sample, double* en_avg,
                 double* heat_cap, double* stat_atom, double* stat_exc);
/* radial distribution sampling (rdfsave, Sampling.jl:282-345): on/off, and
 * the R x 5 n_bin histogram with its bin width delta_r2 */
int orc_set_rdf(orc_run* r, int on);
int orc_get_rdf(orc_run* r, double* rdf, double* dr2);
/* NNVT: accepted atom swaps so far (all slots) */
long orc_get_swaps(orc_run* r);
/* NN only: G matrix (nsf x N, column per atom) of walker w */
int orc_get_nn_state(orc_run* r, int w, double* G, double* eatom);

/* ---- pure functions (known-answer tests) ---- */
double orc_dimer_energy(int kind, const double* c, int K, double r2);
double orc_distance2(const double* a, const double* b, int bc_kind,
                     double L);
double orc_lrc(int N, double r_cut2, const double* c, int K);
/* distance2, get_r_cut, get_volume of a box with length L and height H */
double orc_distance2_box(const double* a, const double* b, int bc_kind, double L, double H);
double orc_box_rcut(int bc_kind, double L, double H);
/* get_tan, dimer_energy of ELJPotentialB and LookupTablePotential */
double orc_get_tan(const double* a, const double* b, int bc_kind, double L, double H);
double orc_eljb_energy(const double* a, const double* b, const double* c, int K, double r2,
                       double tn);
double orc_lut_energy(const double* table, int l_angle, int l_dist, double start_dist,
                      double d_dist, double d_angle, double c6, double r2, double tn);
double orc_box_volume(int bc_kind, double L, double H);
/* dimer_energy_config over all pairs; cut != 0 applies get_r_cut and the
 * box-scaled long-range correction */
double orc_elj_config_energy_box(const double* xyz, int N, int kind, const double* c, int K,
                                 int bc_kind, double L, double H, int cut);
double orc_eam_config_energy(const double* xyz, int N, double n, double m,
                             double ean, double ecam);
double orc_elj_config_energy(const double* xyz, int N, int kind,
                             const double* c, int K, int bc_kind, double L,
                             double r_cut2);
void orc_tempgrid(double ti, double tf, int R, int tdistr, double* T,
                  double* beta);
double orc_u01(uint64_t seed, uint32_t stream, uint32_t run, uint64_t idx);
/* raw Philox4x32-10 block (known-answer test) */
void orc_philox4x32(const uint32_t* ctr, const uint32_t* key, uint32_t* out);
/* per-atom MLP forward (ForwardPass.jl:50-84 math), FP64 */
int orc_mlp_forward(const double* input, int n_in, int batch,
                    const double* weights, int nw, const int* nodes,
                    int n_layers, double* eatom);

/* ---- learned pair surrogate of the delayed-acceptance move (no counterpart
 * in the reference).  cfg = {r_lo, r_hi, gamma, r_cut, escale}; params: the
 * orc_sur_nparams() values W1[16][32], b1[32], W2[32][32], b2[32], w3[32], b3;
 * rows: n records of 128 floats (0..63 new distances |t - x_j|, 64..127 old
 * |x_i - x_j|, negative = no pair).  bf16 != 0 rounds the matrix-product
 * operands to BF16 as the GPU's tensor cores see them. ---- */
int orc_sur_nparams(void);
int orc_sur_forward(const double* cfg, const double* params, const float* rows,
                    int n, int bf16, double* dEs);
/* Huber (delta 1) loss of (dE_s - target)/escale averaged over the records,
 * and its gradient (grad may be NULL) */
int orc_sur_loss_grad(const double* cfg, const double* params,
                      const float* rows, const float* targets, int n, int bf16,
                      double* loss, double* grad);
/* delayed-acceptance atom moves for an NN run (params NULL switches it off);
 * stats: {first-stage rejections, exact evaluations} */
int orc_set_surrogate(orc_run* r, const double* cfg, const double* params,
                      int bf16);
int orc_get_sur_stats(orc_run* r, long* out);

/* ---- multihistogram (multihist_NVT.jl:95, multihist_NPT.jl:113) ---- */
int orc_multihist_nvt(int R, int n_bin, const double* en_hist,
                      const double* t_grid, const double* beta, double en_min,
                      double en_max, double thr, double* T_out, double* cv_out,
                      int* iters);
int orc_multihist_npt(int R, int n_bin, const double* ev_hist,
                      const double* t_grid, const double* beta, double en_min,
                      double en_max, double v_min, double v_max,
                      double pressure, double thr, double* T_out,
                      double* cp_out, int* iters);

/* linear-solve multihistogram (multihistogram(output, Tvec), src/multihist.jl):
 * en_hist [R][n_bin+2]; outputs energies/S_E [n_bin] (the first *n_kept are
 * used), alpha [R], and T/Z/U/Cv/dCv/S_T [npoints].  The gauge alpha[R-1] = 0
 * replaces the singular system's last equation. */
int orc_multihist_linear(int R, int n_bin, const double* en_hist, const double* beta,
                         double en_min, double en_max, int npoints, double* energies,
                         double* S_E, int* n_kept, double* alpha, double* T_out,
                         double* Z, double* U, double* Cv, double* dCv, double* S_T);

#ifdef __cplusplus
}
#endif
#endif
