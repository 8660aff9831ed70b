/*
 * ptmc_gb300.h — C ABI of the GB300 parallel-tempering Monte Carlo engine.
 *
 * One context holds a batch of independent PT runs that share the potential,
 * the ensemble, the temperature grid and the MC parameters (each run may have
 * its own atom count and start configurations).  All replica state lives on the
 * GPU; every entry point takes plain host pointers owned by the caller
 * (column-major Julia arrays map 1:1: xyz is 3 x N per configuration).  No entry
 * point keeps a caller pointer after it returns.  Errors are negative return
 * codes; ptmc_last_error() gives the message.  There is no CPU fallback: every
 * compute entry point fails with PTMC_ERR_CUDA when no usable GPU is present.
 *
 * Each declaration names the reference interface it replaces
 * (ParallelTemperingMonteCarlo.jl v0.3.5, paths relative to the package root).
 */
#ifndef PTMC_GB300_H
#define PTMC_GB300_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

#define PTMC_OK 0
#define PTMC_ERR_ARG -1      /* bad argument (ArgumentError in the reference) */
#define PTMC_ERR_STATE -2    /* call out of order */
#define PTMC_ERR_CUDA -3     /* CUDA failure or no GPU; also a bounded device wait that ran out
                                (tensor-core completion, exchange partner): see ptmc_last_error */
#define PTMC_ERR_SPHERE -4   /* "too many moves out of binding sphere" (src/MCMoves.jl:132) */
#define PTMC_ERR_IO -5       /* checkpoint file error */
#define PTMC_ERR_LIMIT -6    /* size beyond a documented limit */

/* ensembles: NVT (src/Ensembles.jl:42), NPT (src/Ensembles.jl:75), NNVT (two
 * species with atom swaps, src/Ensembles.jl:138-151) */
#define PTMC_NVT 0
#define PTMC_NPT 1
#define PTMC_NNVT 2
/* boundary conditions: SphericalBC (src/BoundaryConditions.jl:44),
 * CubicBC (src/BoundaryConditions.jl:72), RectangularBC (:89) and RhombicBC
 * (:110), the last two with a box length (x, y) and a height (z) */
#define PTMC_BC_SPHERE 0
#define PTMC_BC_CUBIC 1
#define PTMC_BC_RECTANGULAR 2
#define PTMC_BC_RHOMBIC 3
/* arithmetic forms */
#define PTMC_FP64 0          /* plain form: FP64 everywhere */
#define PTMC_FP32_RESYNC 1   /* FP32 move rows, FP64 running total, FP64 resync */
/* temperature distributions (src/InputParams.jl:77-95) */
#define PTMC_TGEOMETRIC 0
#define PTMC_TLINEAR 1

typedef struct ptmc_ctx ptmc_ctx;

/* MCParams (src/InputParams.jl:35-63) + TempGrid (src/InputParams.jl:77-95)
 * + ensemble + engine options. */
typedef struct ptmc_params {
  int n_runs;         /* independent PT runs batched in one context (>= 1) */
  int n_traj;         /* replicas per run, MCParams.n_traj (1..1024; the FP32 form of the
                         pair and EAM potentials runs R > 32 on a cluster of C <= 8 CTAs,
                         so R needs a divisor C with R / C <= 32) */
  long long mc_cycles;/* MCParams.mc_cycles */
  long long eq_cycles;/* MCParams.eq_cycles (round(eq_percentage*cycles)) */
  int mc_sample;      /* MCParams.mc_sample */
  int n_adjust;       /* MCParams.n_adjust */
  int n_bin;          /* MCParams.n_bin */
  double min_acc;     /* MCParams.min_acc */
  double max_acc;     /* MCParams.max_acc */
  int ensemble;       /* PTMC_NVT or PTMC_NPT */
  double pressure;    /* NPT.pressure (Eh/bohr^3) */
  double t_i, t_f;    /* TempGrid end points (K) */
  int tdistr;         /* PTMC_TGEOMETRIC or PTMC_TLINEAR */
  double exch_prob;   /* exchange attempt probability per cycle: 0.1 in
                         src/MCRun.jl:203; 1.0 attempts one exchange every cycle */
  int precision;      /* PTMC_FP64 or PTMC_FP32_RESYNC */
  int resync_every;   /* FP32 form: cycles between FP64 recomputes (0 = never) */
  uint64_t seed;      /* Philox key for every draw stream of this context */
  int cycles_per_launch; /* cycles fused in one kernel launch (0 = auto) */
  int device;         /* CUDA device ordinal */
} ptmc_params;

/* Result bag, Output (src/InputParams.jl:114-176), for one run.  Every array
 * is caller-allocated with the length given; NULL skips it. */
typedef struct ptmc_output {
  double* en_avg;          /* [R]  Output.en_avg */
  double* heat_cap;        /* [R]  Output.heat_cap (C/kB convention of Sampling.jl:386) */
  double* count_stat_atom; /* [R]  Output.count_stat_atom */
  double* count_stat_vol;  /* [R]  accepted volume moves / mc_cycles */
  double* count_stat_exc;  /* [R]  Output.count_stat_exc */
  double* max_displ;       /* [2R] per slot: atom, volume step (MCState.max_displ[1:2]) */
  double* en_histogram;    /* [R*(n_bin+2)]  NVT Output.en_histogram */
  double* ev_histogram;    /* [R*(n_bin+2)^2] NPT Output.ev_histogram, [slot][e][v] */
  double hist_params[6];   /* en_min, en_max, v_min, v_max, delta_en_hist, delta_v_hist */
  double* rdf;             /* [R*5*n_bin] Output.rdf (needs ptmc_set_rdf), NULL skips it */
  double delta_r2;         /* Output.delta_r2, the rdf bin width in r^2 */
} ptmc_output;

/* Engine counters for measurement. */
typedef struct ptmc_stats {
  long long kernel_launches;   /* kernels launched by this context so far */
  long long graph_launches;    /* CUDA graph replays */
  long long atom_moves;        /* attempted atom moves (all replicas, all runs) */
  long long volume_moves;      /* attempted volume moves */
  double max_drift;            /* FP32 form: largest |E_running - E_fp64| seen at a resync (Eh) */
  double last_cycles_ms;       /* device time of the last ptmc_run_cycles / ptmc_equilibrate */
} ptmc_stats;

/* --- set-up (replaces MCParams/TempGrid/ensemble construction and
 *     initialisation(), src/Initialization.jl:70-100) --- */
int ptmc_create(ptmc_ctx** out, const ptmc_params* p);
/* ELJPotential / ELJPotentialEven (src/EnergyEvaluation.jl:923-942);
 * c has K <= 16 coefficients for powers 6,7,8,... (even=0) or 6,8,10,... (even=1) */
int ptmc_set_potential_elj(ptmc_ctx* c, const double* coeff, int K, int even);
/* ELJPotentialB(a, b, c) (src/EnergyEvaluation.jl:161-183): the extended
 * Lennard-Jones dimer in a magnetic field, c_k r^-p_k (1 + a_k cos 2theta +
 * b_k cos 4theta) with theta the pair angle to z (dimer_energy, :943-958);
 * K = 2..16.  Plain FP64 form; NVT with SphericalBC/CubicBC, NPT with
 * CubicBC/RectangularBC/RhombicBC. */
int ptmc_set_potential_eljb(ptmc_ctx* c, const double* a, const double* b,
                            const double* coeff_c, int K);
/* LookupTablePotential (src/EnergyEvaluation.jl:210-298): the fields of the
 * reference's struct; table is its Matrix{Float64}(l_angle, l_dist) in Julia's
 * column-major order (entry (angle a, distance d) at (d-1)*l_angle + (a-1)),
 * so a Julia caller passes pot.table as is.  Same ensembles and boxes as
 * ELJPotentialB. */
int ptmc_set_potential_lookup(ptmc_ctx* c, const double* table, int l_angle,
                              int l_dist, double start_dist, double start_angle,
                              double d_dist, double d_angle, double c6coeff);
/* RuNNerPotential2Atom (src/EnergyEvaluation.jl:1287-1314) for the NNVT
 * ensemble: n1 atoms of species 1 (indices 0..n1-1 of every configuration),
 * the rest species 2.  rad: nrad rows {eta, r_cut, G_offset[4], G_norm[4]}
 * (RadialType2a, MachineLearningPotential/SymmFunc.jl:54-85); ang: nang rows
 * {eta, lambda, zeta, r_cut, tpz[6], G_offset[6]} (AngularType3a, :114-175);
 * w1 / w2: the two species' networks in the layout of ptmc_set_potential_nn
 * with nodes = {2 nrad + 3 nang, H1, H2, 1}.  SphericalBC, at most 64 atoms,
 * plain FP64 form. */
int ptmc_set_potential_nn2(ptmc_ctx* c, const double* rad, int nrad,
                           const double* ang, int nang, const double* w1,
                           const double* w2, int nw, const int* nodes,
                           int n_layers, int n1);
/* NNVT.n_atom_swaps (src/Ensembles.jl:144-151): swaps per cycle (default 1);
 * each picks one atom of each species (swap_atoms, src/MCMoves.jl:363-370). */
int ptmc_set_atom_swaps(ptmc_ctx* c, int n_swaps);
/* Accepted atom swaps of run `run` so far (all its walkers). */
int ptmc_get_swaps(ptmc_ctx* c, int run, long long* accepted);
/* EmbeddedAtomPotential(n, m, ean, eCam) (src/EnergyEvaluation.jl:1059-1073) */
int ptmc_set_potential_eam(ptmc_ctx* c, double n, double m, double ean,
                           double ecam);
/* RuNNerPotential (src/EnergyEvaluation.jl:1182-1213) with the per-atom MLP of
 * MachineLearningPotential/ForwardPass.jl:23-84 (which calls the closed
 * librunnerjulia.so `forward`).  sf: nsf rows of 8 doubles {kind (0 radial
 * G2, 1 angular G4), type (11/10 radial, 111/110/100 angular; only 11 and 111
 * are active for one element, SymmFunc.jl:261,281), eta, lambda, zeta, r_cut,
 * G_min, G_max}.  weights: per layer W[n_in][n_out] (input-major) then
 * b[n_out].  nodes: n_layers counts, nodes[0] == nsf, last == 1, hidden tanh.
 * boundary: hard-core distance (bohr), E = 100 below it
 * (src/EnergyEvaluation.jl:1602-1606). */
int ptmc_set_potential_nn(ptmc_ctx* c, const double* sf, int nsf,
                          const double* weights, int nw, const int* nodes,
                          int n_layers, double boundary);
/* Start configurations of run `run`: n_start configs of N atoms (xyz 3 x N
 * each, bohr); replica i starts from config (i mod n_start)
 * (src/Initialization.jl:88-96).  bc_param: sphere radius or cube side. */
int ptmc_set_run_configs(ptmc_ctx* c, int run, const double* xyz, int N,
                         int n_start, int bc_kind, double bc_param);
/* Start configurations in a RectangularBC or RhombicBC box
 * (src/BoundaryConditions.jl:80-116): box_length (x, y side; for the rhombic
 * box the side of the rhombus) and box_height (z).  For the sphere and the cube
 * box_height is ignored (ptmc_set_run_configs is this call with
 * box_height = bc_param).  These boxes run in the plain FP64 form with the ELJ
 * potentials. */
int ptmc_set_run_configs_box(ptmc_ctx* c, int run, const double* xyz, int N,
                             int n_start, int bc_kind, double box_length,
                             double box_height);
/* Start configurations of the n_runs runs first .. first + n_runs - 1 in one
 * call: one configuration of N atoms per run (xyz [n_runs][N][3], bohr), all
 * with the same boundary; the same as ptmc_set_run_configs_box with n_start = 1
 * for each run (the batched form of the per-run call that
 * src/Initialization.jl:88-96 replaces). */
int ptmc_set_runs_configs(ptmc_ctx* c, int first, int n_runs, const double* xyz, int N,
                          int bc_kind, double box_length, double box_height);
/* NPT(n_atoms, pressure, separated_volume) (src/Ensembles.jl:75-86): volume
 * moves change z (probability 1/6), x and y (1/3) or all directions (1/2)
 * (volume_change_separated, src/MCMoves.jl:298-343) with their own step sizes
 * max_displ[3:4] and counters count_vol_xy / count_vol_z.  RectangularBC or
 * RhombicBC boxes only.  Set it before ptmc_init. */
int ptmc_set_separated_volume(ptmc_ctx* c, int on);
/* Optional initial step sizes, 2 per slot (atom, volume); default 0.1, 0.1
 * (src/MCStates.jl:104). */
int ptmc_set_max_displ(ptmc_ctx* c, int run, const double* max_displ);
/* Optional initial separated-volume step sizes max_displ[3:4], 2 per slot
 * (xy, z); default 0.1, 0.1 (src/MCStates.jl:101). */
int ptmc_set_max_displ_sep(ptmc_ctx* c, int run, const double* max_displ_sep);
/* Radial distribution sampling, the rdfsave option of ptmc_run! (update_rdf!,
 * src/Sampling.jl:282-316): every 1000th production cycle each slot's
 * configuration adds its pair distances to 5 n_bin bins of width
 * delta_r2 = 4 r^2 / n_bin / 5 (sphere) or 3/4 L^2 / n_bin / 5 (cube).  Set it
 * before ptmc_init. */
int ptmc_set_rdf(ptmc_ctx* c, int on);
/* Uploads everything and computes the initial energies on the GPU
 * (MCState constructor, src/MCStates.jl:137-162). */
int ptmc_init(ptmc_ctx* c);

/* --- the hot loop (replaces equilibration/mc_cycle!/ptmc_run! main loop,
 *     src/MCRun.jl:192-253, 282-344, 363-432) --- */
/* equilibration_cycle! (src/MCRun.jl:282-313): eq_cycles/2 cycles, energy
 * bounds from the final energies, counter reset, histogram set-up
 * (src/Sampling.jl:141-194). */
int ptmc_equilibrate(ptmc_ctx* c);
/* n production cycles (mc_cycle! with sampling_step!, src/MCRun.jl:215-253),
 * continuing the cycle index where the previous call stopped. */
int ptmc_run_cycles(ptmc_ctx* c, long long n);
/* plain cycles without sampling (mc_cycle!, src/MCRun.jl:192-213), advancing
 * a separate cycle index starting at 1; used for parity tests. */
int ptmc_cycles_nosample(ptmc_ctx* c, long long n);
/* FP32 form: recompute every running total in FP64 now. */
int ptmc_resync(ptmc_ctx* c);

/* --- results (finalise_results, src/Sampling.jl:377-399) --- */
int ptmc_get_output(ptmc_ctx* c, int run, ptmc_output* out);
/* Slot-ordered replica state: xyz [R][N][3], en_tot [R], box [R] (cube side
 * or sphere radius), max_displ [2R], counts [R][6] = count_atom[1:2],
 * count_vol[1:2], count_exc[1:2] (src/MCStates.jl:33-53), ham [2R]. */
int ptmc_get_states(ptmc_ctx* c, int run, double* xyz, double* en_tot,
                    double* box, double* max_displ, long long* counts,
                    double* ham);
/* Slot-ordered energies of every run in one read: en_tot [n_runs][R]. */
int ptmc_get_energies(ptmc_ctx* c, double* en_tot);
/* Slot-ordered box state of RectangularBC / RhombicBC runs: box_height [R],
 * max_displ_sep [2R] = max_displ[3:4], counts_sep [R][4] = count_vol_xy[1:2],
 * count_vol_z[1:2] (src/MCStates.jl:33-47).  NULL skips an array. */
int ptmc_get_box_states(ptmc_ctx* c, int run, double* box_height,
                        double* max_displ_sep, long long* counts_sep);
int ptmc_get_stats(ptmc_ctx* c, ptmc_stats* s);

/* --- checkpoint / resume (src/ReadSave.jl:93-218, 330-481) --- */
/* Writes the reference's text formats into dir (params.data, hist_info.data,
 * histograms.data, volume_hist.data, index.txt, configT<i>.xyz) for run 0,
 * plus engine.bin with the full binary state of every run (exact resume). */
int ptmc_checkpoint(ptmc_ctx* c, const char* dir);
/* Restores the full state written by ptmc_checkpoint into a context created
 * with the same parameters and potential. */
int ptmc_restore(ptmc_ctx* c, const char* dir);

/* --- multihistogram reweighting on the GPU (FP64 log-sum-exp) --- */
/* multihistogram_NVT (src/multihist_NVT.jl:95-221): en_hist [R][n_bin+2]
 * counts, t_grid/beta [R]; T_out/cv_out [10R]; returns iterations in *iters. */
int ptmc_multihist_nvt(int R, int n_bin, const double* en_hist,
                       const double* t_grid, const double* beta, double en_min,
                       double en_max, double thr, double* T_out, double* cv_out,
                       int* iters);
/* multihistogram_NPT (src/multihist_NPT.jl:113-338): ev_hist
 * [R][n_bin+2][n_bin+2]; T_out/cp_out [10R]. */
int ptmc_multihist_npt(int R, int n_bin, const double* ev_hist,
                       const double* t_grid, const double* beta, double en_min,
                       double en_max, double v_min, double v_max,
                       double pressure, double thr, double* T_out,
                       double* cp_out, int* iters);

/* --- delayed acceptance with a learned pair surrogate (no counterpart in the
 *     reference; Christen & Fox 2005 two-stage Metropolis-Hastings) ---
 * Surrogate: E_s = sum over pairs phi(r), phi = escale*(w3.h2 + b3),
 * h2 = tanh(W2^T h1 + b2), h1 = tanh(W1^T g + b1), g_k = fc(r)*exp(-gamma
 * (r - mu_k)^2) with 16 centres mu_k evenly spaced on [r_lo, r_hi] and the
 * cosine cut-off fc at r_cut.  Parameters: PTMC_SUR_NPARAMS floats W1[16][32]
 * (input-major), b1[32], W2[32][32], b2[32], w3[32], b3.  A move record is 128
 * floats: [0..63] new distances |t - x_j|, [64..127] old distances |x_i - x_j|
 * (negative = no pair); dE_s = sum phi(new) - sum phi(old).  The two matrix
 * products per record run on the tensor cores (BF16 operands, FP32
 * accumulation).  A delayed-acceptance atom move draws, after the proposal,
 * u1 and accepts stage 1 iff min(1, exp(-beta dE_s)) >= u1; only then is the
 * exact NN energy computed and the move accepted iff
 * min(1, exp(-beta (dE - dE_s))) >= u2 (a second draw).  The chain stays exact
 * for any fixed surrogate: train, then freeze, then enable. */
typedef struct ptmc_surrogate_cfg {
  double r_lo, r_hi;  /* first and last Gaussian centre (bohr) */
  double gamma;       /* Gaussian width parameter (1/bohr^2) */
  double r_cut;       /* cosine cut-off of the features (bohr) */
  double escale;      /* output scale (Eh); 0 = set from the recorded dE at the first training */
} ptmc_surrogate_cfg;
#define PTMC_SUR_NPARAMS 1633
/* dE_s of n move records on `device` (host arrays in and out). */
int ptmc_surrogate_eval(const ptmc_surrogate_cfg* cfg, const float* params,
                        const float* rows, int n, double* dEs_out, int device);
/* Huber loss (delta 1) of (dE_s - targets)/escale averaged over the n records
 * and its gradient grad[PTMC_SUR_NPARAMS] (host arrays), computed on `device`
 * by the training kernels (tensor-core forward, FP32 backward). */
int ptmc_surrogate_loss_grad(const ptmc_surrogate_cfg* cfg, const float* params,
                             const float* rows, const float* targets, int n,
                             double* loss, float* grad, int device);
/* Attach a surrogate to an NN context (after ptmc_init): cfg, initial
 * parameters (NULL = seeded uniform(+-1/sqrt(fan_in)) weights, zero biases),
 * a ring of `capacity` training records, and the capture stride: move m of a
 * walker in cycle c is recorded when (c*N + m) % record_every == 0.  Calling
 * it again re-initialises the parameters, the optimiser and the counters and
 * keeps the captured records when the capacity is unchanged. */
int ptmc_surrogate_set(ptmc_ctx* c, const ptmc_surrogate_cfg* cfg,
                       const float* params, int capacity, int record_every);
/* Record (config, dE) pairs from the exact chain during the following cycle
 * calls (on = 1) or stop (0).  Not allowed while delayed acceptance is on. */
int ptmc_surrogate_record(ptmc_ctx* c, int on);
/* `steps` Adam steps (learning rate lr) on minibatches of `batch` records drawn
 * from the ring; *loss_out = mean minibatch loss of the last 10 % of steps. */
int ptmc_surrogate_train(ptmc_ctx* c, int steps, int batch, double lr,
                         double* loss_out);
/* Switch delayed-acceptance moves on (1) or off (0); the surrogate is frozen
 * while on.  Switching on tabulates the network's pair function phi(r) on 4097
 * grid distances over [0, r_cut] (phi is constant beyond r_cut); the first
 * stage of a move interpolates linearly in that table, a fixed pair function of
 * the distance, so the two-stage chain stays exact. */
int ptmc_surrogate_enable(ptmc_ctx* c, int on);
/* Current parameters (params may be NULL), the configuration in use (cfg may
 * be NULL) and counters stats[4] = {records captured, first-stage
 * rejections, exact evaluations, 0} summed over every walker. */
int ptmc_surrogate_get(ptmc_ctx* c, float* params, ptmc_surrogate_cfg* cfg,
                       long long* stats);
/* Screening strength per temperature slot.  With kappa_s the first stage
 * accepts iff min(1, exp(-kappa_s beta_s dE_s)) >= u1 and the second iff
 * min(1, exp(-beta_s (dE - kappa_s dE_s))) >= u2 (exact for any fixed kappa);
 * kappa_s = 0 skips the surrogate for that slot (no first-stage draw).  The
 * default after ptmc_surrogate_set is 1.  This call picks kappa_s in
 * {0, 1/16, ..., 1} per slot to maximise accepted moves per unit time: the sum
 * over slots of the two-stage acceptance a_s(kappa_s) divided by the summed
 * cost per move, r + p1_s(kappa_s) (1 for kappa_s = 0; the walker CTAs share
 * the SMs, so a cycle's time follows the total cost); a and p1 are estimated on the slot's captured
 * records (exact dE and the surrogate's dE_s), r is the cost of a surrogate
 * stage relative to an exact evaluation: cost_ratio if > 0, else measured by
 * timing timing_cycles plain cycles without, with and again without screening
 * (these cycles advance the chain, without sampling).  kappa_out [R] (may be NULL) receives the
 * choice.  The delayed-acceptance on/off state is left as it was. */
int ptmc_surrogate_calibrate(ptmc_ctx* c, double cost_ratio, int timing_cycles,
                             double* kappa_out);
/* Set the screening strength per temperature slot directly: kappa [R], each in
 * [0, 1], the same for every run (for instance a choice ptmc_surrogate_calibrate
 * made on an earlier engine).  No counterpart in the reference (delayed
 * acceptance is this engine's addition). */
int ptmc_surrogate_set_kappa(ptmc_ctx* c, const double* kappa);
/* Copy up to max_n captured records (rows [n][128], targets [n]); *n_out = count. */
int ptmc_surrogate_records(ptmc_ctx* c, float* rows, float* targets, int max_n,
                           int* n_out);

/* multihistogram(output, Tvec) of src/multihist.jl (the linear-solve
 * multihistogram, used by postprocess): histograms en_hist [R][n_bin+2]
 * (interior bins used, divided by n_bin, empty bins dropped), beta [R].
 * Outputs: energies and S_E [n_bin] (entropy per kept bin, the first *n_kept
 * are set), alpha [R], and on npoints temperatures T_1 + k (T_R - T_1)/npoints:
 * T, Z, U, Cv, dCv, S_T [npoints] (analysis, :292-375, with the reference's
 * rescaling of Z into [1, 100]).  The system A alpha = b is singular; the
 * reference's A \ b fixes the free constant by LAPACK's rounding, this call by
 * alpha[R-1] = 0: U, Cv and dCv are unaffected, Z and S_T scale / shift. */
int ptmc_multihist_linear(int R, int n_bin, const double* en_hist, const double* beta,
                          double en_min, double en_max, int npoints, double* energies,
                          double* S_E, int* n_kept, double* alpha, double* T, double* Z,
                          double* U, double* Cv, double* dCv, double* S_T);

/* Allocation-free multihistogram_NVT, no counterpart in the reference (which
 * has no device memory at all).  For callers that cannot call cudaMalloc: a
 * Julia program whose GPU memory belongs to CUDA.jl's pool, code enqueueing
 * inside a stream capture, or a service that reserves all device memory up
 * front.  Every pointer is caller-owned DEVICE memory: d_hist [R][n_bin+2],
 * d_t_grid and d_beta [R] in, d_T_out and d_cv_out [10R] and d_iters [1] out.
 * The work is enqueued on `stream` (a cudaStream_t, NULL = default stream) and
 * the call returns without waiting.  The iteration's scratch is a fixed
 * file-scope device array of PTMC_NOALLOC_SCRATCH_DOUBLES doubles (128 KiB,
 * held by every GPU that loads the library until exit); inputs that need more
 * (3R + 3 n_bin + 20R + 2 doubles) return PTMC_ERR_LIMIT.  All calls share
 * that array, so calls that overlap on the GPU race.  The first call on a
 * device looks up the array's device address (cudaGetSymbolAddress); make
 * that first call before any stream capture.  Results equal
 * ptmc_multihist_nvt's to rounding.  Every failure sets the message of
 * ptmc_last_error(NULL); a CUDA error left pending by an earlier launch of the
 * caller's makes the call return PTMC_ERR_CUDA before it launches anything,
 * and that error stays pending for the caller. */
#define PTMC_NOALLOC_SCRATCH_DOUBLES 16384
int ptmc_multihist_nvt_noalloc(int R, int n_bin, const double* d_hist,
                               const double* d_t_grid, const double* d_beta,
                               double en_min, double en_max, double thr,
                               double* d_T_out, double* d_cv_out, int* d_iters,
                               void* stream);

/* --- launch shapes (no counterpart in the reference: the reference runs one
 *     replica per Julia task) ---
 * FP32 form of the pair and EAM potentials.  C: the R walkers of a run may be
 * spread over a thread-block cluster of C CTAs (C SMs, R/C walkers each); the
 * replica exchange, step adaptation and sampling then read the other CTAs'
 * walkers through distributed shared memory; results are bit-identical for
 * every C.  L: lanes per walker, 32 (one warp per walker), 16 (two walkers per
 * warp), 8 or 4 (four or eight walkers per warp, NVT with C = 1: the move's
 * scalar work is shared by the warp's walkers and a walker needs less shared
 * memory, so more walkers fit an SM); the pair sums then add in another order
 * (FP32 rounding), the chains stay statistically equivalent and every L
 * consumes the same draw streams.  Default C = 1, L = 32. */
/* Set (C, L) for the runs with N atoms (C <= 8, R % C == 0, L in {32, 16, 8, 4},
 * (R / C) % (32 / L) == 0; L <= 8 only with C = 1 in NVT). */
int ptmc_set_launch_shape(ptmc_ctx* c, int N, int ctas_per_run, int lanes_per_walker);
/* Pick (C, L) per atom count by timing `trial_cycles` plain cycles of the whole
 * batch for candidate shapes (coordinate descent over C in {1, 2, 4, 8} x L
 * in {32, 16, 8, 4} per atom count, largest N first) on a snapshot of the device
 * state that is restored after every trial, so the chain is not advanced.
 * cache_path (may be NULL): JSON-lines file of earlier choices, keyed by
 * device, potential, boundary, ensemble, R and the (N, runs) mix; a hit skips
 * the trials, a miss appends the result.  shape_out [2 n_runs] (may be NULL)
 * receives (C, L) per run.  Other forms keep C = 1, L = 32. */
int ptmc_autotune(ptmc_ctx* c, int trial_cycles, const char* cache_path,
                  int* shape_out);

/* Resident CTAs per SM of the cycle kernel for runs of N atoms in this
 * context's form, with launch shape (C, L) in the FP32 form (ignored by the
 * plain form): a batch of a multiple of ctas_per_sm x SMs / C runs fills the
 * GPU in whole waves.  Pair and EAM potentials; callable before ptmc_init
 * once the potential and the first run's configurations are set.  No
 * counterpart in the reference (one CPU thread per replica there). */
int ptmc_occupancy(ptmc_ctx* c, int N, int ctas_per_run, int lanes_per_walker,
                   int* ctas_per_sm);

/* Engine utility, no counterpart in the reference: measured FP32 FMA, FP64
 * FMA (TFLOP/s) and MUFU ex2 (Tops/s) peaks of `device`, the roofline
 * denominators of the replica-cycle kernels. */
int ptmc_measure_peaks(int device, double* fp32_tflops, double* fp64_tflops,
                       double* mufu_tops);

/* --- diagnostics of the bounded device waits (no counterpart in the
 *     reference, which has no device code) ---
 * The FP32 form's exchange handshake waits for the partner walker with a
 * bounded spin (default 2^33 clocks); when it runs out the walker stops with
 * status 3, both walkers of the pair keep their slots, and the call returns
 * PTMC_ERR_CUDA naming the wait.  The context's chains are then incomplete:
 * destroy it and build a new one.  Test hook: `clocks` > 0 sets the limit
 * (0 restores the default); never_set = 1 makes every partner wait target a
 * flag value that no walker writes, so the failure path runs without any
 * fault.  Takes effect at the next launch. */
int ptmc_set_wait_test(ptmc_ctx* c, long long clocks, int never_set);
/* Walker status words of run `run` in walker order, status[R]: 0 running,
 * 1 too many moves out of the sphere, 2 a tensor-core wait ran out, 3 an
 * exchange-partner wait ran out. */
int ptmc_get_walker_status(ptmc_ctx* c, int run, int* status);

const char* ptmc_last_error(ptmc_ctx* c); /* c may be NULL (global last error) */
void ptmc_destroy(ptmc_ctx* c);
const char* ptmc_version(void);

#ifdef __cplusplus
}
#endif
#endif
