// ptmc_engine.cuh — structures shared between the host orchestration
// (ptmc_capi.cu) and the replica-cycle kernels (ptmc_cycles.cu).
//
// HBM layout (structure of arrays, one allocation per field, walkers of all
// runs concatenated; "walker" = configuration-bound data, "slot" =
// temperature-bound data, see the walker/slot note in ptmc_cycles.cu):
//   pos   f64 [sum_r R_r*N_r*3]   positions, walker-major, atom-major, xyz
//   mat   f64 [sum_r R_r*N_r*N_r] NPT plain form and the B potentials:
//                                 squared-distance matrix
//   tan   f64 [same as mat]       B potentials: |tan| of the pair angle to z
//   comp  f64 [sum_r R_r*N_r*2]   EAM (phi_i, rho_i) components
//   pe    f64 [sum_r R_r*N_r*N_r*w] plain form, NVT: pair cache (w = 1 ELJ V(r_ij),
//                                 w = 2 EAM (r_ij^-n, r_ij^-m))
//   en/box/rc2/drift f64 [W], ctr u64 [W], status i32 [W]   per walker
//   boxh f64 [W]  box height (RectangularBC / RhombicBC)     per walker
//   beta/maxbox f64 [W], maxd f64 [2W], ham f64 [2W], cnt i64 [6W],
//   wos i32 [W]                                              per slot
//   maxboxh f64 [W], maxd_sep f64 [2W], cnt_sep i64 [4W]     per slot,
//   separated volume moves (max_displ[3:4], count_vol_xy/_z)
//   hist u32 [sum_r R_r*stride_r]  NVT: (n_bin+2) per slot, NPT: (n_bin+2)^2
#pragma once
#include <cstdint>
#include <string>

namespace ptmc {

enum { POT_ELJ = 0, POT_ELJEVEN = 1, POT_EAM = 2, POT_NN = 3, POT_ELJB = 4, POT_LUT = 5,
       POT_NN2 = 6 };  // POT_NN2: two-species RuNNer potential (NNVT)
// pair potentials with an angle to z (ELJPotentialB, LookupTablePotential)
__host__ __device__ constexpr bool pot_b(int pot) { return pot == POT_ELJB || pot == POT_LUT; }
enum { BC_SPH = 0, BC_CUB = 1, BC_RECT = 2, BC_RHB = 3 };  // RECT/RHB: length L, height H
enum { ENS_NVT = 0, ENS_NPT = 1 };
// the plain form keeps an NVT pair cache (pair energies in HBM) for the ELJ
// and EAM potentials; NPT and the angle-dependent potentials keep distances
__host__ __device__ constexpr bool pair_cache(int pot, int ens) {
  return ens == ENS_NVT && (pot == POT_ELJ || pot == POT_ELJEVEN || pot == POT_EAM);
}
enum { PHASE_PLAIN = 0, PHASE_EQ = 1, PHASE_PROD = 2 };
// TIMEOUT: a bounded tensor-core wait ran out; XWAIT: a bounded wait for an
// exchange partner ran out
enum { ST_OK = 0, ST_SPHERE = 1, ST_TIMEOUT = 2, ST_XWAIT = 3 };
constexpr int MAX_COEFF = 16;
constexpr int DRAW_BUF = 16;
// devices whose per-kernel attributes (shared-memory opt-in) are tracked
constexpr int MAX_DEVICES = 64;

struct RunDesc {
  int N, R;                 // atoms, replicas
  int wk;                   // first global walker (= slot) index of the run
  int run_id;               // Philox run word (global run index)
  long long pos_off;        // element offsets of walker 0 in pos / mat / comp
  long long mat_off;
  long long comp_off;
  long long hist_off;       // element offset of slot 0 in hist
  int hist_stride;          // hist elements per slot
  int n_start;              // distinct start configurations (walker w starts from w mod n_start)
  double en_min, en_max, dE;  // energy histogram (Sampling.jl:141-194)
  double v_min, v_max, dV;    // volume histogram (NPT)
  long long cyc[3];         // next cycle index (1-based) per phase
  unsigned long long run_ctr;  // run-level draw counter
  double dr2;               // radial-distribution bin width in r^2 (Sampling.jl:151,185)
  long long pe_off;         // element offset of walker 0 in pe (plain form, NVT pair cache)
};

// update_rdf! (src/Sampling.jl:282, 301-316): bin = floor(r2 / delta_r2), kept
// when 1 <= bin <= 5 n_bin (1-based; the diagonal, r2 = 0, falls in bin 0)
__device__ __forceinline__ void rdf_add(unsigned int* row, int nb5, double r2, double dr2) {
  const double b = floor(r2 / dr2);
  if (b >= 1.0 && b <= (double)nb5) atomicAdd(row + ((int)b - 1), 1u);
}
// every 1000th production cycle (Sampling.jl:341-345)
constexpr int RDF_EVERY = 1000;

struct KParams {
  RunDesc* runs;
  // walker-bound
  double* pos;
  double* mat;
  double* comp;
  float* lo;                // FP32 form, 4 or 8 lanes per walker: lo halves of the
                            // float-float positions during a launch, float4 per
                            // atom at (pos_off / 3 + walker * N)
  // plain form, runs whose replica state exceeds a CTA's shared memory: the
  // per-atom state stays in HBM (glob = 1) and each walker has scr_stride
  // doubles of scratch for its trial rows
  int glob;
  long long scr_stride;
  double* scr;
  double* pe;               // plain form, NVT: pair cache, ELJ N x N V(r_ij) or EAM
                            // N x N (r_ij^-n, r_ij^-m) per walker (see pair_cache)
  double* en;
  double* box;
  double* rc2;
  double* drift;
  unsigned long long* ctr;
  int* status;
  // slot-bound
  double* beta;
  double* maxd;
  double* maxbox;
  double* ham;
  long long* cnt;
  int* wos;
  unsigned int* hist;
  unsigned int* rdf;        // [slots][5 n_bin] radial distribution (NULL = off)
  // RectangularBC / RhombicBC and NPT separated volume moves
  double* boxh;             // [W] walker box height
  double* maxboxh;          // [W] slot max_boxheight (MCStates.jl:79-87)
  double* maxd_sep;         // [2W] slot max_displ[3] (xy), max_displ[4] (z)
  long long* cnt_sep;       // [4W] slot count_vol_xy[1:2], count_vol_z[1:2]
  int sep_vol;              // NPT.separated_volume
  // ELJPotentialB (coeff_c in c) and LookupTablePotential
  double ca[MAX_COEFF], cb[MAX_COEFF];  // coeff_a, coeff_b
  double* tan;              // tangent matrices, same offsets as mat
  const double* lut;        // table, Julia's Matrix(l_angle, l_dist) column-major
  int lut_na, lut_nd;       // l_angle, l_dist
  double lut_start, lut_dd, lut_da, lut_c6;  // start_dist, d_dist, d_angle, c6coeff
  // potential
  double c[MAX_COEFF];
  int K;
  double eam_n, eam_m, eam_ean, eam_ecam;
  // ensemble / MC parameters
  double pressure;
  double exch_prob;
  double min_acc, max_acc;
  int n_bin, n_adjust, mc_sample, resync_every;
  unsigned long long seed;
  // FP32 copies of the potential constants (FP32 form).  Precomputed on the
  // host so that no use inside the move loop converts from FP64: under
  // register pressure the compiler rematerialises constants from their source
  // expression, and an FP64 -> FP32 conversion issues to the FP64 pipe.
  float f_hn, f_hm, f_ean, f_ecam;  // -n/2, -m/2, ean, eCam
  float cf[MAX_COEFF];              // ELJ coefficients in FP32 (constant-bank operands)
  // bounded exchange-partner waits of the FP32 form: the limit in clocks, and
  // a test switch that makes every such wait target a flag value nobody writes
  long long xwait_clocks;
  int xwait_never;
};
// default limit of an exchange-partner wait (~4 s at 2 GHz; legitimate waits
// last a few cycles)
constexpr long long XWAIT_CLOCKS = 1ll << 33;

// pair terms per unrolled chunk of the FP32 form with 4 or 8 lanes per walker
constexpr int NARROW_CH = 4;
// walker stride (atoms) of that form's shared position array: N padded to
// whole chunks (NARROW_CH * lpr atoms; the pad atoms are far-away sentinels),
// plus lpr, so that the stride is lpr mod 2 lpr and the walkers read by one
// 128-byte shared-memory wavefront fall into disjoint banks
__host__ __device__ inline int narrow_stride(int N, int lpr) {
  const int q = NARROW_CH * lpr;
  return (N + q - 1) / q * q + lpr;
}

// shared-memory bytes of one run CTA
inline long long cycles_smem_bytes(int pot, int ens, bool f32, int R, int N) {
  auto al = [](long long b) { return (b + 15) / 16 * 16; };
  long long b = 0;
  b += al((long long)R * N * 3 * 8);                 // FP64 positions
  if (f32) b += al((long long)R * N * 16);           // FP32 positions (float4)
  if (pot == POT_EAM) {
    b += al((long long)R * N * (f32 ? 8 : 16));      // components
    b += al((long long)R * N * (f32 ? 8 : 16));      // per-move trial pair terms
  }
  if ((ens == ENS_NPT || pot_b(pot) || pot != POT_EAM) && !f32)
    b += al((long long)R * N * 8);                   // trial row (distances or pair energies)
  if (pot_b(pot) && !f32) b += al((long long)R * N * 8);    // trial tangent row
  b += al((long long)R * DRAW_BUF * 8);              // draw buffers
  b += al((long long)R * 8) * 6;                     // beta, maxbox, en, box, ham(2)
  b += al((long long)R * 16);                        // maxd
  b += al((long long)R * 6 * 8);                     // counters
  b += al((long long)R * 8) * 2;                     // boxh, maxboxh
  b += al((long long)R * 16);                        // maxd_sep
  b += al((long long)R * 4 * 8);                     // cnt_sep
  b += al((long long)R * 4) * 2;                     // wos, sow
  b += al((long long)R * 8) * 4 + al((long long)R * 4);  // walker rc2, drift, ctr, base, status
  return b;
}

}  // namespace ptmc

// kernel launch entry points (ptmc_cycles.cu, ptmc_cycles32.cu)
namespace ptmc {
long long cycles32_smem_bytes(int pot, int R, int N, int ncta);
// FP32 form with lpr = 4 or 8 lanes per walker (NVT, one CTA of R * lpr
// threads per run, ptmc_cycles32n.cu)
long long cycles32n_smem_bytes(int pot, int R, int N, int lpr);
int launch_cycles32n(int pot, int bc, const KParams& P, int run0, int nruns, int R, int maxN,
                     int ncycles, int phase, int lpr, void* stream);
// resident CTAs per SM of a cycle kernel (cudaOccupancyMaxActiveBlocksPerMultiprocessor)
int occupancy_cycles(int pot, int bc, int ens, int R, int N, int* ctas_per_sm);
int occupancy_cycles32(int pot, int bc, int ens, int R, int N, int ncta, int lpr, int* ctas_per_sm);
int occupancy_cycles32n(int pot, int bc, int R, int N, int lpr, int* ctas_per_sm);
// ncta: CTAs per run (a thread-block cluster when > 1; FP32 form only)
// lpr: lanes per walker (32 or 16; FP32 form only)
int launch_cycles32(int pot, int bc, int ens, const KParams& P, int run0, int nruns, int R,
                    int maxN, int ncycles, int phase, int ncta, int lpr, void* stream);
int launch_cycles(int pot, int bc, int ens, bool f32, const KParams& P,
                  int run0, int nruns, int R, int maxN, int ncycles, int phase,
                  void* stream, int ncta = 1, int lpr = 32);
int launch_init(int pot, int bc, int ens, bool f32, const KParams& P,
                int run0, int nruns, int R, void* stream);
int launch_resync(int pot, int bc, int ens, bool f32, const KParams& P,
                  int run0, int nruns, int R, void* stream);
// multihistogram (ptmc_wham.cu); scratch is caller-provided device memory
int wham_nvt_device(int R, int n_bin, const double* d_hist, const double* d_beta,
                    double en_min, double en_max, double thr,
                    const double* d_beta_out, int n_out, double* d_work,
                    double* d_out, int* d_iters, void* stream);
int wham_npt_device(int R, int n_bin, const double* d_hist, const double* d_beta,
                    double en_min, double en_max, double v_min, double v_max,
                    double p, double thr, const double* d_beta_out, int n_out,
                    double* d_work, double* d_out, int* d_iters, void* stream);
long long wham_work_doubles(int R, int n_bins_total);
// sets the message returned by ptmc_last_error(NULL) (ptmc_capi.cu)
void set_last_error(const std::string& msg);
}  // namespace ptmc
