// ptmc_capi.cu — the C ABI (include/ptmc_gb300.h): context, HBM layout,
// orchestration of the replica cycles, outputs and checkpoints.
//
// What replaces what: ptmc_create/ptmc_set_*/ptmc_init replace MCParams,
// TempGrid, the ensemble/potential constructors and initialisation()
// (src/Initialization.jl:70-100); ptmc_equilibrate replaces equilibration()
// (src/MCRun.jl:322-344); ptmc_run_cycles replaces the main loop of
// ptmc_run! (src/MCRun.jl:397-419); ptmc_get_output replaces
// finalise_results (src/Sampling.jl:377-399); ptmc_checkpoint/ptmc_restore
// replace checkpoint/save_configs/rebuild_states (src/ReadSave.jl:93-218,
// 330-481).
//
// Runs are grouped by atom count.  One group = one kernel launch per chunk of
// cycles (grid = runs of the group, block = 32 x replicas).  Groups run on
// forked streams so uneven-N batches execute concurrently; a chunk sequence of
// every group is captured once into a CUDA graph and replayed.
#include <cuda_runtime.h>

#include <algorithm>
#include <charconv>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <sys/stat.h>
#include <vector>

#include "../../include/ptmc_gb300.h"
#include "ptmc_engine.cuh"
#include "ptmc_nn.cuh"
#include "ptmc_nn2.cuh"
#include "ptmc_surrogate.cuh"

using namespace ptmc;

namespace {
thread_local std::string g_err;
const double kB = 3.16681196E-6;  // src/InputParams.jl:19

struct HostRun {
  int N = 0;
  int n_start = 0;
  int bc = -1;
  double bc_param = 0;       // sphere radius, cube side, box_length
  double bc_height = 0;      // box_height (RectangularBC, RhombicBC)
  std::vector<double> xyz;   // n_start * N * 3
  std::vector<double> maxd;  // 2R (optional)
  std::vector<double> maxd_sep;  // 2R (optional): max_displ[3:4]
};

struct Group {
  int N;
  int dev0;    // first device run index
  int nruns;
  cudaStream_t st = nullptr;
  int ncta = 1;  // CTAs per run (thread-block cluster size; FP32 form), set by ptmc_autotune
  int lpr = 32;  // lanes per walker (32, 16, 8 or 4; FP32 form)
};

template <typename T>
struct DBuf {
  T* p = nullptr;
  size_t n = 0;
  bool own = true;  // false: a slice of the context's state block
  int alloc(size_t count) {
    n = count;
    own = true;
    if (count == 0) count = 1;
    return (int)cudaMalloc(&p, count * sizeof(T));
  }
  void free_() {
    if (p && own) cudaFree(p);
    p = nullptr;
    own = true;
  }
  // bytes of a slice of `count` elements (at least one), 256-byte aligned
  static size_t span(size_t count) {
    return ((count ? count : 1) * sizeof(T) + 255) / 256 * 256;
  }
  void place(unsigned char*& cur, size_t count) {
    n = count;
    p = (T*)cur;
    own = false;
    cur += span(count);
  }
};

// Shortest round-trip text of a double in Julia's print style ("0.1",
// "100.0", "1.0e6", "-5.62340834334278e7", "1.0e-5"), so that checkpoint files
// read like the reference's writedlm output (src/ReadSave.jl).
std::string fmt_double(double v) {
  if (v == 0) return std::signbit(v) ? "-0.0" : "0.0";
  if (std::isnan(v)) return "NaN";
  if (std::isinf(v)) return v > 0 ? "Inf" : "-Inf";
  char buf[64];
  auto r = std::to_chars(buf, buf + sizeof(buf), v, std::chars_format::scientific);
  std::string sc(buf, r.ptr);  // [-]d[.ddd]e(+|-)XX
  bool neg = sc[0] == '-';
  if (neg) sc = sc.substr(1);
  size_t ep = sc.find('e');
  std::string mant = sc.substr(0, ep);
  int ex = std::stoi(sc.substr(ep + 1));
  std::string digits;
  for (char ch : mant)
    if (ch != '.') digits += ch;
  while (digits.size() > 1 && digits.back() == '0') digits.pop_back();
  std::string out;
  if (ex >= -4 && ex < 6) {  // Julia: 0.0001 fixed, 1.0e-5 and 1.0e6 scientific
    if (ex >= 0) {
      std::string ip = digits.substr(0, std::min<size_t>(digits.size(), ex + 1));
      while ((int)ip.size() < ex + 1) ip += '0';
      std::string fp = (int)digits.size() > ex + 1 ? digits.substr(ex + 1) : "0";
      out = ip + "." + fp;
    } else {
      out = "0." + std::string(-ex - 1, '0') + digits;
    }
  } else {
    out = digits.substr(0, 1) + "." + (digits.size() > 1 ? digits.substr(1) : "0") + "e" +
          std::to_string(ex);
  }
  return neg ? "-" + out : out;
}

bool write_file_atomic(const std::string& path, const std::string& data) {
  std::string tmp = path + ".tmp";
  FILE* f = std::fopen(tmp.c_str(), "wb");
  if (!f) return false;
  bool ok = std::fwrite(data.data(), 1, data.size(), f) == data.size();
  ok = (std::fclose(f) == 0) && ok;
  if (!ok) return false;
  return std::rename(tmp.c_str(), path.c_str()) == 0;
}
}  // namespace

struct ptmc_ctx {
  void* state_block = nullptr;  // one device allocation for the state set up by ptmc_init
  ptmc_params p{};
  std::string err;
  int pot = -1;
  std::vector<double> coeff;
  double eam[4] = {0, 0, 0, 0};
  std::vector<HostRun> runs;
  // layout
  std::vector<int> dev_of_run, run_of_dev;
  std::vector<Group> groups;
  std::vector<RunDesc> rd;  // device-ordered
  int W = 0;                // total walkers
  bool inited = false, equilibrated = false;
  // device state
  DBuf<RunDesc> d_runs;
  DBuf<double> d_pos, d_mat, d_comp, d_en, d_box, d_rc2, d_drift, d_beta, d_maxd,
      d_maxbox, d_ham;
  bool sep_vol = false;        // NPT.separated_volume
  DBuf<double> d_boxh, d_maxboxh, d_maxd_sep;  // box height, max_boxheight, max_displ[3:4]
  DBuf<long long> d_cnt_sep;   // count_vol_xy[1:2], count_vol_z[1:2] per slot
  // ELJPotentialB (coeff_c in coeff) and LookupTablePotential
  std::vector<double> eljb_a, eljb_b, lut;
  int lut_na = 0, lut_nd = 0;
  double lut_par[4] = {0, 0, 0, 0};  // start_dist, d_dist, d_angle, c6coeff
  DBuf<double> d_tan, d_lut;
  DBuf<double> d_pe;           // plain form, NVT: pair cache (pair_cache in ptmc_engine.cuh)
  DBuf<float> d_lo;            // FP32 form: lo halves of positions during a narrow launch
  bool glob = false;           // plain form: per-atom state in HBM (runs beyond shared memory)
  DBuf<double> d_scr;          // its per-walker trial-row scratch
  // two-species RuNNer potential (NNVT ensemble)
  std::vector<double> nn2_rad, nn2_ang, nn2_W1, nn2_W2;
  int nn2_n1 = 0, nn2_H1 = 0, nn2_H2 = 0, n_swaps = 1;
  NN2Params Q2{};
  DBuf<double> d_nn2_rad, d_nn2_ang, d_nn2_W1, d_nn2_W2;
  DBuf<long long> d_nn2_swaps;
  DBuf<unsigned long long> d_ctr;
  DBuf<int> d_status, d_wos;
  DBuf<long long> d_cnt;
  DBuf<unsigned int> d_hist;
  // exchange-partner wait of the FP32 form: limit in clocks, test switch
  long long xwait_clocks = XWAIT_CLOCKS;
  int xwait_never = 0;
  bool rdf_on = false;         // radial distribution sampling (rdfsave of ptmc_run!)
  DBuf<unsigned int> d_rdf;    // [W][5 n_bin]
  KParams K{};
  // neural-network potential
  std::vector<NNSF> nn_sf;    // active functions (radial, then angular sorted by eta)
  std::vector<double> nn_W;   // gathered MLP parameters
  int nn_H1 = 0, nn_H2 = 0, nn_Nmax = 0;
  double nn_rcut = 0, nn_boundary2 = 0;
  DBuf<NNSF> d_nn_sf;
  DBuf<double> d_nn_W, d_nn_G;
  DBuf<int> d_nn_row, d_nn_sow;
  NNParams Q{};
  // delayed-acceptance surrogate (ptmc_surrogate.cuh)
  bool sur_set = false;
  ptmc_surrogate_cfg sur_cfg{};
  DBuf<float> d_sur_P, d_sur_m, d_sur_v, d_sur_g, d_rec_rows, d_rec_y;
  DBuf<double> d_sur_loss;
  DBuf<unsigned long long> d_rec_n;
  DBuf<long long> d_da_cnt;
  DBuf<int> d_sur_err, d_rec_slot;
  DBuf<float> d_da_kappa;
  DBuf<float> d_sur_tab;  // phi on the grid (first stage of screened moves)
  std::vector<double> sur_kappa;  // per slot index
  int sur_step = 0;  // Adam steps taken
  cudaStream_t st = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr, evfork = nullptr;
  std::vector<cudaEvent_t> evjoin;
  std::map<long long, cudaGraphExec_t> graphs;  // key: phase*2^40 + chunk*2^8 + reps
  ptmc_stats stats{};
  std::vector<double> T, beta;

  int fail(int code, const std::string& m) {
    err = m;
    g_err = m;
    return code;
  }
  int cuda_fail(cudaError_t e, const char* where) {
    return fail(PTMC_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
  }
  int R() const { return p.n_traj; }
  int bc() const { return runs.empty() ? 0 : runs[0].bc; }
  bool boxh() const { return bc() == PTMC_BC_RECTANGULAR || bc() == PTMC_BC_RHOMBIC; }
  bool f32() const { return p.precision == PTMC_FP32_RESYNC; }
};

#define CK(call)                                              \
  do {                                                        \
    cudaError_t e_ = (call);                                  \
    if (e_ != cudaSuccess) return c->cuda_fail(e_, #call);    \
  } while (0)

namespace {

// replica start positions from the runs' start configurations: walker w of a
// run starts from configuration w mod n_start (src/Initialization.jl:88-96);
// only the distinct configurations cross the host link
__global__ void k_expand_starts(const RunDesc* runs, const double* starts,
                                const long long* start_off, const int* n_start, double* pos) {
  const RunDesc rd = runs[blockIdx.x];
  const double* src = starts + start_off[blockIdx.x];
  const int per = rd.N * 3, ns = n_start[blockIdx.x];
  double* dst = pos + rd.pos_off;
  for (long long k = threadIdx.x; k < (long long)rd.R * per; k += blockDim.x) {
    const int w = (int)(k / per), e = (int)(k % per);
    dst[k] = src[(long long)(w % ns) * per + e];
  }
}

int check_status(ptmc_ctx* c) {
  std::vector<int> st(c->W);
  CK(cudaMemcpyAsync(st.data(), c->d_status.p, sizeof(int) * c->W, cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  for (int i = 0; i < c->W; ++i) {
    if (st[i] == ST_SPHERE)
      return c->fail(PTMC_ERR_SPHERE, "Error: too many moves out of binding sphere");
    if (st[i] == ST_TIMEOUT)
      return c->fail(PTMC_ERR_CUDA, "a tensor-core completion wait ran out (surrogate stage)");
    if (st[i] == ST_XWAIT)
      return c->fail(PTMC_ERR_CUDA, "a wait for an exchange partner ran out (FP32 cycle kernel)");
  }
  return PTMC_OK;
}

int push_runs(ptmc_ctx* c) {
  CK(cudaMemcpyAsync(c->d_runs.p, c->rd.data(), sizeof(RunDesc) * c->rd.size(),
                     cudaMemcpyHostToDevice, c->st));
  return PTMC_OK;
}
int pull_runs(ptmc_ctx* c) {
  CK(cudaMemcpyAsync(c->rd.data(), c->d_runs.p, sizeof(RunDesc) * c->rd.size(),
                     cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  return PTMC_OK;
}

// one chunk of `ncyc` cycles for every group, groups on forked streams
int enqueue_chunk(ptmc_ctx* c, int ncyc, int phase) {
  if (c->pot == POT_NN2) {  // one cycle kernel + one run epilogue per cycle
    for (int k = 0; k < ncyc; ++k) {
      int rc = nn2_launch_cycle(c->K, c->Q2, c->Q, c->W, (int)c->rd.size(), c->R(), c->nn_Nmax,
                                phase, c->st);
      if (rc) return c->cuda_fail((cudaError_t)rc, "k_nn2_cycle launch");
      c->stats.kernel_launches += 2;
    }
    return PTMC_OK;
  }
  if (c->pot == POT_NN) {  // one cycle kernel + one run epilogue per cycle
    for (int k = 0; k < ncyc; ++k) {
      int rc = nn_launch_cycle(c->K, c->Q, c->W, (int)c->rd.size(), c->R(), c->nn_Nmax,
                               !c->f32(), phase, c->st);
      if (rc) return c->cuda_fail((cudaError_t)rc, "k_nn_cycle launch");
      c->stats.kernel_launches += 2;
    }
    return PTMC_OK;
  }
  CK(cudaEventRecord(c->evfork, c->st));
  for (size_t g = 0; g < c->groups.size(); ++g) {
    Group& G = c->groups[g];
    CK(cudaStreamWaitEvent(G.st, c->evfork, 0));
    int rc = launch_cycles(c->pot, c->bc(), c->p.ensemble, c->f32(), c->K, G.dev0,
                           G.nruns, c->R(), G.N, ncyc, phase, G.st, c->f32() ? G.ncta : 1,
                           c->f32() ? G.lpr : 32);
    if (rc) return c->cuda_fail((cudaError_t)rc, "k_cycles launch");
    CK(cudaEventRecord(c->evjoin[g], G.st));
    CK(cudaStreamWaitEvent(c->st, c->evjoin[g], 0));
    c->stats.kernel_launches += 1;
  }
  return PTMC_OK;
}

int default_chunk(ptmc_ctx* c) {
  if (c->p.cycles_per_launch > 0) return c->p.cycles_per_launch;
  if (c->pot == POT_NN || c->pot == POT_NN2) return 16;  // cycles per chunk (2 launches each)
  // aim at a few milliseconds of work per launch
  int maxN = 0;
  for (auto& G : c->groups) maxN = std::max(maxN, G.N);
  long long per_cycle = (long long)maxN * maxN;  // pair terms per walker-cycle
  long long chunk = std::max(1LL, 4000000LL / std::max(1LL, per_cycle));
  return (int)std::min(chunk, 2000LL);
}

int run_phase(ptmc_ctx* c, long long n, int phase) {
  if (n <= 0) return PTMC_OK;
  int chunk = default_chunk(c);
  CK(cudaEventRecord(c->ev0, c->st));
  long long done = 0;
  const int reps = 8;
  long long nfull = n / ((long long)chunk * reps);
  if (nfull > 0) {
    long long key = ((long long)phase << 40) | ((long long)chunk << 8) | reps;
    auto it = c->graphs.find(key);
    if (it == c->graphs.end()) {
      cudaGraph_t graph;
      CK(cudaStreamBeginCapture(c->st, cudaStreamCaptureModeThreadLocal));
      long long saved = c->stats.kernel_launches;
      for (int r = 0; r < reps; ++r) {
        int rc = enqueue_chunk(c, chunk, phase);
        if (rc) {
          cudaStreamEndCapture(c->st, &graph);
          return rc;
        }
      }
      c->stats.kernel_launches = saved;
      CK(cudaStreamEndCapture(c->st, &graph));
      cudaGraphExec_t ex;
      CK(cudaGraphInstantiate(&ex, graph, 0));
      cudaGraphDestroy(graph);
      it = c->graphs.emplace(key, ex).first;
    }
    for (long long k = 0; k < nfull; ++k) {
      CK(cudaGraphLaunch(it->second, c->st));
      c->stats.graph_launches += 1;
      c->stats.kernel_launches +=
          (c->pot == POT_NN || c->pot == POT_NN2) ? 2LL * reps * chunk
                                                  : (long long)reps * c->groups.size();
    }
    done = nfull * chunk * reps;
  }
  while (done < n) {
    int m = (int)std::min<long long>(chunk, n - done);
    int rc = enqueue_chunk(c, m, phase);
    if (rc) return rc;
    done += m;
  }
  CK(cudaEventRecord(c->ev1, c->st));
  CK(cudaEventSynchronize(c->ev1));
  float ms = 0;
  CK(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
  c->stats.last_cycles_ms = ms;
  long long atom_slots = 0, vol_slots = 0;
  for (auto& G : c->groups) {
    atom_slots += (long long)G.nruns * c->R() * G.N;
    if (c->p.ensemble == PTMC_NPT) vol_slots += (long long)G.nruns * c->R();
  }
  // attempted moves: n_steps per walker-cycle split by the slot draw; the
  // expected split is exact on average, report the nominal counts
  c->stats.atom_moves += atom_slots * n;
  c->stats.volume_moves += vol_slots * n;
  CK(cudaGetLastError());
  return check_status(c);
}

}  // namespace

namespace ptmc {
void set_last_error(const std::string& msg) { g_err = msg; }
}  // namespace ptmc

// ================================================================ C ABI
extern "C" {

const char* ptmc_version(void) { return "ptmc-gb300 0.1 (sm_103a)"; }

const char* ptmc_last_error(ptmc_ctx* c) { return c ? c->err.c_str() : g_err.c_str(); }

int ptmc_create(ptmc_ctx** out, const ptmc_params* p) {
  if (!out || !p) {
    g_err = "ptmc_create: null argument";
    return PTMC_ERR_ARG;
  }
  *out = nullptr;
  if (p->n_runs < 1 || p->n_traj < 1) {
    g_err = "ptmc_create: need n_runs >= 1 and n_traj >= 1";
    return PTMC_ERR_ARG;
  }
  if (p->n_traj > 1024) {
    g_err = "ptmc_create: at most 1024 replicas per run";
    return PTMC_ERR_LIMIT;
  }
  if (p->n_bin < 2 || p->n_adjust < 1 || p->mc_sample < 1 || p->mc_cycles < 0 || p->eq_cycles < 0) {
    g_err = "ptmc_create: invalid MCParams";
    return PTMC_ERR_ARG;
  }
  if (p->ensemble != PTMC_NVT && p->ensemble != PTMC_NPT && p->ensemble != PTMC_NNVT) {
    g_err = "ptmc_create: unknown ensemble";
    return PTMC_ERR_ARG;
  }
  if (p->tdistr != PTMC_TGEOMETRIC && p->tdistr != PTMC_TLINEAR) {
    g_err = "chosen temperature distribution does not exist";  // InputParams.jl:91
    return PTMC_ERR_ARG;
  }
  if (p->precision != PTMC_FP64 && p->precision != PTMC_FP32_RESYNC) {
    g_err = "ptmc_create: unknown precision";
    return PTMC_ERR_ARG;
  }
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0) {
    g_err = std::string("ptmc_create: no CUDA device: ") + cudaGetErrorString(e);
    return PTMC_ERR_CUDA;
  }
  if (p->device < 0 || p->device >= ndev) {
    g_err = "ptmc_create: bad device ordinal";
    return PTMC_ERR_ARG;
  }
  e = cudaSetDevice(p->device);
  if (e != cudaSuccess) {
    g_err = std::string("cudaSetDevice: ") + cudaGetErrorString(e);
    return PTMC_ERR_CUDA;
  }
  ptmc_ctx* c = new ptmc_ctx();
  c->p = *p;
  c->runs.resize(p->n_runs);
  // TempGrid (src/InputParams.jl:77-95)
  int R = p->n_traj;
  c->T.resize(R);
  c->beta.resize(R);
  for (int i = 0; i < R; ++i) {
    if (R == 1) c->T[i] = p->t_i;
    else if (p->tdistr == PTMC_TLINEAR) c->T[i] = p->t_i + i * ((p->t_f - p->t_i) / (R - 1));
    else c->T[i] = p->t_i * std::pow(p->t_f / p->t_i, (double)i / (double)(R - 1));
    c->beta[i] = 1.0 / (kB * c->T[i]);
  }
  if (cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&c->ev0) != cudaSuccess || cudaEventCreate(&c->ev1) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->evfork, cudaEventDisableTiming) != cudaSuccess) {
    g_err = "ptmc_create: stream/event creation failed";
    delete c;
    return PTMC_ERR_CUDA;
  }
  *out = c;
  return PTMC_OK;
}

int ptmc_set_potential_elj(ptmc_ctx* c, const double* coeff, int K, int even) {
  if (!c || !coeff) return PTMC_ERR_ARG;
  if (K < 1 || K > MAX_COEFF) return c->fail(PTMC_ERR_LIMIT, "ELJ: 1..16 coefficients supported");
  if (c->p.ensemble == PTMC_NPT && !even)
    return c->fail(PTMC_ERR_ARG, "NPT long-range correction is defined for ELJPotentialEven only");
  c->pot = even ? POT_ELJEVEN : POT_ELJ;
  c->coeff.assign(coeff, coeff + K);
  return PTMC_OK;
}

int ptmc_set_potential_eljb(ptmc_ctx* c, const double* a, const double* b, const double* cc,
                            int K) {
  if (!c || !a || !b || !cc) return PTMC_ERR_ARG;
  if (K < 2 || K > MAX_COEFF) return c->fail(PTMC_ERR_ARG, "ELJPotentialB: 2..16 coefficients");
  c->pot = POT_ELJB;
  c->eljb_a.assign(a, a + K);
  c->eljb_b.assign(b, b + K);
  c->coeff.assign(cc, cc + K);
  return PTMC_OK;
}

int ptmc_set_potential_lookup(ptmc_ctx* c, const double* table, int l_angle, int l_dist,
                              double start_dist, double start_angle, double d_dist,
                              double d_angle, double c6coeff) {
  if (!c || !table) return PTMC_ERR_ARG;
  if (l_angle < 1 || l_dist < 1 || !(d_dist > 0) || !(d_angle > 0))
    return c->fail(PTMC_ERR_ARG, "LookupTablePotential: bad table dimensions or steps");
  (void)start_angle;  // the angle index starts at 0 degrees (EnergyEvaluation.jl:279-285)
  c->pot = POT_LUT;
  c->lut.assign(table, table + (size_t)l_angle * l_dist);
  c->lut_na = l_angle;
  c->lut_nd = l_dist;
  c->lut_par[0] = start_dist;
  c->lut_par[1] = d_dist;
  c->lut_par[2] = d_angle;
  c->lut_par[3] = c6coeff;
  c->coeff.clear();
  return PTMC_OK;
}

int ptmc_set_potential_nn2(ptmc_ctx* c, const double* rad, int nrad, const double* ang, int nang,
                           const double* w1, const double* w2, int nw, const int* nodes,
                           int n_layers, int n1) {
  if (!c || !rad || (nang > 0 && !ang) || !w1 || !w2 || !nodes) return PTMC_ERR_ARG;
  if (c->p.ensemble != PTMC_NNVT)
    return c->fail(PTMC_ERR_ARG, "RuNNerPotential2Atom runs in the NNVT ensemble");
  if (nrad < 1 || nang < 0 || n1 < 1) return c->fail(PTMC_ERR_ARG, "NNVT: bad symmetry-function counts");
  const int Ng = 2 * nrad + 3 * nang;
  if (n_layers != 4 || nodes[0] != Ng || nodes[3] != 1)
    return c->fail(PTMC_ERR_ARG, "RuNNerPotential2Atom: nodes = [2 nrad + 3 nang, H1, H2, 1]");
  if (nodes[1] < 1 || nodes[2] < 1 || nodes[1] > MAX_NN2_HIDDEN || nodes[2] > MAX_NN2_HIDDEN)
    return c->fail(PTMC_ERR_LIMIT, "RuNNerPotential2Atom: 1..64 units per hidden layer");
  const long need = (long)Ng * nodes[1] + nodes[1] + (long)nodes[1] * nodes[2] + nodes[2] + nodes[2] + 1;
  if (nw != need) return c->fail(PTMC_ERR_ARG, "RuNNerPotential2Atom: weight count does not match nodes");
  c->pot = POT_NN2;
  c->nn2_rad.assign(rad, rad + 10 * (size_t)nrad);
  c->nn2_ang.assign(ang, ang + 16 * (size_t)nang);
  c->nn2_W1.assign(w1, w1 + nw);
  c->nn2_W2.assign(w2, w2 + nw);
  c->nn2_n1 = n1;
  c->nn2_H1 = nodes[1];
  c->nn2_H2 = nodes[2];
  c->Q2.nrad = nrad;
  c->Q2.nang = nang;
  return PTMC_OK;
}

int ptmc_set_atom_swaps(ptmc_ctx* c, int n_swaps) {
  if (!c) return PTMC_ERR_ARG;
  if (c->inited) return c->fail(PTMC_ERR_STATE, "atom swaps are set before ptmc_init");
  if (n_swaps < 0) return c->fail(PTMC_ERR_ARG, "n_atom_swaps must be >= 0");
  c->n_swaps = n_swaps;
  return PTMC_OK;
}

int ptmc_get_swaps(ptmc_ctx* c, int run, long long* accepted) {
  if (!c || !accepted) return PTMC_ERR_ARG;
  if (!c->inited) return c->fail(PTMC_ERR_STATE, "ptmc_init not called");
  if (run < 0 || run >= c->p.n_runs) return c->fail(PTMC_ERR_ARG, "run index out of range");
  *accepted = 0;
  if (c->pot != POT_NN2) return PTMC_OK;
  const RunDesc& r = c->rd[c->dev_of_run[run]];
  std::vector<long long> sw(c->R());
  CK(cudaMemcpy(sw.data(), c->d_nn2_swaps.p + r.wk, sizeof(long long) * c->R(), cudaMemcpyDeviceToHost));
  for (long long v : sw) *accepted += v;
  return PTMC_OK;
}

int ptmc_set_potential_eam(ptmc_ctx* c, double n, double m, double ean, double ecam) {
  if (!c) return PTMC_ERR_ARG;
  if (c->p.ensemble == PTMC_NPT) return c->fail(PTMC_ERR_ARG, "EAM is supported in the NVT ensemble only");
  c->pot = POT_EAM;
  c->eam[0] = n;
  c->eam[1] = m;
  c->eam[2] = ean;
  c->eam[3] = ecam;
  return PTMC_OK;
}

int ptmc_set_potential_nn(ptmc_ctx* c, const double* sf, int nsf, const double* weights, int nw,
                          const int* nodes, int n_layers, double boundary) {
  if (!c || !sf || !weights || !nodes) return PTMC_ERR_ARG;
  if (c->p.ensemble == PTMC_NPT) return c->fail(PTMC_ERR_ARG, "NN potential is supported in the NVT ensemble only");
  if (n_layers != 4 || nodes[0] != nsf || nodes[3] != 1)
    return c->fail(PTMC_ERR_ARG, "NN: layers must be {n_sf, H1, H2, 1} (ForwardPass.jl:21)");
  int H1 = nodes[1], H2 = nodes[2];
  if (H1 < 1 || H2 < 1 || H1 > 64 || H2 > 64) return c->fail(PTMC_ERR_LIMIT, "NN: hidden layers of 1..64 nodes");
  long long need = (long long)nsf * H1 + H1 + (long long)H1 * H2 + H2 + H2 + 1;
  if (need != nw) return c->fail(PTMC_ERR_ARG, "NN: weight count does not match the layer sizes");
  // active functions: radial type 11 in table order, angular type 111 sorted by
  // (eta, lambda, zeta)
  std::vector<int> rad, ang;
  double rc = -1;
  for (int k = 0; k < nsf; ++k) {
    const double* q = sf + 8 * k;
    int kind = (int)q[0], type = (int)q[1];
    if (rc < 0) rc = q[5];
    if (q[5] != rc) return c->fail(PTMC_ERR_ARG, "NN: all symmetry functions must share one cut-off");
    if (kind == 0 && type == 11) rad.push_back(k);
    if (kind == 1 && type == 111) ang.push_back(k);
  }
  std::stable_sort(ang.begin(), ang.end(), [&](int a, int b) {
    const double* x = sf + 8 * a;
    const double* y = sf + 8 * b;
    if (x[2] != y[2]) return x[2] < y[2];
    if (x[3] != y[3]) return x[3] < y[3];
    return x[4] < y[4];
  });
  if ((int)ang.size() > MAX_NN_ANG) return c->fail(PTMC_ERR_LIMIT, "NN: at most 32 active angular functions");
  std::vector<int> act(rad);
  act.insert(act.end(), ang.begin(), ang.end());
  c->nn_sf.clear();
  for (int k : act) {
    const double* q = sf + 8 * k;
    NNSF f{};
    f.eta = q[2];
    f.lambda = q[3];
    f.zeta = q[4];
    double gmin = q[6], gmax = q[7];
    f.gnorm = 1 / (gmax - gmin);  // RadialType2 / AngularType3 with [max, min]
    f.goffset = -gmin * f.gnorm;
    f.tpz = std::pow(2.0, 1 - f.zeta) * f.gnorm;
    f.zc = f.zeta == 1 ? 1 : f.zeta == 2 ? 2 : f.zeta == 4 ? 3 : f.zeta == 8 ? 4 : f.zeta == 16 ? 5 : 0;
    c->nn_sf.push_back(f);
  }
  // gather the MLP: W1 rows of the active inputs, the rest unchanged
  int S = (int)act.size();
  std::vector<double>& W = c->nn_W;
  W.clear();
  for (int q = 0; q < S; ++q)
    for (int h = 0; h < H1; ++h) W.push_back(weights[(size_t)act[q] * H1 + h]);
  const double* rest = weights + (size_t)nsf * H1;
  W.insert(W.end(), rest, rest + (H1 + (size_t)H1 * H2 + H2 + H2 + 1));
  c->nn_H1 = H1;
  c->nn_H2 = H2;
  c->nn_rcut = rc;
  c->nn_boundary2 = boundary * boundary;
  c->Q.SR = (int)rad.size();
  c->Q.SA = (int)ang.size();
  // a sorted angular set whose structure (eta groups, lambda signs, zeta
  // powers) matches a compiled pattern runs the table-specialised FP32 kernel;
  // the eta values themselves are runtime parameters
  c->Q.ang_pat = NN_PAT_GENERIC;
  for (int pat : {NN_PAT_CU55}) {
    const int n = nn_pat_sa(pat);
    if ((int)ang.size() != n) continue;
    bool ok = true;
    int g = -1;
    float nle[8] = {};
    for (int q = 0; q < n && ok; ++q) {
      const double* r = sf + 8 * ang[q];
      const double eta = r[2], lam = r[3], zeta = r[4];
      if (q == 0 || eta != sf[8 * ang[q - 1] + 2]) {
        if (++g >= 8) break;
        nle[g] = (float)(-eta * 1.4426950408889634);
      }
      const int e = zeta == 1 ? 0 : zeta == 2 ? 1 : zeta == 4 ? 2 : zeta == 8 ? 3 : zeta == 16 ? 4 : -1;
      ok = e >= 0 && (lam == 1.0 || lam == -1.0) &&
           nn_pat_term(pat, q) == (g | ((lam < 0 ? 1 : 0) << 4) | (e << 5));
    }
    if (ok && g + 1 == nn_pat_ng(pat)) {
      c->Q.ang_pat = pat;
      for (int k = 0; k < 8; ++k) c->Q.ang_nle[k] = nle[k];
      break;
    }
  }
  c->pot = POT_NN;
  return PTMC_OK;
}

int ptmc_set_run_configs(ptmc_ctx* c, int run, const double* xyz, int N, int n_start,
                         int bc_kind, double bc_param) {
  return ptmc_set_run_configs_box(c, run, xyz, N, n_start, bc_kind, bc_param, bc_param);
}

namespace {
// the checks of a start-configuration call that do not depend on the run
int check_configs(ptmc_ctx* c, const double* xyz, int N, int n_start, int bc_kind,
                  double bc_param, double box_height) {
  if (!c || !xyz) return PTMC_ERR_ARG;
  if (c->inited) return c->fail(PTMC_ERR_STATE, "configurations must be set before ptmc_init");
  if (N < 2) return c->fail(PTMC_ERR_ARG, "need at least 2 atoms");
  if (N > 1024) return c->fail(PTMC_ERR_LIMIT, "at most 1024 atoms per configuration");
  if (n_start < 1) return c->fail(PTMC_ERR_ARG, "need at least one start configuration");
  if (bc_kind != PTMC_BC_SPHERE && bc_kind != PTMC_BC_CUBIC && bc_kind != PTMC_BC_RECTANGULAR &&
      bc_kind != PTMC_BC_RHOMBIC)
    return c->fail(PTMC_ERR_ARG, "unknown boundary condition");
  if (!(bc_param > 0)) return c->fail(PTMC_ERR_ARG, "boundary parameter must be positive");
  if (!(box_height > 0)) return c->fail(PTMC_ERR_ARG, "box height must be positive");
  if (c->p.ensemble == PTMC_NPT && bc_kind == PTMC_BC_SPHERE)
    return c->fail(PTMC_ERR_ARG, "SphericalBC cannot be used in an NPT ensemble.");  // Ensembles.jl:192
  for (auto& r : c->runs)
    if (r.bc >= 0 && r.bc != bc_kind)
      return c->fail(PTMC_ERR_ARG, "all runs of a context share one boundary kind");
  return PTMC_OK;
}

void store_configs(HostRun& h, const double* xyz, int N, int n_start, int bc_kind,
                   double bc_param, double box_height) {
  h.N = N;
  h.n_start = n_start;
  h.bc = bc_kind;
  h.bc_param = bc_param;
  h.bc_height = (bc_kind == PTMC_BC_RECTANGULAR || bc_kind == PTMC_BC_RHOMBIC) ? box_height : bc_param;
  h.xyz.assign(xyz, xyz + (size_t)n_start * N * 3);
}
}  // namespace

int ptmc_set_runs_configs(ptmc_ctx* c, int first, int n_runs, const double* xyz, int N,
                          int bc_kind, double box_length, double box_height) {
  int rc = check_configs(c, xyz, N, 1, bc_kind, box_length, box_height);
  if (rc) return rc;
  if (n_runs < 1 || first < 0 || first + n_runs > c->p.n_runs)
    return c->fail(PTMC_ERR_ARG, "run range out of bounds");
  for (int r = 0; r < n_runs; ++r)
    store_configs(c->runs[first + r], xyz + (size_t)r * N * 3, N, 1, bc_kind, box_length,
                  box_height);
  return PTMC_OK;
}

int ptmc_set_run_configs_box(ptmc_ctx* c, int run, const double* xyz, int N, int n_start,
                             int bc_kind, double box_length, double box_height) {
  const double bc_param = box_length;
  if (!c || !xyz) return PTMC_ERR_ARG;
  if (c->inited) return c->fail(PTMC_ERR_STATE, "configurations must be set before ptmc_init");
  if (run < 0 || run >= c->p.n_runs) return c->fail(PTMC_ERR_ARG, "run index out of range");
  if (N < 2) return c->fail(PTMC_ERR_ARG, "need at least 2 atoms");
  if (N > 1024) return c->fail(PTMC_ERR_LIMIT, "at most 1024 atoms per configuration");
  if (n_start < 1) return c->fail(PTMC_ERR_ARG, "need at least one start configuration");
  if (bc_kind != PTMC_BC_SPHERE && bc_kind != PTMC_BC_CUBIC && bc_kind != PTMC_BC_RECTANGULAR &&
      bc_kind != PTMC_BC_RHOMBIC)
    return c->fail(PTMC_ERR_ARG, "unknown boundary condition");
  if (!(bc_param > 0)) return c->fail(PTMC_ERR_ARG, "boundary parameter must be positive");
  if (!(box_height > 0)) return c->fail(PTMC_ERR_ARG, "box height must be positive");
  if (c->p.ensemble == PTMC_NPT && bc_kind == PTMC_BC_SPHERE)
    return c->fail(PTMC_ERR_ARG, "SphericalBC cannot be used in an NPT ensemble.");  // Ensembles.jl:192
  for (auto& r : c->runs)
    if (r.bc >= 0 && r.bc != bc_kind)
      return c->fail(PTMC_ERR_ARG, "all runs of a context share one boundary kind");
  HostRun& h = c->runs[run];
  h.N = N;
  h.n_start = n_start;
  h.bc = bc_kind;
  h.bc_param = bc_param;
  h.bc_height = (bc_kind == PTMC_BC_RECTANGULAR || bc_kind == PTMC_BC_RHOMBIC) ? box_height : bc_param;
  h.xyz.assign(xyz, xyz + (size_t)n_start * N * 3);
  return PTMC_OK;
}

int ptmc_set_separated_volume(ptmc_ctx* c, int on) {
  if (!c) return PTMC_ERR_ARG;
  if (c->inited) return c->fail(PTMC_ERR_STATE, "separated volume moves are set before ptmc_init");
  c->sep_vol = on != 0;
  return PTMC_OK;
}

int ptmc_set_max_displ_sep(ptmc_ctx* c, int run, const double* md) {
  if (!c || !md) return PTMC_ERR_ARG;
  if (run < 0 || run >= c->p.n_runs) return c->fail(PTMC_ERR_ARG, "run index out of range");
  c->runs[run].maxd_sep.assign(md, md + 2 * c->R());
  return PTMC_OK;
}

int ptmc_set_max_displ(ptmc_ctx* c, int run, const double* md) {
  if (!c || !md) return PTMC_ERR_ARG;
  if (run < 0 || run >= c->p.n_runs) return c->fail(PTMC_ERR_ARG, "run index out of range");
  c->runs[run].maxd.assign(md, md + 2 * c->R());
  return PTMC_OK;
}

int ptmc_set_rdf(ptmc_ctx* c, int on) {
  if (!c) return PTMC_ERR_ARG;
  if (c->inited) return c->fail(PTMC_ERR_STATE, "radial distribution sampling is set before ptmc_init");
  c->rdf_on = on != 0;
  return PTMC_OK;
}

int ptmc_init(ptmc_ctx* c) {
  if (!c) return PTMC_ERR_ARG;
  if (c->inited) return c->fail(PTMC_ERR_STATE, "ptmc_init called twice");
  if (c->pot < 0) return c->fail(PTMC_ERR_STATE, "no potential set");
  for (auto& r : c->runs)
    if (r.N == 0) return c->fail(PTMC_ERR_STATE, "every run needs start configurations");
  const int R = c->R();
  const bool nn2 = c->pot == POT_NN2;
  const bool nn = c->pot == POT_NN || nn2;  // one CTA per walker, per-cycle epilogue
  if (c->p.ensemble == PTMC_NNVT && !nn2)
    return c->fail(PTMC_ERR_ARG, "the NNVT ensemble needs RuNNerPotential2Atom");
  if (nn2) {
    if (c->f32())
      return c->fail(PTMC_ERR_ARG, "RuNNerPotential2Atom runs in the plain FP64 form (precision PTMC_FP64)");
    for (auto& r : c->runs) {
      if (r.N > MAX_NN2_ATOMS) return c->fail(PTMC_ERR_LIMIT, "RuNNerPotential2Atom: at most 64 atoms");
      if (r.N <= c->nn2_n1)
        return c->fail(PTMC_ERR_ARG, "NNVT: every run needs atoms of both species (N > n1)");
    }
  }
  // the FP32 form runs more than 32 replicas of a run on a thread-block
  // cluster of C CTAs (R / C <= 32 walkers each): the smallest such C <= 8
  int ncta0 = 1;
  if (!nn && c->f32()) {
    while (ncta0 <= 8 && (R % ncta0 != 0 || R / ncta0 > 32)) ++ncta0;
    if (ncta0 > 8)
      return c->fail(PTMC_ERR_LIMIT, "FP32 form: the replica count needs a divisor C <= 8 with "
                                     "R / C <= 32 (one thread-block cluster of C CTAs per run)");
  }
  if (nn) {
    for (auto& r : c->runs) {
      if (r.N > MAX_NN_ATOMS) return c->fail(PTMC_ERR_LIMIT, "NN potential: at most 64 atoms");
      if (r.bc != PTMC_BC_SPHERE) return c->fail(PTMC_ERR_ARG, "NN potential: SphericalBC only");
    }
  }
  const bool npt = c->p.ensemble == PTMC_NPT;
  const bool bpot = pot_b(c->pot);
  if (c->boxh()) {  // RectangularBC / RhombicBC: the plain FP64 form with the dimer potentials
    if (c->f32())
      return c->fail(PTMC_ERR_ARG,
                     "RectangularBC/RhombicBC run in the plain FP64 form (precision PTMC_FP64)");
    if (c->pot != POT_ELJ && c->pot != POT_ELJEVEN && !bpot)
      return c->fail(PTMC_ERR_ARG, "RectangularBC/RhombicBC: ELJ, ELJPotentialB or "
                                   "LookupTablePotential only");
    if (bpot && !npt)
      return c->fail(PTMC_ERR_ARG, "ELJPotentialB/LookupTablePotential in RectangularBC/RhombicBC: "
                                   "NPT only");
  }
  if (bpot && c->f32())
    return c->fail(PTMC_ERR_ARG,
                   "ELJPotentialB/LookupTablePotential run in the plain FP64 form (precision PTMC_FP64)");
  if (c->sep_vol && (!npt || !c->boxh()))
    return c->fail(PTMC_ERR_ARG,
                   "separated volume moves need the NPT ensemble with a RectangularBC or RhombicBC");
  if (npt && c->pot != POT_ELJEVEN && !bpot)
    return c->fail(PTMC_ERR_ARG, "NPT: ELJPotentialEven, ELJPotentialB or LookupTablePotential "
                                 "(the potentials with a long-range correction, "
                                 "src/EnergyEvaluation.jl:968-1009)");
  // group runs by N: device order sorted by N (stable)
  int nr = c->p.n_runs;
  c->run_of_dev.resize(nr);
  for (int i = 0; i < nr; ++i) c->run_of_dev[i] = i;
  std::stable_sort(c->run_of_dev.begin(), c->run_of_dev.end(),
                   [&](int a, int b) { return c->runs[a].N < c->runs[b].N; });
  c->dev_of_run.resize(nr);
  for (int d = 0; d < nr; ++d) c->dev_of_run[c->run_of_dev[d]] = d;
  c->groups.clear();
  for (int d = 0; d < nr; ++d) {
    int N = c->runs[c->run_of_dev[d]].N;
    if (c->groups.empty() || c->groups.back().N != N) c->groups.push_back({N, d, 0, nullptr});
    c->groups.back().nruns++;
  }
  // Replica state beyond a CTA's shared memory: the FP32 form spreads the run
  // over a larger cluster (fewer walkers per CTA); the plain form keeps the
  // per-atom state in HBM (glob).
  const long long smem_cap = 227 * 1024;
  c->glob = false;
  for (auto& G : c->groups) {
    G.ncta = ncta0;
    if (!nn && c->f32()) {
      while (G.ncta <= 8 && (R % G.ncta != 0 || R / G.ncta > 32 ||
                             cycles32_smem_bytes(c->pot, R, G.N, G.ncta) > smem_cap))
        ++G.ncta;
      if (G.ncta > 8)
        return c->fail(PTMC_ERR_LIMIT, "FP32 form: the replica state of a run does not fit a "
                                       "cluster of 8 CTAs (R * N too large)");
    } else if (!nn && cycles_smem_bytes(c->pot, c->p.ensemble, false, R, G.N) > smem_cap) {
      c->glob = true;
    }
  }
  if (c->glob && cycles_smem_bytes(c->pot, c->p.ensemble, false, R, 0) > smem_cap)
    return c->fail(PTMC_ERR_LIMIT, "the slot tables of a run exceed a CTA's shared memory");
  for (auto& G : c->groups) {
    CK(cudaStreamCreateWithFlags(&G.st, cudaStreamNonBlocking));
    cudaEvent_t e;
    CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    c->evjoin.push_back(e);
  }
  // offsets
  c->rd.assign(nr, RunDesc{});
  long long po = 0, mo = 0, co = 0, ho = 0, peo = 0;
  // the plain form's NVT pair cache: N x N values (ELJ) or pairs (EAM) per walker
  const int pe_w = (!c->f32() && !nn && pair_cache(c->pot, npt ? ENS_NPT : ENS_NVT))
                       ? (c->pot == POT_EAM ? 2 : 1) : 0;
  int wk = 0;
  int nb = c->p.n_bin + 2;
  int hstride = npt ? nb * nb : nb;
  for (int d = 0; d < nr; ++d) {
    const HostRun& h = c->runs[c->run_of_dev[d]];
    RunDesc& r = c->rd[d];
    r.N = h.N;
    r.R = R;
    r.wk = wk;
    r.run_id = c->run_of_dev[d];
    r.pos_off = po;
    r.mat_off = mo;
    r.comp_off = co;
    r.pe_off = peo;
    r.hist_off = ho;
    r.hist_stride = hstride;
    r.n_start = h.n_start;
    r.cyc[0] = r.cyc[1] = r.cyc[2] = 1;
    r.run_ctr = 0;
    po += (long long)R * h.N * 3;
    if ((npt || bpot) && !c->f32()) mo += (long long)R * h.N * h.N;
    if (c->pot == POT_EAM) co += (long long)R * h.N * 2;
    peo += (long long)R * h.N * h.N * pe_w;
    ho += (long long)R * hstride;
    wk += R;
  }
  c->W = wk;
  int W = wk;
  int maxN_all = 0;
  for (auto& G : c->groups) maxN_all = std::max(maxN_all, G.N);
  // host images of the start configurations (they go up once per run and are
  // expanded into replicas on the device)
  std::vector<long long> start_off(nr);
  std::vector<int> n_start(nr);
  long long n_starts = 0;
  for (int d = 0; d < nr; ++d) {
    const HostRun& h = c->runs[c->run_of_dev[d]];
    start_off[d] = n_starts;
    n_start[d] = h.n_start;
    n_starts += (long long)h.n_start * h.N * 3;
  }
  // the context's device state as slices of one allocation (a cudaMalloc per
  // buffer costs tens of microseconds at creation and again at destruction)
  DBuf<double> d_starts;
  DBuf<long long> d_soff;
  DBuf<int> d_ns;
  {
    size_t total = 0;
    unsigned char* cur = nullptr;
    auto take = [&](auto& b, size_t count) {
      if (cur) b.place(cur, count);
      else total += b.span(count);
    };
    auto plan = [&]() {
      take(c->d_runs, nr);
      take(c->d_pos, po);
      take(c->d_mat, mo);
      take(c->d_comp, co);
      take(c->d_en, W);
      take(c->d_box, W);
      take(c->d_rc2, W);
      take(c->d_drift, W);
      take(c->d_beta, W);
      take(c->d_maxd, 2 * (size_t)W);
      take(c->d_maxbox, W);
      take(c->d_ham, 2 * (size_t)W);
      take(c->d_ctr, W);
      take(c->d_status, W);
      take(c->d_wos, W);
      take(c->d_cnt, 6 * (size_t)W);
      take(c->d_hist, ho);
      if (c->rdf_on) take(c->d_rdf, (size_t)W * 5 * c->p.n_bin);
      take(c->d_boxh, W);
      take(c->d_maxboxh, W);
      take(c->d_maxd_sep, 2 * (size_t)W);
      take(c->d_cnt_sep, 4 * (size_t)W);
      if (bpot) take(c->d_tan, mo);
      if (c->pot == POT_LUT) take(c->d_lut, c->lut.size());
      take(c->d_pe, peo);
      take(c->d_lo, c->f32() && !nn ? po / 3 * 4 : 0);
      take(c->d_scr, c->glob ? (size_t)W * 4 * maxN_all : 0);
      take(d_starts, n_starts);
      take(d_soff, nr);
      take(d_ns, nr);
    };
    plan();
    if (cudaMalloc(&c->state_block, total) != cudaSuccess) {
      c->state_block = nullptr;
      return c->fail(PTMC_ERR_CUDA, "device allocation failed");
    }
    cur = (unsigned char*)c->state_block;
    plan();
  }
  // host images (the start configurations go up once per run and are
  // expanded into replicas on the device)
  std::vector<double> box(W), rc2(W), beta(W), maxd(2 * W), maxbox(W), boxh(W),
      maxboxh(W), maxd_sep(2 * W);
  std::vector<int> wos(W);
  std::vector<double> starts(n_starts);
  for (int d = 0; d < nr; ++d) {
    const HostRun& h = c->runs[c->run_of_dev[d]];
    std::copy(h.xyz.begin(), h.xyz.end(), starts.begin() + start_off[d]);
  }
  for (int d = 0; d < nr; ++d) {
    const HostRun& h = c->runs[c->run_of_dev[d]];
    const RunDesc& r = c->rd[d];
    for (int w = 0; w < R; ++w) {
      int g = r.wk + w;
      const double Lb = h.bc_param, Hb = h.bc_height;
      box[g] = Lb;
      boxh[g] = Hb;
      // get_r_cut (Ensembles.jl:118-155)
      rc2[g] = h.bc == PTMC_BC_CUBIC         ? Lb * Lb / 4
               : h.bc == PTMC_BC_RECTANGULAR ? std::min(Lb * Lb / 4, Hb * Hb / 4)
               : h.bc == PTMC_BC_RHOMBIC     ? std::min(Lb * Lb * 3 / 16, Hb * Hb / 4)
                                             : 0.0;
      beta[g] = c->beta[w];
      maxd[2 * g] = h.maxd.empty() ? 0.1 : h.maxd[2 * w];       // MCStates.jl:104
      maxd[2 * g + 1] = h.maxd.empty() ? 0.1 : h.maxd[2 * w + 1];
      maxd_sep[2 * g] = h.maxd_sep.empty() ? 0.1 : h.maxd_sep[2 * w];
      maxd_sep[2 * g + 1] = h.maxd_sep.empty() ? 0.1 : h.maxd_sep[2 * w + 1];
      // max_length / max_height (MCStates.jl:63-87)
      maxbox[g] = h.bc == PTMC_BC_SPHERE ? 30.0 : Lb * 1.8;
      maxboxh[g] = h.bc == PTMC_BC_SPHERE ? 30.0 : Hb * 1.8;
      wos[g] = w;
    }
  }
  cudaStream_t s = c->st;
  int rc = push_runs(c);
  if (rc) return rc;
  {
    cudaError_t e = cudaMemcpyAsync(d_starts.p, starts.data(), sizeof(double) * n_starts,
                                    cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(d_soff.p, start_off.data(), sizeof(long long) * nr, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(d_ns.p, n_start.data(), sizeof(int) * nr, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) {
      k_expand_starts<<<nr, 256, 0, s>>>(c->d_runs.p, d_starts.p, d_soff.p, d_ns.p, c->d_pos.p);
      e = cudaGetLastError();
      c->stats.kernel_launches += 1;
    }
    if (e != cudaSuccess) return c->cuda_fail(e, "start configurations");
  }
  CK(cudaMemcpyAsync(c->d_box.p, box.data(), sizeof(double) * W, cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(c->d_rc2.p, rc2.data(), sizeof(double) * W, cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(c->d_beta.p, beta.data(), sizeof(double) * W, cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(c->d_maxd.p, maxd.data(), sizeof(double) * 2 * W, cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(c->d_maxbox.p, maxbox.data(), sizeof(double) * W, cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(c->d_boxh.p, boxh.data(), sizeof(double) * W, cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(c->d_maxboxh.p, maxboxh.data(), sizeof(double) * W, cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(c->d_maxd_sep.p, maxd_sep.data(), sizeof(double) * 2 * W, cudaMemcpyHostToDevice, s));
  CK(cudaMemsetAsync(c->d_cnt_sep.p, 0, sizeof(long long) * 4 * W, s));
  CK(cudaMemcpyAsync(c->d_wos.p, wos.data(), sizeof(int) * W, cudaMemcpyHostToDevice, s));
  CK(cudaMemsetAsync(c->d_ctr.p, 0, sizeof(unsigned long long) * W, s));
  CK(cudaMemsetAsync(c->d_ham.p, 0, sizeof(double) * 2 * W, s));
  CK(cudaMemsetAsync(c->d_cnt.p, 0, sizeof(long long) * 6 * W, s));
  CK(cudaMemsetAsync(c->d_hist.p, 0, sizeof(unsigned int) * std::max<long long>(ho, 1), s));
  if (c->rdf_on) CK(cudaMemsetAsync(c->d_rdf.p, 0, sizeof(unsigned int) * c->d_rdf.n, s));
  KParams& K = c->K;
  K.runs = c->d_runs.p;
  K.pos = c->d_pos.p;
  K.mat = c->d_mat.p;
  K.comp = c->d_comp.p;
  K.pe = c->d_pe.p;
  K.lo = c->d_lo.p;
  K.glob = c->glob ? 1 : 0;
  K.scr = c->d_scr.p;
  K.scr_stride = 4LL * maxN_all;  // trial row, tangent row, EAM trial terms (2 N)
  K.en = c->d_en.p;
  K.box = c->d_box.p;
  K.rc2 = c->d_rc2.p;
  K.drift = c->d_drift.p;
  K.ctr = c->d_ctr.p;
  K.status = c->d_status.p;
  K.beta = c->d_beta.p;
  K.maxd = c->d_maxd.p;
  K.maxbox = c->d_maxbox.p;
  K.ham = c->d_ham.p;
  K.cnt = c->d_cnt.p;
  K.wos = c->d_wos.p;
  K.hist = c->d_hist.p;
  K.rdf = c->rdf_on ? c->d_rdf.p : nullptr;
  K.boxh = c->d_boxh.p;
  K.maxboxh = c->d_maxboxh.p;
  K.maxd_sep = c->d_maxd_sep.p;
  K.cnt_sep = c->d_cnt_sep.p;
  K.sep_vol = c->sep_vol ? 1 : 0;
  K.tan = c->d_tan.p;
  for (int k = 0; k < MAX_COEFF; ++k) {
    K.ca[k] = k < (int)c->eljb_a.size() ? c->eljb_a[k] : 0.0;
    K.cb[k] = k < (int)c->eljb_b.size() ? c->eljb_b[k] : 0.0;
  }
  if (c->pot == POT_LUT) {
    CK(cudaMemcpyAsync(c->d_lut.p, c->lut.data(), sizeof(double) * c->lut.size(),
                       cudaMemcpyHostToDevice, s));
    K.lut = c->d_lut.p;
    K.lut_na = c->lut_na;
    K.lut_nd = c->lut_nd;
    K.lut_start = c->lut_par[0];
    K.lut_dd = c->lut_par[1];
    K.lut_da = c->lut_par[2];
    K.lut_c6 = c->lut_par[3];
  }
  K.K = (int)c->coeff.size();
  for (int k = 0; k < MAX_COEFF; ++k) K.c[k] = k < K.K ? c->coeff[k] : 0.0;
  for (int k = 0; k < MAX_COEFF; ++k) K.cf[k] = (float)K.c[k];
  K.eam_n = c->eam[0];
  K.eam_m = c->eam[1];
  K.eam_ean = c->eam[2];
  K.eam_ecam = c->eam[3];
  K.f_hn = (float)(-0.5 * c->eam[0]);
  K.f_hm = (float)(-0.5 * c->eam[1]);
  K.f_ean = (float)c->eam[2];
  K.f_ecam = (float)c->eam[3];
  K.pressure = c->p.pressure;
  K.exch_prob = c->p.exch_prob;
  K.min_acc = c->p.min_acc;
  K.max_acc = c->p.max_acc;
  K.n_bin = c->p.n_bin;
  K.n_adjust = c->p.n_adjust;
  K.mc_sample = c->p.mc_sample;
  K.resync_every = c->p.resync_every;
  K.seed = c->p.seed;
  K.xwait_clocks = c->xwait_clocks;
  K.xwait_never = c->xwait_never;
  if (nn2) {
    int Nmax = 0;
    for (auto& G : c->groups) Nmax = std::max(Nmax, G.N);
    c->nn_Nmax = Nmax;
    std::vector<int> row(W), sow(W);
    for (int d = 0; d < nr; ++d)
      for (int w = 0; w < R; ++w) {
        row[c->rd[d].wk + w] = d;
        sow[c->rd[d].wk + w] = w;
      }
    if (c->d_nn_row.alloc(W) || c->d_nn_sow.alloc(W) || c->d_nn2_rad.alloc(c->nn2_rad.size()) ||
        c->d_nn2_ang.alloc(c->nn2_ang.size()) || c->d_nn2_W1.alloc(c->nn2_W1.size()) ||
        c->d_nn2_W2.alloc(c->nn2_W2.size()) || c->d_nn2_swaps.alloc(W))
      return c->fail(PTMC_ERR_CUDA, "device allocation failed");
    CK(cudaMemcpyAsync(c->d_nn_row.p, row.data(), sizeof(int) * W, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(c->d_nn_sow.p, sow.data(), sizeof(int) * W, cudaMemcpyHostToDevice, s));
    for (auto pr : {std::make_pair(&c->d_nn2_rad, &c->nn2_rad), std::make_pair(&c->d_nn2_ang, &c->nn2_ang),
                    std::make_pair(&c->d_nn2_W1, &c->nn2_W1), std::make_pair(&c->d_nn2_W2, &c->nn2_W2)})
      if (!pr.second->empty())
        CK(cudaMemcpyAsync(pr.first->p, pr.second->data(), sizeof(double) * pr.second->size(),
                           cudaMemcpyHostToDevice, s));
    CK(cudaMemsetAsync(c->d_nn2_swaps.p, 0, sizeof(long long) * W, s));
    NN2Params& Q2 = c->Q2;
    Q2.n1 = c->nn2_n1;
    Q2.H1 = c->nn2_H1;
    Q2.H2 = c->nn2_H2;
    Q2.n_swaps = c->n_swaps;
    Q2.rcut = c->nn2_rad[1];  // r_cut of the first radial function (EnergyEvaluation.jl:1297)
    Q2.rad = c->d_nn2_rad.p;
    Q2.ang = c->d_nn2_ang.p;
    Q2.W1 = c->d_nn2_W1.p;
    Q2.W2 = c->d_nn2_W2.p;
    Q2.run_of_walker = c->d_nn_row.p;
    Q2.sow = c->d_nn_sow.p;
    Q2.swaps_acc = c->d_nn2_swaps.p;
    c->Q.run_of_walker = c->d_nn_row.p;  // the run epilogue's walker <-> slot tables
    c->Q.sow = c->d_nn_sow.p;
    if (nn2_smem_bytes(Q2, Nmax) > 227 * 1024)
      return c->fail(PTMC_ERR_LIMIT, "NNVT walker state exceeds 227 KB of shared memory");
    int e = nn2_launch_init(K, Q2, W, Nmax, s);
    if (e) return c->cuda_fail((cudaError_t)e, "k_nn2_init launch");
    c->stats.kernel_launches += 1;
  } else if (nn) {
    int S = (int)c->nn_sf.size();
    int Nmax = 0;
    for (auto& G : c->groups) Nmax = std::max(Nmax, G.N);
    c->nn_Nmax = Nmax;
    std::vector<int> row(W), sow(W);
    for (int d = 0; d < nr; ++d)
      for (int w = 0; w < R; ++w) {
        row[c->rd[d].wk + w] = d;
        sow[c->rd[d].wk + w] = w;
      }
    if (c->d_nn_sf.alloc(S) || c->d_nn_W.alloc(c->nn_W.size()) ||
        c->d_nn_G.alloc((size_t)W * S * Nmax) || c->d_nn_row.alloc(W) || c->d_nn_sow.alloc(W))
      return c->fail(PTMC_ERR_CUDA, "device allocation failed");
    CK(cudaMemcpyAsync(c->d_nn_sf.p, c->nn_sf.data(), sizeof(NNSF) * S, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(c->d_nn_W.p, c->nn_W.data(), sizeof(double) * c->nn_W.size(), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(c->d_nn_row.p, row.data(), sizeof(int) * W, cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(c->d_nn_sow.p, sow.data(), sizeof(int) * W, cudaMemcpyHostToDevice, s));
    NNParams& Q = c->Q;
    Q.S = S;
    Q.H1 = c->nn_H1;
    Q.H2 = c->nn_H2;
    Q.nW = (int)c->nn_W.size();
    Q.Nmax = Nmax;
    Q.rcut = c->nn_rcut;
    Q.boundary2 = c->nn_boundary2;
    Q.sf = c->d_nn_sf.p;
    Q.W = c->d_nn_W.p;
    Q.G = c->d_nn_G.p;
    Q.run_of_walker = c->d_nn_row.p;
    Q.sow = c->d_nn_sow.p;
    if (nn_smem_bytes(Q, Nmax, !c->f32()) > 227 * 1024)
      return c->fail(PTMC_ERR_LIMIT, "NN walker state exceeds 227 KB of shared memory");
    if (c->f32() && (S > 32 || Q.H1 > 32 || Q.H2 > 32))
      return c->fail(PTMC_ERR_LIMIT,
                     "FP32 NN form: at most 32 active symmetry functions and 32 units per hidden "
                     "layer (one tensor-core tile)");
    int e = nn_launch_init(K, Q, W, Nmax, !c->f32(), s);
    if (e) return c->cuda_fail((cudaError_t)e, "k_nn_init launch");
    c->stats.kernel_launches += 1;
  } else {
    for (auto& G : c->groups) {
      int e = launch_init(c->pot, c->bc(), c->p.ensemble, c->f32(), K, G.dev0, G.nruns, R, s);
      if (e) return c->cuda_fail((cudaError_t)e, "k_init launch");
      c->stats.kernel_launches += 1;
    }
  }
  CK(cudaStreamSynchronize(s));
  c->inited = true;
  return PTMC_OK;
}

int ptmc_cycles_nosample(ptmc_ctx* c, long long n) {
  if (!c) return PTMC_ERR_ARG;
  if (!c->inited) return c->fail(PTMC_ERR_STATE, "ptmc_init not called");
  return run_phase(c, n, PHASE_PLAIN);
}

int ptmc_equilibrate(ptmc_ctx* c) {
  if (!c) return PTMC_ERR_ARG;
  if (!c->inited) return c->fail(PTMC_ERR_STATE, "ptmc_init not called");
  if (c->equilibrated) return c->fail(PTMC_ERR_STATE, "already equilibrated");
  long long eq = c->p.eq_cycles;
  int rc = run_phase(c, eq / 2, PHASE_EQ);  // only half is simulated (MCRun.jl:296-298)
  if (rc) return rc;
  int R = c->R(), W = c->W;
  std::vector<double> en(W), box(W), boxh(W);
  std::vector<int> wos(W);
  CK(cudaMemcpyAsync(en.data(), c->d_en.p, sizeof(double) * W, cudaMemcpyDeviceToHost, c->st));
  CK(cudaMemcpyAsync(box.data(), c->d_box.p, sizeof(double) * W, cudaMemcpyDeviceToHost, c->st));
  CK(cudaMemcpyAsync(boxh.data(), c->d_boxh.p, sizeof(double) * W, cudaMemcpyDeviceToHost, c->st));
  CK(cudaMemcpyAsync(wos.data(), c->d_wos.p, sizeof(int) * W, cudaMemcpyDeviceToHost, c->st));
  rc = pull_runs(c);
  if (rc) return rc;
  for (auto& r : c->rd) {
    double eb[2] = {100.0, -100.0};  // check_e_bounds (MCRun.jl:258-265, 299-303)
    for (long long i = eq / 2 + 1; i <= eq; ++i)
      for (int s = 0; s < R; ++s) {
        double e = en[r.wk + wos[r.wk + s]];
        if (e < eb[0]) eb[0] = e;
        else if (e > eb[1]) eb[1] = e;
      }
    // initialise_histograms! (Sampling.jl:141-194)
    r.en_min = eb[0];
    r.en_max = eb[1];
    r.dE = (r.en_max - r.en_min) / (c->p.n_bin - 1);
    // the first state's box (Sampling.jl:141-245)
    const double b = box[r.wk + wos[r.wk + 0]], bh = boxh[r.wk + wos[r.wk + 0]];
    const int bc = c->bc();
    if (c->p.ensemble == PTMC_NPT) {
      double V = bc == PTMC_BC_RECTANGULAR ? b * b * bh
                 : bc == PTMC_BC_RHOMBIC   ? b * b * bh * 1.7320508075688772 / 2
                                           : b * b * b;
      r.v_min = V * 0.8;
      r.v_max = V * 2.0;
      r.dV = (r.v_max - r.v_min) / c->p.n_bin;
    }
    // delta_r2 (Sampling.jl:151 sphere, :185 cube, :210 rhombic, :240 rectangular)
    if (bc == PTMC_BC_CUBIC) r.dr2 = 3.0 / 4.0 * (b * b) / c->p.n_bin / 5;
    else if (bc == PTMC_BC_RHOMBIC) r.dr2 = (3.0 / 8.0 * (b * b) + 1.0 / 4.0 * (bh * bh)) / c->p.n_bin / 5;
    else if (bc == PTMC_BC_RECTANGULAR) r.dr2 = (1.0 / 2.0 * (b * b) + 1.0 / 4.0 * (bh * bh)) / c->p.n_bin / 5;
    else r.dr2 = 4 * (b * b) / c->p.n_bin / 5;
  }
  c->equilibrated = true;
  rc = push_runs(c);
  if (rc) return rc;
  // reset_counters (MCRun.jl:271-277)
  CK(cudaMemsetAsync(c->d_cnt.p, 0, sizeof(long long) * 6 * W, c->st));
  CK(cudaMemsetAsync(c->d_cnt_sep.p, 0, sizeof(long long) * 4 * W, c->st));
  CK(cudaMemsetAsync(c->d_hist.p, 0, sizeof(unsigned int) * std::max<size_t>(c->d_hist.n, 1), c->st));
  if (c->rdf_on) CK(cudaMemsetAsync(c->d_rdf.p, 0, sizeof(unsigned int) * c->d_rdf.n, c->st));
  CK(cudaStreamSynchronize(c->st));
  return PTMC_OK;
}

int ptmc_run_cycles(ptmc_ctx* c, long long n) {
  if (!c) return PTMC_ERR_ARG;
  if (!c->equilibrated) return c->fail(PTMC_ERR_STATE, "ptmc_equilibrate not called");
  return run_phase(c, n, PHASE_PROD);
}

int ptmc_resync(ptmc_ctx* c) {
  if (!c) return PTMC_ERR_ARG;
  if (!c->inited) return c->fail(PTMC_ERR_STATE, "ptmc_init not called");
  if (c->pot == POT_NN2) {  // recompute the energies from the positions
    int e = nn2_launch_init(c->K, c->Q2, c->W, c->nn_Nmax, c->st);
    if (e) return c->cuda_fail((cudaError_t)e, "k_nn2_init launch");
    c->stats.kernel_launches += 1;
    CK(cudaStreamSynchronize(c->st));
    return PTMC_OK;
  }
  if (c->pot == POT_NN) {  // recompute G and the energies from the positions
    int e = nn_launch_init(c->K, c->Q, c->W, c->nn_Nmax, !c->f32(), c->st);
    if (e) return c->cuda_fail((cudaError_t)e, "k_nn_init launch");
    c->stats.kernel_launches += 1;
    CK(cudaStreamSynchronize(c->st));
    return PTMC_OK;
  }
  for (auto& G : c->groups) {
    int e = launch_resync(c->pot, c->bc(), c->p.ensemble, c->f32(), c->K, G.dev0, G.nruns, c->R(), c->st);
    if (e) return c->cuda_fail((cudaError_t)e, "k_resync launch");
    c->stats.kernel_launches += 1;
  }
  CK(cudaStreamSynchronize(c->st));
  return PTMC_OK;
}

int ptmc_get_states(ptmc_ctx* c, int run, double* xyz, double* en_tot, double* box,
                    double* max_displ, long long* counts, double* ham) {
  if (!c) return PTMC_ERR_ARG;
  if (!c->inited) return c->fail(PTMC_ERR_STATE, "ptmc_init not called");
  if (run < 0 || run >= c->p.n_runs) return c->fail(PTMC_ERR_ARG, "run index out of range");
  const RunDesc& r = c->rd[c->dev_of_run[run]];
  int R = c->R(), N = r.N;
  std::vector<double> pos((size_t)R * N * 3), en(R), bx(R), md(2 * R), hm(2 * R);
  std::vector<int> wos(R);
  std::vector<long long> cnt(6 * R);
  cudaStream_t s = c->st;
  CK(cudaMemcpyAsync(pos.data(), c->d_pos.p + r.pos_off, sizeof(double) * pos.size(), cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(en.data(), c->d_en.p + r.wk, sizeof(double) * R, cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(bx.data(), c->d_box.p + r.wk, sizeof(double) * R, cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(md.data(), c->d_maxd.p + 2 * r.wk, sizeof(double) * 2 * R, cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(hm.data(), c->d_ham.p + 2 * r.wk, sizeof(double) * 2 * R, cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(cnt.data(), c->d_cnt.p + 6 * (size_t)r.wk, sizeof(long long) * 6 * R, cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(wos.data(), c->d_wos.p + r.wk, sizeof(int) * R, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  for (int slot = 0; slot < R; ++slot) {
    int w = wos[slot];
    if (xyz) std::copy(&pos[(size_t)w * N * 3], &pos[(size_t)w * N * 3] + (size_t)N * 3, xyz + (size_t)slot * N * 3);
    if (en_tot) en_tot[slot] = en[w];
    if (box) box[slot] = bx[w];
  }
  if (max_displ) std::copy(md.begin(), md.end(), max_displ);
  if (counts) std::copy(cnt.begin(), cnt.end(), counts);
  if (ham) std::copy(hm.begin(), hm.end(), ham);
  return PTMC_OK;
}

int ptmc_get_energies(ptmc_ctx* c, double* en_tot) {
  if (!c || !en_tot) return PTMC_ERR_ARG;
  if (!c->inited) return c->fail(PTMC_ERR_STATE, "ptmc_init not called");
  const int R = c->R(), W = c->W;
  std::vector<double> en(W);
  std::vector<int> wos(W);
  CK(cudaMemcpyAsync(en.data(), c->d_en.p, sizeof(double) * W, cudaMemcpyDeviceToHost, c->st));
  CK(cudaMemcpyAsync(wos.data(), c->d_wos.p, sizeof(int) * W, cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  for (int run = 0; run < c->p.n_runs; ++run) {
    const int wk = c->rd[c->dev_of_run[run]].wk;
    for (int s = 0; s < R; ++s) en_tot[(size_t)run * R + s] = en[wk + wos[wk + s]];
  }
  return PTMC_OK;
}

int ptmc_get_box_states(ptmc_ctx* c, int run, double* box_height, double* max_displ_sep,
                        long long* counts_sep) {
  if (!c) return PTMC_ERR_ARG;
  if (!c->inited) return c->fail(PTMC_ERR_STATE, "ptmc_init not called");
  if (run < 0 || run >= c->p.n_runs) return c->fail(PTMC_ERR_ARG, "run index out of range");
  const RunDesc& r = c->rd[c->dev_of_run[run]];
  const int R = c->R();
  std::vector<double> bh(R), md(2 * R);
  std::vector<long long> cnt(4 * R);
  std::vector<int> wos(R);
  cudaStream_t s = c->st;
  CK(cudaMemcpyAsync(bh.data(), c->d_boxh.p + r.wk, sizeof(double) * R, cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(md.data(), c->d_maxd_sep.p + 2 * r.wk, sizeof(double) * 2 * R, cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(cnt.data(), c->d_cnt_sep.p + 4 * (size_t)r.wk, sizeof(long long) * 4 * R,
                     cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(wos.data(), c->d_wos.p + r.wk, sizeof(int) * R, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  for (int slot = 0; slot < R; ++slot)
    if (box_height) box_height[slot] = bh[wos[slot]];
  if (max_displ_sep) std::copy(md.begin(), md.end(), max_displ_sep);
  if (counts_sep) std::copy(cnt.begin(), cnt.end(), counts_sep);
  return PTMC_OK;
}

int ptmc_get_output(ptmc_ctx* c, int run, ptmc_output* o) {
  if (!c || !o) return PTMC_ERR_ARG;
  if (!c->inited) return c->fail(PTMC_ERR_STATE, "ptmc_init not called");
  if (run < 0 || run >= c->p.n_runs) return c->fail(PTMC_ERR_ARG, "run index out of range");
  int rc = pull_runs(c);
  if (rc) return rc;
  const RunDesc& r = c->rd[c->dev_of_run[run]];
  int R = c->R();
  std::vector<double> md(2 * R), hm(2 * R);
  std::vector<long long> cnt(6 * R);
  std::vector<unsigned int> h((size_t)R * r.hist_stride);
  cudaStream_t s = c->st;
  CK(cudaMemcpyAsync(md.data(), c->d_maxd.p + 2 * r.wk, sizeof(double) * 2 * R, cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(hm.data(), c->d_ham.p + 2 * r.wk, sizeof(double) * 2 * R, cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(cnt.data(), c->d_cnt.p + 6 * (size_t)r.wk, sizeof(long long) * 6 * R, cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(h.data(), c->d_hist.p + r.hist_off, sizeof(unsigned int) * h.size(), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  // finalise_results (Sampling.jl:377-399)
  double n_sample = (double)c->p.mc_cycles / (double)c->p.mc_sample;
  for (int i = 0; i < R; ++i) {
    double ea = hm[2 * i] / n_sample, e2 = hm[2 * i + 1] / n_sample;
    if (o->en_avg) o->en_avg[i] = ea;
    if (o->heat_cap) o->heat_cap[i] = (e2 - ea * ea) * (c->beta[i] * c->beta[i]);
    if (o->count_stat_atom)
      o->count_stat_atom[i] = (double)cnt[6 * i] / (double)((long long)r.N * c->p.mc_cycles);
    if (o->count_stat_vol) o->count_stat_vol[i] = (double)cnt[6 * i + 2] / (double)c->p.mc_cycles;
    if (o->count_stat_exc) o->count_stat_exc[i] = (double)cnt[6 * i + 5] / (double)cnt[6 * i + 4];
  }
  if (o->max_displ) std::copy(md.begin(), md.end(), o->max_displ);
  if (o->en_histogram && c->p.ensemble == PTMC_NVT)
    for (size_t k = 0; k < h.size(); ++k) o->en_histogram[k] = (double)h[k];
  if (o->ev_histogram && c->p.ensemble == PTMC_NPT)
    for (size_t k = 0; k < h.size(); ++k) o->ev_histogram[k] = (double)h[k];
  o->hist_params[0] = r.en_min;
  o->hist_params[1] = r.en_max;
  o->hist_params[2] = r.v_min;
  o->hist_params[3] = r.v_max;
  o->hist_params[4] = r.dE;
  o->hist_params[5] = r.dV;
  o->delta_r2 = r.dr2;
  if (o->rdf && c->rdf_on) {  // Output.rdf: 5 n_bin bins per slot
    const size_t nb5 = (size_t)5 * c->p.n_bin;
    std::vector<unsigned int> rh((size_t)R * nb5);
    CK(cudaMemcpyAsync(rh.data(), c->d_rdf.p + (size_t)r.wk * nb5, sizeof(unsigned int) * rh.size(),
                       cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    for (size_t k = 0; k < rh.size(); ++k) o->rdf[k] = (double)rh[k];
  }
  return PTMC_OK;
}

int ptmc_get_stats(ptmc_ctx* c, ptmc_stats* s) {
  if (!c || !s) return PTMC_ERR_ARG;
  *s = c->stats;
  if (c->inited) {
    std::vector<double> d(c->W);
    CK(cudaMemcpy(d.data(), c->d_drift.p, sizeof(double) * c->W, cudaMemcpyDeviceToHost));
    double m = 0;
    for (double x : d) m = std::max(m, x);
    s->max_drift = m;
  }
  return PTMC_OK;
}

void ptmc_destroy(ptmc_ctx* c) {
  if (!c) return;
  for (auto& kv : c->graphs) cudaGraphExecDestroy(kv.second);
  for (auto& G : c->groups)
    if (G.st) cudaStreamDestroy(G.st);
  for (auto e : c->evjoin) cudaEventDestroy(e);
  if (c->ev0) cudaEventDestroy(c->ev0);
  if (c->ev1) cudaEventDestroy(c->ev1);
  if (c->evfork) cudaEventDestroy(c->evfork);
  c->d_runs.free_();
  c->d_pos.free_();
  c->d_mat.free_();
  c->d_comp.free_();
  c->d_en.free_();
  c->d_box.free_();
  c->d_rc2.free_();
  c->d_drift.free_();
  c->d_beta.free_();
  c->d_maxd.free_();
  c->d_maxbox.free_();
  c->d_ham.free_();
  c->d_ctr.free_();
  c->d_status.free_();
  c->d_wos.free_();
  c->d_cnt.free_();
  c->d_hist.free_();
  c->d_rdf.free_();
  c->d_boxh.free_();
  c->d_maxboxh.free_();
  c->d_maxd_sep.free_();
  c->d_cnt_sep.free_();
  c->d_tan.free_();
  c->d_lut.free_();
  c->d_pe.free_();
  c->d_lo.free_();
  c->d_scr.free_();
  if (c->state_block) cudaFree(c->state_block);
  c->state_block = nullptr;
  for (auto* b : {&c->d_nn2_rad, &c->d_nn2_ang, &c->d_nn2_W1, &c->d_nn2_W2}) b->free_();
  c->d_nn2_swaps.free_();
  c->d_nn_sf.free_();
  c->d_nn_W.free_();
  c->d_nn_G.free_();
  c->d_nn_row.free_();
  c->d_nn_sow.free_();
  for (auto* b : {&c->d_sur_P, &c->d_sur_m, &c->d_sur_v, &c->d_sur_g, &c->d_rec_rows, &c->d_rec_y,
                  &c->d_da_kappa, &c->d_sur_tab})
    b->free_();
  c->d_sur_loss.free_();
  c->d_rec_n.free_();
  c->d_da_cnt.free_();
  c->d_sur_err.free_();
  c->d_rec_slot.free_();
  if (c->st) cudaStreamDestroy(c->st);
  delete c;
}

}  // extern "C"

// ---------------------------------------------------------------- checkpoint
// Reference text formats (src/ReadSave.jl) for run 0, plus engine.bin with the
// complete binary state of every run for exact resume.
namespace {
template <typename T>
void put(std::string& b, const T* p, size_t n) {
  b.append((const char*)p, n * sizeof(T));
}
template <typename T>
int dump(ptmc_ctx* c, std::string& b, const DBuf<T>& d) {
  std::vector<T> h(d.n);
  if (d.n) CK(cudaMemcpy(h.data(), d.p, sizeof(T) * d.n, cudaMemcpyDeviceToHost));
  unsigned long long n = d.n;
  put(b, &n, 1);
  put(b, h.data(), h.size());
  return PTMC_OK;
}
template <typename T>
int undump(ptmc_ctx* c, const std::string& b, size_t& at, DBuf<T>& d) {
  unsigned long long n = 0;
  if (at + sizeof(n) > b.size()) return c->fail(PTMC_ERR_IO, "engine.bin truncated");
  std::memcpy(&n, b.data() + at, sizeof(n));
  at += sizeof(n);
  if (n != d.n) return c->fail(PTMC_ERR_IO, "engine.bin does not match this context's layout");
  if (at + n * sizeof(T) > b.size()) return c->fail(PTMC_ERR_IO, "engine.bin truncated");
  if (n) CK(cudaMemcpy(d.p, b.data() + at, sizeof(T) * n, cudaMemcpyHostToDevice));
  at += n * sizeof(T);
  return PTMC_OK;
}
}  // namespace

// ------------------------------------------------------- reference restart
// rebuild_states (src/ReadSave.jl:436-481) with initialisation's restart
// branch (src/Initialization.jl:103-119): the states of run 0 from the text
// files a reference checkpoint holds, when the directory has no engine.bin.
namespace {

void drop_graphs(ptmc_ctx* c);  // captured launches hold the old kernel parameters

// whitespace-separated tokens of every line of a text file
bool read_table(const std::string& path, std::vector<std::vector<std::string>>& rows) {
  std::ifstream f(path);
  if (!f) return false;
  rows.clear();
  std::string line;
  while (std::getline(f, line)) {
    std::istringstream ls(line);
    std::vector<std::string> t;
    std::string tok;
    while (ls >> tok) t.push_back(tok);
    if (!t.empty()) rows.push_back(t);
  }
  return true;
}

bool to_double(std::string t, double& v) {
  while (!t.empty() && t.back() == ',') t.pop_back();  // "box_dims: L, H" (src/ReadSave.jl:133-135)
  char* end = nullptr;
  v = std::strtod(t.c_str(), &end);
  return end && *end == '\0' && !t.empty();
}

// launches the kernels that evaluate every walker's energy (and the potential
// variables: EAM components, distance matrices, pair caches, symmetry
// functions) from the positions on the device
int init_energies(ptmc_ctx* c) {
  const int W = c->W, R = c->R();
  if (c->pot == POT_NN2) {
    int e = nn2_launch_init(c->K, c->Q2, W, c->nn_Nmax, c->st);
    if (e) return c->cuda_fail((cudaError_t)e, "k_nn2_init launch");
  } else if (c->pot == POT_NN) {
    int e = nn_launch_init(c->K, c->Q, W, c->nn_Nmax, !c->f32(), c->st);
    if (e) return c->cuda_fail((cudaError_t)e, "k_nn_init launch");
  } else {
    for (auto& G : c->groups) {
      int e = launch_init(c->pot, c->bc(), c->p.ensemble, c->f32(), c->K, G.dev0, G.nruns, R, c->st);
      if (e) return c->cuda_fail((cudaError_t)e, "k_init launch");
    }
  }
  c->stats.kernel_launches += c->groups.size();
  CK(cudaStreamSynchronize(c->st));
  return PTMC_OK;
}

int restore_reference_text(ptmc_ctx* c, const std::string& d) {
  if (c->p.n_runs != 1)
    return c->fail(PTMC_ERR_STATE, "a reference checkpoint holds one run: restore it into a context "
                                   "with n_runs = 1");
  const int R = c->R(), W = c->W;
  RunDesc& r = c->rd[0];
  const int N = r.N, nb = c->p.n_bin + 2;
  const bool npt = c->p.ensemble == PTMC_NPT;
  std::vector<std::vector<std::string>> t;
  // hist_info.data: header row, then e_min e_max v_min v_max dE dV dr2
  double hi[7];
  if (!read_table(d + "/hist_info.data", t) || t.size() < 2 || t[1].size() < 7)
    return c->fail(PTMC_ERR_IO, "cannot read " + d + "/hist_info.data");
  for (int k = 0; k < 7; ++k)
    if (!to_double(t[1][k], hi[k])) return c->fail(PTMC_ERR_IO, "hist_info.data: bad number");
  // histograms.data: one row of n_bin + 2 counts per state
  std::vector<unsigned int> hist((size_t)R * r.hist_stride, 0u);
  if (!read_table(d + "/histograms.data", t) || (int)t.size() != R)
    return c->fail(PTMC_ERR_IO, "histograms.data: need " + std::to_string(R) + " rows");
  if (!npt)
    for (int s = 0; s < R; ++s) {
      if ((int)t[s].size() != nb) return c->fail(PTMC_ERR_IO, "histograms.data: row length is not n_bin + 2");
      for (int k = 0; k < nb; ++k) {
        double v;
        if (!to_double(t[s][k], v)) return c->fail(PTMC_ERR_IO, "histograms.data: bad number");
        hist[(size_t)s * r.hist_stride + k] = (unsigned int)std::llround(v);
      }
    }
  if (npt) {  // volume_hist.data: each state's E x V matrix, column-major (V index outer)
    if (!read_table(d + "/volume_hist.data", t) || (int)t.size() != R)
      return c->fail(PTMC_ERR_IO, "volume_hist.data: need " + std::to_string(R) + " rows");
    for (int s = 0; s < R; ++s) {
      if ((long long)t[s].size() != (long long)nb * nb)
        return c->fail(PTMC_ERR_IO, "volume_hist.data: row length is not (n_bin + 2)^2");
      for (int iv = 0; iv < nb; ++iv)
        for (int ie = 0; ie < nb; ++ie) {
          double v;
          if (!to_double(t[s][(size_t)iv * nb + ie], v))
            return c->fail(PTMC_ERR_IO, "volume_hist.data: bad number");
          hist[(size_t)s * r.hist_stride + (size_t)ie * nb + iv] = (unsigned int)std::llround(v);
        }
    }
  }
  std::vector<unsigned int> rdf;
  if (c->rdf_on && read_table(d + "/rdf.data", t)) {
    const int nr = 5 * c->p.n_bin;
    if ((int)t.size() != R) return c->fail(PTMC_ERR_IO, "rdf.data: need one row per state");
    rdf.assign((size_t)W * nr, 0u);
    for (int s = 0; s < R; ++s)
      for (int k = 0; k < nr && k < (int)t[s].size(); ++k) {
        double v;
        if (!to_double(t[s][k], v)) return c->fail(PTMC_ERR_IO, "rdf.data: bad number");
        rdf[(size_t)(r.wk + s) * nr + k] = (unsigned int)std::llround(v);
      }
  }
  long long index = 1;
  if (read_table(d + "/index.txt", t) && !t.empty()) {
    double v;
    if (!to_double(t[0][0], v)) return c->fail(PTMC_ERR_IO, "index.txt: bad number");
    index = (long long)v;
  }
  // configT<i>.xyz: N, then "<BC type> <label> <bc values> max_displ[1:3]
  // count_atom count_vol", then N rows "1 x y z" (src/ReadSave.jl:142-165,
  // read_checkpoint_config :371-396)
  std::vector<double> pos((size_t)R * N * 3), box(R), boxh(R), rc2(R), maxd(2 * R), maxbox(R),
      maxboxh(R), maxd_sep(2 * R);
  std::vector<long long> cnt(6 * (size_t)R, 0);
  const int bc = c->bc();
  for (int s = 0; s < R; ++s) {
    const std::string path = d + "/configT" + std::to_string(s + 1) + ".xyz";
    if (!read_table(path, t) || t.size() < 2) return c->fail(PTMC_ERR_IO, "cannot read " + path);
    double nv;
    if (!to_double(t[0][0], nv) || (int)nv != N || (int)t.size() < 2 + N)
      return c->fail(PTMC_ERR_IO, path + ": not " + std::to_string(N) + " atoms");
    const std::vector<std::string>& h = t[1];
    const bool two = bc == PTMC_BC_RECTANGULAR || bc == PTMC_BC_RHOMBIC;
    const char* want = bc == PTMC_BC_SPHERE ? "SphericalBC" : bc == PTMC_BC_CUBIC ? "CubicBC"
                       : bc == PTMC_BC_RECTANGULAR ? "RectangularBC" : "RhombicBC";
    if (h[0].compare(0, std::strlen(want), want) != 0)
      return c->fail(PTMC_ERR_IO, path + ": boundary condition is not " + want);
    const size_t nv_needed = two ? 9 : 8;
    if (h.size() < nv_needed) return c->fail(PTMC_ERR_IO, path + ": short comment line");
    double b0, b1 = 0.0, md[3], ca, cv;
    bool ok = to_double(h[2], b0);
    size_t at = 3;
    if (two) ok = ok && to_double(h[at++], b1);
    for (int k = 0; k < 3; ++k) ok = ok && to_double(h[at++], md[k]);
    ok = ok && to_double(h[at++], ca) && to_double(h[at++], cv);
    if (!ok) return c->fail(PTMC_ERR_IO, path + ": bad comment line");
    const double L = bc == PTMC_BC_SPHERE ? std::sqrt(b0) : b0;  // the sphere line holds r^2
    box[s] = L;
    boxh[s] = two ? b1 : 0.0;
    rc2[s] = bc == PTMC_BC_CUBIC         ? L * L / 4
             : bc == PTMC_BC_RECTANGULAR ? std::min(L * L / 4, b1 * b1 / 4)
             : bc == PTMC_BC_RHOMBIC     ? std::min(L * L * 3 / 16, b1 * b1 / 4)
                                         : 0.0;
    // MCState(...; max_displ, count_atom = [count, 0], count_vol = [count, 0]):
    // the totals are kept, the adaptation counters start at zero, and the
    // state's box limits follow from the restored box (MCStates.jl:63-87)
    maxd[2 * s] = md[0];
    maxd[2 * s + 1] = md[1];
    maxd_sep[2 * s] = md[2];
    maxd_sep[2 * s + 1] = 0.1;
    maxbox[s] = bc == PTMC_BC_SPHERE ? 30.0 : L * 1.8;
    maxboxh[s] = bc == PTMC_BC_SPHERE ? 30.0 : b1 * 1.8;
    cnt[6 * (size_t)s + 0] = (long long)ca;
    cnt[6 * (size_t)s + 2] = (long long)cv;
    // recentre! of every state (src/Initialization.jl:114-116)
    double cx = 0, cy = 0, cz = 0;
    double* X = &pos[(size_t)s * N * 3];
    for (int a = 0; a < N; ++a) {
      const std::vector<std::string>& row = t[2 + a];
      if (row.size() < 4 || !to_double(row[1], X[3 * a]) || !to_double(row[2], X[3 * a + 1]) ||
          !to_double(row[3], X[3 * a + 2]))
        return c->fail(PTMC_ERR_IO, path + ": bad position row");
      cx += X[3 * a];
      cy += X[3 * a + 1];
      cz += X[3 * a + 2];
    }
    cx /= N;
    cy /= N;
    cz /= N;
    for (int a = 0; a < N; ++a) {
      X[3 * a] -= cx;
      X[3 * a + 1] -= cy;
      X[3 * a + 2] -= cz;
    }
  }
  // device state of run 0: walker s in slot s, fresh draw streams
  const int wk = r.wk;
  std::vector<int> wos(R);
  for (int s = 0; s < R; ++s) wos[s] = s;
  std::vector<double> zero2(2 * (size_t)R, 0.0);
  std::vector<unsigned long long> ctr(R, 0ull);
  std::vector<int> st(R, 0);
  cudaStream_t q = c->st;
  CK(cudaMemcpyAsync(c->d_pos.p + r.pos_off, pos.data(), sizeof(double) * pos.size(), cudaMemcpyHostToDevice, q));
  CK(cudaMemcpyAsync(c->d_box.p + wk, box.data(), sizeof(double) * R, cudaMemcpyHostToDevice, q));
  CK(cudaMemcpyAsync(c->d_boxh.p + wk, boxh.data(), sizeof(double) * R, cudaMemcpyHostToDevice, q));
  CK(cudaMemcpyAsync(c->d_rc2.p + wk, rc2.data(), sizeof(double) * R, cudaMemcpyHostToDevice, q));
  CK(cudaMemcpyAsync(c->d_maxd.p + 2 * wk, maxd.data(), sizeof(double) * 2 * R, cudaMemcpyHostToDevice, q));
  CK(cudaMemcpyAsync(c->d_maxd_sep.p + 2 * wk, maxd_sep.data(), sizeof(double) * 2 * R, cudaMemcpyHostToDevice, q));
  CK(cudaMemcpyAsync(c->d_maxbox.p + wk, maxbox.data(), sizeof(double) * R, cudaMemcpyHostToDevice, q));
  CK(cudaMemcpyAsync(c->d_maxboxh.p + wk, maxboxh.data(), sizeof(double) * R, cudaMemcpyHostToDevice, q));
  CK(cudaMemcpyAsync(c->d_cnt.p + 6 * (size_t)wk, cnt.data(), sizeof(long long) * cnt.size(), cudaMemcpyHostToDevice, q));
  CK(cudaMemsetAsync(c->d_cnt_sep.p + 4 * (size_t)wk, 0, sizeof(long long) * 4 * R, q));
  CK(cudaMemcpyAsync(c->d_ham.p + 2 * wk, zero2.data(), sizeof(double) * 2 * R, cudaMemcpyHostToDevice, q));
  CK(cudaMemcpyAsync(c->d_hist.p + r.hist_off, hist.data(), sizeof(unsigned int) * hist.size(), cudaMemcpyHostToDevice, q));
  if (!rdf.empty())
    CK(cudaMemcpyAsync(c->d_rdf.p, rdf.data(), sizeof(unsigned int) * rdf.size(), cudaMemcpyHostToDevice, q));
  CK(cudaMemcpyAsync(c->d_wos.p + wk, wos.data(), sizeof(int) * R, cudaMemcpyHostToDevice, q));
  CK(cudaMemcpyAsync(c->d_ctr.p + wk, ctr.data(), sizeof(unsigned long long) * R, cudaMemcpyHostToDevice, q));
  CK(cudaMemcpyAsync(c->d_status.p + wk, st.data(), sizeof(int) * R, cudaMemcpyHostToDevice, q));
  r.n_start = R;  // every walker has its own configuration
  r.en_min = hi[0];
  r.en_max = hi[1];
  r.v_min = hi[2];
  r.v_max = hi[3];
  r.dE = hi[4];
  r.dV = hi[5];
  r.dr2 = hi[6];
  // the reference's loop resumes at the saved index (src/MCRun.jl:455: i in
  // start_counter:mc_cycles), so cycle `index` runs again
  r.cyc[PHASE_PROD] = index;
  r.run_ctr = 0;
  int rc = push_runs(c);
  if (rc) return rc;
  rc = init_energies(c);
  if (rc) return rc;
  c->equilibrated = true;
  drop_graphs(c);
  return PTMC_OK;
}

}  // namespace

extern "C" {

int ptmc_checkpoint(ptmc_ctx* c, const char* dir) {
  if (!c || !dir) return PTMC_ERR_ARG;
  if (!c->inited) return c->fail(PTMC_ERR_STATE, "ptmc_init not called");
  CK(cudaStreamSynchronize(c->st));
  ::mkdir(dir, 0755);
  std::string d(dir);
  int rc = pull_runs(c);
  if (rc) return rc;
  const int R = c->R();
  const RunDesc& r0 = c->rd[c->dev_of_run[0]];
  const int N = r0.N;
  const bool npt = c->p.ensemble == PTMC_NPT;
  // params.data (save_init/writeparams/writeensemble/writepotential, :24-110)
  std::string s = "cycles: sample_rate: n_traj: n_atoms: n_adjust n_bins min_acc: max_acc t_i: t_f\n";
  double pv[10] = {(double)c->p.mc_cycles, (double)c->p.mc_sample, (double)R, (double)N,
                   (double)c->p.n_adjust, (double)c->p.n_bin, c->p.min_acc, c->p.max_acc,
                   c->T.front(), c->T.back()};
  for (int k = 0; k < 10; ++k) s += fmt_double(pv[k]) + (k < 9 ? " " : "\n");
  if (npt) {
    s += "ensemble n_atom_moves n_volume_moves n_atom_swaps pressure separated_volume\n";
    s += "NPT " + std::to_string(N) + " " + std::to_string(N) + " 1 0 " + fmt_double(c->p.pressure) +
         (c->sep_vol ? " true\n" : " false\n");
  } else if (c->p.ensemble == PTMC_NNVT) {  // writeensemble NNVT (:51-55)
    s += "ensemble n_1 n_2 n_atom_moves n_atom_swaps\n";
    s += "NNVT " + std::to_string(c->nn2_n1) + " " + std::to_string(N - c->nn2_n1) + " " +
         std::to_string(N) + " " + std::to_string(c->n_swaps) + "\n";
  } else {
    s += "ensemble n_atom_moves n_atom_swaps\n";
    s += "NVT " + std::to_string(N) + " " + std::to_string(N) + " 0\n";
  }
  if (c->pot == POT_EAM) {
    s += "EAM: " + fmt_double(c->eam[0]) + " " + fmt_double(c->eam[1]) + " " + fmt_double(c->eam[2]) +
         " " + fmt_double(c->eam[3]) + " \n";
  } else if (c->pot == POT_NN || c->pot == POT_NN2) {
    s += "runnerpotential \n";
  } else if (c->pot == POT_LUT) {
    s += "LookupTablePotential \n";
  } else if (c->pot == POT_ELJB) {  // writepotential AbstractDimerPotentialB (:71-77)
    s += "ELJB " + std::to_string(c->coeff.size()) + " \n";
    for (const std::vector<double>* v : {&c->eljb_a, &c->eljb_b, &c->coeff}) {
      for (size_t k = 0; k < v->size(); ++k) s += fmt_double((*v)[k]) + (k + 1 < v->size() ? "\t" : "\n");
    }
  } else {
    s += std::string(c->pot == POT_ELJEVEN ? "ELJPotentialEven{" : "ELJPotential{") +
         std::to_string(c->coeff.size()) + ", Float64}";
    for (double x : c->coeff) s += " " + fmt_double(x);
    s += "\n";
  }
  if (!write_file_atomic(d + "/params.data", s)) return c->fail(PTMC_ERR_IO, "cannot write params.data");
  // hist_info.data (save_histparams, :117-127)
  s = "e_min e_max v_min v_max \xce\x94_E \xce\x94_V \xce\x94_r2\n";
  double hv[7] = {r0.en_min, r0.en_max, r0.v_min, r0.v_max, r0.dE, r0.dV, r0.dr2};
  for (int k = 0; k < 7; ++k) s += fmt_double(hv[k]) + (k < 6 ? " " : "\n");
  if (!write_file_atomic(d + "/hist_info.data", s)) return c->fail(PTMC_ERR_IO, "cannot write hist_info.data");
  // histograms (checkpoint, :178-218)
  std::vector<unsigned int> h((size_t)R * r0.hist_stride);
  CK(cudaMemcpy(h.data(), c->d_hist.p + r0.hist_off, sizeof(unsigned int) * h.size(), cudaMemcpyDeviceToHost));
  int nb = c->p.n_bin + 2;
  s.clear();
  for (int i = 0; i < R; ++i) {
    for (int m = 0; m < nb; ++m) {
      double v = npt ? 0.0 : (double)h[(size_t)i * r0.hist_stride + m];
      s += fmt_double(v) + (m < nb - 1 ? "\t" : "\n");
    }
  }
  if (!write_file_atomic(d + "/histograms.data", s)) return c->fail(PTMC_ERR_IO, "cannot write histograms.data");
  if (npt) {  // one row per replica, matrix flattened column-major (setresults :404-412)
    s.clear();
    for (int i = 0; i < R; ++i)
      for (int col = 0; col < nb; ++col)
        for (int rw = 0; rw < nb; ++rw) {
          double v = (double)h[(size_t)i * r0.hist_stride + (size_t)rw * nb + col];
          s += fmt_double(v) + ((col == nb - 1 && rw == nb - 1) ? "\n" : "\t");
        }
    if (!write_file_atomic(d + "/volume_hist.data", s)) return c->fail(PTMC_ERR_IO, "cannot write volume_hist.data");
  }
  if (c->rdf_on) {  // rdf.data (checkpoint with rdfsave, :192-196): one row per replica
    const size_t nb5 = (size_t)5 * c->p.n_bin;
    std::vector<unsigned int> rh((size_t)R * nb5);
    CK(cudaMemcpy(rh.data(), c->d_rdf.p + (size_t)r0.wk * nb5, sizeof(unsigned int) * rh.size(),
                  cudaMemcpyDeviceToHost));
    s.clear();
    for (int i = 0; i < R; ++i)
      for (size_t m = 0; m < nb5; ++m)
        s += fmt_double((double)rh[(size_t)i * nb5 + m]) + (m < nb5 - 1 ? "\t" : "\n");
    if (!write_file_atomic(d + "/rdf.data", s)) return c->fail(PTMC_ERR_IO, "cannot write rdf.data");
  }
  long long index = r0.cyc[PHASE_PROD] - 1;
  if (!write_file_atomic(d + "/index.txt", std::to_string(index) + "\n"))
    return c->fail(PTMC_ERR_IO, "cannot write index.txt");
  // configT<i>.xyz (checkpoint_config, :142-158)
  std::vector<double> xyz((size_t)R * N * 3), en(R), box(R), md(2 * R), ham(2 * R), bh(R), mds(2 * R);
  std::vector<long long> cnt(6 * R);
  rc = ptmc_get_states(c, 0, xyz.data(), en.data(), box.data(), md.data(), cnt.data(), ham.data());
  if (rc) return rc;
  rc = ptmc_get_box_states(c, 0, bh.data(), mds.data(), nullptr);
  if (rc) return rc;
  for (int i = 0; i < R; ++i) {
    std::string t = std::to_string(N) + "\n";
    // bc_info (ReadSave.jl:131-135)
    if (c->bc() == PTMC_BC_SPHERE) t += "SphericalBC{Float64} r2: " + fmt_double(box[i] * box[i]);
    else if (c->bc() == PTMC_BC_CUBIC) t += "CubicBC{Float64} box_length: " + fmt_double(box[i]);
    else
      t += std::string(c->bc() == PTMC_BC_RHOMBIC ? "RhombicBC" : "RectangularBC") +
           "{Float64} box_dims: " + fmt_double(box[i]) + ", " + fmt_double(bh[i]);
    t += " " + fmt_double(md[2 * i]) + " " + fmt_double(md[2 * i + 1]) + " " + fmt_double(mds[2 * i]) +
         " " + std::to_string(cnt[6 * i]) + " " + std::to_string(cnt[6 * i + 2]) + "\n";
    for (int a = 0; a < N; ++a) {
      const double* x = &xyz[((size_t)i * N + a) * 3];
      t += "1  " + fmt_double(x[0]) + " " + fmt_double(x[1]) + " " + fmt_double(x[2]) + " \n";
    }
    if (!write_file_atomic(d + "/configT" + std::to_string(i + 1) + ".xyz", t))
      return c->fail(PTMC_ERR_IO, "cannot write configT.xyz");
  }
  // engine.bin: complete state
  std::string b = "PTMCGB03";
  unsigned long long hdr[4] = {(unsigned long long)c->p.n_runs, (unsigned long long)R,
                               (unsigned long long)c->W, (unsigned long long)c->equilibrated};
  put(b, hdr, 4);
  put(b, c->rd.data(), c->rd.size());
  if ((rc = dump(c, b, c->d_pos)) || (rc = dump(c, b, c->d_mat)) || (rc = dump(c, b, c->d_comp)) ||
      (rc = dump(c, b, c->d_en)) || (rc = dump(c, b, c->d_box)) || (rc = dump(c, b, c->d_rc2)) ||
      (rc = dump(c, b, c->d_drift)) || (rc = dump(c, b, c->d_beta)) || (rc = dump(c, b, c->d_maxd)) ||
      (rc = dump(c, b, c->d_maxbox)) || (rc = dump(c, b, c->d_ham)) || (rc = dump(c, b, c->d_ctr)) ||
      (rc = dump(c, b, c->d_status)) || (rc = dump(c, b, c->d_wos)) || (rc = dump(c, b, c->d_cnt)) ||
      (rc = dump(c, b, c->d_hist)) || (rc = dump(c, b, c->d_nn_G)) || (rc = dump(c, b, c->d_nn_sow)) ||
      (rc = dump(c, b, c->d_rdf)) || (rc = dump(c, b, c->d_boxh)) || (rc = dump(c, b, c->d_maxboxh)) ||
      (rc = dump(c, b, c->d_maxd_sep)) || (rc = dump(c, b, c->d_cnt_sep)) || (rc = dump(c, b, c->d_tan)) ||
      (rc = dump(c, b, c->d_nn2_swaps)) || (rc = dump(c, b, c->d_pe)))
    return rc;
  put(b, "PTMCEND!", 8);
  if (!write_file_atomic(d + "/engine.bin", b)) return c->fail(PTMC_ERR_IO, "cannot write engine.bin");
  return PTMC_OK;
}

int ptmc_restore(ptmc_ctx* c, const char* dir) {
  if (!c || !dir) return PTMC_ERR_ARG;
  if (!c->inited) return c->fail(PTMC_ERR_STATE, "call ptmc_init before ptmc_restore");
  std::string path = std::string(dir) + "/engine.bin";
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) {
    struct stat sb;
    if (::stat((std::string(dir) + "/hist_info.data").c_str(), &sb) == 0)
      return restore_reference_text(c, dir);  // a checkpoint the reference wrote
    return c->fail(PTMC_ERR_IO, "cannot open " + path + " (and no reference checkpoint files)");
  }
  std::string b;
  char buf[1 << 16];
  size_t k;
  while ((k = std::fread(buf, 1, sizeof(buf), f)) > 0) b.append(buf, k);
  std::fclose(f);
  if (b.size() >= 8 && (b.compare(0, 8, "PTMCGB01") == 0 || b.compare(0, 8, "PTMCGB02") == 0))
    return c->fail(PTMC_ERR_IO, "engine.bin: written by an earlier format (" + b.substr(0, 8) +
                                    "), not restorable");
  if (b.size() < 8 + 32 || b.compare(0, 8, "PTMCGB03") != 0)
    return c->fail(PTMC_ERR_IO, "engine.bin: bad magic");
  if (b.size() < 8 || b.compare(b.size() - 8, 8, "PTMCEND!") != 0)
    return c->fail(PTMC_ERR_IO, "engine.bin truncated (no end marker)");
  unsigned long long hdr[4];
  std::memcpy(hdr, b.data() + 8, sizeof(hdr));
  if (hdr[0] != (unsigned long long)c->p.n_runs || hdr[1] != (unsigned long long)c->R() ||
      hdr[2] != (unsigned long long)c->W)
    return c->fail(PTMC_ERR_IO, "engine.bin was written by a context with other dimensions");
  size_t at = 8 + sizeof(hdr);
  if (at + sizeof(RunDesc) * c->rd.size() > b.size()) return c->fail(PTMC_ERR_IO, "engine.bin truncated");
  std::vector<RunDesc> rd(c->rd.size());
  std::memcpy(rd.data(), b.data() + at, sizeof(RunDesc) * rd.size());
  at += sizeof(RunDesc) * rd.size();
  for (size_t i = 0; i < rd.size(); ++i)
    if (rd[i].N != c->rd[i].N || rd[i].pos_off != c->rd[i].pos_off)
      return c->fail(PTMC_ERR_IO, "engine.bin run layout does not match");
  int rc;
  if ((rc = undump(c, b, at, c->d_pos)) || (rc = undump(c, b, at, c->d_mat)) ||
      (rc = undump(c, b, at, c->d_comp)) || (rc = undump(c, b, at, c->d_en)) ||
      (rc = undump(c, b, at, c->d_box)) || (rc = undump(c, b, at, c->d_rc2)) ||
      (rc = undump(c, b, at, c->d_drift)) || (rc = undump(c, b, at, c->d_beta)) ||
      (rc = undump(c, b, at, c->d_maxd)) || (rc = undump(c, b, at, c->d_maxbox)) ||
      (rc = undump(c, b, at, c->d_ham)) || (rc = undump(c, b, at, c->d_ctr)) ||
      (rc = undump(c, b, at, c->d_status)) || (rc = undump(c, b, at, c->d_wos)) ||
      (rc = undump(c, b, at, c->d_cnt)) || (rc = undump(c, b, at, c->d_hist)) ||
      (rc = undump(c, b, at, c->d_nn_G)) || (rc = undump(c, b, at, c->d_nn_sow)) ||
      (rc = undump(c, b, at, c->d_rdf)) || (rc = undump(c, b, at, c->d_boxh)) ||
      (rc = undump(c, b, at, c->d_maxboxh)) || (rc = undump(c, b, at, c->d_maxd_sep)) ||
      (rc = undump(c, b, at, c->d_cnt_sep)) || (rc = undump(c, b, at, c->d_tan)) ||
      (rc = undump(c, b, at, c->d_nn2_swaps)) || (rc = undump(c, b, at, c->d_pe)))
    return rc;
  c->rd = rd;
  c->equilibrated = hdr[3] != 0;
  rc = push_runs(c);
  if (rc) return rc;
  CK(cudaStreamSynchronize(c->st));
  return PTMC_OK;
}

}  // extern "C"

extern "C" {

// ---------------------------------------------------------------- WHAM
static int wham_common(bool npt, int R, int n_bin, const double* hist,
                       const double* t_grid, const double* beta, double en_min,
                       double en_max, double v_min, double v_max, double pr,
                       double thr, double* T_out, double* cv_out, int* iters) {
  if (R < 1 || n_bin < 1 || !hist || !t_grid || !beta || !T_out || !cv_out) {
    g_err = "multihistogram: bad arguments";
    return PTMC_ERR_ARG;
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    g_err = "multihistogram: no CUDA device";
    return PTMC_ERR_CUDA;
  }
  int n_out = 10 * R;  // temp_trajectories (multihist_NVT.jl:11-15)
  std::vector<double> tb(2 * n_out);
  for (int i = 0; i < n_out; ++i) {  // TempGrid{10R}(t_1, t_R) geometric (:29-34)
    double T = n_out == 1 ? t_grid[0]
                          : t_grid[0] * std::pow(t_grid[R - 1] / t_grid[0], (double)i / (double)(n_out - 1));
    tb[i] = 1.0 / (kB * T);
    tb[n_out + i] = T;
  }
  long long nb = n_bin + 2;
  long long hn = npt ? (long long)R * nb * nb : (long long)R * nb;
  long long B = npt ? (long long)n_bin * n_bin : n_bin;
  long long nwork = wham_work_doubles(R, (int)B);
  double *dh = nullptr, *db = nullptr, *dtb = nullptr, *dw = nullptr, *dout = nullptr;
  int* dit = nullptr;
  cudaError_t e = cudaSuccess;
  auto chk = [&](cudaError_t x) { if (e == cudaSuccess) e = x; };
  chk(cudaMalloc(&dh, sizeof(double) * hn));
  chk(cudaMalloc(&db, sizeof(double) * R));
  chk(cudaMalloc(&dtb, sizeof(double) * 2 * n_out));
  chk(cudaMalloc(&dw, sizeof(double) * nwork));
  chk(cudaMalloc(&dout, sizeof(double) * n_out));
  chk(cudaMalloc(&dit, sizeof(int)));
  if (e == cudaSuccess) {
    chk(cudaMemcpy(dh, hist, sizeof(double) * hn, cudaMemcpyHostToDevice));
    chk(cudaMemcpy(db, beta, sizeof(double) * R, cudaMemcpyHostToDevice));
    chk(cudaMemcpy(dtb, tb.data(), sizeof(double) * 2 * n_out, cudaMemcpyHostToDevice));
  }
  if (e == cudaSuccess) {
    int rc = npt ? wham_npt_device(R, n_bin, dh, db, en_min, en_max, v_min, v_max, pr, thr, dtb,
                                   n_out, dw, dout, dit, nullptr)
                 : wham_nvt_device(R, n_bin, dh, db, en_min, en_max, thr, dtb, n_out, dw, dout,
                                   dit, nullptr);
    if (rc) e = (cudaError_t)rc;
  }
  if (e == cudaSuccess) chk(cudaMemcpy(cv_out, dout, sizeof(double) * n_out, cudaMemcpyDeviceToHost));
  int it = 0;
  if (e == cudaSuccess) chk(cudaMemcpy(&it, dit, sizeof(int), cudaMemcpyDeviceToHost));
  cudaFree(dh);
  cudaFree(db);
  cudaFree(dtb);
  cudaFree(dw);
  cudaFree(dout);
  cudaFree(dit);
  if (e != cudaSuccess) {
    g_err = std::string("multihistogram: ") + cudaGetErrorString(e);
    return PTMC_ERR_CUDA;
  }
  for (int i = 0; i < n_out; ++i) T_out[i] = tb[n_out + i];
  if (iters) *iters = it;
  return PTMC_OK;
}

int ptmc_multihist_nvt(int R, int n_bin, const double* en_hist, const double* t_grid,
                       const double* beta, double en_min, double en_max, double thr,
                       double* T_out, double* cv_out, int* iters) {
  return wham_common(false, R, n_bin, en_hist, t_grid, beta, en_min, en_max, 0, 0, 0, thr,
                     T_out, cv_out, iters);
}

int ptmc_multihist_npt(int R, int n_bin, const double* ev_hist, const double* t_grid,
                       const double* beta, double en_min, double en_max, double v_min,
                       double v_max, double pressure, double thr, double* T_out,
                       double* cp_out, int* iters) {
  return wham_common(true, R, n_bin, ev_hist, t_grid, beta, en_min, en_max, v_min, v_max,
                     pressure, thr, T_out, cp_out, iters);
}

}  // extern "C"

// ---------------------------------------------------------------- surrogate
// Delayed-acceptance pair surrogate (ptmc_surrogate.cuh, ptmc_surrogate.cu):
// record capture from the exact chain, training on the GPU, frozen use as the
// first stage of two-stage moves in the NN cycle kernel.
namespace {

SurCfgDev sur_dev(const ptmc_surrogate_cfg& c) {
  SurCfgDev d;
  d.r_lo = (float)c.r_lo;
  d.dmu = (float)((c.r_hi - c.r_lo) / (SUR_F - 1));
  d.gamma = (float)c.gamma;
  d.r_cut = (float)c.r_cut;
  d.escale = (float)c.escale;
  return d;
}

bool sur_cfg_ok(const ptmc_surrogate_cfg* c, bool allow_auto_scale) {
  if (!c) return false;
  if (!(c->r_hi > c->r_lo) || !(c->gamma > 0) || !(c->r_cut > 0)) return false;
  return c->escale > 0 || (allow_auto_scale && c->escale == 0);
}

// seeded initial parameters: W ~ U(-1/sqrt(fan_in), 1/sqrt(fan_in)), zero biases
void sur_init_params(std::vector<float>& P, uint64_t seed) {
  uint64_t x = seed ^ 0x9E3779B97F4A7C15ull;
  auto u = [&]() {  // splitmix64 -> [0, 1)
    x += 0x9E3779B97F4A7C15ull;
    uint64_t z = x;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (double)(z >> 11) * (1.0 / 9007199254740992.0);
  };
  P.assign(SUR_NP, 0.0f);
  for (int k = 0; k < SUR_B1; ++k) P[k] = (float)((2 * u() - 1) / std::sqrt((double)SUR_F));
  for (int k = 0; k < SUR_H * SUR_H; ++k)
    P[SUR_W2 + k] = (float)((2 * u() - 1) / std::sqrt((double)SUR_H));
  for (int k = 0; k < SUR_H; ++k) P[SUR_W3 + k] = (float)((2 * u() - 1) / std::sqrt((double)SUR_H));
}

void drop_graphs(ptmc_ctx* c) {
  for (auto& kv : c->graphs) cudaGraphExecDestroy(kv.second);
  c->graphs.clear();
}

int sur_err_check(ptmc_ctx* c) {
  int e = 0;
  CK(cudaMemcpyAsync(&e, c->d_sur_err.p, sizeof(int), cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  if (e) return c->fail(PTMC_ERR_CUDA, "a tensor-core completion wait ran out (surrogate kernels)");
  return PTMC_OK;
}

// phi of the frozen surrogate on the grid of the first stage (built whenever
// screening is switched on: the parameters cannot change while it is on)
int build_sur_table(ptmc_ctx* c) {
  int e = sur_launch_table(sur_dev(c->sur_cfg), c->d_sur_P.p, c->d_sur_tab.p, c->d_sur_err.p, c->st);
  if (e) return c->cuda_fail((cudaError_t)e, "k_sur_table launch");
  int rc = sur_err_check(c);
  if (rc) return rc;
  c->Q.sur_tab = c->d_sur_tab.p;
  c->Q.sur_tab_inv_h = (float)((SUR_TAB_N - 1) / (double)c->sur_cfg.r_cut);
  return PTMC_OK;
}

int sm_count() {
  int dev = 0, n = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
  return n > 0 ? n : 1;
}

// standalone helpers: device buffers owned by one call
struct Scratch {
  std::vector<void*> ptrs;
  template <typename T>
  T* get(size_t n) {
    void* p = nullptr;
    if (cudaMalloc(&p, std::max<size_t>(n, 1) * sizeof(T)) != cudaSuccess) return nullptr;
    ptrs.push_back(p);
    return (T*)p;
  }
  ~Scratch() {
    for (void* p : ptrs) cudaFree(p);
  }
};

int standalone_device(int device) {
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0) {
    g_err = std::string("no CUDA device: ") + cudaGetErrorString(e);
    return PTMC_ERR_CUDA;
  }
  if (device < 0 || device >= ndev) {
    g_err = "bad device ordinal";
    return PTMC_ERR_ARG;
  }
  if ((e = cudaSetDevice(device)) != cudaSuccess) {
    g_err = std::string("cudaSetDevice: ") + cudaGetErrorString(e);
    return PTMC_ERR_CUDA;
  }
  return PTMC_OK;
}

#define SCK(call)                                                           \
  do {                                                                      \
    cudaError_t e_ = (call);                                                \
    if (e_ != cudaSuccess) {                                                \
      g_err = std::string(#call) + ": " + cudaGetErrorString(e_);           \
      return PTMC_ERR_CUDA;                                                 \
    }                                                                       \
  } while (0)

}  // namespace

extern "C" {

int ptmc_surrogate_eval(const ptmc_surrogate_cfg* cfg, const float* params, const float* rows,
                        int n, double* dEs_out, int device) {
  if (!sur_cfg_ok(cfg, false) || !params || (n > 0 && (!rows || !dEs_out)) || n < 0) {
    g_err = "ptmc_surrogate_eval: bad argument";
    return PTMC_ERR_ARG;
  }
  int rc = standalone_device(device);
  if (rc) return rc;
  if (n == 0) return PTMC_OK;
  Scratch sc;
  float* dP = sc.get<float>(SUR_NP);
  float* dR = sc.get<float>((size_t)n * SUR_ROWS);
  double* dO = sc.get<double>(n);
  int* dE = sc.get<int>(1);
  if (!dP || !dR || !dO || !dE) {
    g_err = "ptmc_surrogate_eval: device allocation failed";
    return PTMC_ERR_CUDA;
  }
  SCK(cudaMemcpy(dP, params, sizeof(float) * SUR_NP, cudaMemcpyHostToDevice));
  SCK(cudaMemcpy(dR, rows, sizeof(float) * n * SUR_ROWS, cudaMemcpyHostToDevice));
  SCK(cudaMemset(dE, 0, sizeof(int)));
  int e = sur_launch_eval(sur_dev(*cfg), dP, dR, n, dO, dE, 8 * sm_count(), nullptr);
  if (e) {
    g_err = std::string("k_sur_eval launch: ") + cudaGetErrorString((cudaError_t)e);
    return PTMC_ERR_CUDA;
  }
  SCK(cudaDeviceSynchronize());
  int herr = 0;
  SCK(cudaMemcpy(&herr, dE, sizeof(int), cudaMemcpyDeviceToHost));
  if (herr) {
    g_err = "a tensor-core completion wait ran out (k_sur_eval)";
    return PTMC_ERR_CUDA;
  }
  SCK(cudaMemcpy(dEs_out, dO, sizeof(double) * n, cudaMemcpyDeviceToHost));
  return PTMC_OK;
}

int ptmc_surrogate_loss_grad(const ptmc_surrogate_cfg* cfg, const float* params, const float* rows,
                             const float* targets, int n, double* loss, float* grad, int device) {
  if (!sur_cfg_ok(cfg, false) || !params || !rows || !targets || !loss || !grad || n < 1) {
    g_err = "ptmc_surrogate_loss_grad: bad argument";
    return PTMC_ERR_ARG;
  }
  int rc = standalone_device(device);
  if (rc) return rc;
  Scratch sc;
  float* dP = sc.get<float>(SUR_NP);
  float* dR = sc.get<float>((size_t)n * SUR_ROWS);
  float* dY = sc.get<float>(n);
  int* dI = sc.get<int>(n);
  float* dG = sc.get<float>(SUR_NP);
  double* dL = sc.get<double>(1);
  int* dE = sc.get<int>(1);
  if (!dP || !dR || !dY || !dI || !dG || !dL || !dE) {
    g_err = "ptmc_surrogate_loss_grad: device allocation failed";
    return PTMC_ERR_CUDA;
  }
  std::vector<int> idx(n);
  for (int k = 0; k < n; ++k) idx[k] = k;
  SCK(cudaMemcpy(dP, params, sizeof(float) * SUR_NP, cudaMemcpyHostToDevice));
  SCK(cudaMemcpy(dR, rows, sizeof(float) * n * SUR_ROWS, cudaMemcpyHostToDevice));
  SCK(cudaMemcpy(dY, targets, sizeof(float) * n, cudaMemcpyHostToDevice));
  SCK(cudaMemcpy(dI, idx.data(), sizeof(int) * n, cudaMemcpyHostToDevice));
  SCK(cudaMemset(dG, 0, sizeof(float) * SUR_NP));
  SCK(cudaMemset(dL, 0, sizeof(double)));
  SCK(cudaMemset(dE, 0, sizeof(int)));
  int e = sur_launch_grad(sur_dev(*cfg), dP, dR, dY, n, dI, n, 0, 0, dG, dL, dE, 3 * sm_count(),
                          nullptr);
  if (e) {
    g_err = std::string("k_sur_grad launch: ") + cudaGetErrorString((cudaError_t)e);
    return PTMC_ERR_CUDA;
  }
  SCK(cudaDeviceSynchronize());
  int herr = 0;
  SCK(cudaMemcpy(&herr, dE, sizeof(int), cudaMemcpyDeviceToHost));
  if (herr) {
    g_err = "a tensor-core completion wait ran out (k_sur_grad)";
    return PTMC_ERR_CUDA;
  }
  SCK(cudaMemcpy(grad, dG, sizeof(float) * SUR_NP, cudaMemcpyDeviceToHost));
  SCK(cudaMemcpy(loss, dL, sizeof(double), cudaMemcpyDeviceToHost));
  return PTMC_OK;
}

int ptmc_surrogate_set(ptmc_ctx* c, const ptmc_surrogate_cfg* cfg, const float* params,
                       int capacity, int record_every) {
  if (!c) return PTMC_ERR_ARG;
  if (!c->inited) return c->fail(PTMC_ERR_STATE, "ptmc_init not called");
  if (c->pot != POT_NN) return c->fail(PTMC_ERR_ARG, "delayed acceptance needs the NN potential");
  if (!sur_cfg_ok(cfg, true)) return c->fail(PTMC_ERR_ARG, "surrogate: bad configuration");
  if (capacity < 1 || record_every < 1)
    return c->fail(PTMC_ERR_ARG, "surrogate: capacity and record_every must be >= 1");
  if ((long long)capacity * SUR_ROWS > (1LL << 31))
    return c->fail(PTMC_ERR_LIMIT, "surrogate: at most 2^24 records");
  const int W = c->W;
  // the record ring survives a new set-up with the same capacity (re-training
  // from other initial parameters on the same records)
  const bool keep_ring = c->sur_set && c->Q.rec_cap == capacity;
  for (auto* b : {&c->d_sur_P, &c->d_sur_m, &c->d_sur_v, &c->d_sur_g, &c->d_da_kappa, &c->d_sur_tab})
    b->free_();
  c->d_sur_loss.free_();
  c->d_da_cnt.free_();
  c->d_sur_err.free_();
  if (!keep_ring) {
    c->d_rec_rows.free_();
    c->d_rec_y.free_();
    c->d_rec_n.free_();
    c->d_rec_slot.free_();
  }
  if (c->d_sur_P.alloc(SUR_NP) || c->d_sur_m.alloc(SUR_NP) || c->d_sur_v.alloc(SUR_NP) ||
      c->d_sur_g.alloc(SUR_NP) || c->d_sur_loss.alloc(1) || c->d_da_cnt.alloc(2 * (size_t)W) ||
      c->d_sur_err.alloc(1) || c->d_da_kappa.alloc(W) || c->d_sur_tab.alloc(SUR_TAB_N))
    return c->fail(PTMC_ERR_CUDA, "surrogate: device allocation failed");
  if (!keep_ring && (c->d_rec_rows.alloc((size_t)capacity * SUR_ROWS) ||
                     c->d_rec_y.alloc(capacity) || c->d_rec_n.alloc(1) ||
                     c->d_rec_slot.alloc(capacity)))
    return c->fail(PTMC_ERR_CUDA, "surrogate: device allocation failed");
  c->sur_kappa.assign(c->R(), 1.0);
  {
    std::vector<float> k1(W, 1.0f);
    CK(cudaMemcpyAsync(c->d_da_kappa.p, k1.data(), sizeof(float) * W, cudaMemcpyHostToDevice, c->st));
  }
  std::vector<float> P;
  if (params) P.assign(params, params + SUR_NP);
  else sur_init_params(P, c->p.seed);
  CK(cudaMemcpyAsync(c->d_sur_P.p, P.data(), sizeof(float) * SUR_NP, cudaMemcpyHostToDevice, c->st));
  CK(cudaMemsetAsync(c->d_sur_m.p, 0, sizeof(float) * SUR_NP, c->st));
  CK(cudaMemsetAsync(c->d_sur_v.p, 0, sizeof(float) * SUR_NP, c->st));
  CK(cudaMemsetAsync(c->d_sur_g.p, 0, sizeof(float) * SUR_NP, c->st));
  CK(cudaMemsetAsync(c->d_sur_loss.p, 0, sizeof(double), c->st));
  if (!keep_ring) CK(cudaMemsetAsync(c->d_rec_n.p, 0, sizeof(unsigned long long), c->st));
  CK(cudaMemsetAsync(c->d_da_cnt.p, 0, sizeof(long long) * 2 * W, c->st));
  CK(cudaMemsetAsync(c->d_sur_err.p, 0, sizeof(int), c->st));
  CK(cudaStreamSynchronize(c->st));
  c->sur_cfg = *cfg;
  c->sur_set = true;
  c->sur_step = 0;
  NNParams& Q = c->Q;
  Q.da = 0;
  Q.sc = sur_dev(*cfg);
  Q.surP = c->d_sur_P.p;
  Q.da_cnt = c->d_da_cnt.p;
  Q.da_kappa = c->d_da_kappa.p;
  Q.rec_rows = nullptr;
  Q.rec_y = c->d_rec_y.p;
  Q.rec_slot = c->d_rec_slot.p;
  Q.rec_n = c->d_rec_n.p;
  Q.rec_cap = capacity;
  Q.rec_every = record_every;
  drop_graphs(c);
  return PTMC_OK;
}

int ptmc_surrogate_record(ptmc_ctx* c, int on) {
  if (!c) return PTMC_ERR_ARG;
  if (!c->sur_set) return c->fail(PTMC_ERR_STATE, "ptmc_surrogate_set not called");
  if (on && c->Q.da)
    return c->fail(PTMC_ERR_STATE, "records come from the exact chain: switch delayed acceptance off first");
  c->Q.rec_rows = on ? c->d_rec_rows.p : nullptr;
  drop_graphs(c);
  return PTMC_OK;
}

int ptmc_surrogate_train(ptmc_ctx* c, int steps, int batch, double lr, double* loss_out) {
  if (!c) return PTMC_ERR_ARG;
  if (!c->sur_set) return c->fail(PTMC_ERR_STATE, "ptmc_surrogate_set not called");
  if (c->Q.da) return c->fail(PTMC_ERR_STATE, "the surrogate is frozen while delayed acceptance is on");
  if (steps < 0 || batch < 1 || !(lr > 0)) return c->fail(PTMC_ERR_ARG, "surrogate: bad training arguments");
  unsigned long long nrec = 0;
  CK(cudaMemcpyAsync(&nrec, c->d_rec_n.p, sizeof(nrec), cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  const int n = (int)std::min<unsigned long long>(nrec, (unsigned long long)c->Q.rec_cap);
  if (n < 1) return c->fail(PTMC_ERR_STATE, "surrogate: no training records captured");
  if (c->sur_cfg.escale == 0) {  // output scale from the data: 1.4826 x median |dE - median|
    std::vector<float> y(n);
    CK(cudaMemcpyAsync(y.data(), c->d_rec_y.p, sizeof(float) * n, cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    std::vector<float> t(y);
    std::nth_element(t.begin(), t.begin() + n / 2, t.end());
    const float med = t[n / 2];
    for (auto& v : t) v = std::fabs(v - med);
    std::nth_element(t.begin(), t.begin() + n / 2, t.end());
    double sc = 1.4826 * t[n / 2];
    if (!(sc > 0)) sc = 1e-3;
    c->sur_cfg.escale = sc;
    c->Q.sc.escale = (float)sc;
  }
  const SurCfgDev sd = sur_dev(c->sur_cfg);
  const int k0 = steps - std::max(1, steps / 10);
  const int grid = std::min(batch, 3 * sm_count());
  for (int k = 0; k < steps; ++k) {
    if (k == k0) CK(cudaMemsetAsync(c->d_sur_loss.p, 0, sizeof(double), c->st));
    int e = sur_launch_grad(sd, c->d_sur_P.p, c->d_rec_rows.p, c->d_rec_y.p, n, nullptr, batch,
                            c->p.seed ^ 0x5A17ull, c->sur_step, c->d_sur_g.p, c->d_sur_loss.p,
                            c->d_sur_err.p, grid, c->st);
    if (e) return c->cuda_fail((cudaError_t)e, "k_sur_grad launch");
    c->sur_step += 1;
    e = sur_launch_adam(c->d_sur_P.p, c->d_sur_g.p, c->d_sur_m.p, c->d_sur_v.p, c->sur_step,
                        (float)lr, c->st);
    if (e) return c->cuda_fail((cudaError_t)e, "k_sur_adam launch");
    c->stats.kernel_launches += 2;
  }
  int rc = sur_err_check(c);
  if (rc) return rc;
  if (loss_out) {
    double L = 0;
    CK(cudaMemcpyAsync(&L, c->d_sur_loss.p, sizeof(double), cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    *loss_out = steps > 0 ? L / (steps - k0) : 0.0;
  }
  return PTMC_OK;
}

int ptmc_surrogate_enable(ptmc_ctx* c, int on) {
  if (!c) return PTMC_ERR_ARG;
  if (!c->sur_set) return c->fail(PTMC_ERR_STATE, "ptmc_surrogate_set not called");
  if (on) {
    if (c->Q.rec_rows) return c->fail(PTMC_ERR_STATE, "stop recording before enabling delayed acceptance");
    if (!(c->sur_cfg.escale > 0))
      return c->fail(PTMC_ERR_STATE, "surrogate output scale unset: train first or give escale");
    int rc = build_sur_table(c);
    if (rc) return rc;
  }
  c->Q.da = on ? 1 : 0;
  drop_graphs(c);
  return PTMC_OK;
}

int ptmc_surrogate_get(ptmc_ctx* c, float* params, ptmc_surrogate_cfg* cfg, long long* stats) {
  if (!c) return PTMC_ERR_ARG;
  if (!c->sur_set) return c->fail(PTMC_ERR_STATE, "ptmc_surrogate_set not called");
  if (params)
    CK(cudaMemcpyAsync(params, c->d_sur_P.p, sizeof(float) * SUR_NP, cudaMemcpyDeviceToHost, c->st));
  std::vector<long long> cnt(2 * (size_t)c->W);
  unsigned long long nrec = 0;
  CK(cudaMemcpyAsync(cnt.data(), c->d_da_cnt.p, sizeof(long long) * cnt.size(), cudaMemcpyDeviceToHost, c->st));
  CK(cudaMemcpyAsync(&nrec, c->d_rec_n.p, sizeof(nrec), cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  if (cfg) *cfg = c->sur_cfg;
  if (stats) {
    stats[0] = (long long)nrec;
    stats[1] = stats[2] = stats[3] = 0;
    for (int g = 0; g < c->W; ++g) {
      stats[1] += cnt[2 * (size_t)g];
      stats[2] += cnt[2 * (size_t)g + 1];
    }
  }
  return PTMC_OK;
}

int ptmc_surrogate_records(ptmc_ctx* c, float* rows, float* targets, int max_n, int* n_out) {
  if (!c || !n_out || max_n < 0) return PTMC_ERR_ARG;
  if (!c->sur_set) return c->fail(PTMC_ERR_STATE, "ptmc_surrogate_set not called");
  unsigned long long nrec = 0;
  CK(cudaMemcpyAsync(&nrec, c->d_rec_n.p, sizeof(nrec), cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  int n = (int)std::min<unsigned long long>(std::min<unsigned long long>(nrec, c->Q.rec_cap),
                                            (unsigned long long)max_n);
  if (n > 0 && rows)
    CK(cudaMemcpyAsync(rows, c->d_rec_rows.p, sizeof(float) * SUR_ROWS * n, cudaMemcpyDeviceToHost, c->st));
  if (n > 0 && targets)
    CK(cudaMemcpyAsync(targets, c->d_rec_y.p, sizeof(float) * n, cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  *n_out = n;
  return PTMC_OK;
}


int ptmc_surrogate_set_kappa(ptmc_ctx* c, const double* kappa) {
  if (!c || !kappa) return PTMC_ERR_ARG;
  if (!c->sur_set) return c->fail(PTMC_ERR_STATE, "ptmc_surrogate_set not called");
  const int R = c->R(), W = c->W;
  for (int s2 = 0; s2 < R; ++s2)
    if (!(kappa[s2] >= 0.0 && kappa[s2] <= 1.0))
      return c->fail(PTMC_ERR_ARG, "kappa must lie in [0, 1]");
  std::vector<float> kw(W);
  for (const auto& r : c->rd)
    for (int s2 = 0; s2 < R; ++s2) kw[r.wk + s2] = (float)kappa[s2];
  CK(cudaMemcpyAsync(c->d_da_kappa.p, kw.data(), sizeof(float) * W, cudaMemcpyHostToDevice, c->st));
  CK(cudaStreamSynchronize(c->st));
  c->sur_kappa.assign(kappa, kappa + R);
  return PTMC_OK;
}

int ptmc_surrogate_calibrate(ptmc_ctx* c, double cost_ratio, int timing_cycles, double* kappa_out) {
  if (!c) return PTMC_ERR_ARG;
  if (!c->sur_set) return c->fail(PTMC_ERR_STATE, "ptmc_surrogate_set not called");
  if (c->Q.rec_rows) return c->fail(PTMC_ERR_STATE, "stop recording before calibrating");
  if (!(c->sur_cfg.escale > 0)) return c->fail(PTMC_ERR_STATE, "train the surrogate before calibrating");
  unsigned long long nrec = 0;
  CK(cudaMemcpyAsync(&nrec, c->d_rec_n.p, sizeof(nrec), cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  const int n = (int)std::min<unsigned long long>(nrec, (unsigned long long)c->Q.rec_cap);
  if (n < 1) return c->fail(PTMC_ERR_STATE, "surrogate: no records to calibrate on");
  const int R = c->R(), W = c->W;
  const int da_before = c->Q.da;
  {
    int rc = build_sur_table(c);
    if (rc) return rc;
  }
  auto set_kappa = [&](const std::vector<double>& k) -> int {
    std::vector<float> kw(W);
    for (const auto& r : c->rd)
      for (int s2 = 0; s2 < R; ++s2) kw[r.wk + s2] = (float)k[s2];
    CK(cudaMemcpyAsync(c->d_da_kappa.p, kw.data(), sizeof(float) * W, cudaMemcpyHostToDevice, c->st));
    CK(cudaStreamSynchronize(c->st));
    return PTMC_OK;
  };
  double r = cost_ratio;
  if (!(r > 0)) {  // cost of a surrogate stage relative to an exact evaluation, measured
    if (timing_cycles < 1) return c->fail(PTMC_ERR_ARG, "need timing_cycles >= 1 to measure the cost ratio");
    int rc = set_kappa(std::vector<double>(R, 1.0));
    if (rc) return rc;
    c->Q.da = 0;
    drop_graphs(c);
    rc = run_phase(c, timing_cycles, PHASE_PLAIN);
    if (rc) return rc;
    double t_ex = c->stats.last_cycles_ms;
    std::vector<long long> k0(2 * (size_t)W), k1(2 * (size_t)W);
    CK(cudaMemcpyAsync(k0.data(), c->d_da_cnt.p, sizeof(long long) * k0.size(), cudaMemcpyDeviceToHost, c->st));
    c->Q.da = 1;
    drop_graphs(c);
    rc = run_phase(c, timing_cycles, PHASE_PLAIN);
    if (rc) return rc;
    const double t_da = c->stats.last_cycles_ms;
    CK(cudaMemcpyAsync(k1.data(), c->d_da_cnt.p, sizeof(long long) * k1.size(), cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    c->Q.da = 0;  // a second exact segment after the screened one (the chain drifts)
    drop_graphs(c);
    rc = run_phase(c, timing_cycles, PHASE_PLAIN);
    if (rc) return rc;
    t_ex = 0.5 * (t_ex + c->stats.last_cycles_ms);
    double rej = 0, ex = 0;
    for (int g = 0; g < W; ++g) {
      rej += (double)(k1[2 * (size_t)g] - k0[2 * (size_t)g]);
      ex += (double)(k1[2 * (size_t)g + 1] - k0[2 * (size_t)g + 1]);
    }
    const double f = ex / std::max(1.0, rej + ex);
    r = t_ex > 0 ? t_da / t_ex - f : 0.05;
    r = std::min(2.0, std::max(0.002, r));
  }
  // dE_s of every record on the GPU, then the choice per slot on the host
  double* d_out = nullptr;
  CK(cudaMalloc(&d_out, sizeof(double) * n));
  int e = sur_launch_eval(sur_dev(c->sur_cfg), c->d_sur_P.p, c->d_rec_rows.p, n, d_out,
                          c->d_sur_err.p, 8 * sm_count(), c->st);
  std::vector<double> des(n);
  std::vector<float> y(n);
  std::vector<int> sl(n);
  cudaError_t ce = e ? (cudaError_t)e
                     : cudaMemcpyAsync(des.data(), d_out, sizeof(double) * n, cudaMemcpyDeviceToHost, c->st);
  if (ce == cudaSuccess)
    ce = cudaMemcpyAsync(y.data(), c->d_rec_y.p, sizeof(float) * n, cudaMemcpyDeviceToHost, c->st);
  if (ce == cudaSuccess)
    ce = cudaMemcpyAsync(sl.data(), c->d_rec_slot.p, sizeof(int) * n, cudaMemcpyDeviceToHost, c->st);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(c->st);
  cudaFree(d_out);
  if (ce != cudaSuccess) return c->cuda_fail(ce, "surrogate calibration");
  int rc = sur_err_check(c);
  if (rc) return rc;
  // Per slot and kappa in {0, 1/16, ..., 1}: the two-stage acceptance a and the
  // cost per move c (r + p1 with p1 the first-stage acceptance; 1 for kappa = 0,
  // no screening), estimated on the slot's records.  The walker CTAs share the
  // SMs and the cycle kernel is throughput-bound, so a cycle's time follows the
  // summed cost of all walkers (measured: uniform kappa = 1 ran in r + mean p1
  // of the exact time).  Objective: accepted moves per unit time,
  // sum_s a_s / sum_s c_s, maximised over the per-slot choices by Dinkelbach's
  // iteration (each step maximises sum_s (a_s - lambda c_s) slot by slot, then
  // lambda = sum a / sum c).
  constexpr int NK = 17;
  std::vector<double> A((size_t)R * NK, -1.0), Cc((size_t)R * NK, 0.0);
  for (int s2 = 0; s2 < R; ++s2) {
    const double b = c->beta[s2];
    for (int q = 0; q < NK; ++q) {
      const double k = q / 16.0;
      double a = 0, p1s = 0;
      long cnt = 0;
      for (int m = 0; m < n; ++m) {
        if (sl[m] != s2) continue;
        const double d = (double)y[m], ds = des[m];
        const double p1 = std::min(1.0, std::exp(-k * b * ds));
        const double p2 = std::min(1.0, std::exp(-b * (d - k * ds)));
        a += p1 * p2;
        p1s += p1;
        ++cnt;
      }
      if (cnt == 0) break;  // no records for this slot: it keeps kappa = 1
      A[(size_t)s2 * NK + q] = a / cnt;
      Cc[(size_t)s2 * NK + q] = q == 0 ? 1.0 : r + p1s / cnt;
    }
  }
  std::vector<double> kap(R, 1.0);
  std::vector<int> pick(R, NK - 1);
  auto totals = [&](double& sa, double& sc) {
    sa = sc = 0;
    for (int s2 = 0; s2 < R; ++s2) {
      if (A[(size_t)s2 * NK] < 0) continue;
      sa += A[(size_t)s2 * NK + pick[s2]];
      sc += Cc[(size_t)s2 * NK + pick[s2]];
    }
  };
  double sa = 0, sc = 0;
  totals(sa, sc);
  double lambda = sc > 0 ? sa / sc : 0;
  for (int it = 0; it < 50; ++it) {
    for (int s2 = 0; s2 < R; ++s2) {
      if (A[(size_t)s2 * NK] < 0) continue;
      double bv = -1e300;
      for (int q = 0; q < NK; ++q) {
        const double v = A[(size_t)s2 * NK + q] - lambda * Cc[(size_t)s2 * NK + q];
        if (v > bv + 1e-15) {
          bv = v;
          pick[s2] = q;
        }
      }
    }
    totals(sa, sc);
    const double nl = sc > 0 ? sa / sc : 0;
    if (std::fabs(nl - lambda) <= 1e-12 * std::max(1.0, nl)) break;
    lambda = nl;
  }
  for (int s2 = 0; s2 < R; ++s2)
    if (A[(size_t)s2 * NK] >= 0) kap[s2] = pick[s2] / 16.0;
  rc = set_kappa(kap);
  if (rc) return rc;
  c->sur_kappa = kap;
  c->Q.da = da_before;
  drop_graphs(c);
  if (kappa_out)
    for (int s2 = 0; s2 < R; ++s2) kappa_out[s2] = kap[s2];
  return PTMC_OK;
}

}  // extern "C"

// ---------------------------------------------------------------- autotuner
// Launch shape per atom-count group: CTAs per run C (a thread-block cluster of
// C CTAs on C SMs holds the R walkers of a run, R/C per CTA) and lanes per
// walker L (32, or 16 with two walkers per warp); FP32 form.
// Coordinate descent on the whole batch's device time: starting from C = 1
// everywhere, each group in turn (largest N first) tries every C in
// {1, 2, 4, 8} x L in {32, 16} (R % C == 0, shared memory permitting) with
// the other groups fixed, and takes the best if it cuts the batch time of `trial_cycles`
// cycles by more than 2 %; at most 3 passes.  Every trial
// runs on a snapshot of the device state that is restored afterwards, so the
// chain continues as if no trial had run.  Results are cached by key (device
// name, potential, boundary, ensemble, R, the (N, runs) multiset) as JSON
// lines {"key": "...", "ncta": {"N": 100 C + L, ...}} (L = lanes per walker).
namespace {

std::string tune_key(ptmc_ctx* c) {
  cudaDeviceProp prop{};
  int dev = 0;
  cudaGetDevice(&dev);
  cudaGetDeviceProperties(&prop, dev);
  std::ostringstream k;
  k << prop.name << "|sm" << prop.multiProcessorCount << "|shape=100C+L|pot" << c->pot << "|bc" << c->bc()
    << "|ens" << c->p.ensemble << "|R" << c->R() << "|groups";
  for (auto& G : c->groups) k << ":" << G.N << "x" << G.nruns;
  return k.str();
}

bool tune_cache_read(const char* path, const std::string& key, std::map<int, int>& out) {
  if (!path) return false;
  std::ifstream f(path);
  if (!f) return false;
  std::string line, want = "{\"key\": \"" + key + "\"";
  while (std::getline(f, line)) {
    if (line.compare(0, want.size(), want) != 0) continue;
    size_t at = line.find("\"ncta\": {");
    if (at == std::string::npos) continue;
    out.clear();
    const char* p = line.c_str() + at + 9;
    int n = 0, v = 0, used = 0;
    while (std::sscanf(p, " \"%d\": %d%n", &n, &v, &used) == 2) {
      out[n] = v;
      p += used;
      while (*p == ',' || *p == ' ') ++p;
    }
    return !out.empty();
  }
  return false;
}

void tune_cache_write(const char* path, const std::string& key, const std::map<int, int>& m) {
  if (!path) return;
  std::ofstream f(path, std::ios::app);
  if (!f) return;
  f << "{\"key\": \"" << key << "\", \"ncta\": {";
  bool first = true;
  for (auto& kv : m) {
    f << (first ? "" : ", ") << "\"" << kv.first << "\": " << kv.second;
    first = false;
  }
  f << "}}\n";
}

struct Snapshot {
  std::vector<std::pair<void*, std::vector<unsigned char>>> bufs;  // device ptr, host copy
};

template <typename T>
int snap_one(ptmc_ctx* c, Snapshot& s, DBuf<T>& d) {
  if (!d.p || d.n == 0) return PTMC_OK;
  std::vector<unsigned char> h(d.n * sizeof(T));
  CK(cudaMemcpyAsync(h.data(), d.p, h.size(), cudaMemcpyDeviceToHost, c->st));
  s.bufs.emplace_back((void*)d.p, std::move(h));
  return PTMC_OK;
}

int snapshot(ptmc_ctx* c, Snapshot& s) {
  int rc = 0;
  rc |= snap_one(c, s, c->d_runs);
  for (auto* b : {&c->d_pos, &c->d_mat, &c->d_comp, &c->d_en, &c->d_box, &c->d_rc2, &c->d_drift,
                  &c->d_beta, &c->d_maxd, &c->d_maxbox, &c->d_ham, &c->d_boxh, &c->d_maxboxh,
                  &c->d_maxd_sep})
    rc |= snap_one(c, s, *b);
  rc |= snap_one(c, s, c->d_cnt_sep);
  rc |= snap_one(c, s, c->d_tan);
  rc |= snap_one(c, s, c->d_ctr);
  rc |= snap_one(c, s, c->d_status);
  rc |= snap_one(c, s, c->d_wos);
  rc |= snap_one(c, s, c->d_cnt);
  rc |= snap_one(c, s, c->d_hist);
  if (rc) return PTMC_ERR_CUDA;
  CK(cudaStreamSynchronize(c->st));
  return PTMC_OK;
}

int restore_snapshot(ptmc_ctx* c, const Snapshot& s) {
  for (auto& b : s.bufs)
    CK(cudaMemcpyAsync(b.first, b.second.data(), b.second.size(), cudaMemcpyHostToDevice, c->st));
  CK(cudaStreamSynchronize(c->st));
  return PTMC_OK;
}

}  // namespace

extern "C" int ptmc_autotune(ptmc_ctx* c, int trial_cycles, const char* cache_path,
                             int* shape_out) {
  if (!c) return PTMC_ERR_ARG;
  if (!c->inited) return c->fail(PTMC_ERR_STATE, "ptmc_init not called");
  if (trial_cycles < 1) return c->fail(PTMC_ERR_ARG, "trial_cycles must be >= 1");
  const int R = c->R();
  // shape code: 100 * CTAs per run + lanes per walker
  std::map<int, int> best;  // N -> shape code
  for (auto& G : c->groups) best[G.N] = 100 * G.ncta + G.lpr;
  auto apply = [&](const std::map<int, int>& m) {
    for (auto& G : c->groups) {
      G.ncta = m.at(G.N) / 100;
      G.lpr = m.at(G.N) % 100;
    }
    drop_graphs(c);
  };
  if (c->f32() && c->pot != POT_NN) {
    const std::string key = tune_key(c);
    std::map<int, int> cached;
    if (tune_cache_read(cache_path, key, cached) && cached.size() == best.size()) {
      best = cached;
    } else {
      int optin = 0, dev = 0;
      cudaGetDevice(&dev);
      cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
      Snapshot snap;
      int rc = snapshot(c, snap);
      if (rc) return rc;
      const ptmc_stats saved = c->stats;
      auto trial = [&](const std::map<int, int>& m, double& ms) -> int {
        apply(m);
        int r = run_phase(c, 2, PHASE_PLAIN);  // warm-up (attributes, first launch)
        if (!r) r = run_phase(c, trial_cycles, PHASE_PLAIN);
        ms = c->stats.last_cycles_ms;
        int r2 = restore_snapshot(c, snap);
        return r ? r : r2;
      };
      double t_best = 0;
      rc = trial(best, t_best);
      if (rc) return rc;
      std::vector<int> order;
      for (auto& kv : best) order.push_back(kv.first);
      std::sort(order.rbegin(), order.rend());  // largest N first
      // coordinate descent: every candidate shape of one group with the others
      // fixed (the batch time is not monotonic in the shape: co-residency of the
      // groups' CTAs on the SMs changes with it), at most 3 passes
      for (int pass = 0; pass < 3; ++pass) {
        bool improved = false;
        for (int N : order) {
          int pick = best[N];
          double t_pick = t_best;
          for (int cc : {1, 2, 4, 8})
            for (int ll : {32, 16, 8, 4}) {
              const int code = 100 * cc + ll;
              if (code == best[N] || R % cc != 0 || (R / cc) % (32 / ll) != 0) continue;
              if (R / cc * ll > 1024) continue;  // threads of a CTA
              if (ll <= 8 && (cc != 1 || c->p.ensemble != PTMC_NVT || R > 32)) continue;
              const long long smem = ll <= 8 ? cycles32n_smem_bytes(c->pot, R, N, ll)
                                             : cycles32_smem_bytes(c->pot, R, N, cc);
              if (smem > optin) continue;
              std::map<int, int> cand = best;
              cand[N] = code;
              double t = 0;
              rc = trial(cand, t);
              if (rc) {  // a shape the device cannot launch: skip it
                apply(best);
                cudaGetLastError();
                continue;
              }
              if (t < 0.98 * t_pick) {
                pick = code;
                t_pick = t;
              }
            }
          if (pick != best[N]) {
            best[N] = pick;
            t_best = t_pick;
            improved = true;
          }
        }
        if (!improved) break;
      }
      c->stats = saved;
      tune_cache_write(cache_path, key, best);
    }
  }
  apply(best);
  if (shape_out)
    for (int r = 0; r < c->p.n_runs; ++r) {
      shape_out[2 * r] = best[c->runs[r].N] / 100;
      shape_out[2 * r + 1] = best[c->runs[r].N] % 100;
    }
  return PTMC_OK;
}

extern "C" int ptmc_set_launch_shape(ptmc_ctx* c, int N, int ctas_per_run, int lanes_per_walker) {
  if (!c) return PTMC_ERR_ARG;
  if (!c->inited) return c->fail(PTMC_ERR_STATE, "ptmc_init not called");
  if (!c->f32() || c->pot == POT_NN)
    return c->fail(PTMC_ERR_ARG, "launch shapes apply to the FP32 form of the pair/EAM potentials");
  const int R = c->R();
  if (ctas_per_run < 1 || ctas_per_run > 8 || R % ctas_per_run != 0)
    return c->fail(PTMC_ERR_ARG, "ctas_per_run must divide the replica count and be <= 8");
  if (lanes_per_walker != 32 && lanes_per_walker != 16 && lanes_per_walker != 8 &&
      lanes_per_walker != 4)
    return c->fail(PTMC_ERR_ARG, "lanes_per_walker must be 32, 16, 8 or 4");
  if ((R / ctas_per_run) % (32 / lanes_per_walker) != 0)
    return c->fail(PTMC_ERR_ARG, "the walkers of a CTA must fill whole warps (R / C a multiple of "
                                 "32 / lanes_per_walker)");
  if (R / ctas_per_run * lanes_per_walker > 1024)
    return c->fail(PTMC_ERR_ARG, "a CTA holds at most 1024 threads (R / C * lanes_per_walker)");
  if (lanes_per_walker <= 8 && (ctas_per_run != 1 || c->p.ensemble != PTMC_NVT || R > 32))
    return c->fail(PTMC_ERR_ARG, "8 or 4 lanes per walker: NVT with one CTA of at most 32 "
                                 "walkers per run");
  int optin = 0, dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  bool found = false;
  for (auto& G : c->groups) {
    if (G.N != N) continue;
    const long long smem = lanes_per_walker <= 8 ? cycles32n_smem_bytes(c->pot, R, N, lanes_per_walker)
                                                 : cycles32_smem_bytes(c->pot, R, N, ctas_per_run);
    if (smem > optin) return c->fail(PTMC_ERR_LIMIT, "launch shape exceeds the shared memory of a CTA");
    G.ncta = ctas_per_run;
    G.lpr = lanes_per_walker;
    found = true;
  }
  if (!found) return c->fail(PTMC_ERR_ARG, "no run with that atom count");
  drop_graphs(c);
  return PTMC_OK;
}

extern "C" int ptmc_set_wait_test(ptmc_ctx* c, long long clocks, int never_set) {
  if (!c) return PTMC_ERR_ARG;
  if (clocks < 0) return c->fail(PTMC_ERR_ARG, "ptmc_set_wait_test: clocks must be >= 0");
  c->xwait_clocks = clocks == 0 ? XWAIT_CLOCKS : clocks;
  c->xwait_never = never_set ? 1 : 0;
  c->K.xwait_clocks = c->xwait_clocks;
  c->K.xwait_never = c->xwait_never;
  drop_graphs(c);  // captured launches hold the old kernel parameters
  return PTMC_OK;
}

extern "C" int ptmc_get_walker_status(ptmc_ctx* c, int run, int* status) {
  if (!c || !status) return PTMC_ERR_ARG;
  if (!c->inited) return c->fail(PTMC_ERR_STATE, "ptmc_init not called");
  if (run < 0 || run >= c->p.n_runs) return c->fail(PTMC_ERR_ARG, "run index out of range");
  const RunDesc& r = c->rd[c->dev_of_run[run]];
  CK(cudaMemcpyAsync(status, c->d_status.p + r.wk, sizeof(int) * c->R(), cudaMemcpyDeviceToHost, c->st));
  CK(cudaStreamSynchronize(c->st));
  return PTMC_OK;
}

extern "C" int ptmc_occupancy(ptmc_ctx* c, int N, int ctas_per_run, int lanes_per_walker,
                              int* ctas_per_sm) {
  if (!c || !ctas_per_sm) return PTMC_ERR_ARG;
  if (c->pot < 0) return c->fail(PTMC_ERR_STATE, "no potential set");
  if (c->pot == POT_NN || c->pot == POT_NN2 || pot_b(c->pot))
    return c->fail(PTMC_ERR_ARG, "ptmc_occupancy: pair and EAM potentials only");
  if (N < 2) return c->fail(PTMC_ERR_ARG, "ptmc_occupancy: N >= 2");
  const int bc = c->runs.empty() ? PTMC_BC_SPHERE : c->runs[0].bc;
  *ctas_per_sm = 0;
  // the plain form keeps the per-atom state in HBM when it exceeds a CTA's
  // shared memory: then only the tables (N = 0) are in shared memory
  const int Nq = cycles_smem_bytes(c->pot, c->p.ensemble, false, c->R(), N) > 227 * 1024 ? 0 : N;
  int e = c->f32() ? occupancy_cycles32(c->pot, bc, c->p.ensemble, c->R(), N, ctas_per_run,
                                        lanes_per_walker, ctas_per_sm)
                   : occupancy_cycles(c->pot, bc, c->p.ensemble, c->R(), Nq, ctas_per_sm);
  if (e < 0) return c->fail(PTMC_ERR_ARG, "ptmc_occupancy: no cycle kernel for this combination");
  if (e) return c->cuda_fail((cudaError_t)e, "ptmc_occupancy");
  return PTMC_OK;
}
