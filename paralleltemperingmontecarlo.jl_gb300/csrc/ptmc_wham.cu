// ptmc_wham.cu — multihistogram reweighting (WHAM) on the GPU, FP64.
//
// multihistogram_NVT (src/multihist_NVT.jl:95-221) and multihistogram_NPT
// (src/multihist_NPT.jl:113-338) iterate free energies f_i over R replica
// histograms until sum_i (f_i' - f_i)^2 < thr (at most 1000 iterations), then
// reweight to 10R temperatures.  The reference evaluates quasiprob(beta, m)
// (multihist_NVT.jl:59-85) afresh for every (beta, m), an O(R) loop each; the
// offset and denominator of a bin do not depend on the target beta, so here
// one pass over the bins computes, per bin, w_m = num_m / den_m and off_m with
// the reference's arithmetic, and every quasiprob becomes
// w_m * exp(-beta * X_m - off_m) (X = E for NVT, E + pV for NPT).  This turns
// O(R^2 B) exp per iteration into O(R B) + O(R B) and keeps the whole
// iteration inside one CTA (no host round trips, no spin-waits: the loop is
// bounded by 1000 iterations and every barrier is a __syncthreads).
//
// Energy origin: the iteration first runs with the reference's arithmetic
// (absolute energies).  The per-bin offset is set by the replica with the
// largest -beta_i X - f_i, so with large |E| (Cu55 EAM: E ~ -9 Eh, beta up to
// 1580 / Eh) the other replicas' terms exp(-(beta_j - beta_1) X) underflow to
// zero in the first iteration, their f_j become -inf and every Cv is NaN (on
// the CPU restatement as in the reference).  When the iteration ends with a
// non-finite free energy, it is repeated with energies measured from en_min
// (X = E - en_min (+ pV)); Cv/Cp are unchanged by a constant shift of the
// energy (the free energies absorb -beta_i * shift), and |beta X| then stays
// below beta * (en_max - en_min).  Cases the reference handles keep its exact
// iteration.
//
// Scratch (caller-provided device memory, wham_work_doubles() doubles):
//   f[R], nf[R], nc[R], num[B], w[B], off[B], red[2] where B = n_bin (NVT) or
//   n_bin^2 (NPT).
#include <cuda_runtime.h>

#include "ptmc_device.cuh"
#include "ptmc_engine.cuh"

namespace ptmc {

constexpr int WHAM_THREADS = 1024;

long long wham_work_doubles(int R, int n_bins_total) {
  return 3LL * R + 3LL * n_bins_total + 2;
}

// bin m (0-based over the n_bin interior bins, or n_bin^2 for NPT)
struct BinGeo {
  int npt, n_bin;
  double en_min, dE, v_min, dV, p;
  __device__ __forceinline__ double X(int m) const {
    if (!npt) return en_min + ((m + 1) - 0.5) * dE;  // energy_t (:70)
    int a = m / n_bin, b = m % n_bin;
    double E = en_min + ((a + 1) - 0.5) * dE;
    double V = v_min + ((b + 1) - 0.5) * dV;
    return E + p * V;                                // multihist_NPT.jl:79-99
  }
  __device__ __forceinline__ double E(int m) const {
    int a = npt ? m / n_bin : m;
    return en_min + ((a + 1) - 0.5) * dE;
  }
  __device__ __forceinline__ long long hidx(int i, int m) const {  // hist[i][m+1](, [n+1])
    long long nb = n_bin + 2;
    if (!npt) return (long long)i * nb + (m + 1);
    int a = m / n_bin, b = m % n_bin;
    return ((long long)i * nb + (a + 1)) * nb + (b + 1);
  }
};

__device__ void bin_pass(const BinGeo& G, int R, int B, const double* hist,
                         const double* beta, const double* f, const double* nc,
                         const double* num, double* w, double* off) {
  for (int m = threadIdx.x; m < B; m += blockDim.x) {
    double X = G.X(m);
    double o = -1e6;  // offset (:73-77)
    for (int i = 0; i < R; ++i) o = fmax(o, -beta[i] * X - f[i]);
    o = o + log(1000.0);
    double den = 0.0;
    for (int i = 0; i < R; ++i) den = den + nc[i] * exp(-beta[i] * X - f[i] - o);
    w[m] = num[m] / den;
    off[m] = o;
  }
}

// sum_m w_m exp(-bt X_m - off_m) by one warp
__device__ double warp_qsum(const BinGeo& G, int B, double bt, const double* w,
                            const double* off, int lane) {
  double s = 0.0;
  for (int m = lane; m < B; m += 32)
    if (w[m] != 0.0) s += w[m] * exp(-bt * G.X(m) - off[m]);
  return warp_sum(s);
}

__global__ void __launch_bounds__(WHAM_THREADS)
    k_wham(BinGeo G0, int R, const double* hist, const double* beta, double thr,
           const double* tb_out, int n_out, double* work, double* out,
           int* iters) {
  BinGeo G = G0;
  const int B = G.npt ? G.n_bin * G.n_bin : G.n_bin;
  double* f = work;
  double* nf = f + R;
  double* nc = nf + R;
  double* num = nc + R;
  double* w = num + B;
  double* off = w + B;
  __shared__ int s_stop, s_finite;
  const int tid = threadIdx.x, wid = tid >> 5, lane = tid & 31;
  const int nw = blockDim.x >> 5;
  int it = 0;
  for (int attempt = 0; attempt < 2; ++attempt) {
    if (attempt == 1) G.en_min = 0.0;  // energies measured from en_min
    // free_energy_initialise (:37-57): f = 0, ncycles_i = sum of interior bins
    for (int i = tid; i < R; i += blockDim.x) {
      f[i] = 0.0;
      double s = 0.0;
      for (int m = 0; m < B; ++m) s = s + hist[G.hidx(i, m)];
      nc[i] = s;
    }
    for (int m = tid; m < B; m += blockDim.x) {  // sum_i n_im, order i = 1..R
      double q = 0.0;
      for (int i = 0; i < R; ++i) q = q + hist[G.hidx(i, m)];
      num[m] = q;
    }
    __syncthreads();
    for (it = 1; it <= 1000; ++it) {
      bin_pass(G, R, B, hist, beta, f, nc, num, w, off);
      __syncthreads();
      for (int i = wid; i < R; i += nw) {
        double s = warp_qsum(G, B, beta[i], w, off, lane);
        if (lane == 0) nf[i] = log(s);
      }
      __syncthreads();
      if (tid == 0) {
        double delta = 0.0;
        for (int i = 0; i < R; ++i) {
          double d = fabs(nf[i] - f[i]);
          delta = delta + d * d;
          f[i] = nf[i];
        }
        s_stop = delta < thr;
      }
      __syncthreads();
      if (s_stop) break;
    }
    if (tid == 0) {
      int ok = 1;
      for (int i = 0; i < R; ++i) ok &= isfinite(f[i]) ? 1 : 0;
      s_finite = ok;
    }
    __syncthreads();
    if (s_finite) break;
  }
  // reweighting with the final free energies (:158-216)
  bin_pass(G, R, B, hist, beta, f, nc, num, w, off);
  __syncthreads();
  for (int t = wid; t < n_out; t += nw) {
    double bt = tb_out[t], T = tb_out[n_out + t];
    double norm = warp_qsum(G, B, bt, w, off, lane);
    double e1 = 0.0, e2 = 0.0;
    for (int m = lane; m < B; m += 32) {
      if (w[m] == 0.0) continue;
      double q = w[m] * exp(-bt * G.X(m) - off[m]) / norm;
      double x = G.X(m);  // NVT: E, NPT: enthalpy E + pV
      e1 += q * x;
      e2 += q * (x * x);
    }
    e1 = warp_sum(e1);
    e2 = warp_sum(e2);
    if (lane == 0) out[t] = (e2 - e1 * e1) / ((3.166811429 / 1e6) * (T * T));
  }
  if (tid == 0) *iters = it > 1000 ? 1000 : it;
}

static int wham_launch(const BinGeo& G, int R, const double* d_hist,
                       const double* d_beta, double thr, const double* d_tb,
                       int n_out, double* d_work, double* d_out, int* d_iters,
                       void* stream) {
  k_wham<<<1, WHAM_THREADS, 0, (cudaStream_t)stream>>>(G, R, d_hist, d_beta, thr, d_tb,
                                                        n_out, d_work, d_out, d_iters);
  return (int)cudaGetLastError();
}

int wham_nvt_device(int R, int n_bin, const double* d_hist, const double* d_beta,
                    double en_min, double en_max, double thr,
                    const double* d_tb, int n_out, double* d_work,
                    double* d_out, int* d_iters, void* stream) {
  BinGeo G{0, n_bin, en_min, (en_max - en_min) / n_bin, 0.0, 0.0, 0.0};
  return wham_launch(G, R, d_hist, d_beta, thr, d_tb, n_out, d_work, d_out, d_iters, stream);
}

int wham_npt_device(int R, int n_bin, const double* d_hist, const double* d_beta,
                    double en_min, double en_max, double v_min, double v_max,
                    double p, double thr, const double* d_tb, int n_out,
                    double* d_work, double* d_out, int* d_iters, void* stream) {
  BinGeo G{1, n_bin, en_min, (en_max - en_min) / n_bin, v_min, (v_max - v_min) / n_bin, p};
  return wham_launch(G, R, d_hist, d_beta, thr, d_tb, n_out, d_work, d_out, d_iters, stream);
}

}  // namespace ptmc
