// ptmc_mhlin.cu — the linear-solve multihistogram on the GPU, FP64.
//
// multihistogram(output, Tvec) of src/multihist.jl: the histograms (interior
// bins, divided by n_bin) with the empty energy bins removed (processhist!,
// :89-114); the b vector (:166-210) and the A matrix (:215-232); alpha solving
// A alpha = b (systemsolver, :237-270); the entropy S(E) (Entropycalc,
// :275-283); and on `npoints` temperatures evenly spaced from T_1 (T_R - T_1)
// / npoints apart, the partition function with the reference's rescaling of
// the Boltzmann factors into [1, 100] (nexp steps of -1 / +0.7 carried from one
// temperature to the next), U, Cv, dCv and S(T) (analysis, :292-375).
//
// A is singular (its rows sum to zero and b is consistent), so the reference's
// A \ b returns alpha up to an additive constant chosen by LAPACK's rounding.
// Here the last equation is replaced by alpha[R-1] = 0 and the system is solved
// by Gaussian elimination with partial pivoting (rows eliminated in parallel).
// A constant in alpha shifts S(E) by a constant: U, Cv and dCv do not change; Z
// and S(T) change by the corresponding factor / offset.
//
// One CTA does everything (a few dozen replicas, a few hundred bins); every sum
// is taken in a fixed order so results are deterministic.  The rescaling loop
// is bounded: a status word reports when it does not settle.
#include <cuda_runtime.h>

#include <cmath>
#include <string>
#include <vector>

#include "../../include/ptmc_gb300.h"
#include "ptmc_engine.cuh"

namespace ptmc {

namespace {

constexpr int MH_THREADS = 256;
constexpr long long MH_RESCALE_LIMIT = 10000000;

struct MhScratch {  // device arrays, sizes in elements
  double* H;     // [R][n_bin] normalised histograms, then compacted [R][B]
  double* nsum;  // [n_bin]
  double* ev;    // [n_bin] energies of the kept bins
  double* bmat;  // [R][n_bin]
  double* rh;    // [n_bin]
  double* A;     // [R][R]
  double* b;     // [R]
  double* S;     // [n_bin]
  double* part;  // [MH_THREADS]
  int* keep;     // [n_bin]
};

// sum of v over the CTA in a fixed order (per-thread partials, then thread 0)
__device__ double fixed_sum(double v, double* part, double* out) {
  part[threadIdx.x] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int k = 0; k < blockDim.x; ++k) t += part[k];
    *out = t;
  }
  __syncthreads();
  return *out;
}

__global__ void __launch_bounds__(MH_THREADS)
    k_mhlin(int R, int n_bin, const double* __restrict__ hist, const double* __restrict__ beta,
            double en_min, double en_max, int npoints, MhScratch w, double* energies,
            double* S_E, int* n_kept, double* alpha, double* T_out, double* Z_out, double* U_out,
            double* Cv_out, double* dCv_out, double* ST_out, int* status) {
  __shared__ double s_red[4];
  __shared__ int s_B, s_flag;
  __shared__ double s_nexp;
  const int tid = threadIdx.x, nt = blockDim.x;
  const double kB = 3.16681196E-6;  // multihist.jl:57
  const int nb = n_bin + 2;
  const double de = (en_max - en_min) / (n_bin - 1);
  // readfile + processhist!: interior bins / n_bin, bin sums in replica order
  for (int t = tid; t < R * n_bin; t += nt) {
    const int i = t / n_bin, j = t % n_bin;
    w.H[t] = hist[(size_t)i * nb + j + 1] / n_bin;
  }
  __syncthreads();
  for (int j = tid; j < n_bin; j += nt) {
    double s = 0.0;
    for (int i = 0; i < R; ++i) s += w.H[(size_t)i * n_bin + j];
    w.nsum[j] = s;
  }
  __syncthreads();
  if (tid == 0) {  // keep the non-empty bins in order
    int B = 0;
    for (int j = 0; j < n_bin; ++j)
      if (w.nsum[j] != 0.0) w.keep[B++] = j;
    s_B = B;
    *status = B == 0 ? 1 : 0;
  }
  __syncthreads();
  const int B = s_B;
  if (B == 0) return;
  // compacted copies (bmat doubles as the staging buffer of H's kept columns)
  for (int t = tid; t < R * B; t += nt) {
    const int i = t / B, k = t % B;
    w.bmat[t] = w.H[(size_t)i * n_bin + w.keep[k]];
  }
  for (int k = tid; k < B; k += nt) {
    w.ev[k] = __dadd_rn(__dmul_rn((double)w.keep[k], de), en_min);  // (j-1) de + emin, unfused
    w.S[k] = w.nsum[w.keep[k]];  // staged nsum
  }
  __syncthreads();
  for (int t = tid; t < R * B; t += nt) w.H[t] = w.bmat[t];
  for (int k = tid; k < B; k += nt) w.nsum[k] = w.S[k];
  __syncthreads();
  // bvector: bmat = n (ln n + beta E) (0 where n = 0), rh_k = sum_i bmat_ik,
  // b_i = sum_k (bmat_ik - n_ik rh_k / nsum_k)
  for (int t = tid; t < R * B; t += nt) {
    const int i = t / B, k = t % B;
    const double x = w.H[t];
    w.bmat[t] = x == 0.0 ? 0.0 : x * (log(x) + beta[i] * w.ev[k]);
  }
  __syncthreads();
  for (int k = tid; k < B; k += nt) {
    double s = 0.0;
    for (int i = 0; i < R; ++i) s += w.bmat[(size_t)i * B + k];
    w.rh[k] = s;
  }
  __syncthreads();
  for (int i = tid; i < R; i += nt) {
    double s = 0.0;
    for (int k = 0; k < B; ++k) s += w.bmat[(size_t)i * B + k] - w.H[(size_t)i * B + k] * w.rh[k] / w.nsum[k];
    w.b[i] = s;
  }
  // amatrix: A_ii' = -sum_k n_ik n_i'k / nsum_k (+ sum_k n_ik on the diagonal)
  for (int t = tid; t < R * R; t += nt) {
    const int i = t / R, ip = t % R;
    double s = 0.0;
    for (int k = 0; k < B; ++k) s += w.H[(size_t)i * B + k] * w.H[(size_t)ip * B + k] / w.nsum[k];
    double a = -s;
    if (i == ip) {
      double d = 0.0;
      for (int k = 0; k < B; ++k) d += w.H[(size_t)i * B + k];
      a += d;
    }
    w.A[t] = a;
  }
  __syncthreads();
  // gauge alpha[R-1] = 0 in place of the dependent last equation
  for (int ip = tid; ip < R; ip += nt) w.A[(size_t)(R - 1) * R + ip] = ip == R - 1 ? 1.0 : 0.0;
  if (tid == 0) w.b[R - 1] = 0.0;
  __syncthreads();
  for (int col = 0; col < R; ++col) {  // Gaussian elimination, partial pivoting
    if (tid == 0) {
      int piv = col;
      for (int r = col + 1; r < R; ++r)
        if (fabs(w.A[(size_t)r * R + col]) > fabs(w.A[(size_t)piv * R + col])) piv = r;
      s_flag = w.A[(size_t)piv * R + col] == 0.0;
      if (!s_flag && piv != col) {
        for (int c = 0; c < R; ++c) {
          const double tmp = w.A[(size_t)piv * R + c];
          w.A[(size_t)piv * R + c] = w.A[(size_t)col * R + c];
          w.A[(size_t)col * R + c] = tmp;
        }
        const double tb = w.b[piv];
        w.b[piv] = w.b[col];
        w.b[col] = tb;
      }
    }
    __syncthreads();
    if (s_flag) {
      if (tid == 0) *status = 2;
      return;
    }
    for (int r = col + 1 + tid; r < R; r += nt) {
      const double f = w.A[(size_t)r * R + col] / w.A[(size_t)col * R + col];
      for (int c = col; c < R; ++c) w.A[(size_t)r * R + c] -= f * w.A[(size_t)col * R + c];
      w.b[r] -= f * w.b[col];
    }
    __syncthreads();
  }
  if (tid == 0)
    for (int r = R - 1; r >= 0; --r) {
      double t = w.b[r];
      for (int c = r + 1; c < R; ++c) t -= w.A[(size_t)r * R + c] * w.b[c];
      w.b[r] = t / w.A[(size_t)r * R + r];
    }
  __syncthreads();
  // Entropycalc: S_k = (sum_i bmat_ik - n_ik alpha_i) / nsum_k
  for (int k = tid; k < B; k += nt) {
    double t = 0.0;
    for (int i = 0; i < R; ++i) t += w.bmat[(size_t)i * B + k] - w.H[(size_t)i * B + k] * w.b[i];
    w.S[k] = t / w.nsum[k];
  }
  if (tid == 0) s_nexp = 0.0;
  __syncthreads();
  // analysis
  const double T0 = 1 / (kB * beta[0]), T1 = 1 / (kB * beta[R - 1]);
  const double dT = (T1 - T0) / npoints;
  for (int p = 0; p < npoints; ++p) {
    const double T = __dadd_rn(__dmul_rn((double)p, dT), T0);
    double z = 0.0;
    for (long long guard = 0;; ++guard) {
      const double nexp = s_nexp;
      double v = 0.0;
      for (int k = tid; k < B; k += nt) v += exp((w.S[k] - w.ev[k] / (T * kB)) - nexp);
      z = fixed_sum(v, w.part, &s_red[0]);
      if (tid == 0) {
        s_flag = 0;
        if (guard > MH_RESCALE_LIMIT) s_flag = 2;
        else if (z < 1.0) s_nexp = nexp - 1.0, s_flag = 1;
        else if (z > 100.0) s_nexp = nexp + 0.7, s_flag = 1;
      }
      __syncthreads();
      const int f = s_flag;
      __syncthreads();
      if (f == 2) {
        if (tid == 0) *status = 3;
        return;
      }
      if (f == 0) break;
    }
    const double nexp = s_nexp;
    double a1 = 0.0, a2 = 0.0;
    for (int k = tid; k < B; k += nt) {
      const double xp = exp((w.S[k] - w.ev[k] / (T * kB)) - nexp);
      a1 += xp * w.ev[k];
      a2 += xp * w.ev[k] * w.ev[k];
    }
    const double u = fixed_sum(a1, w.part, &s_red[1]) / z;
    const double u2 = fixed_sum(a2, w.part, &s_red[2]) / z;
    double q2 = 0.0, q3 = 0.0;
    for (int k = tid; k < B; k += nt) {
      const double xp = exp((w.S[k] - w.ev[k] / (T * kB)) - nexp);
      const double d = w.ev[k] - u;
      q2 += xp * d * d;
      q3 += xp * d * d * d;
    }
    const double r2 = fixed_sum(q2, w.part, &s_red[3]) / z;
    const double r3 = fixed_sum(q3, w.part, &s_red[3]) / z;
    if (tid == 0) {
      T_out[p] = T;
      Z_out[p] = z;
      U_out[p] = u;
      Cv_out[p] = (u2 - u * u) / kB / (T * T);
      ST_out[p] = u / T + kB * log(z);
      dCv_out[p] = r3 / (kB * kB) / (T * T * T * T) - 2 * r2 / kB / (T * T * T);
    }
  }
  for (int k = tid; k < B; k += nt) {
    energies[k] = w.ev[k];
    S_E[k] = w.S[k];
  }
  for (int i = tid; i < R; i += nt) alpha[i] = w.b[i];
  if (tid == 0) *n_kept = B;
}

}  // namespace
}  // namespace ptmc

extern "C" int ptmc_multihist_linear(int R, int n_bin, const double* en_hist, const double* beta,
                                     double en_min, double en_max, int npoints, double* energies,
                                     double* S_E, int* n_kept, double* alpha, double* T_out,
                                     double* Z, double* U, double* Cv, double* dCv,
                                     double* S_T) {
  using namespace ptmc;
  if (R < 2 || R > 1024 || n_bin < 2 || npoints < 1 || !en_hist || !beta || !energies || !S_E ||
      !n_kept || !alpha || !T_out || !Z || !U || !Cv || !dCv || !S_T) {
    set_last_error("multihistogram (linear): bad arguments");
    return PTMC_ERR_ARG;
  }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    set_last_error("multihistogram (linear): no CUDA device");
    return PTMC_ERR_CUDA;
  }
  const size_t nbt = (size_t)n_bin, nb = (size_t)n_bin + 2;
  // one device block: inputs, scratch, outputs
  const size_t nd = (size_t)R * nb + R                                   // hist, beta
                    + 2 * (size_t)R * nbt + 4 * nbt + (size_t)R * R + R + MH_THREADS  // scratch
                    + 2 * nbt + R + 6 * (size_t)npoints;                  // outputs
  double* d = nullptr;
  int* di = nullptr;
  if (cudaMalloc(&d, sizeof(double) * nd) != cudaSuccess) {
    set_last_error("multihistogram (linear): device allocation failed");
    return PTMC_ERR_CUDA;
  }
  if (cudaMalloc(&di, sizeof(int) * (nbt + 2)) != cudaSuccess) {
    cudaFree(d);
    set_last_error("multihistogram (linear): device allocation failed");
    return PTMC_ERR_CUDA;
  }
  double* p = d;
  auto take = [&](size_t n) {
    double* q = p;
    p += n;
    return q;
  };
  double* d_hist = take((size_t)R * nb);
  double* d_beta = take(R);
  MhScratch w;
  w.H = take((size_t)R * nbt);
  w.bmat = take((size_t)R * nbt);
  w.nsum = take(nbt);
  w.ev = take(nbt);
  w.rh = take(nbt);
  w.S = take(nbt);
  w.A = take((size_t)R * R);
  w.b = take(R);
  w.part = take(MH_THREADS);
  w.keep = di;
  int* d_nk = di + nbt;
  int* d_status = di + nbt + 1;
  double* o_E = take(nbt);
  double* o_S = take(nbt);
  double* o_alpha = take(R);
  double* o_T = take(npoints);
  double* o_Z = take(npoints);
  double* o_U = take(npoints);
  double* o_Cv = take(npoints);
  double* o_dCv = take(npoints);
  double* o_ST = take(npoints);
  cudaError_t e = cudaMemcpy(d_hist, en_hist, sizeof(double) * R * nb, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(d_beta, beta, sizeof(double) * R, cudaMemcpyHostToDevice);
  int status = 0, nk = 0;
  if (e == cudaSuccess) {
    k_mhlin<<<1, MH_THREADS>>>(R, n_bin, d_hist, d_beta, en_min, en_max, npoints, w, o_E, o_S, d_nk,
                               o_alpha, o_T, o_Z, o_U, o_Cv, o_dCv, o_ST, d_status);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(&status, d_status, sizeof(int), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && status == 0) {
    e = cudaMemcpy(&nk, d_nk, sizeof(int), cudaMemcpyDeviceToHost);
    auto cp = [&](double* dst, const double* src, size_t n) {
      if (e == cudaSuccess) e = cudaMemcpy(dst, src, sizeof(double) * n, cudaMemcpyDeviceToHost);
    };
    cp(energies, o_E, nk);
    cp(S_E, o_S, nk);
    cp(alpha, o_alpha, R);
    cp(T_out, o_T, npoints);
    cp(Z, o_Z, npoints);
    cp(U, o_U, npoints);
    cp(Cv, o_Cv, npoints);
    cp(dCv, o_dCv, npoints);
    cp(S_T, o_ST, npoints);
  }
  cudaFree(d);
  cudaFree(di);
  if (e != cudaSuccess) {
    set_last_error(std::string("multihistogram (linear): ") + cudaGetErrorString(e));
    return PTMC_ERR_CUDA;
  }
  if (status == 1) {
    set_last_error("multihistogram (linear): every histogram bin is empty");
    return PTMC_ERR_ARG;
  }
  if (status == 2) {
    set_last_error("multihistogram (linear): singular system");
    return PTMC_ERR_ARG;
  }
  if (status == 3) {
    set_last_error("multihistogram (linear): partition-function rescaling did not settle");
    return PTMC_ERR_LIMIT;
  }
  *n_kept = nk;
  return PTMC_OK;
}
