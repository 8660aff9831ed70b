// ptmc_noalloc.cu — an allocation-free variant of the NVT multihistogram entry
// point, for callers that cannot allocate device memory themselves.
//
// ptmc_multihist_nvt() allocates its device buffers with cudaMalloc.  Some
// callers must not do that: a Julia program whose GPU memory is owned by
// CUDA.jl's pool (a foreign cudaMalloc bypasses the pool's accounting and can
// fail once the pool has taken the free memory), code that enqueues work
// inside a stream capture (where cudaMalloc is not a legal call), or a service
// that pre-reserves all device memory at start-up.  Such a caller passes its
// own device buffers for the inputs and outputs; the per-call scratch of the
// WHAM iteration lives in a fixed file-scope __device__ array instead.
//
// Limits and sharing: the scratch array holds PTMC_NOALLOC_SCRATCH_DOUBLES
// doubles (each GPU that loads the library keeps it until the process exits);
// sizes that need more are rejected with PTMC_ERR_LIMIT.  Every call uses the
// same array and the array keeps the previous call's contents, so the kernels
// initialise everything they read, and two calls that run at the same time on
// the GPU (for example on different streams) race on it.
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>
#include <string>

#include "../../include/ptmc_gb300.h"
#include "ptmc_engine.cuh"

namespace {

constexpr int kMaxDevices = 64;
// the scratch of every call: f, nf, nc (R each), num, w, off (n_bin each),
// then the output grid (10R betas and 10R temperatures)
__device__ __align__(256) double g_wham_scratch[PTMC_NOALLOC_SCRATCH_DOUBLES];

std::mutex g_mu;
double* g_scratch_ptr[kMaxDevices] = {nullptr};

// Output temperature grid TempGrid{10R}(t_1, t_R) (src/multihist_NVT.jl:29-34),
// geometric, with kB of src/InputParams.jl:19.
__global__ void k_tgrid(const double* t_grid, int R, int n_out, double* tb, double* T_out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_out) return;
  double t0 = t_grid[0], t1 = t_grid[R - 1];
  double T = n_out == 1 ? t0 : t0 * pow(t1 / t0, (double)i / (double)(n_out - 1));
  tb[i] = 1.0 / (3.16681196E-6 * T);
  tb[n_out + i] = T;
  T_out[i] = T;
}

// every failure return names the entry point in the global last error
// (ptmc_last_error(NULL)), as the allocating entry points do
int fail(int code, const std::string& msg) {
  ptmc::set_last_error("ptmc_multihist_nvt_noalloc: " + msg);
  return code;
}

}  // namespace

extern "C" int ptmc_multihist_nvt_noalloc(int R, int n_bin, const double* d_hist,
                                          const double* d_t_grid, const double* d_beta,
                                          double en_min, double en_max, double thr,
                                          double* d_T_out, double* d_cv_out, int* d_iters,
                                          void* stream) {
  if (R < 1 || n_bin < 1 || !d_hist || !d_t_grid || !d_beta || !d_T_out || !d_cv_out || !d_iters)
    return fail(PTMC_ERR_ARG, "need R >= 1, n_bin >= 1 and non-null device buffers");
  const long long n_out = 10LL * R;
  const long long need = ptmc::wham_work_doubles(R, n_bin) + 2 * n_out;
  if (need > PTMC_NOALLOC_SCRATCH_DOUBLES)
    return fail(PTMC_ERR_LIMIT, "R = " + std::to_string(R) + ", n_bin = " + std::to_string(n_bin) +
                                    " need " + std::to_string(need) + " scratch doubles, the fixed array holds " +
                                    std::to_string(PTMC_NOALLOC_SCRATCH_DOUBLES));
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail(PTMC_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return fail(PTMC_ERR_CUDA, "device ordinal beyond 63");
  // An error left pending by an earlier launch of the caller's is reported,
  // not consumed: the launch checks below would otherwise read (and clear) it
  // as if this call had caused it.
  e = cudaPeekAtLastError();
  if (e != cudaSuccess)
    return fail(PTMC_ERR_CUDA, std::string("a CUDA error was pending before the call (left for the caller): ") +
                                   cudaGetErrorString(e));
  double* base;
  {
    // once per device, with that device current: the array's device address
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_scratch_ptr[dev]) {
      void* p = nullptr;
      e = cudaGetSymbolAddress(&p, g_wham_scratch);
      if (e != cudaSuccess || !p)
        return fail(PTMC_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
      g_scratch_ptr[dev] = (double*)p;
    }
    base = g_scratch_ptr[dev];
  }
  double* work = base;
  double* tb = base + ptmc::wham_work_doubles(R, n_bin);
  cudaStream_t st = (cudaStream_t)stream;
  k_tgrid<<<(int)((n_out + 127) / 128), 128, 0, st>>>(d_t_grid, R, (int)n_out, tb, d_T_out);
  e = cudaGetLastError();  // nothing was pending, so an error here is this launch's
  if (e != cudaSuccess) return fail(PTMC_ERR_CUDA, std::string("k_tgrid launch: ") + cudaGetErrorString(e));
  int rc = ptmc::wham_nvt_device(R, n_bin, d_hist, d_beta, en_min, en_max, thr, tb, (int)n_out,
                                 work, d_cv_out, d_iters, stream);
  if (rc != 0)
    return fail(PTMC_ERR_CUDA, std::string("k_wham launch: ") + cudaGetErrorString((cudaError_t)rc));
  return PTMC_OK;
}
