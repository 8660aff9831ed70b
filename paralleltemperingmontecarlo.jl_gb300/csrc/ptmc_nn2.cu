// ptmc_nn2.cu — the two-species RuNNer potential (RuNNerPotential2Atom) in
// the NNVT ensemble: atom moves and atom swaps, plain FP64 form.
//
// The reference (src/EnergyEvaluation.jl:1276-1448, MachineLearningPotential/
// SymmFunc.jl:326-541, DeltaMatrix.jl:256-635) keeps a symmetry matrix G of
// 2 nrad + 3 nang rows per atom: radial function k gives rows 2k and 2k+1 (the
// neighbour's species), angular function k rows 2 nrad + 3k + m with m the
// number of species-2 atoms among the centre's two neighbours; every row is
// scaled and offset by the centre's species.  Species-1 atoms (indices
// 0..n1-1) go through nnp1, the others through nnp2.
//
// Execution: one CTA per walker.  A move (atom displacement or swap of one
// atom of each species) rebuilds G of the trial configuration, each centre
// atom's columns summed by a fixed set of threads in a fixed order (so runs
// are deterministic); every triangle's term is formed from its sorted
// indices exactly as the reference's loops form it.  The state that outlives
// a launch is the positions and energies: the distance, cutoff and symmetry
// matrices are rebuilt from the positions when a launch starts.  Exchange,
// step adaptation and sampling run in the NN path's run epilogue.
#include <cuda_runtime.h>

#include "ptmc_device.cuh"
#include "ptmc_engine.cuh"
#include "ptmc_nn.cuh"
#include "ptmc_nn2.cuh"

namespace ptmc {

namespace {

constexpr int NN2_THREADS = 256;

struct Nn2Smem {
  double* X;     // [N*3] positions
  double* Xt;    // [N*3] trial positions
  double* D;     // [N*N] squared distances
  double* F;     // [N*N] cutoff values
  double* G;     // [Ng*N]
  double* Gt;    // [Ng*N] trial
  double* row;   // [N] trial distances of the moved atom
  double* frow;  // [N] trial cutoffs
  double* part;  // [NN2_THREADS * 3] partial sums
  double* ea;    // [N] atomic energies
  int* perm;     // [N] trial atom a sits where atom perm[a] sat (swaps)
  int* flags;    // [8]
  double* dd;    // [8]
};

__host__ __device__ size_t carve(Nn2Smem& s, unsigned char* base, int N, int Ng) {
  size_t off = 0;
  auto take = [&](size_t bytes) {
    unsigned char* p = base + off;
    off += (bytes + 15) / 16 * 16;
    return p;
  };
  s.X = (double*)take(8 * N * 3);
  s.Xt = (double*)take(8 * N * 3);
  s.D = (double*)take(8 * (size_t)N * N);
  s.F = (double*)take(8 * (size_t)N * N);
  s.G = (double*)take(8 * (size_t)Ng * N);
  s.Gt = (double*)take(8 * (size_t)Ng * N);
  s.row = (double*)take(8 * N);
  s.frow = (double*)take(8 * N);
  s.part = (double*)take(8 * NN2_THREADS * 3);
  s.ea = (double*)take(8 * N);
  s.perm = (int*)take(4 * N);
  s.flags = (int*)take(4 * 8);
  s.dd = (double*)take(8 * 8);
  return off;
}

// cutoff_function (MachineLearningPotential/Cutoff.jl:79-90)
__device__ __forceinline__ double cutoff2(double r, double rc) {
  return r < rc ? 0.5 * (cos(3.141592653589793 * (r / rc)) + 1) : 0.0;
}

// The symmetry matrix of a configuration given by accessors x(a) (positions),
// d(a,b), f(a,b).  Thread t sums centre a = t mod N over the neighbour pairs
// p = t / N, t / N + Q, ... (Q = threads / N); the partials of a centre are
// then added in slice order.
template <class XA, class DA, class FA>
__device__ void build_G(const NN2Params& Q, int N, XA x, DA d, FA f, double* G, double* part) {
  const int tid = threadIdx.x, nt = blockDim.x;
  const int n1 = Q.n1, nr = Q.nrad, na = Q.nang;
  const int QS = nt / N;                      // slices per centre
  const int a = tid % N, q = tid / N;
  const bool act = q < QS;
  for (int k = 0; k < nr; ++k) {
    const double* r = Q.rad + 10 * k;
    double s0 = 0.0, s1 = 0.0;
    if (act)
      for (int j = q; j < N; j += QS) {
        if (j == a) continue;
        const double fc = f(a, j);
        const double v = (fc != 0.0 && fc != 1.0) ? fc * exp(-r[0] * d(a, j)) : 0.0;
        if (j < n1) s0 += v;
        else s1 += v;
      }
    part[tid] = s0;
    part[nt + tid] = s1;
    __syncthreads();
    for (int c = tid; c < N; c += nt) {
      double t0 = 0.0, t1 = 0.0;
      for (int qq = 0; qq < QS; ++qq) {
        t0 += part[qq * N + c];
        t1 += part[nt + qq * N + c];
      }
      const int o = c < n1 ? 0 : 2;
      G[(size_t)(2 * k) * N + c] = t0 * r[6 + o] + r[2 + o];
      G[(size_t)(2 * k + 1) * N + c] = t1 * r[7 + o] + r[3 + o];
    }
    __syncthreads();
  }
  for (int k = 0; k < na; ++k) {
    const double* r = Q.ang + 16 * k;
    const double eta = r[0], lam = r[1], zeta = r[2];
    double s[3] = {0.0, 0.0, 0.0};
    if (act) {
      int p = 0;
      for (int j = 0; j < N; ++j) {
        if (j == a) continue;
        for (int l = j + 1; l < N; ++l) {
          if (l == a) continue;
          if (p++ % QS != q) continue;
          // the triangle in sorted order, as the reference's loops form it
          int lo = a, mi = j, hi = l;
          if (lo > mi) { int t = lo; lo = mi; mi = t; }
          if (mi > hi) { int t = mi; mi = hi; hi = t; }
          if (lo > mi) { int t = lo; lo = mi; mi = t; }
          const double rsum = (d(lo, mi) + d(lo, hi)) + d(mi, hi);
          const double e = exp(-eta * rsum) * f(lo, mi) * f(lo, hi) * f(mi, hi);
          // cos of the angle at a between a-j and a-l (Cutoff.jl:48-57)
          double v1[3], v2[3];
          for (int c = 0; c < 3; ++c) {
            v1[c] = x(a)[c] - x(j)[c];
            v2[c] = x(a)[c] - x(l)[c];
          }
          const double th = ((v1[0] * v2[0] + v1[1] * v2[1]) + v1[2] * v2[2]) /
                            (sqrt(d(a, j)) * sqrt(d(a, l)));
          const int m = (j >= n1) + (l >= n1);
          s[m] += e * pow(1.0 + lam * th, zeta);
        }
      }
    }
    part[tid] = s[0];
    part[nt + tid] = s[1];
    part[2 * nt + tid] = s[2];
    __syncthreads();
    for (int c = tid; c < N; c += nt) {
      const int o = c < n1 ? 0 : 3;
      for (int m = 0; m < 3; ++m) {
        double t = 0.0;
        for (int qq = 0; qq < QS; ++qq) t += part[m * nt + qq * N + c];
        G[(size_t)(2 * nr + 3 * k + m) * N + c] = t * r[4 + o + m] + r[10 + o + m];
      }
    }
    __syncthreads();
  }
}

// forward_pass of the species' network (two tanh hidden layers), one atom
// per thread, summed in atom order by thread 0
__device__ double mlp_energy2(const NN2Params& Q, int N, const double* G, double* ea) {
  const int Ng = 2 * Q.nrad + 3 * Q.nang, H1 = Q.H1, H2 = Q.H2;
  for (int a = threadIdx.x; a < N; a += blockDim.x) {
    const double* w = a < Q.n1 ? Q.W1 : Q.W2;
    const double* W1 = w;
    const double* b1 = W1 + (size_t)Ng * H1;
    const double* W2 = b1 + H1;
    const double* b2 = W2 + (size_t)H1 * H2;
    const double* w3 = b2 + H2;
    const double b3 = w3[H2];
    double h1[64], out = 0.0;
    for (int u = 0; u < H1; ++u) {
      double t = 0.0;
      for (int s = 0; s < Ng; ++s) t += G[(size_t)s * N + a] * W1[(size_t)s * H1 + u];
      h1[u] = tanh(t + b1[u]);
    }
    for (int v = 0; v < H2; ++v) {
      double t = 0.0;
      for (int u = 0; u < H1; ++u) t += h1[u] * W2[(size_t)u * H2 + v];
      out += tanh(t + b2[v]) * w3[v];
    }
    ea[a] = out + b3;
  }
  __syncthreads();
  __shared__ double tot;
  if (threadIdx.x == 0) {
    double e = 0.0;
    for (int a = 0; a < N; ++a) e += ea[a];
    tot = e;
  }
  __syncthreads();
  return tot;
}

// distances and cutoffs of the current positions (get_distance2_mat, f_matrix)
__device__ void build_DF(const NN2Params& Q, int N, const double* X, double* D, double* F) {
  for (int p = threadIdx.x; p < N * N; p += blockDim.x) {
    const int a = p / N, b = p % N;
    const int lo = a < b ? a : b, hi = a < b ? b : a;
    const double v = a == b ? 0.0
                            : d2_sph(X[3 * lo], X[3 * lo + 1], X[3 * lo + 2], X[3 * hi],
                                     X[3 * hi + 1], X[3 * hi + 2]);
    D[p] = v;
    F[p] = cutoff2(sqrt(v), Q.rcut);
  }
  __syncthreads();
}

__global__ void __launch_bounds__(NN2_THREADS) k_nn2_init(KParams P, NN2Params Q) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int gw = blockIdx.x;
  const RunDesc* rd = P.runs + Q.run_of_walker[gw];
  const int N = rd->N, w = gw - rd->wk, g = rd->wk + w;
  const int Ng = 2 * Q.nrad + 3 * Q.nang;
  Nn2Smem s;
  carve(s, smem_raw, N, Ng);
  const double* Xg = P.pos + rd->pos_off + (size_t)w * N * 3;
  for (int k = threadIdx.x; k < N * 3; k += blockDim.x) s.X[k] = Xg[k];
  __syncthreads();
  build_DF(Q, N, s.X, s.D, s.F);
  build_G(Q, N, [&](int a) { return s.X + 3 * a; }, [&](int a, int b) { return s.D[a * N + b]; },
          [&](int a, int b) { return s.F[a * N + b]; }, s.G, s.part);
  const double e = mlp_energy2(Q, N, s.G, s.ea);
  if (threadIdx.x == 0) {
    P.en[g] = e;
    P.status[g] = ST_OK;
    P.drift[g] = 0.0;
  }
}

// one cycle (N + n_swaps moves, mc_step!) of every walker
__global__ void __launch_bounds__(NN2_THREADS) k_nn2_cycle(KParams P, NN2Params Q) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int gw = blockIdx.x;
  const RunDesc* rd = P.runs + Q.run_of_walker[gw];
  const int N = rd->N, w = gw - rd->wk, g = rd->wk + w;
  const int tid = threadIdx.x;
  const int Ng = 2 * Q.nrad + 3 * Q.nang, n1 = Q.n1;
  if (P.status[g] != ST_OK) return;
  Nn2Smem s;
  carve(s, smem_raw, N, Ng);
  double* Xg = P.pos + rd->pos_off + (size_t)w * N * 3;
  for (int k = tid; k < N * 3; k += blockDim.x) s.X[k] = Xg[k];
  __syncthreads();
  build_DF(Q, N, s.X, s.D, s.F);
  build_G(Q, N, [&](int a) { return s.X + 3 * a; }, [&](int a, int b) { return s.D[a * N + b]; },
          [&](int a, int b) { return s.F[a * N + b]; }, s.G, s.part);
  const int slot = Q.sow[g];
  const int gs = rd->wk + slot;
  const double beta = P.beta[gs];
  const double md = P.maxd[2 * gs];
  const double R2 = P.box[g] * P.box[g];
  double en = P.en[g];
  unsigned long long ctr = P.ctr[g];  // thread 0's copy is the one that counts
  const uint32_t run_word = (uint32_t)rd->run_id;
  auto draw = [&]() -> double { return philox_u01(P.seed, (uint32_t)w, run_word, ctr++); };
  long long acc = 0, swaps = 0;
  int status = ST_OK;
  const int n_steps = N + Q.n_swaps;
  for (int step = 0; step < n_steps; ++step) {
    // ---- 1. the move (thread 0 draws): atom displacement with the sphere's
    // retry loop (src/MCMoves.jl:115-143), or a swap (src/MCMoves.jl:363-370)
    if (tid == 0) {
      const int k = randint(draw(), n_steps);
      s.flags[0] = k;
      s.flags[1] = 0;  // error
      if (k < N) {
        const int i = k;
        double xi = s.X[3 * i], yi = s.X[3 * i + 1], zi = s.X[3 * i + 2];
        double tx, ty, tz;
        auto propose = [&]() {
          double ux = draw(), uy = draw(), uz = draw();
          tx = dadd(xi, dmul(dsub(ux, 0.5), md));
          ty = dadd(yi, dmul(dsub(uy, 0.5), md));
          tz = dadd(zi, dmul(dsub(uz, 0.5), md));
        };
        propose();
        int count = 0;
        while (dot3(tx, ty, tz) > R2) {
          ++count;
          if (count == 50) {  // recentre! (src/Configurations.jl:79-85)
            double cx = 0, cy = 0, cz = 0;
            for (int a = 0; a < N; ++a) {
              cx += s.X[3 * a];
              cy += s.X[3 * a + 1];
              cz += s.X[3 * a + 2];
            }
            cx /= N;
            cy /= N;
            cz /= N;
            for (int a = 0; a < N; ++a) {
              s.X[3 * a] -= cx;
              s.X[3 * a + 1] -= cy;
              s.X[3 * a + 2] -= cz;
            }
            xi = s.X[3 * i];
            yi = s.X[3 * i + 1];
            zi = s.X[3 * i + 2];
          } else {
            propose();
            if (count == 100) {
              s.flags[1] = 1;
              break;
            }
          }
        }
        s.dd[0] = tx;
        s.dd[1] = ty;
        s.dd[2] = tz;
      } else {
        s.flags[2] = randint(draw(), n1);
        s.flags[3] = n1 + randint(draw(), N - n1);
      }
    }
    __syncthreads();
    if (s.flags[1]) {
      status = ST_SPHERE;
      break;
    }
    const int k = s.flags[0];
    const bool is_swap = k >= N;
    const int i = k, i1 = s.flags[2], i2 = s.flags[3];
    // ---- 2. the trial configuration: positions, distance and cutoff rows
    for (int a = tid; a < N; a += blockDim.x) {
      const int src = !is_swap ? a : (a == i1 ? i2 : (a == i2 ? i1 : a));
      s.perm[a] = src;
      for (int c = 0; c < 3; ++c) s.Xt[3 * a + c] = s.X[3 * src + c];
      if (!is_swap && a == i) {
        s.Xt[3 * a] = s.dd[0];
        s.Xt[3 * a + 1] = s.dd[1];
        s.Xt[3 * a + 2] = s.dd[2];
      }
    }
    __syncthreads();
    if (!is_swap) {
      for (int j = tid; j < N; j += blockDim.x) {
        const double v = j == i ? 0.0
                                : d2_sph(s.Xt[3 * i], s.Xt[3 * i + 1], s.Xt[3 * i + 2], s.X[3 * j],
                                         s.X[3 * j + 1], s.X[3 * j + 2]);
        s.row[j] = v;
        s.frow[j] = j == i ? 1.0 : cutoff2(sqrt(v), Q.rcut);
      }
      __syncthreads();
    }
    auto dt = [&](int a, int b) -> double {
      if (!is_swap) return a == i ? s.row[b] : (b == i ? s.row[a] : s.D[a * N + b]);
      return s.D[s.perm[a] * N + s.perm[b]];
    };
    auto ft = [&](int a, int b) -> double {
      if (!is_swap) return a == i ? s.frow[b] : (b == i ? s.frow[a] : s.F[a * N + b]);
      return s.F[s.perm[a] * N + s.perm[b]];
    };
    // ---- 3. trial symmetry matrix and energy (energy_update! / swap_energy_update,
    // src/EnergyEvaluation.jl:1622-1642, 1438-1446)
    build_G(Q, N, [&](int a) { return s.Xt + 3 * a; }, dt, ft, s.Gt, s.part);
    const double new_en = mlp_energy2(Q, N, s.Gt, s.ea);
    // ---- 4. Metropolis (src/Exchange.jl:53-57) and commit (swap_config!,
    // src/swap_config.jl:14-51, 237-276); swaps change no counter
    if (tid == 0) {
      double prob = exp(-(new_en - en) * beta);
      if (prob > 1) prob = 1.0;
      s.flags[4] = prob >= draw();
    }
    __syncthreads();
    if (s.flags[4]) {
      // D and F: a move changes row and column i, a swap exchanges two rows
      // and two columns
      if (!is_swap) {
        for (int j = tid; j < N; j += blockDim.x) {
          s.D[i * N + j] = s.row[j];
          s.D[j * N + i] = s.row[j];
          s.F[i * N + j] = s.frow[j];
          s.F[j * N + i] = s.frow[j];
        }
      } else {
        for (int j = tid; j < N; j += blockDim.x) {  // rows first
          double t = s.D[i1 * N + j];
          s.D[i1 * N + j] = s.D[i2 * N + j];
          s.D[i2 * N + j] = t;
          t = s.F[i1 * N + j];
          s.F[i1 * N + j] = s.F[i2 * N + j];
          s.F[i2 * N + j] = t;
        }
        __syncthreads();
        for (int j = tid; j < N; j += blockDim.x) {  // then columns
          double t = s.D[j * N + i1];
          s.D[j * N + i1] = s.D[j * N + i2];
          s.D[j * N + i2] = t;
          t = s.F[j * N + i1];
          s.F[j * N + i1] = s.F[j * N + i2];
          s.F[j * N + i2] = t;
        }
        __syncthreads();
        if (tid == 0) {
          s.D[i1 * N + i1] = s.D[i2 * N + i2] = 0.0;
          s.F[i1 * N + i1] = s.F[i2 * N + i2] = 1.0;
        }
      }
      for (int p = tid; p < N * 3; p += blockDim.x) s.X[p] = s.Xt[p];
      for (int p = tid; p < Ng * N; p += blockDim.x) s.G[p] = s.Gt[p];
      en = new_en;
      if (is_swap) ++swaps;
      else ++acc;
    }
    __syncthreads();
  }
  // ---- write back
  for (int k = tid; k < N * 3; k += blockDim.x) Xg[k] = s.X[k];
  if (tid == 0) {
    P.en[g] = en;
    P.ctr[g] = ctr;
    P.status[g] = status;
    P.cnt[6 * (size_t)gs + 0] += acc;
    P.cnt[6 * (size_t)gs + 1] += acc;
    Q.swaps_acc[g] += swaps;
  }
}

}  // namespace

size_t nn2_smem_bytes(const NN2Params& Q, int N) {
  Nn2Smem s;
  return carve(s, nullptr, N, 2 * Q.nrad + 3 * Q.nang) + 64;
}

template <typename K>
static int set_smem2(K kern, size_t smem) {
  if (smem <= 48 * 1024) return 0;
  return (int)cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

int nn2_launch_init(const KParams& P, const NN2Params& Q, int n_walkers, int maxN, void* stream) {
  const size_t smem = nn2_smem_bytes(Q, maxN);
  int e = set_smem2(k_nn2_init, smem);
  if (e) return e;
  k_nn2_init<<<n_walkers, NN2_THREADS, smem, (cudaStream_t)stream>>>(P, Q);
  return (int)cudaGetLastError();
}

int nn2_launch_cycle(const KParams& P, const NN2Params& Q, const NNParams& Q1, int n_walkers,
                     int n_runs, int R, int maxN, int phase, void* stream) {
  const size_t smem = nn2_smem_bytes(Q, maxN);
  int e = set_smem2(k_nn2_cycle, smem);
  if (e) return e;
  k_nn2_cycle<<<n_walkers, NN2_THREADS, smem, (cudaStream_t)stream>>>(P, Q);
  if ((e = (int)cudaGetLastError())) return e;
  return nn_launch_epilogue(P, Q1, n_runs, R, phase, stream);
}

}  // namespace ptmc
