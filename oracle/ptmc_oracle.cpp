// ptmc_oracle.cpp — CPU ORACLE (test infrastructure only; see ptmc_oracle.h).
//
// A plain FP64 restatement of ParallelTemperingMonteCarlo.jl's hot path.  Every
// function cites the reference file:line it follows.  Arithmetic keeps the
// reference's operation order (no fused multiply-add: build with
// -ffp-contract=off) so that squared distances, proposals and ELJ pair energies
// are bit-identical to what the reference computes for the same inputs.
//
// Walker/slot formulation: the reference swaps whole configurations between
// temperature-indexed MCState objects on an accepted exchange
// (src/Exchange.jl:115-124).  Here a "walker" owns the configuration-bound data
// (positions, distance matrix, energy, potential variables, box, draw stream)
// and a "slot" owns the temperature-bound data (beta, max_displ, counters,
// E/E^2 accumulators, histogram row).  An accepted exchange swaps the
// walker<->slot mapping, which is the same state transition.
#include "ptmc_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace {

thread_local std::string g_err;
int fail(const std::string& m) {
  g_err = m;
  return -1;
}

// ---------------------------------------------------------------- Philox4x32-10
// Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy as 1, 2, 3"
// (SC'11).  Counter = {idx lo, idx hi, stream, run}; key = seed.
inline void philox(uint32_t c[4], uint32_t k0, uint32_t k1) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
  const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
  for (int r = 0; r < 10; ++r) {
    if (r > 0) {
      k0 += W0;
      k1 += W1;
    }
    uint64_t p0 = (uint64_t)M0 * c[0];
    uint64_t p1 = (uint64_t)M1 * c[2];
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    uint32_t n0 = hi1 ^ c[1] ^ k0;
    uint32_t n2 = hi0 ^ c[3] ^ k1;
    c[0] = n0;
    c[1] = lo1;
    c[2] = n2;
    c[3] = lo0;
  }
}
// Draw k of a stream is half (k & 1) of Philox block k >> 1: half 0 takes 53
// bits from words (0,1), half 1 from words (2,3).
inline double u01(uint64_t seed, uint32_t stream, uint32_t run, uint64_t idx) {
  uint64_t blk = idx >> 1;
  uint32_t c[4] = {(uint32_t)blk, (uint32_t)(blk >> 32), stream, run};
  philox(c, (uint32_t)seed, (uint32_t)(seed >> 32));
  int h = (int)(idx & 1) * 2;
  uint64_t b = ((uint64_t)c[h] << 21) | (uint64_t)(c[h + 1] >> 11);
  return (double)b * 0x1.0p-53;
}
// rand(1:n) (0-based result): floor(u*n), clamped
inline int randint(double u, int n) {
  int k = (int)(u * (double)n);
  return k >= n ? n - 1 : k;
}

const double kB = 3.16681196E-6;  // src/InputParams.jl:19

// ---------------------------------------------------------------- distances
// distance2 (src/Configurations.jl:101-109): (a-b).(a-b) summed left to right
inline double dot3(double x, double y, double z) {
  return (x * x + y * y) + z * z;
}
inline double dist2_sph(const double* a, const double* b) {
  return dot3(a[0] - b[0], a[1] - b[1], a[2] - b[2]);
}
// cubic minimum image (src/Configurations.jl:103-109)
inline double dist2_cub(const double* a, const double* b, double L) {
  double bx = b[0] + L * std::nearbyint((a[0] - b[0]) / L);
  double by = b[1] + L * std::nearbyint((a[1] - b[1]) / L);
  double bz = b[2] + L * std::nearbyint((a[2] - b[2]) / L);
  return dot3(a[0] - bx, a[1] - by, a[2] - bz);
}
// RectangularBC minimum image: side L in x and y, height H in z
// (src/Configurations.jl:121-126)
inline double dist2_rect(const double* a, const double* b, double L, double H) {
  double bx = b[0] + L * std::nearbyint((a[0] - b[0]) / L);
  double by = b[1] + L * std::nearbyint((a[1] - b[1]) / L);
  double bz = b[2] + H * std::nearbyint((a[2] - b[2]) / H);
  return dot3(a[0] - bx, a[1] - by, a[2] - bz);
}
// RhombicBC minimum image (src/Configurations.jl:110-120): y on the rhombus
// height sqrt(3)/2 L, x on the sheared axis, z as the rectangular box.  3^0.5
// is the double nearest sqrt(3) (Julia's pow is within 0.05 ulp of it there).
const double S3 = 1.7320508075688772;
inline double dist2_rhb(const double* a, const double* b, double L, double H) {
  const double hy = S3 / 2 * L, is3 = 1 / S3;
  double by = b[1] + hy * std::nearbyint((a[1] - b[1]) / hy);
  double bx = ((b[0] - b[1] / S3) + L * std::nearbyint(((a[0] - b[0]) - is3 * (a[1] - b[1])) / L)) +
              is3 * by;
  double bz = b[2] + H * std::nearbyint((a[2] - b[2]) / H);
  return dot3(a[0] - bx, a[1] - by, a[2] - bz);
}
inline double dist2_bc(int bc, const double* a, const double* b, double L, double H) {
  switch (bc) {
    case ORC_BC_CUBIC: return dist2_cub(a, b, L);
    case ORC_BC_RECT: return dist2_rect(a, b, L, H);
    case ORC_BC_RHOMBIC: return dist2_rhb(a, b, L, H);
    default: return dist2_sph(a, b);
  }
}
// get_r_cut (src/Ensembles.jl:118-155): squared cut-off implied by the box
inline double box_rcut(int bc, double L, double H) {
  if (bc == ORC_BC_RHOMBIC) return std::min(L * L * 3 / 16, H * H / 4);
  if (bc == ORC_BC_RECT) return std::min(L * L / 4, H * H / 4);
  if (bc == ORC_BC_CUBIC) return L * L / 4;
  return 0.0;
}
// get_volume (src/Configurations.jl:246-256)
inline double box_volume(int bc, double L, double H) {
  if (bc == ORC_BC_RHOMBIC) return L * L * H * S3 / 2;
  if (bc == ORC_BC_RECT) return L * L * H;
  return L * L * L;
}

// get_tan (src/Configurations.jl:181-215): |tan| of the angle between the
// (minimum-image) pair vector and z, sqrt(dx^2 + dy^2) / dz
inline double tan_bc(int bc, const double* a, const double* b, double L, double H) {
  double bx = b[0], by = b[1], bz = b[2];
  if (bc == ORC_BC_CUBIC || bc == ORC_BC_RECT) {
    const double Hz = bc == ORC_BC_RECT ? H : L;
    bx = b[0] + L * std::nearbyint((a[0] - b[0]) / L);
    by = b[1] + L * std::nearbyint((a[1] - b[1]) / L);
    bz = b[2] + Hz * std::nearbyint((a[2] - b[2]) / Hz);
  } else if (bc == ORC_BC_RHOMBIC) {
    const double hy = S3 / 2 * L, is3 = 1 / S3;
    by = b[1] + hy * std::nearbyint((a[1] - b[1]) / hy);
    bx = ((b[0] - b[1] / S3) + L * std::nearbyint(((a[0] - b[0]) - is3 * (a[1] - b[1])) / L)) +
         is3 * by;
    bz = b[2] + H * std::nearbyint((a[2] - b[2]) / H);
  }
  const double dx = a[0] - bx, dy = a[1] - by;
  return std::fabs(std::sqrt(dx * dx + dy * dy) / (a[2] - bz));
}

// ---------------------------------------------------------------- potentials
struct SF {
  int kind, type;
  double eta, lambda, zeta, rcut, gnorm, goffset, tpz;
};

struct Pot {
  int kind = -1;
  std::vector<double> c;  // ELJ coefficients (ELJPotentialB: coeff_c)
  std::vector<double> a, b;  // ELJPotentialB coeff_a, coeff_b
  // LookupTablePotential: table [l_dist][l_angle] (Julia's column-major
  // Matrix(l_angle, l_dist)), first distance, steps, c6 tail coefficient
  std::vector<double> lut;
  int l_dist = 0, l_angle = 0;
  // RuNNerPotential2Atom: species 1 = atoms 0..n1-1; radial rows {eta, r_cut,
  // G_offset[4], G_norm[4]}, angular rows {eta, lambda, zeta, r_cut, tpz[6],
  // G_offset[6]}; w = species-1 weights, w_b = species-2 weights
  int n1 = 0, nrad2 = 0, nang2 = 0;
  std::vector<double> rad2, ang2, w_b;
  double start_dist = 0, start_angle = 0, d_dist = 0, d_angle = 0, c6 = 0;
  double n = 0, m = 0, ean = 0, ecam = 0;
  // NN
  std::vector<SF> sf;
  std::vector<double> w;
  std::vector<int> nodes;
  double rcut = 0, boundary2 = 0;
};

// dimer_energy ELJPotential (EnergyEvaluation.jl:923-932)
double elj_all(const double* c, int K, double r2) {
  double r = std::sqrt(r2);
  double r6inv = 1 / (r2 * r2 * r2);
  double s = 0.0;
  for (int i = 0; i < K; ++i) {
    s += c[i] * r6inv;
    r6inv /= r;
  }
  return s;
}
// dimer_energy ELJPotentialEven (EnergyEvaluation.jl:934-942)
double elj_even(const double* c, int K, double r2) {
  double r6inv = 1 / (r2 * r2 * r2);
  double s = 0.0;
  for (int i = 0; i < K; ++i) {
    s += c[i] * r6inv;
    r6inv /= r2;
  }
  return s;
}
// dimer_energy ELJPotentialB (EnergyEvaluation.jl:943-958): terms r^-6, r^-8,
// then one more power of 1/r each, scaled by 1 + a cos 2theta + b cos 4theta
double eljb(const Pot& p, double r2, double tn) {
  if (!(r2 >= 5.30)) return 0.1;
  double r6inv = 1 / (r2 * r2 * r2);
  const double t2 = 2 / (tn * tn + 1) - 1;  // cos(2 theta)
  const double t4 = 2 * (t2 * t2) - 1;
  double s = p.c[0] * r6inv * (1 + p.a[0] * t2 + p.b[0] * t4);
  r6inv /= r2;
  for (size_t i = 1; i < p.c.size(); ++i) {
    s += p.c[i] * r6inv * (1 + p.a[i] * t2 + p.b[i] * t4);
    r6inv /= std::sqrt(r2);
  }
  return s;
}
// dimer_energy LookupTablePotential (EnergyEvaluation.jl:277-298); Julia's
// round is half-to-even (nearbyint); the indices are kept inside the table
double lut_energy(const Pot& p, double r2, double tn) {
  int ia = 1;
  const double at = std::fabs(tn);
  if (at > 0.00872687153 && at <= 114.592845357)
    ia = (int)std::nearbyint(std::atan(at) / p.d_angle * 180.0 / M_PI + 1.0);
  else if (at > 114.592845357)
    ia = 91;
  ia = std::min(std::max(ia, 1), p.l_angle);
  const double r0 = p.start_dist + 0.5 * p.d_dist, r1 = p.start_dist + p.l_dist * p.d_dist;
  if (r2 <= r0 * r0) return p.lut[(size_t)(ia - 1)];
  if (r2 <= r1 * r1) {
    int id = (int)std::nearbyint((std::sqrt(r2) - p.start_dist) / p.d_dist);
    id = std::min(std::max(id, 1), p.l_dist);
    return p.lut[(size_t)(id - 1) * p.l_angle + (ia - 1)];
  }
  return p.c6 / (r2 * r2 * r2);
}
inline bool is_b(const Pot& p) { return p.kind == ORC_POT_ELJB || p.kind == ORC_POT_LUT; }
inline double dimer_b(const Pot& p, double r2, double tn) {
  return p.kind == ORC_POT_ELJB ? eljb(p, r2, tn) : lut_energy(p, r2, tn);
}
inline double dimer(const Pot& p, double r2) {
  return p.kind == ORC_POT_ELJ ? elj_all(p.c.data(), (int)p.c.size(), r2)
                               : elj_even(p.c.data(), (int)p.c.size(), r2);
}
// lrc (EnergyEvaluation.jl:968-982); r_cut is the squared cut-off
double lrc_even(int N, double r_cut, const double* c, int K) {
  if (r_cut <= 50) return 0.0;
  double rcs = std::sqrt(r_cut);  // r_cut^0.5, correctly rounded
  double rc3 = r_cut * rcs;
  double e = 0.0;
  for (int i = 1; i <= K; ++i) {
    e += c[i - 1] / rc3 / (2 * i + 1);
    rc3 *= r_cut;
  }
  e *= M_PI * (double)(N * N) / 4 / (rcs * rcs * rcs);
  return e;
}
// lrc of ELJPotentialB (EnergyEvaluation.jl:983-998): fixed coefficients
double lrc_eljb(int N, double r_cut) {
  static const double cf[4] = {-0.1279111890228638, -1.328138539967966, 12.260941135261255,
                               41.12212408251662};
  if (r_cut <= 16) return 0.0;
  double rcs = std::sqrt(r_cut);
  double rc3 = r_cut * rcs;
  double e = 0.0;
  for (int i = 1; i <= 4; ++i) {
    e += cf[i - 1] / rc3 / (2 * i + 1);
    rc3 *= r_cut;
  }
  e *= M_PI * (double)(N * N) / 4 / (rcs * rcs * rcs);
  return e;
}
// lrc of LookupTablePotential (EnergyEvaluation.jl:999-1009): 1.0 below r_cut = 10
double lrc_lut(int N, double r_cut, double c6) {
  if (r_cut <= 10) return 1.0;
  double rcs = std::sqrt(r_cut);
  double rc3 = r_cut * rcs;
  double e = c6 / rc3 / 3;
  e *= M_PI * (double)(N * N) / 4 / (rcs * rcs * rcs);
  return e;
}
// the potential's long-range correction with the box factor of
// dimer_energy_config (EnergyEvaluation.jl:419, 444, 469-472, 587, 634-637, 743)
double lrc_pot(const Pot& p, int N, double rc2, int bc, double L, double H) {
  double l = p.kind == ORC_POT_ELJB  ? lrc_eljb(N, rc2)
             : p.kind == ORC_POT_LUT ? lrc_lut(N, rc2, p.c6)
                                     : lrc_even(N, rc2, p.c.data(), (int)p.c.size());
  if (bc == ORC_BC_RHOMBIC) l = l * 3 / 4 * L / H;
  else if (bc == ORC_BC_RECT) l = L < H ? l * L / H : l * (H * H) / (L * L);
  return l;
}
// dimer_energy_atom with the tangent row (EnergyEvaluation.jl:334-361)
double dimer_atom_b(const Pot& p, int i, const double* d2, const double* tn, int N, bool cut,
                    double rc2) {
  double s = 0.0;
  for (int j = 0; j < N; ++j) {
    if (j == i) continue;
    if (cut && !(d2[j] <= rc2)) continue;
    s += dimer_b(p, d2[j], tn[j]);
  }
  return s;
}
// dimer_energy_config with the tangent matrix (EnergyEvaluation.jl:476-640, 657-780)
double dimer_config_b(const Pot& p, const double* d2, const double* tn, int N, bool cut,
                      double rc2, int bc, double L, double H) {
  double e = 0.0;
  for (int i = 0; i < N; ++i)
    for (int j = i + 1; j < N; ++j) {
      const double x = d2[(size_t)i * N + j];
      if (cut && !(x <= rc2)) continue;
      e += dimer_b(p, x, tn[(size_t)i * N + j]);
    }
  if (cut) e = e + lrc_pot(p, N, rc2, bc, L, H);
  return e;
}
// dimer_energy_atom (EnergyEvaluation.jl:313-345): sum over j != i in order
double dimer_atom(const Pot& p, int i, const double* d2, int N, bool cut,
                  double rc2) {
  double s = 0.0;
  for (int j = 0; j < N; ++j) {
    if (j == i) continue;
    if (cut && !(d2[j] <= rc2)) continue;
    s += dimer(p, d2[j]);
  }
  return s;
}
// dimer_energy_config (EnergyEvaluation.jl:378-473); with a cut-off the long-range
// correction, which assumes a cube, is rescaled for the other boxes
// (:444, :469-472)
double dimer_config(const Pot& p, const double* d2, int N, bool cut,
                    double rc2, int bc = ORC_BC_CUBIC, double L = 0, double H = 0) {
  double e = 0.0;
  for (int i = 0; i < N; ++i)
    for (int j = i + 1; j < N; ++j) {
      double x = d2[(size_t)i * N + j];
      if (cut && !(x <= rc2)) continue;
      e += dimer(p, x);
    }
  if (cut) {
    e = e + lrc_pot(p, N, rc2, bc, L, H);
  }
  return e;
}
// invrexp (EnergyEvaluation.jl:1088-1095)
inline void invrexp(double r2, double n, double m, double& a, double& b) {
  if (r2 != 0.0) {
    double rt = 1 / std::sqrt(r2);
    a = std::pow(rt, n);
    b = std::pow(rt, m);
  } else {
    a = 0.0;
    b = 0.0;
  }
}
// calc_energies_from_components (EnergyEvaluation.jl:1156-1162)
double eam_energy(const double* comp, int N, double ean, double ecam) {
  double e = 0.0;
  for (int i = 0; i < N; ++i)
    e += ean * comp[2 * i] - ecam * std::sqrt(comp[2 * i + 1]);
  return e;
}

// cutoff_function (MachineLearningPotential/Cutoff.jl:79-90)
inline double cutoff(double r, double rc) {
  return r < rc ? 0.5 * (std::cos(M_PI * (r / rc)) + 1) : 0.0;
}
// all_angular_measure (Cutoff.jl:48-57): the three cosines of triangle abc
inline void angles(const double* a, const double* b, const double* c,
                   double r2ab, double r2ac, double r2bc, double th[3]) {
  double ab[3], ac[3], bc[3];
  for (int k = 0; k < 3; ++k) {
    ab[k] = a[k] - b[k];
    ac[k] = a[k] - c[k];
    bc[k] = b[k] - c[k];
  }
  double dab = std::sqrt(r2ab), dac = std::sqrt(r2ac), dbc = std::sqrt(r2bc);
  th[0] = ((ab[0] * ac[0] + ab[1] * ac[1]) + ab[2] * ac[2]) / (dab * dac);
  th[1] = (((-ab[0]) * bc[0] + (-ab[1]) * bc[1]) + (-ab[2]) * bc[2]) /
          (dab * dbc);
  th[2] = (((-ac[0]) * (-bc[0]) + (-ac[1]) * (-bc[1])) + (-ac[2]) * (-bc[2])) /
          (dac * dbc);
}
inline double theta_part(double th, double lam, double zeta) {
  return std::pow(1 + lam * th, zeta);  // SymmFunc.jl:166
}

// ---- two-species RuNNer potential (EnergyEvaluation.jl:1276-1448,
// SymmFunc.jl:326-471, 508-541): the symmetry matrix of a configuration.
// Radial function k fills rows 2k (neighbour of species 1) and 2k+1 (species
// 2); angular function k fills rows 2 nrad + 3k + m, m = the number of
// species-2 atoms among the centre's two neighbours.  Each row is scaled and
// offset by the centre atom's species.  Loops in the reference's order.
void nn2_G(const Pot& p, const double* X, const double* D, const double* F, int N, double* G) {
  const int n1 = p.n1, nr = p.nrad2, na = p.nang2;
  std::fill(G, G + (size_t)(2 * nr + 3 * na) * N, 0.0);
  for (int k = 0; k < nr; ++k) {
    const double* q = &p.rad2[10 * (size_t)k];
    const double eta = q[0];
    double* g0 = G + (size_t)(2 * k) * N;
    double* g1 = G + (size_t)(2 * k + 1) * N;
    auto v = [&](int a, int b) {  // calc_one_symm_val (SymmFunc.jl:228-230)
      const double fc = F[(size_t)a * N + b];
      return (fc != 0.0 && fc != 1.0) ? fc * std::exp(-eta * D[(size_t)a * N + b]) : 0.0;
    };
    for (int a = 0; a < n1; ++a)
      for (int b = a + 1; b < n1; ++b) {
        const double x = v(a, b);
        g0[a] += x;
        g0[b] += x;
      }
    for (int a = n1; a < N; ++a)
      for (int b = a + 1; b < N; ++b) {
        const double x = v(a, b);
        g1[a] += x;
        g1[b] += x;
      }
    for (int a = 0; a < n1; ++a)
      for (int b = n1; b < N; ++b) {
        const double x = v(a, b);
        g1[a] += x;
        g0[b] += x;
      }
    for (int a = 0; a < N; ++a) {
      const int t = a < n1 ? 0 : 2;
      g0[a] = g0[a] * q[6 + t] + q[2 + t];
      g1[a] = g1[a] * q[7 + t] + q[3 + t];
    }
  }
  for (int k = 0; k < na; ++k) {
    const double* q = &p.ang2[16 * (size_t)k];
    const double eta = q[0], lam = q[1], zeta = q[2];
    double* g = G + (size_t)(2 * nr + 3 * k) * N;  // rows m = 0, 1, 2
    auto tri = [&](int a, int b, int c, int ma, int mb, int mc) {
      const double rab = D[(size_t)a * N + b], rac = D[(size_t)a * N + c], rbc = D[(size_t)b * N + c];
      double th[3];
      angles(X + 3 * a, X + 3 * b, X + 3 * c, rab, rac, rbc, th);
      const double e = std::exp(-eta * (rab + rac + rbc)) * F[(size_t)a * N + b] *
                       F[(size_t)a * N + c] * F[(size_t)b * N + c];
      g[(size_t)ma * N + a] += e * theta_part(th[0], lam, zeta);
      g[(size_t)mb * N + b] += e * theta_part(th[1], lam, zeta);
      g[(size_t)mc * N + c] += e * theta_part(th[2], lam, zeta);
    };
    for (int a = 0; a < n1; ++a)  // 111
      for (int b = a + 1; b < n1; ++b)
        for (int c = b + 1; c < n1; ++c) tri(a, b, c, 0, 0, 0);
    for (int a = n1; a < N; ++a)  // 222
      for (int b = a + 1; b < N; ++b)
        for (int c = b + 1; c < N; ++c) tri(a, b, c, 2, 2, 2);
    for (int a = 0; a < n1; ++a)  // 112
      for (int b = a + 1; b < n1; ++b)
        for (int c = n1; c < N; ++c) tri(a, b, c, 1, 1, 0);
    for (int a = 0; a < n1; ++a)  // 122
      for (int b = n1; b < N; ++b)
        for (int c = b + 1; c < N; ++c) tri(a, b, c, 2, 1, 1);
    for (int a = 0; a < N; ++a) {
      const int t = a < n1 ? 0 : 3;
      for (int m = 0; m < 3; ++m) {
        double& x = g[(size_t)m * N + a];
        x = x * q[4 + t + m] + q[10 + t + m];
      }
    }
  }
}
// calc_new_runner_energy! (EnergyEvaluation.jl:1419-1432): species-1 atoms
// through nnp1, species-2 atoms through nnp2
double nn2_energy(const Pot& p, const double* G, int N, double* eatom);

// per-atom MLP forward (ForwardPass.jl:50-84 math: activations
// linear/tanh/.../linear).  Weight layout (ours): per layer W[n_in][n_out]
// input-major, then bias[n_out].
double mlp_atom(const double* x, const double* w, const int* nodes, int nl) {
  double buf0[256], buf1[256];
  const double* in = x;
  double* out = buf0;
  size_t off = 0;
  for (int l = 1; l < nl; ++l) {
    int ni = nodes[l - 1], no = nodes[l];
    const double* W = w + off;
    const double* B = w + off + (size_t)ni * no;
    for (int j = 0; j < no; ++j) {
      double s = 0.0;
      for (int i = 0; i < ni; ++i) s += in[i] * W[(size_t)i * no + j];
      s += B[j];
      out[j] = (l < nl - 1) ? std::tanh(s) : s;
    }
    off += (size_t)ni * no + no;
    in = out;
    out = (out == buf0) ? buf1 : buf0;
  }
  return in[0];
}


// ---------------------------------------------------------------- surrogate
// Learned pair surrogate of the delayed-acceptance move (no counterpart in the
// reference; Christen & Fox, J. Comput. Graph. Stat. 14 (2005) 795, two-stage
// Metropolis-Hastings).  E_s(x) = sum_{i<j} phi(r_ij) with
//   g_k(r) = fc(r) exp(-gamma (r - mu_k)^2),  mu_k = r_lo + k (r_hi - r_lo)/15,
//   h1 = tanh(W1^T g + b1),  h2 = tanh(W2^T h1 + b2),
//   phi = escale (w3 . h2 + b3)
// (16 features, 32 + 32 hidden units).  A move of atom i has the record
// rows[0..63] = |t - x_j| (new), rows[64..127] = |x_i - x_j| (old), negative =
// no pair; dE_s = sum_new phi - sum_old phi.  With `bf` set, the operands of
// the two matrix products (g, W1, h1, W2) are rounded to BF16 as the tensor
// cores see them; sums and activations stay FP64 here.
struct SurCfg {
  double r_lo = 0, r_hi = 0, gamma = 0, r_cut = 0, escale = 1;
};
constexpr int SUR_F = 16, SUR_H = 32, SUR_ROWS = 128;
constexpr int SUR_B1 = SUR_F * SUR_H, SUR_W2 = SUR_B1 + SUR_H, SUR_B2 = SUR_W2 + SUR_H * SUR_H,
              SUR_W3 = SUR_B2 + SUR_H, SUR_B3 = SUR_W3 + SUR_H, SUR_NP = SUR_B3 + 1;

// round to float, then to the nearest BF16 (ties to even)
inline double bf16r(double x) {
  float f = (float)x;
  uint32_t u;
  std::memcpy(&u, &f, 4);
  if ((u & 0x7F800000u) != 0x7F800000u) u = (u + 0x7FFFu + ((u >> 16) & 1u)) & 0xFFFF0000u;
  std::memcpy(&f, &u, 4);
  return (double)f;
}

struct SurRow {
  double g[SUR_F], h1[SUR_H], h2[SUR_H], phi;
};

void sur_row(const SurCfg& c, const double* P, double r, bool bf, SurRow& st) {
  const double fc = r < c.r_cut ? 0.5 * (std::cos(3.141592653589793 * (r / c.r_cut)) + 1) : 0.0;
  for (int k = 0; k < SUR_F; ++k) {
    double mu = c.r_lo + k * ((c.r_hi - c.r_lo) / (SUR_F - 1));
    double d = r - mu;
    double g = fc * std::exp(-c.gamma * (d * d));
    st.g[k] = bf ? bf16r(g) : g;
  }
  for (int n = 0; n < SUR_H; ++n) {
    double z = 0;
    for (int k = 0; k < SUR_F; ++k) {
      double w = P[k * SUR_H + n];
      z += st.g[k] * (bf ? bf16r(w) : w);
    }
    st.h1[n] = std::tanh(z + P[SUR_B1 + n]);
  }
  double phi = 0;
  for (int n = 0; n < SUR_H; ++n) {
    double z = 0;
    for (int k = 0; k < SUR_H; ++k) {
      double w = P[SUR_W2 + k * SUR_H + n];
      z += (bf ? bf16r(st.h1[k]) : st.h1[k]) * (bf ? bf16r(w) : w);
    }
    st.h2[n] = std::tanh(z + P[SUR_B2 + n]);
    phi += P[SUR_W3 + n] * st.h2[n];
  }
  st.phi = c.escale * (phi + P[SUR_B3]);
}

double sur_delta(const SurCfg& c, const double* P, const float* rows, bool bf) {
  SurRow st;
  double e = 0;
  for (int q = 0; q < SUR_ROWS; ++q) {
    if (!(rows[q] >= 0)) continue;
    sur_row(c, P, rows[q], bf, st);
    e += q < SUR_ROWS / 2 ? st.phi : -st.phi;
  }
  return e;
}

// Huber loss (delta 1) of the scaled residual (dE_s - y)/escale, averaged
// over the n records, and its gradient with respect to the parameters (the
// BF16 rounding, when on, is treated as the identity in the backward pass).
double sur_loss_grad(const SurCfg& c, const double* P, const float* rows, const float* y, int n,
                     bool bf, double* grad) {
  std::vector<SurRow> st(SUR_ROWS);
  double L = 0;
  if (grad) std::fill(grad, grad + SUR_NP, 0.0);
  for (int b = 0; b < n; ++b) {
    const float* rr = rows + (size_t)b * SUR_ROWS;
    double e = 0;
    for (int q = 0; q < SUR_ROWS; ++q) {
      if (!(rr[q] >= 0)) continue;
      sur_row(c, P, rr[q], bf, st[q]);
      e += q < SUR_ROWS / 2 ? st[q].phi : -st[q].phi;
    }
    double res = (e - (double)y[b]) / c.escale;
    double a = std::fabs(res);
    L += a <= 1 ? 0.5 * res * res : a - 0.5;
    if (!grad) continue;
    double G = (res > 1 ? 1.0 : res < -1 ? -1.0 : res) / (c.escale * n);  // dL/d dE_s
    for (int q = 0; q < SUR_ROWS; ++q) {
      if (!(rr[q] >= 0)) continue;
      const SurRow& s = st[q];
      double dphi = (q < SUR_ROWS / 2 ? G : -G) * c.escale;
      grad[SUR_B3] += dphi;
      double dz2[SUR_H];
      for (int m = 0; m < SUR_H; ++m) {
        grad[SUR_W3 + m] += dphi * s.h2[m];
        dz2[m] = dphi * P[SUR_W3 + m] * (1 - s.h2[m] * s.h2[m]);
        grad[SUR_B2 + m] += dz2[m];
      }
      for (int k = 0; k < SUR_H; ++k) {
        double h1k = bf ? bf16r(s.h1[k]) : s.h1[k];
        double dh = 0;
        for (int m = 0; m < SUR_H; ++m) {
          double w = P[SUR_W2 + k * SUR_H + m];
          grad[SUR_W2 + k * SUR_H + m] += h1k * dz2[m];
          dh += (bf ? bf16r(w) : w) * dz2[m];
        }
        double dz1 = dh * (1 - s.h1[k] * s.h1[k]);
        grad[SUR_B1 + k] += dz1;
        for (int f = 0; f < SUR_F; ++f) grad[f * SUR_H + k] += s.g[f] * dz1;
      }
    }
  }
  return L / n;
}

}  // namespace

// ================================================================ run state
struct orc_run {
  int N, R, ens, bc;
  double pressure, exch_prob, min_acc, max_acc;
  int n_bin, n_adjust, mc_sample;
  uint64_t seed;
  int run_index;
  Pot pot;
  // walker-bound
  std::vector<double> pos;    // R*N*3
  std::vector<double> d2;     // R*N*N
  std::vector<double> tn;     // R*N*N tangent matrix (ELJPotentialB, LookupTablePotential)
  std::vector<double> en;     // R
  std::vector<double> box;    // R (cubic side, box_length of the other boxes)
  std::vector<double> boxh;   // R (box_height of RectangularBC / RhombicBC)
  std::vector<double> rcut2;  // R
  std::vector<double> comp;   // R*N*2 (EAM)
  std::vector<double> G;      // R*nsf*N (NN, column per atom)
  std::vector<double> F;      // R*N*N (NN cut-off matrix)
  std::vector<double> eatom;  // R*N
  std::vector<uint64_t> ctr;  // R
  // slot-bound
  std::vector<double> T, beta, maxd, ham, max_box;  // R, R, 2R, 2R, R
  std::vector<long> cnt_atom, cnt_vol, cnt_exc;     // 2R each
  // separated volume moves (NPT separated_volume): max_displ[3:4] (xy, z),
  // max_boxheight, count_vol_xy, count_vol_z (MCStates.jl:33-47)
  bool sep = false;
  int n_swaps = 0;          // NNVT: atom swaps per cycle
  long n_swaps_acc = 0;     // accepted swaps (all slots)
  std::vector<double> maxd_sep, max_boxh;          // 2R, R
  std::vector<long> cnt_xy, cnt_z;                 // 2R each
  std::vector<int> wos;                             // walker of slot
  uint64_t run_ctr = 0;
  // delayed acceptance (NN only): surrogate parameters, stage counters
  bool da = false, da_bf = true;
  SurCfg sc;
  std::vector<double> sp;
  long da_reject1 = 0, da_exact = 0;
  // results
  double en_min = 0, en_max = 0, v_min = 0, v_max = 0, dE = 0, dV = 0;
  std::vector<double> en_hist, ev_hist;
  bool rdf_on = false;       // rdfsave
  double dr2 = 0;            // delta_r2
  std::vector<double> rdf;   // R * 5 n_bin
  bool inited = false;
  // scratch
  std::vector<double> trial_trow, sc_tn, sc_f;
  std::vector<double> trial_row, new_comp, newG, newF, new_eatom, sc_pos,
      sc_d2;

  double draw(int w) {
    return u01(seed, (uint32_t)w, (uint32_t)run_index, ctr[w]++);
  }
  double draw_run() {
    return u01(seed, 0xFFFFFFFFu, (uint32_t)run_index, run_ctr++);
  }
  double* P(int w) { return &pos[(size_t)w * N * 3]; }
  double* D(int w) { return &d2[(size_t)w * N * N]; }
  double* TN(int w) { return &tn[(size_t)w * N * N]; }
};

namespace {

int nsf(const orc_run* r) { return (int)r->pot.sf.size(); }

// get_distance2_mat! (Configurations.jl:146-162)
void build_d2(orc_run* r, int w) {
  int N = r->N;
  double* p = r->P(w);
  double* d = r->D(w);
  for (int i = 0; i < N; ++i)
    for (int j = i + 1; j < N; ++j) {
      double x = dist2_bc(r->bc, p + 3 * i, p + 3 * j, r->box[w], r->boxh[w]);
      d[(size_t)i * N + j] = x;
      d[(size_t)j * N + i] = x;
    }
  for (int i = 0; i < N; ++i) d[(size_t)i * N + i] = 0;
  if (is_b(r->pot)) {  // get_tantheta_mat! (Configurations.jl:225-240)
    double* t = r->TN(w);
    for (int i = 0; i < N; ++i) {
      t[(size_t)i * N + i] = 0;
      for (int j = i + 1; j < N; ++j) {
        double x = tan_bc(r->bc, p + 3 * i, p + 3 * j, r->box[w], r->boxh[w]);
        t[(size_t)i * N + j] = x;
        t[(size_t)j * N + i] = x;
      }
    }
  }
}

// total_symm_calc (SymmFunc.jl:494-510), all angular rows computed (the
// reference's (Nrad+1):Nang loop bound skips the last Nrad angular rows).
void nn_full(orc_run* r, int w) {
  int N = r->N, S = nsf(r);
  const double* p = r->P(w);
  const double* d = r->D(w);
  double* F = &r->F[(size_t)w * N * N];
  double* G = &r->G[(size_t)w * S * N];
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < N; ++j)
      F[(size_t)i * N + j] = cutoff(std::sqrt(d[(size_t)i * N + j]), r->pot.rcut);
  std::fill(G, G + (size_t)S * N, 0.0);
  for (int s = 0; s < S; ++s) {
    const SF& f = r->pot.sf[s];
    double* g = G + (size_t)s * N;
    if (f.kind == 0) {
      if (f.type != 11) continue;  // calc_symm_vals! :259-278 -> zeros(N)
      for (int a = 0; a < N; ++a)
        for (int b = a + 1; b < N; ++b) {
          double fc = F[(size_t)a * N + b];
          double gv = (fc != 0.0 && fc != 1.0)
                          ? fc * std::exp(-f.eta * d[(size_t)a * N + b]) * f.gnorm
                          : 0.0;  // calc_one_symm_val :234
          g[a] += gv;
          g[b] += gv;
        }
    } else {
      if (f.type != 111) continue;  // :280-312
      for (int a = 0; a < N; ++a)
        for (int b = a + 1; b < N; ++b)
          for (int c = b + 1; c < N; ++c) {
            double rab = d[(size_t)a * N + b], rac = d[(size_t)a * N + c],
                   rbc = d[(size_t)b * N + c];
            double th[3];
            angles(p + 3 * a, p + 3 * b, p + 3 * c, rab, rac, rbc, th);
            double ex = std::exp(-f.eta * (rab + rac + rbc)) *
                        F[(size_t)a * N + b] * F[(size_t)a * N + c] *
                        F[(size_t)b * N + c];
            g[a] += ex * theta_part(th[0], f.lambda, f.zeta) * f.tpz;
            g[b] += ex * theta_part(th[1], f.lambda, f.zeta) * f.tpz;
            g[c] += ex * theta_part(th[2], f.lambda, f.zeta) * f.tpz;
          }
    }
    for (int a = 0; a < N; ++a) g[a] = g[a] + f.goffset;
  }
}

double nn2_energy(const Pot& p, const double* G, int N, double* eatom) {
  const int Ng = 2 * p.nrad2 + 3 * p.nang2;
  std::vector<double> x(Ng);
  double e = 0.0;
  for (int a = 0; a < N; ++a) {
    for (int s = 0; s < Ng; ++s) x[s] = G[(size_t)s * N + a];
    eatom[a] = mlp_atom(x.data(), (a < p.n1 ? p.w : p.w_b).data(), p.nodes.data(),
                        (int)p.nodes.size());
    e += eatom[a];
  }
  return e;
}

double nn_energy(orc_run* r, const double* G, double* eatom) {
  int N = r->N, S = nsf(r);
  std::vector<double> x(S);
  double e = 0.0;
  for (int a = 0; a < N; ++a) {
    for (int s = 0; s < S; ++s) x[s] = G[(size_t)s * N + a];
    eatom[a] = mlp_atom(x.data(), r->pot.w.data(), r->pot.nodes.data(),
                        (int)r->pot.nodes.size());
    e += eatom[a];
  }
  return e;
}

// initialise_energy (EnergyEvaluation.jl:1662-1747) for walker w
double init_energy(orc_run* r, int w) {
  int N = r->N;
  const Pot& p = r->pot;
  if (p.kind == ORC_POT_EAM) {
    double* comp = &r->comp[(size_t)w * N * 2];
    const double* d = r->D(w);
    for (int i = 0; i < N; ++i) {  // set_variables :1800-1810
      double a = 0, b = 0;
      for (int j = 0; j < N; ++j) {
        double x, y;
        invrexp(d[(size_t)i * N + j], p.n, p.m, x, y);
        a += x;
        b += y;
      }
      comp[2 * i] = a;
      comp[2 * i + 1] = b;
    }
    return eam_energy(comp, N, p.ean, p.ecam);
  }
  if (p.kind == ORC_POT_NN2) {  // set_variables + initialise_energy (:1823-1849, 1750-1766)
    const double rc = p.rad2[1];
    double* F = &r->F[(size_t)w * N * N];
    const double* d = r->D(w);
    for (size_t k = 0; k < (size_t)N * N; ++k) F[k] = cutoff(std::sqrt(d[k]), rc);
    double* G = &r->G[(size_t)w * (2 * p.nrad2 + 3 * p.nang2) * N];
    nn2_G(p, r->P(w), d, F, N, G);
    return nn2_energy(p, G, N, &r->eatom[(size_t)w * N]);
  }
  if (p.kind == ORC_POT_NN) {
    nn_full(r, w);
    return nn_energy(r, &r->G[(size_t)w * nsf(r) * N], &r->eatom[(size_t)w * N]);
  }
  bool cut = r->ens == ORC_NPT;
  if (is_b(p)) return dimer_config_b(p, r->D(w), r->TN(w), N, cut, r->rcut2[w], r->bc, r->box[w], r->boxh[w]);
  return dimer_config(p, r->D(w), N, cut, r->rcut2[w], r->bc, r->box[w], r->boxh[w]);
}

// ---------------------------------------------------------------- moves
// atom move: mc_move! (MCRun.jl:142-162) with index < N
int atom_move(orc_run* r, int w, int slot, int i) {
  int N = r->N;
  double md = r->maxd[2 * slot];
  double* p = r->P(w);
  double* xi = p + 3 * i;
  double t[3];
  // atom_displacement (MCMoves.jl:33-64, 100-143)
  auto propose = [&]() {
    double dx = (r->draw(w) - 0.5) * md;
    double dy = (r->draw(w) - 0.5) * md;
    double dz = (r->draw(w) - 0.5) * md;
    t[0] = xi[0] + dx;
    t[1] = xi[1] + dy;
    t[2] = xi[2] + dz;
  };
  propose();
  if (r->bc == ORC_BC_SPHERE) {
    double R2 = r->box[w] * r->box[w];  // SphericalBC stores radius^2
    int count = 0;
    while (dot3(t[0], t[1], t[2]) > R2) {
      ++count;
      if (count == 50) {  // recentre!(config) (Configurations.jl:79-85)
        double cx = 0, cy = 0, cz = 0;
        for (int a = 0; a < N; ++a) {
          cx += p[3 * a];
          cy += p[3 * a + 1];
          cz += p[3 * a + 2];
        }
        cx /= N;
        cy /= N;
        cz /= N;
        for (int a = 0; a < N; ++a) {
          p[3 * a] -= cx;
          p[3 * a + 1] -= cy;
          p[3 * a + 2] -= cz;
        }
      } else {
        propose();
        if (count == 100) return fail("Error: too many moves out of binding sphere");
      }
    }
  } else if (r->bc == ORC_BC_RHOMBIC) {  // rhombic wrap (MCMoves.jl:66-83)
    double L = r->box[w], H = r->boxh[w];
    double ky = std::nearbyint((t[1] - L * S3 / 4) / (L * S3 / 2));
    double sx = L * std::nearbyint((t[0] - t[1] / S3 - L / 2) / L) + L / 2 * ky;
    double sy = L * S3 / 2 * ky;
    double sz = H * std::nearbyint((t[2] - H / 2) / H);
    t[0] -= sx;
    t[1] -= sy;
    t[2] -= sz;
  } else {  // cubic / rectangular wrap (MCMoves.jl:50-64, 85-98)
    double L = r->box[w], H = r->bc == ORC_BC_RECT ? r->boxh[w] : L;
    t[0] -= L * std::nearbyint(t[0] / L);
    t[1] -= L * std::nearbyint(t[1] / L);
    t[2] -= H * std::nearbyint(t[2] / H);
  }
  double* row = r->trial_row.data();
  for (int j = 0; j < N; ++j) row[j] = dist2_bc(r->bc, t, p + 3 * j, r->box[w], r->boxh[w]);
  row[i] = 0.0;
  const double* old = r->D(w) + (size_t)i * N;
  const Pot& pot = r->pot;
  double new_en;
  bool hard = false;
  // delayed acceptance, stage 1: the surrogate screens the proposal; the
  // first-stage draw follows the proposal draws (a rejected proposal costs no
  // exact energy evaluation)
  double dEs = 0.0;
  if (r->da) {
    float rows[SUR_ROWS];
    for (int q = 0; q < SUR_ROWS; ++q) rows[q] = -1.0f;
    for (int j = 0; j < N; ++j) {
      if (j == i) continue;
      rows[j] = (float)std::sqrt(row[j]);
      rows[SUR_ROWS / 2 + j] = (float)std::sqrt(old[j]);
    }
    dEs = sur_delta(r->sc, r->sp.data(), rows, r->da_bf);
    double p1 = std::exp(-dEs * r->beta[slot]);
    if (p1 > 1) p1 = 1.0;
    if (!(p1 >= r->draw(w))) {
      r->da_reject1 += 1;
      return 0;
    }
    r->da_exact += 1;
  }
  if (pot.kind == ORC_POT_NN2) {  // energy_update! RuNNerPotential2Atom (:1622-1642)
    // the trial's distance and cutoff matrices (row and column i), then its
    // symmetry matrix and energy
    const size_t NN = (size_t)N * N;
    const int Ng = 2 * pot.nrad2 + 3 * pot.nang2;
    r->sc_d2.assign(r->D(w), r->D(w) + NN);
    r->sc_f.assign(&r->F[(size_t)w * NN], &r->F[(size_t)w * NN] + NN);
    r->sc_pos.assign(p, p + 3 * (size_t)N);
    r->sc_pos[3 * i] = t[0];
    r->sc_pos[3 * i + 1] = t[1];
    r->sc_pos[3 * i + 2] = t[2];
    for (int j = 0; j < N; ++j) {
      if (j == i) continue;
      const double f = cutoff(std::sqrt(row[j]), pot.rad2[1]);
      r->sc_d2[(size_t)i * N + j] = r->sc_d2[(size_t)j * N + i] = row[j];
      r->sc_f[(size_t)i * N + j] = r->sc_f[(size_t)j * N + i] = f;
    }
    r->newG.resize((size_t)Ng * N);
    nn2_G(pot, r->sc_pos.data(), r->sc_d2.data(), r->sc_f.data(), N, r->newG.data());
    new_en = nn2_energy(pot, r->newG.data(), N, r->new_eatom.data());
  } else if (pot.kind == ORC_POT_EAM) {  // energy_update! EAM (:1567-1591)
    int S2 = 2 * N;
    double* nc = r->new_comp.data();
    std::memcpy(nc, &r->comp[(size_t)w * S2], sizeof(double) * S2);
    for (int j = 0; j < N; ++j) {  // calc_components :1129-1148
      double a1, b1, a0, b0;
      invrexp(row[j], pot.n, pot.m, a1, b1);
      invrexp(old[j], pot.n, pot.m, a0, b0);
      double ja = a1 - a0, jb = b1 - b0;
      nc[2 * j] += ja;
      nc[2 * j + 1] += jb;
      nc[2 * i] += ja;
      nc[2 * i + 1] += jb;
    }
    new_en = eam_energy(nc, N, pot.ean, pot.ecam);
  } else if (pot.kind == ORC_POT_NN) {  // energy_update! RuNNer (:1593-1621)
    for (int j = 0; j < N; ++j)
      if (j != i && row[j] < pot.boundary2) hard = true;
    if (hard) {
      new_en = 100.0;
    } else {
      int S = nsf(r);
      double* nF = r->newF.data();
      for (int j = 0; j < N; ++j) nF[j] = cutoff(std::sqrt(row[j]), pot.rcut);
      double* nG = r->newG.data();
      std::memcpy(nG, &r->G[(size_t)w * S * N], sizeof(double) * S * N);
      const double* F = &r->F[(size_t)w * N * N];
      const double* d = r->D(w);
      for (int s = 0; s < S; ++s) {  // total_thr_symm! (DeltaMatrix.jl:933)
        const SF& f = pot.sf[s];
        double* g = nG + (size_t)s * N;
        if (f.kind == 0) {
          if (f.type != 11) continue;  // radial_symmetry_calculation! :794
          for (int j = 0; j < N; ++j) {
            if (j == i) continue;
            double gn = std::exp(-f.eta * row[j]) * (nF[j] * f.gnorm);
            double go = std::exp(-f.eta * old[j]) * ((-F[(size_t)i * N + j]) * f.gnorm);
            g[i] = g[i] + gn;
            g[j] = g[j] + gn;
            g[i] = g[i] + go;
            g[j] = g[j] + go;
          }
        } else {
          if (f.type != 111) continue;  // angular_symmetry_calculation! :827
          for (int j = 0; j < N; ++j) {
            if (j == i) continue;
            for (int k = j + 1; k < N; ++k) {
              if (k == i) continue;
              double rjk = d[(size_t)j * N + k];
              double tn[3], to[3];
              angles(t, p + 3 * j, p + 3 * k, row[j], row[k], rjk, tn);
              angles(p + 3 * i, p + 3 * j, p + 3 * k, old[j], old[k], rjk, to);
              double en_ = std::exp(-f.eta * (row[j] + row[k] + rjk)) * nF[j] *
                           nF[k] * F[(size_t)j * N + k];
              double eo_ = std::exp(-f.eta * (old[j] + old[k] + rjk)) *
                           F[(size_t)i * N + j] * F[(size_t)i * N + k] *
                           F[(size_t)j * N + k];
              int idx[3] = {i, j, k};
              for (int q = 0; q < 3; ++q) {
                double vo = theta_part(to[q], f.lambda, f.zeta);
                double vn = theta_part(tn[q], f.lambda, f.zeta);
                double gv = g[idx[q]];
                gv += en_ * vn * f.tpz;
                gv -= eo_ * vo * f.tpz;
                g[idx[q]] = gv;
              }
            }
          }
        }
      }
      new_en = nn_energy(r, nG, r->new_eatom.data());
    }
  } else if (is_b(pot)) {  // energy_update! for the B potentials (:1508-1564)
    double* trow = r->trial_trow.data();
    for (int j = 0; j < N; ++j) trow[j] = tan_bc(r->bc, t, p + 3 * j, r->box[w], r->boxh[w]);
    trow[i] = 0.0;
    const bool cut = r->ens == ORC_NPT;
    const double rc2 = r->rcut2[w];
    const double* told = r->TN(w) + (size_t)i * N;
    double dE = dimer_atom_b(pot, i, row, trow, N, cut, rc2) - dimer_atom_b(pot, i, old, told, N, cut, rc2);
    new_en = dE + r->en[w];
  } else {  // dimer_energy_update! (:804-821)
    bool cut = r->ens == ORC_NPT;
    double rc2 = r->rcut2[w];
    double dE = dimer_atom(pot, i, row, N, cut, rc2) - dimer_atom(pot, i, old, N, cut, rc2);
    new_en = dE + r->en[w];
  }
  // acc_test! (MCRun.jl:122-132), metropolis_condition (Exchange.jl:53-57);
  // with delayed acceptance the second stage uses exp(-beta (dE - dE_s))
  double prob = std::exp(-((new_en - r->en[w]) - dEs) * r->beta[slot]);
  if (prob > 1) prob = 1.0;
  double u = r->draw(w);
  if (prob >= u) {  // swap_atom_config! (swap_config.jl:40-51)
    xi[0] = t[0];
    xi[1] = t[1];
    xi[2] = t[2];
    double* d = r->D(w);
    for (int j = 0; j < N; ++j) {
      d[(size_t)i * N + j] = row[j];
      d[(size_t)j * N + i] = row[j];
    }
    r->en[w] = new_en;
    r->cnt_atom[2 * slot] += 1;
    r->cnt_atom[2 * slot + 1] += 1;
    if (is_b(pot)) {  // swap_vars! B potentials (swap_config.jl:198-206)
      double* tm = r->TN(w);
      for (int j = 0; j < N; ++j) {
        tm[(size_t)i * N + j] = r->trial_trow[j];
        tm[(size_t)j * N + i] = r->trial_trow[j];
      }
    }
    if (pot.kind == ORC_POT_NN2) {  // swap_atom_config! + swap_vars! (swap_config.jl:40-51, 213-235)
      const size_t NN = (size_t)N * N;
      const int Ng = 2 * pot.nrad2 + 3 * pot.nang2;
      std::memcpy(&r->F[(size_t)w * NN], r->sc_f.data(), sizeof(double) * NN);
      std::memcpy(&r->G[(size_t)w * Ng * N], r->newG.data(), sizeof(double) * Ng * N);
      std::memcpy(&r->eatom[(size_t)w * N], r->new_eatom.data(), sizeof(double) * N);
    }
    if (pot.kind == ORC_POT_EAM) {  // swap_vars! EAM (:208-211)
      std::memcpy(&r->comp[(size_t)w * N * 2], r->new_comp.data(), sizeof(double) * 2 * N);
    } else if (pot.kind == ORC_POT_NN && !hard) {  // swap_vars! NNP (:213-221)
      int S = nsf(r);
      std::memcpy(&r->G[(size_t)w * S * N], r->newG.data(), sizeof(double) * S * N);
      std::memcpy(&r->eatom[(size_t)w * N], r->new_eatom.data(), sizeof(double) * N);
      double* F = &r->F[(size_t)w * N * N];
      for (int j = 0; j < N; ++j) {
        F[(size_t)i * N + j] = r->newF[j];
        F[(size_t)j * N + i] = r->newF[j];
      }
    }
  }
  return 0;
}

// volume move: volume_change (MCMoves.jl:350-356) with the NPT energy
// (MCRun.jl:76-85) and metropolis_condition NPT (Exchange.jl:58-70).
// Uniform (volume_change_uniform, :277-287): positions and box scaled by
// exp((u - 1/2) max_displ[2])^(1/3), distances scaled by scale^2.  Separated
// (volume_change_separated, :298-343): rand(1:6) picks z (1), xy (2-3) or all
// directions (4-6); the trial distance matrix is recomputed from the scaled
// positions in every case.
int volume_move(orc_run* r, int w, int slot) {
  int N = r->N;
  const double L = r->box[w], H = r->boxh[w];
  int xy_or_z = 0;
  double fx = 1.0, fz = 1.0;  // trial factors of x, y and of z
  double Ln = L, Hn = H;
  const bool rect = r->bc == ORC_BC_RECT || r->bc == ORC_BC_RHOMBIC;
  auto change_xyz = [&]() {  // volume_change_xyz (:169-177)
    double u = r->draw(w);
    double scale = std::pow(std::exp((u - 0.5) * r->maxd[2 * slot + 1]), 1.0 / 3.0);
    if (L >= r->max_box[slot] && scale > 1.0) scale = 1.0;
    fx = fz = scale;
    Ln = scale * L;
    Hn = rect ? scale * H : Ln;
  };
  if (r->sep) {
    const double lh = r->max_box[slot] / r->max_boxh[slot];  // lh_ratio (MCStates.jl:103)
    int ra = randint(r->draw(w), 6) + 1;
    if (ra == 1) {  // volume_change_z (:257-271)
      xy_or_z = 2;
      double u = r->draw(w);
      double scale = std::exp((u - 0.5) * r->maxd_sep[2 * slot + 1]);
      if (L / H <= lh * 1.1 && scale > 1.0) scale = 1 / scale;
      else if (L / H >= lh * 0.909 && scale < 1.0) scale = 1 / scale;
      if (H >= r->max_boxh[slot] && scale > 1.0) scale = 1 / scale;
      fz = scale;
      Hn = H * scale;
    } else if (ra <= 3) {  // volume_change_xy (:231-247)
      xy_or_z = 1;
      double u = r->draw(w);
      double scale = std::pow(std::exp((u - 0.5) * r->maxd_sep[2 * slot]), 0.5);
      if (L / H >= lh * 1.1 && scale > 1.0) scale = 1 / scale;
      else if (L / H <= lh * 0.909 && scale < 1.0) scale = 1 / scale;
      if (L >= r->max_box[slot] && scale > 1.0) scale = 1 / scale;
      fx = scale;
      Ln = L * scale;
    } else {
      change_xyz();
    }
  } else {
    change_xyz();
  }
  const double rc_new = box_rcut(r->bc, Ln, Hn);
  std::vector<double>& nd = r->sc_d2;
  std::vector<double>& np = r->sc_pos;
  const double* p = r->P(w);
  const bool bpot = is_b(r->pot);
  // tangents of the trial: recomputed for separated z / xy moves
  // (get_tantheta_mat!, MCMoves.jl:336-341), unchanged otherwise
  std::vector<double>& nt = r->sc_tn;
  if (bpot) {
    nt.resize((size_t)N * N);
    std::memcpy(nt.data(), r->TN(w), sizeof(double) * N * N);
  }
  if (r->sep) {  // get_distance2_mat! of the trial configuration
    np.resize((size_t)3 * N);
    for (int a = 0; a < N; ++a) {
      np[3 * a] = p[3 * a] * fx;
      np[3 * a + 1] = p[3 * a + 1] * fx;
      np[3 * a + 2] = p[3 * a + 2] * fz;
    }
    for (int i = 0; i < N; ++i) {
      nd[(size_t)i * N + i] = 0.0;
      for (int j = i + 1; j < N; ++j) {
        double x = dist2_bc(r->bc, &np[3 * i], &np[3 * j], Ln, Hn);
        nd[(size_t)i * N + j] = x;
        nd[(size_t)j * N + i] = x;
        if (bpot && xy_or_z != 0) {
          double y = tan_bc(r->bc, &np[3 * i], &np[3 * j], Ln, Hn);
          nt[(size_t)i * N + j] = y;
          nt[(size_t)j * N + i] = y;
        }
      }
    }
  } else {  // dist2_mat .* scale^2
    const double s2 = fx * fx;
    const double* d = r->D(w);
    for (size_t k = 0; k < (size_t)N * N; ++k) nd[k] = d[k] * s2;
  }
  double new_en = bpot ? dimer_config_b(r->pot, nd.data(), nt.data(), N, true, rc_new, r->bc, Ln, Hn)
                       : dimer_config(r->pot, nd.data(), N, true, rc_new, r->bc, Ln, Hn);
  double Vn = box_volume(r->bc, Ln, Hn), Vo = box_volume(r->bc, L, H);
  double dh = (new_en - r->en[w]) + r->pressure * (Vn - Vo);
  double prob = std::exp(-dh * r->beta[slot] + (double)N * std::log(Vn / Vo));
  if (prob > 1) prob = 1.0;
  double ua = r->draw(w);
  if (prob >= ua) {  // swap_config_v! (swap_config.jl:113-141)
    double* pw = r->P(w);
    if (r->sep) {
      std::memcpy(pw, np.data(), sizeof(double) * 3 * N);
    } else {
      for (int k = 0; k < 3 * N; ++k) pw[k] = fx * pw[k];
    }
    r->box[w] = Ln;
    r->boxh[w] = Hn;
    std::memcpy(r->D(w), nd.data(), sizeof(double) * N * N);
    if (bpot) std::memcpy(r->TN(w), nt.data(), sizeof(double) * N * N);
    r->en[w] = new_en;
    std::vector<long>& cv = xy_or_z == 0 ? r->cnt_vol : xy_or_z == 1 ? r->cnt_xy : r->cnt_z;
    cv[2 * slot] += 1;
    cv[2 * slot + 1] += 1;
    r->rcut2[w] = rc_new;
  }
  return 0;
}

// atom swap of the NNVT ensemble: swap_atoms (MCMoves.jl:363-370) draws one
// atom of each species, swap_energy_update (EnergyEvaluation.jl:1438-1446)
// gives the energy with the two positions exchanged, swap_move_config!
// (swap_config.jl:237-276) commits; swaps change no counter
int swap_move(orc_run* r, int w, int slot) {
  const int N = r->N;
  const Pot& pot = r->pot;
  const int n1 = pot.n1;
  const int i1 = randint(r->draw(w), n1);
  const int i2 = n1 + randint(r->draw(w), N - n1);
  const size_t NN = (size_t)N * N;
  const int Ng = 2 * pot.nrad2 + 3 * pot.nang2;
  const double* p = r->P(w);
  r->sc_pos.assign(p, p + 3 * (size_t)N);
  for (int k = 0; k < 3; ++k) std::swap(r->sc_pos[3 * i1 + k], r->sc_pos[3 * i2 + k]);
  // rows and columns i1 <-> i2 of the distance and cutoff matrices
  auto swapped = [&](const double* M, std::vector<double>& out, double diag) {
    out.assign(M, M + NN);
    for (int j = 0; j < N; ++j) {
      std::swap(out[(size_t)i1 * N + j], out[(size_t)i2 * N + j]);
    }
    for (int j = 0; j < N; ++j) {
      std::swap(out[(size_t)j * N + i1], out[(size_t)j * N + i2]);
    }
    out[(size_t)i1 * N + i1] = diag;
    out[(size_t)i2 * N + i2] = diag;
  };
  swapped(r->D(w), r->sc_d2, 0.0);
  swapped(&r->F[(size_t)w * NN], r->sc_f, 1.0);
  r->newG.resize((size_t)Ng * N);
  nn2_G(pot, r->sc_pos.data(), r->sc_d2.data(), r->sc_f.data(), N, r->newG.data());
  const double new_en = nn2_energy(pot, r->newG.data(), N, r->new_eatom.data());
  double prob = std::exp(-(new_en - r->en[w]) * r->beta[slot]);  // metropolis_condition
  if (prob > 1) prob = 1.0;
  if (prob >= r->draw(w)) {
    std::memcpy(r->P(w), r->sc_pos.data(), sizeof(double) * 3 * N);
    std::memcpy(r->D(w), r->sc_d2.data(), sizeof(double) * NN);
    std::memcpy(&r->F[(size_t)w * NN], r->sc_f.data(), sizeof(double) * NN);
    std::memcpy(&r->G[(size_t)w * Ng * N], r->newG.data(), sizeof(double) * Ng * N);
    std::memcpy(&r->eatom[(size_t)w * N], r->new_eatom.data(), sizeof(double) * N);
    r->en[w] = new_en;
    r->n_swaps_acc += 1;
  }
  return 0;
}

// mc_cycle! (MCRun.jl:192-213)
int cycle(orc_run* r, long index) {
  int R = r->R, N = r->N;
  int n_steps = r->ens == ORC_NPT ? N + 1 : r->ens == ORC_NNVT ? N + r->n_swaps : N;
  for (int s = 0; s < R; ++s) {  // mc_step! over states
    int w = r->wos[s];
    for (int k = 0; k < n_steps; ++k) {
      int idx = randint(r->draw(w), n_steps);
      int rc = idx < N                 ? atom_move(r, w, s, idx)
               : r->ens == ORC_NNVT ? swap_move(r, w, s)
                                    : volume_move(r, w, s);
      if (rc) return rc;
    }
  }
  // parallel_tempering_exchange! (Exchange.jl:132-180)
  if (R > 1 && r->draw_run() < r->exch_prob) {
    int k = randint(r->draw_run(), R - 1);
    r->cnt_exc[2 * k] += 1;
    r->cnt_exc[2 * (k + 1)] += 1;
    int w1 = r->wos[k], w2 = r->wos[k + 1];
    double e1 = r->en[w1], e2 = r->en[w2];
    if (r->ens == ORC_NPT) {
      e1 = e1 + r->pressure * box_volume(r->bc, r->box[w1], r->boxh[w1]);
      e2 = e2 + r->pressure * box_volume(r->bc, r->box[w2], r->boxh[w2]);
    }
    double acc = std::exp((r->beta[k] - r->beta[k + 1]) * (e1 - e2));
    if (acc > 1.0) acc = 1.0;
    if (acc > r->draw_run()) {
      r->cnt_exc[2 * k + 1] += 1;
      r->cnt_exc[2 * (k + 1) + 1] += 1;
      r->wos[k] = w2;
      r->wos[k + 1] = w1;
    }
  }
  // update_max_stepsize! (Exchange.jl:198-257)
  if (index % r->n_adjust == 0) {
    for (int s = 0; s < R; ++s) {
      double acc = (double)r->cnt_atom[2 * s + 1] / (double)(r->n_adjust * N);
      if (acc < r->min_acc) r->maxd[2 * s] *= 0.9;
      else if (acc > r->max_acc) r->maxd[2 * s] *= 1.1;
      r->cnt_atom[2 * s + 1] = 0;
      if (r->ens == ORC_NPT && !r->sep) {
        double av = (double)r->cnt_vol[2 * s + 1] / (double)(r->n_adjust * 1);
        if (av < r->min_acc) r->maxd[2 * s + 1] *= 0.9;
        else if (av > r->max_acc) r->maxd[2 * s + 1] *= 1.1;
        r->cnt_vol[2 * s + 1] = 0;
      } else if (r->ens == ORC_NPT) {  // separated: all, xy, z (Exchange.jl:221-244)
        auto adapt = [&](std::vector<long>& cv, double& md, double den) {
          double av = (double)cv[2 * s + 1] / den;
          if (av < r->min_acc) md *= 0.9;
          else if (av > r->max_acc) md *= 1.1;
          cv[2 * s + 1] = 0;
        };
        const double nu = (double)(r->n_adjust * 1);
        adapt(r->cnt_vol, r->maxd[2 * s + 1], nu * 1 / 2);
        adapt(r->cnt_xy, r->maxd_sep[2 * s], nu * 1 / 3);
        adapt(r->cnt_z, r->maxd_sep[2 * s + 1], nu / 6);
      }
    }
  }
  return 0;
}

// find_hist_index (Sampling.jl:53-62)
inline long hist_index(double h, int n_bin) {
  if (!(h >= 1)) return 1;  // NaN lands in the underflow bin (the reference throws)
  if (h > n_bin) return n_bin + 2;
  return (long)std::floor(h) + 1;
}

// sampling_step! (Sampling.jl:330-371)
// update_rdf! (Sampling.jl:282, 301-316): dist2_mat[i, k], k <= i, of each
// slot's configuration; rdf_index = floor(r2 / delta_r2), kept when != 0 and
// <= 5 n_bin (1-based)
void update_rdf(orc_run* r) {
  const int N = r->N, nb5 = 5 * r->n_bin;
  for (int s = 0; s < r->R; ++s) {
    const double* d = r->D(r->wos[s]);
    for (int i = 0; i < N; ++i)
      for (int k = 0; k <= i; ++k) {
        const double idx = std::floor(d[(size_t)i * N + k] / r->dr2);
        if (idx != 0 && idx <= nb5) r->rdf[(size_t)s * nb5 + (size_t)idx - 1] += 1;
      }
  }
}

// sampling_step! (Sampling.jl:330-371) of production cycle `idx`
void sample(orc_run* r, long idx) {
  if (r->rdf_on && idx % 1000 == 0) update_rdf(r);
  int R = r->R, nb = r->n_bin + 2;
  for (int s = 0; s < R; ++s) {
    int w = r->wos[s];
    double e = r->en[w];
    if (r->ens == ORC_NPT) {
      double L = r->box[w], Hb = r->boxh[w];
      double H = e + r->pressure * box_volume(r->bc, L, Hb);  // update_energy_tot :35-46
      r->ham[2 * s] += H;
      r->ham[2 * s + 1] += H * H;
      double he = std::floor((e - r->en_min) / r->dE) + 1;  // :98-130
      // the volume of the histogram index: L^3, L^2 H, and for the rhombic
      // box L^2 * 3 H^0.5 / 2 as written at Sampling.jl:119-121
      double vh = r->bc == ORC_BC_RECT      ? L * L * Hb
                  : r->bc == ORC_BC_RHOMBIC ? L * L * (3 * std::sqrt(Hb)) / 2
                                            : L * L * L;
      double hv = std::floor((vh - r->v_min) / r->dV) + 1;
      long ie = hist_index(he, r->n_bin), iv = hist_index(hv, r->n_bin);
      r->ev_hist[((size_t)s * nb + (ie - 1)) * nb + (iv - 1)] += 1;
    } else {
      r->ham[2 * s] += e;
      r->ham[2 * s + 1] += e * e;
      long ie = hist_index((e - r->en_min) / r->dE + 1, r->n_bin);
      r->en_hist[(size_t)s * nb + (ie - 1)] += 1;
    }
  }
}

}  // namespace

// ================================================================ C API
extern "C" {

const char* orc_last_error(void) { return g_err.c_str(); }

double orc_u01(uint64_t seed, uint32_t stream, uint32_t run, uint64_t idx) {
  return u01(seed, stream, run, idx);
}
void orc_philox4x32(const uint32_t* ctr, const uint32_t* key, uint32_t* out) {
  uint32_t c[4] = {ctr[0], ctr[1], ctr[2], ctr[3]};
  philox(c, key[0], key[1]);
  for (int k = 0; k < 4; ++k) out[k] = c[k];
}

orc_run* orc_create(int N, int R, int ensemble, double pressure, int bc_kind,
                    double bc_param, const double* xyz, const double* T,
                    const double* max_displ, int n_bin, int n_adjust,
                    int mc_sample, double min_acc, double max_acc,
                    double exch_prob, uint64_t seed, int run_index) {
  if (N < 2 || R < 1) {
    fail("orc_create: need N >= 2 and R >= 1");
    return nullptr;
  }
  if (ensemble == ORC_NPT && bc_kind == ORC_BC_SPHERE) {
    fail("SphericalBC cannot be used in an NPT ensemble.");  // Ensembles.jl:192
    return nullptr;
  }
  orc_run* r = new orc_run();
  r->N = N;
  r->R = R;
  r->ens = ensemble;
  r->bc = bc_kind;
  r->pressure = pressure;
  r->exch_prob = exch_prob;
  r->min_acc = min_acc;
  r->max_acc = max_acc;
  r->n_bin = n_bin;
  r->n_adjust = n_adjust;
  r->mc_sample = mc_sample;
  r->seed = seed;
  r->run_index = run_index;
  r->pos.assign(xyz, xyz + (size_t)R * N * 3);
  r->d2.assign((size_t)R * N * N, 0.0);
  r->en.assign(R, 0.0);
  r->box.assign(R, bc_param);
  r->boxh.assign(R, bc_param);
  r->rcut2.assign(R, box_rcut(bc_kind, bc_param, bc_param));
  r->ctr.assign(R, 0);
  r->T.assign(T, T + R);
  r->beta.resize(R);
  for (int s = 0; s < R; ++s) r->beta[s] = 1.0 / (kB * T[s]);  // InputParams.jl:93
  r->maxd.assign(max_displ, max_displ + 2 * R);
  r->max_box.assign(R, bc_param * 1.8);  // max_length (MCStates.jl:66-75)
  r->max_boxh.assign(R, bc_param * 1.8);  // max_height (MCStates.jl:79-87)
  r->maxd_sep.assign(2 * R, 0.1);         // max_displ[3:4] (MCStates.jl:101)
  r->ham.assign(2 * R, 0.0);
  r->cnt_atom.assign(2 * R, 0);
  r->cnt_vol.assign(2 * R, 0);
  r->cnt_exc.assign(2 * R, 0);
  r->cnt_xy.assign(2 * R, 0);
  r->cnt_z.assign(2 * R, 0);
  r->wos.resize(R);
  for (int s = 0; s < R; ++s) r->wos[s] = s;
  r->trial_row.resize(N);
  r->trial_trow.resize(N);
  r->new_comp.resize(2 * N);
  r->sc_d2.resize((size_t)N * N);
  r->newF.resize(N);
  r->new_eatom.resize(N);
  return r;
}

void orc_destroy(orc_run* r) { delete r; }

int orc_set_box(orc_run* r, double height, int separated, const double* max_displ_sep) {
  if (r->inited) return fail("orc_set_box: call before orc_init");
  if (r->bc != ORC_BC_RECT && r->bc != ORC_BC_RHOMBIC) {
    if (separated) return fail("separated volume moves need a RectangularBC or RhombicBC");
    return 0;
  }
  if (!(height > 0)) return fail("box height must be positive");
  if (separated && r->ens != ORC_NPT) return fail("separated volume moves are NPT moves");
  for (int w = 0; w < r->R; ++w) {
    r->boxh[w] = height;
    r->rcut2[w] = box_rcut(r->bc, r->box[w], height);
    r->max_boxh[w] = height * 1.8;
  }
  r->sep = separated != 0;
  if (max_displ_sep) r->maxd_sep.assign(max_displ_sep, max_displ_sep + 2 * r->R);
  return 0;
}
int orc_get_box(orc_run* r, double* height, double* max_displ_sep, long* count_xy, long* count_z) {
  int R = r->R;
  if (height) std::memcpy(height, r->boxh.data(), sizeof(double) * R);
  if (max_displ_sep) std::memcpy(max_displ_sep, r->maxd_sep.data(), sizeof(double) * 2 * R);
  if (count_xy) std::memcpy(count_xy, r->cnt_xy.data(), sizeof(long) * 2 * R);
  if (count_z) std::memcpy(count_z, r->cnt_z.data(), sizeof(long) * 2 * R);
  return 0;
}

int orc_set_pot_elj(orc_run* r, const double* c, int K, int even) {
  if (K < 1) return fail("ELJ needs at least one coefficient");
  r->pot.kind = even ? ORC_POT_ELJEVEN : ORC_POT_ELJ;
  r->pot.c.assign(c, c + K);
  if (r->ens == ORC_NPT && !even)
    return fail("NPT long-range correction is defined for ELJPotentialEven only");
  return 0;
}
int orc_set_pot_eljb(orc_run* r, const double* a, const double* b, const double* c, int K) {
  if (K < 2) return fail("ELJPotentialB needs at least two coefficients");
  r->pot.kind = ORC_POT_ELJB;
  r->pot.a.assign(a, a + K);
  r->pot.b.assign(b, b + K);
  r->pot.c.assign(c, c + K);
  r->tn.assign((size_t)r->R * r->N * r->N, 0.0);
  return 0;
}
int orc_set_pot_lut(orc_run* r, const double* table, int l_angle, int l_dist, double start_dist,
                    double start_angle, double d_dist, double d_angle, double c6) {
  if (l_angle < 1 || l_dist < 1 || !(d_dist > 0) || !(d_angle > 0))
    return fail("lookup table: bad dimensions");
  r->pot.kind = ORC_POT_LUT;
  r->pot.lut.assign(table, table + (size_t)l_angle * l_dist);
  r->pot.l_angle = l_angle;
  r->pot.l_dist = l_dist;
  r->pot.start_dist = start_dist;
  r->pot.start_angle = start_angle;
  r->pot.d_dist = d_dist;
  r->pot.d_angle = d_angle;
  r->pot.c6 = c6;
  r->tn.assign((size_t)r->R * r->N * r->N, 0.0);
  return 0;
}
int orc_set_pot_nn2(orc_run* r, const double* rad, int nrad, const double* ang, int nang,
                    const double* w1, const double* w2, int nw, const int* nodes, int n_layers,
                    int n1, int n_swaps) {
  if (r->ens != ORC_NNVT) return fail("RuNNerPotential2Atom runs in the NNVT ensemble");
  if (r->bc != ORC_BC_SPHERE) return fail("RuNNerPotential2Atom: SphericalBC only");
  if (nrad < 1 || n1 < 1 || n1 >= r->N) return fail("NNVT: need radial functions and both species");
  const int Ng = 2 * nrad + 3 * nang;
  if (n_layers < 2 || nodes[0] != Ng || nodes[n_layers - 1] != 1)
    return fail("NN2: node counts must start at 2 nrad + 3 nang and end at 1");
  long need = 0;
  for (int l = 1; l < n_layers; ++l) need += (long)nodes[l - 1] * nodes[l] + nodes[l];
  if (need != nw) return fail("NN2: weight count does not match the layer sizes");
  Pot& p = r->pot;
  p.kind = ORC_POT_NN2;
  p.n1 = n1;
  p.nrad2 = nrad;
  p.nang2 = nang;
  p.rad2.assign(rad, rad + 10 * (size_t)nrad);
  p.ang2.assign(ang, ang + 16 * (size_t)nang);
  p.w.assign(w1, w1 + nw);
  p.w_b.assign(w2, w2 + nw);
  p.nodes.assign(nodes, nodes + n_layers);
  r->n_swaps = n_swaps;
  r->G.assign((size_t)r->R * Ng * r->N, 0.0);
  r->F.assign((size_t)r->R * r->N * r->N, 0.0);
  r->eatom.assign((size_t)r->R * r->N, 0.0);
  r->new_eatom.resize(r->N);
  return 0;
}
int orc_set_pot_eam(orc_run* r, double n, double m, double ean, double ecam) {
  if (r->ens == ORC_NPT) return fail("EAM is supported in the NVT ensemble only");
  r->pot.kind = ORC_POT_EAM;
  r->pot.n = n;
  r->pot.m = m;
  r->pot.ean = ean;
  r->pot.ecam = ecam;
  return 0;
}
int orc_set_pot_nn(orc_run* r, const double* sf, int nsf_, const double* weights,
                   int nw, const int* nodes, int n_layers, double boundary) {
  if (r->ens == ORC_NPT) return fail("NN potential is supported in the NVT ensemble only");
  if (n_layers < 2 || nodes[0] != nsf_ || nodes[n_layers - 1] != 1)
    return fail("NN: node counts must start at the number of symmetry functions and end at 1");
  long need = 0;
  for (int l = 1; l < n_layers; ++l) need += (long)nodes[l - 1] * nodes[l] + nodes[l];
  if (need != nw) return fail("NN: weight count does not match the layer sizes");
  for (int l = 0; l < n_layers; ++l)
    if (nodes[l] > 256) return fail("NN: layers wider than 256 are not supported");
  r->pot.kind = ORC_POT_NN;
  r->pot.sf.clear();
  for (int s = 0; s < nsf_; ++s) {
    const double* q = sf + 8 * s;
    SF f;
    f.kind = (int)q[0];
    f.type = (int)q[1];
    f.eta = q[2];
    f.lambda = q[3];
    f.zeta = q[4];
    f.rcut = q[5];
    double gmin = q[6], gmax = q[7];
    // RadialType2 / AngularType3 with G_vals = [max, min] (SymmFunc.jl:37-44,104-112)
    f.gnorm = 1 / (gmax - gmin);
    f.goffset = -gmin * f.gnorm;
    f.tpz = std::pow(2.0, 1 - f.zeta) * f.gnorm;
    r->pot.sf.push_back(f);
  }
  r->pot.rcut = r->pot.sf.empty() ? 0.0 : r->pot.sf[0].rcut;
  r->pot.w.assign(weights, weights + nw);
  r->pot.nodes.assign(nodes, nodes + n_layers);
  r->pot.boundary2 = boundary * boundary;
  r->G.assign((size_t)r->R * nsf_ * r->N, 0.0);
  r->F.assign((size_t)r->R * r->N * r->N, 0.0);
  r->eatom.assign((size_t)r->R * r->N, 0.0);
  r->newG.resize((size_t)nsf_ * r->N);
  return 0;
}

int orc_init(orc_run* r) {
  if (r->pot.kind < 0) return fail("no potential set");
  if (r->pot.kind == ORC_POT_EAM) r->comp.assign((size_t)r->R * r->N * 2, 0.0);
  for (int w = 0; w < r->R; ++w) {
    build_d2(r, w);
    r->en[w] = init_energy(r, w);
  }
  r->inited = true;
  return 0;
}

int orc_cycles(orc_run* r, long first, long n) {
  if (!r->inited) return fail("orc_init not called");
  for (long i = first; i < first + n; ++i) {
    int rc = cycle(r, i);
    if (rc) return rc;
  }
  return 0;
}

int orc_equilibrate(orc_run* r, int eq_cycles) {
  if (!r->inited) return fail("orc_init not called");
  for (long i = 1; i <= eq_cycles / 2; ++i) {
    int rc = cycle(r, i);
    if (rc) return rc;
  }
  double eb[2] = {100.0, -100.0};  // check_e_bounds (MCRun.jl:258-265)
  for (long i = eq_cycles / 2 + 1; i <= eq_cycles; ++i)
    for (int s = 0; s < r->R; ++s) {
      double e = r->en[r->wos[s]];
      if (e < eb[0]) eb[0] = e;
      else if (e > eb[1]) eb[1] = e;
    }
  for (int k = 0; k < 2 * r->R; ++k) {  // reset_counters (MCRun.jl:271-277)
    r->cnt_atom[k] = 0;
    r->cnt_vol[k] = 0;
    r->cnt_exc[k] = 0;
    r->cnt_xy[k] = 0;
    r->cnt_z[k] = 0;
  }
  // initialise_histograms! (Sampling.jl:141-194)
  r->en_min = eb[0];
  r->en_max = eb[1];
  r->dE = (r->en_max - r->en_min) / (r->n_bin - 1);
  int nb = r->n_bin + 2;
  r->en_hist.assign((size_t)r->R * nb, 0.0);
  const double b = r->box[r->wos[0]], bh = r->boxh[r->wos[0]];  // the first state's box
  if (r->ens == ORC_NPT) {
    const double V = box_volume(r->bc, b, bh);
    r->v_min = V * 0.8;
    r->v_max = V * 2.0;
    r->dV = (r->v_max - r->v_min) / r->n_bin;
    r->ev_hist.assign((size_t)r->R * nb * nb, 0.0);
  }
  // delta_r2 (Sampling.jl:151 sphere, :185 cube, :210 rhombic, :240 rectangular)
  if (r->bc == ORC_BC_CUBIC) r->dr2 = 3.0 / 4.0 * (b * b) / r->n_bin / 5;
  else if (r->bc == ORC_BC_RHOMBIC) r->dr2 = (3.0 / 8.0 * (b * b) + 1.0 / 4.0 * (bh * bh)) / r->n_bin / 5;
  else if (r->bc == ORC_BC_RECT) r->dr2 = (1.0 / 2.0 * (b * b) + 1.0 / 4.0 * (bh * bh)) / r->n_bin / 5;
  else r->dr2 = 4 * (b * b) / r->n_bin / 5;
  r->rdf.assign((size_t)r->R * 5 * r->n_bin, 0.0);
  return 0;
}

int orc_set_rdf(orc_run* r, int on) {
  r->rdf_on = on != 0;
  return 0;
}
int orc_get_rdf(orc_run* r, double* rdf, double* dr2) {
  if (rdf && !r->rdf.empty()) std::memcpy(rdf, r->rdf.data(), sizeof(double) * r->rdf.size());
  if (dr2) *dr2 = r->dr2;
  return 0;
}

int orc_production(orc_run* r, long first, long n) {
  if (r->en_hist.empty()) return fail("orc_equilibrate not called");
  for (long i = first; i < first + n; ++i) {
    int rc = cycle(r, i);
    if (rc) return rc;
    if (i % r->mc_sample == 0) sample(r, i);
  }
  return 0;
}

int orc_get_walkers(orc_run* r, double* xyz, double* en_tot, double* box) {
  if (xyz) std::memcpy(xyz, r->pos.data(), sizeof(double) * r->pos.size());
  if (en_tot) std::memcpy(en_tot, r->en.data(), sizeof(double) * r->R);
  if (box) std::memcpy(box, r->box.data(), sizeof(double) * r->R);
  return 0;
}

int orc_get_slots(orc_run* r, int* wos, double* max_displ, long* ca, long* cv,
                  long* ce, double* ham) {
  int R = r->R;
  if (wos) std::memcpy(wos, r->wos.data(), sizeof(int) * R);
  if (max_displ) std::memcpy(max_displ, r->maxd.data(), sizeof(double) * 2 * R);
  if (ca) std::memcpy(ca, r->cnt_atom.data(), sizeof(long) * 2 * R);
  if (cv) std::memcpy(cv, r->cnt_vol.data(), sizeof(long) * 2 * R);
  if (ce) std::memcpy(ce, r->cnt_exc.data(), sizeof(long) * 2 * R);
  if (ham) std::memcpy(ham, r->ham.data(), sizeof(double) * 2 * R);
  return 0;
}

int orc_get_hist(orc_run* r, double* en_hist, double* ev_hist, double* hp) {
  if (en_hist && !r->en_hist.empty() && r->ens == ORC_NVT)
    std::memcpy(en_hist, r->en_hist.data(), sizeof(double) * r->en_hist.size());
  if (ev_hist && !r->ev_hist.empty())
    std::memcpy(ev_hist, r->ev_hist.data(), sizeof(double) * r->ev_hist.size());
  if (hp) {
    hp[0] = r->en_min;
    hp[1] = r->en_max;
    hp[2] = r->v_min;
    hp[3] = r->v_max;
    hp[4] = r->dE;
    hp[5] = r->dV;
  }
  return 0;
}

int orc_finalise(orc_run* r, long mc_cycles, int mc_sample, double* en_avg,
                 double* heat_cap, double* stat_atom, double* stat_exc) {
  double n_sample = (double)mc_cycles / (double)mc_sample;
  for (int s = 0; s < r->R; ++s) {
    double ea = r->ham[2 * s] / n_sample;
    double e2 = r->ham[2 * s + 1] / n_sample;
    if (en_avg) en_avg[s] = ea;
    if (heat_cap) heat_cap[s] = (e2 - ea * ea) * (r->beta[s] * r->beta[s]);
    if (stat_atom) stat_atom[s] = (double)r->cnt_atom[2 * s] / (double)((long)r->N * mc_cycles);
    if (stat_exc) stat_exc[s] = (double)r->cnt_exc[2 * s + 1] / (double)r->cnt_exc[2 * s];
  }
  return 0;
}

long orc_get_swaps(orc_run* r) { return r->n_swaps_acc; }

int orc_get_nn_state(orc_run* r, int w, double* G, double* eatom) {
  if (r->pot.kind != ORC_POT_NN && r->pot.kind != ORC_POT_NN2) return fail("not an NN run");
  int S = r->pot.kind == ORC_POT_NN2 ? 2 * r->pot.nrad2 + 3 * r->pot.nang2 : nsf(r), N = r->N;
  if (G) std::memcpy(G, &r->G[(size_t)w * S * N], sizeof(double) * S * N);
  if (eatom) std::memcpy(eatom, &r->eatom[(size_t)w * N], sizeof(double) * N);
  return 0;
}

double orc_dimer_energy(int kind, const double* c, int K, double r2) {
  return kind == ORC_POT_ELJ ? elj_all(c, K, r2) : elj_even(c, K, r2);
}
double orc_distance2(const double* a, const double* b, int bc_kind, double L) {
  return dist2_bc(bc_kind, a, b, L, L);
}
double orc_distance2_box(const double* a, const double* b, int bc_kind, double L, double H) {
  return dist2_bc(bc_kind, a, b, L, H);
}
double orc_box_rcut(int bc_kind, double L, double H) { return box_rcut(bc_kind, L, H); }
double orc_get_tan(const double* a, const double* b, int bc_kind, double L, double H) {
  return tan_bc(bc_kind, a, b, L, H);
}
double orc_eljb_energy(const double* a, const double* b, const double* c, int K, double r2,
                       double tn) {
  Pot p;
  p.kind = ORC_POT_ELJB;
  p.a.assign(a, a + K);
  p.b.assign(b, b + K);
  p.c.assign(c, c + K);
  return eljb(p, r2, tn);
}
double orc_lut_energy(const double* table, int l_angle, int l_dist, double start_dist,
                      double d_dist, double d_angle, double c6, double r2, double tn) {
  Pot p;
  p.kind = ORC_POT_LUT;
  p.lut.assign(table, table + (size_t)l_angle * l_dist);
  p.l_angle = l_angle;
  p.l_dist = l_dist;
  p.start_dist = start_dist;
  p.d_dist = d_dist;
  p.d_angle = d_angle;
  p.c6 = c6;
  return lut_energy(p, r2, tn);
}
double orc_box_volume(int bc_kind, double L, double H) { return box_volume(bc_kind, L, H); }
double orc_lrc(int N, double r_cut2, const double* c, int K) {
  return lrc_even(N, r_cut2, c, K);
}
double orc_eam_config_energy(const double* xyz, int N, double n, double m,
                             double ean, double ecam) {
  std::vector<double> comp(2 * N, 0.0);
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < N; ++j) {
      double a, b;
      invrexp(i == j ? 0.0 : dist2_sph(xyz + 3 * i, xyz + 3 * j), n, m, a, b);
      comp[2 * i] += a;
      comp[2 * i + 1] += b;
    }
  return eam_energy(comp.data(), N, ean, ecam);
}
double orc_elj_config_energy(const double* xyz, int N, int kind,
                             const double* c, int K, int bc_kind, double L,
                             double r_cut2) {
  Pot p;
  p.kind = kind;
  p.c.assign(c, c + K);
  std::vector<double> d((size_t)N * N, 0.0);
  for (int i = 0; i < N; ++i)
    for (int j = i + 1; j < N; ++j) {
      double x = dist2_bc(bc_kind, xyz + 3 * i, xyz + 3 * j, L, L);
      d[(size_t)i * N + j] = d[(size_t)j * N + i] = x;
    }
  return dimer_config(p, d.data(), N, bc_kind == ORC_BC_CUBIC, r_cut2);
}
double orc_elj_config_energy_box(const double* xyz, int N, int kind, const double* c, int K,
                                 int bc_kind, double L, double H, int cut) {
  Pot p;
  p.kind = kind;
  p.c.assign(c, c + K);
  std::vector<double> d((size_t)N * N, 0.0);
  for (int i = 0; i < N; ++i)
    for (int j = i + 1; j < N; ++j) {
      double x = dist2_bc(bc_kind, xyz + 3 * i, xyz + 3 * j, L, H);
      d[(size_t)i * N + j] = d[(size_t)j * N + i] = x;
    }
  return dimer_config(p, d.data(), N, cut != 0, box_rcut(bc_kind, L, H), bc_kind, L, H);
}
void orc_tempgrid(double ti, double tf, int R, int tdistr, double* T, double* beta) {
  // TempGrid (InputParams.jl:77-95)
  for (int i = 0; i < R; ++i) {
    if (tdistr == 1) T[i] = ti + i * ((tf - ti) / (R - 1));
    else T[i] = ti * std::pow(tf / ti, (double)i / (double)(R - 1));
    beta[i] = 1.0 / (kB * T[i]);
  }
}
int orc_mlp_forward(const double* input, int n_in, int batch,
                    const double* weights, int nw, const int* nodes,
                    int n_layers, double* eatom) {
  (void)nw;
  if (nodes[0] != n_in) return fail("input width mismatch");
  for (int b = 0; b < batch; ++b)
    eatom[b] = mlp_atom(input + (size_t)b * n_in, weights, nodes, n_layers);
  return 0;
}

// ---------------------------------------------------------------- surrogate
static SurCfg sur_cfg(const double* cfg) {
  SurCfg c;
  c.r_lo = cfg[0];
  c.r_hi = cfg[1];
  c.gamma = cfg[2];
  c.r_cut = cfg[3];
  c.escale = cfg[4];
  return c;
}
int orc_sur_nparams(void) { return SUR_NP; }
int orc_sur_forward(const double* cfg, const double* params, const float* rows, int n, int bf16,
                    double* dEs) {
  SurCfg c = sur_cfg(cfg);
  for (int b = 0; b < n; ++b) dEs[b] = sur_delta(c, params, rows + (size_t)b * SUR_ROWS, bf16 != 0);
  return 0;
}
int orc_sur_loss_grad(const double* cfg, const double* params, const float* rows,
                      const float* targets, int n, int bf16, double* loss, double* grad) {
  if (n < 1) return fail("need at least one record");
  *loss = sur_loss_grad(sur_cfg(cfg), params, rows, targets, n, bf16 != 0, grad);
  return 0;
}
int orc_set_surrogate(orc_run* r, const double* cfg, const double* params, int bf16) {
  if (!params) {
    r->da = false;
    return 0;
  }
  if (r->pot.kind != ORC_POT_NN) return fail("delayed acceptance needs the NN potential");
  if (r->N > SUR_ROWS / 2) return fail("delayed acceptance: at most 64 atoms");
  r->sc = sur_cfg(cfg);
  r->sp.assign(params, params + SUR_NP);
  r->da_bf = bf16 != 0;
  r->da = true;
  return 0;
}
int orc_get_sur_stats(orc_run* r, long* out) {
  out[0] = r->da_reject1;
  out[1] = r->da_exact;
  return 0;
}

// ---------------------------------------------------------------- linear multihistogram
// multihistogram(output, Tvec) of src/multihist.jl:25-487: readfile (:55-79),
// processhist! (:89-114), bvector (:166-210), amatrix (:215-232), systemsolver
// (:237-270), Entropycalc (:275-283), analysis (:292-375).  The matrix A is
// singular (its rows sum to zero; b is consistent), so the reference's A \ b
// returns alpha up to an additive constant chosen by LAPACK's rounding; here
// the last equation is replaced by alpha[R-1] = 0 (Gaussian elimination with
// partial pivoting).  A constant in alpha shifts S(E) by a constant, which
// leaves U, Cv and dCv unchanged (Z and S(T) change by the factor / offset).
int orc_multihist_linear(int R, int n_bin, const double* en_hist, const double* beta,
                         double en_min, double en_max, int npoints, double* energies,
                         double* S_E, int* n_kept, double* alpha, double* T_out, double* Z,
                         double* U, double* Cv, double* dCv, double* S_T) {
  const double kB = 3.16681196E-6;  // multihist.jl:57
  const int nb = n_bin + 2;
  const double de = (en_max - en_min) / (n_bin - 1);
  std::vector<double> H((size_t)R * n_bin), E(n_bin);
  for (int j = 0; j < n_bin; ++j) E[j] = j * de + en_min;
  for (int i = 0; i < R; ++i)
    for (int j = 0; j < n_bin; ++j) H[(size_t)i * n_bin + j] = en_hist[(size_t)i * nb + j + 1] / n_bin;
  // processhist!: drop bins with no counts
  std::vector<int> keep;
  std::vector<double> nsum;
  for (int j = 0; j < n_bin; ++j) {
    double t = 0;
    for (int i = 0; i < R; ++i) t += H[(size_t)i * n_bin + j];
    if (t != 0) {
      keep.push_back(j);
      nsum.push_back(t);
    }
  }
  const int B = (int)keep.size();
  if (B == 0) return fail("multihistogram: empty histograms");
  std::vector<double> h((size_t)R * B), ev(B), bmat((size_t)R * B), rh(B, 0.0), b(R, 0.0);
  for (int k = 0; k < B; ++k) {
    ev[k] = E[keep[k]];
    for (int i = 0; i < R; ++i) h[(size_t)i * B + k] = H[(size_t)i * n_bin + keep[k]];
  }
  for (int i = 0; i < R; ++i)  // bvector
    for (int k = 0; k < B; ++k) {
      double x = h[(size_t)i * B + k];
      bmat[(size_t)i * B + k] = x == 0.0 ? 0.0 : x * (std::log(x) + beta[i] * ev[k]);
    }
  for (int k = 0; k < B; ++k)
    for (int i = 0; i < R; ++i) rh[k] += bmat[(size_t)i * B + k];
  for (int i = 0; i < R; ++i)
    for (int k = 0; k < B; ++k) b[i] += bmat[(size_t)i * B + k] - h[(size_t)i * B + k] * rh[k] / nsum[k];
  std::vector<double> A((size_t)R * R, 0.0);  // amatrix
  for (int i = 0; i < R; ++i)
    for (int ip = 0; ip < R; ++ip) {
      double t = 0;
      for (int k = 0; k < B; ++k) t += h[(size_t)i * B + k] * h[(size_t)ip * B + k] / nsum[k];
      A[(size_t)i * R + ip] = -t;
      if (i == ip) {
        double d = 0;
        for (int k = 0; k < B; ++k) d += h[(size_t)i * B + k];
        A[(size_t)i * R + ip] += d;
      }
    }
  // gauge: alpha[R-1] = 0 in place of the last (dependent) equation
  for (int ip = 0; ip < R; ++ip) A[(size_t)(R - 1) * R + ip] = ip == R - 1 ? 1.0 : 0.0;
  b[R - 1] = 0.0;
  std::vector<double> x(b);
  for (int col = 0; col < R; ++col) {  // Gaussian elimination, partial pivoting
    int piv = col;
    for (int rr = col + 1; rr < R; ++rr)
      if (std::fabs(A[(size_t)rr * R + col]) > std::fabs(A[(size_t)piv * R + col])) piv = rr;
    if (A[(size_t)piv * R + col] == 0.0) return fail("multihistogram: singular system");
    if (piv != col) {
      for (int cc = 0; cc < R; ++cc) std::swap(A[(size_t)piv * R + cc], A[(size_t)col * R + cc]);
      std::swap(x[piv], x[col]);
    }
    for (int rr = col + 1; rr < R; ++rr) {
      const double f = A[(size_t)rr * R + col] / A[(size_t)col * R + col];
      for (int cc = col; cc < R; ++cc) A[(size_t)rr * R + cc] -= f * A[(size_t)col * R + cc];
      x[rr] -= f * x[col];
    }
  }
  for (int rr = R - 1; rr >= 0; --rr) {
    double t = x[rr];
    for (int cc = rr + 1; cc < R; ++cc) t -= A[(size_t)rr * R + cc] * x[cc];
    x[rr] = t / A[(size_t)rr * R + rr];
  }
  std::vector<double> S(B);  // Entropycalc
  for (int k = 0; k < B; ++k) {
    double t = 0;
    for (int i = 0; i < R; ++i) t += bmat[(size_t)i * B + k] - h[(size_t)i * B + k] * x[i];
    S[k] = t / nsum[k];
  }
  // analysis
  const double T0 = 1 / (kB * beta[0]), T1 = 1 / (kB * beta[R - 1]);
  const double dT = (T1 - T0) / npoints;
  double nexp = 0;
  std::vector<double> XP(B);
  for (int p = 0; p < npoints; ++p) {
    const double T = p * dT + T0;
    double z = 0;
    for (long guard = 0;; ++guard) {
      if (guard > 10000000) return fail("multihistogram: partition-function scaling did not settle");
      z = 0;
      for (int k = 0; k < B; ++k) {
        XP[k] = std::exp((S[k] - ev[k] / (T * kB)) - nexp);
        z += XP[k];
      }
      if (z < 1.0) nexp -= 1.0;
      else if (z > 100.0) nexp += 0.7;
      else break;
    }
    double u = 0, u2 = 0;
    for (int k = 0; k < B; ++k) {
      u += XP[k] * ev[k];
      u2 += XP[k] * ev[k] * ev[k];
    }
    u /= z;
    u2 /= z;
    double r2 = 0, r3 = 0;
    for (int k = 0; k < B; ++k) {
      const double d = ev[k] - u;
      r2 += XP[k] * d * d;
      r3 += XP[k] * d * d * d;
    }
    r2 /= z;
    r3 /= z;
    if (T_out) T_out[p] = T;
    if (Z) Z[p] = z;
    if (U) U[p] = u;
    if (Cv) Cv[p] = (u2 - u * u) / kB / (T * T);
    if (S_T) S_T[p] = u / T + kB * std::log(z);
    if (dCv) dCv[p] = r3 / (kB * kB) / (T * T * T * T) - 2 * r2 / kB / (T * T * T);
  }
  if (n_kept) *n_kept = B;
  if (energies) std::copy(ev.begin(), ev.end(), energies);
  if (S_E) std::copy(S.begin(), S.end(), S_E);
  if (alpha) std::copy(x.begin(), x.end(), alpha);
  return 0;
}

// ---------------------------------------------------------------- WHAM NVT
// multihistogram_NVT (multihist_NVT.jl:11-221), restated literally.
int orc_multihist_nvt(int R, int n_bin, const double* H, const double* t_grid,
                      const double* beta, double en_min, double en_max,
                      double thr, double* T_out, double* cv_out, int* iters) {
  const double k = 3.166811429 / 1e6;  // :18
  int nb = n_bin + 2;
  double dE = (en_max - en_min) / n_bin;  // :24
  std::vector<double> f(R, 0.0), nf(R, 0.0), nc(R, 0.0);
  for (int i = 0; i < R; ++i)
    for (int m = 1; m <= n_bin; ++m) nc[i] = nc[i] + H[(size_t)i * nb + m];
  auto qp = [&](double bt, int m) {  // quasiprob :59-85
    double E = en_min + (m - 0.5) * dE;
    double q = 0, den = 0, off = -1e6;
    for (int i = 0; i < R; ++i) off = std::fmax(off, -beta[i] * E - f[i]);
    off = off + std::log(1e3);
    for (int i = 0; i < R; ++i) {
      q = q + H[(size_t)i * nb + m];
      den = den + nc[i] * std::exp(-beta[i] * E - f[i] - off);
    }
    return q / den * std::exp(-bt * E - off);
  };
  int it = 0;
  for (it = 1; it <= 1000; ++it) {
    for (int i = 0; i < R; ++i) {
      nf[i] = 0;
      for (int m = 1; m <= n_bin; ++m) nf[i] = nf[i] + qp(beta[i], m);
      nf[i] = std::log(nf[i]);
    }
    double delta = 0;
    for (int i = 0; i < R; ++i) {
      double dd = std::fabs(nf[i] - f[i]);
      delta = delta + dd * dd;
      f[i] = nf[i];
    }
    if (delta < thr) break;
  }
  if (iters) *iters = it > 1000 ? 1000 : it;
  int RR = 10 * R;
  std::vector<double> Tr(RR), Br(RR);
  orc_tempgrid(t_grid[0], t_grid[R - 1], RR, 0, Tr.data(), Br.data());
  for (int i = 0; i < RR; ++i) {
    double norm = 0;
    for (int m = 1; m <= n_bin; ++m) norm = norm + qp(Br[i], m);
    double e1 = 0, e2 = 0;
    for (int m = 1; m <= n_bin; ++m) {
      double E = en_min + (m - 0.5) * dE;
      e1 = e1 + qp(Br[i], m) / norm * E;
      e2 = e2 + qp(Br[i], m) / norm * (E * E);
    }
    T_out[i] = Tr[i];
    cv_out[i] = (e2 - e1 * e1) / (k * (Tr[i] * Tr[i]));
  }
  return 0;
}

// ---------------------------------------------------------------- WHAM NPT
// multihistogram_NPT (multihist_NPT.jl:11-338), restated literally.
int orc_multihist_npt(int R, int n_bin, const double* H, const double* t_grid,
                      const double* beta, double en_min, double en_max,
                      double v_min, double v_max, double p, double thr,
                      double* T_out, double* cp_out, int* iters) {
  const double k = 3.166811429 / 1e6;
  int nb = n_bin + 2;
  double dE = (en_max - en_min) / n_bin, dV = (v_max - v_min) / n_bin;
  auto h = [&](int i, int m, int n) { return H[((size_t)i * nb + m) * nb + n]; };
  std::vector<double> f(R, 0.0), nf(R, 0.0), nc(R, 0.0);
  for (int i = 0; i < R; ++i)
    for (int m = 1; m <= n_bin; ++m)
      for (int n = 1; n <= n_bin; ++n) nc[i] = nc[i] + h(i, m, n);
  auto qp = [&](double bt, int m, int n) {  // quasiprob :70-103
    double E = en_min + (m - 0.5) * dE;
    double V = v_min + (n - 0.5) * dV;
    double q = 0, den = 0, off = -1e6;
    for (int i = 0; i < R; ++i) off = std::fmax(off, -beta[i] * (E + p * V) - f[i]);
    off = off + std::log(1e3);
    for (int i = 0; i < R; ++i) {
      q = q + h(i, m, n);
      den = den + nc[i] * std::exp(-beta[i] * (E + p * V) - f[i] - off);
    }
    return q / den * std::exp(-bt * (E + p * V) - off);
  };
  int it = 0;
  for (it = 1; it <= 1000; ++it) {
    for (int i = 0; i < R; ++i) {
      nf[i] = 0;
      for (int m = 1; m <= n_bin; ++m)
        for (int n = 1; n <= n_bin; ++n) nf[i] = nf[i] + qp(beta[i], m, n);
      nf[i] = std::log(nf[i]);
    }
    double delta = 0;
    for (int i = 0; i < R; ++i) {
      double dd = std::fabs(nf[i] - f[i]);
      delta = delta + dd * dd;
      f[i] = nf[i];
    }
    if (delta < thr) break;
  }
  if (iters) *iters = it > 1000 ? 1000 : it;
  int RR = 10 * R;
  std::vector<double> Tr(RR), Br(RR);
  orc_tempgrid(t_grid[0], t_grid[R - 1], RR, 0, Tr.data(), Br.data());
  for (int i = 0; i < RR; ++i) {
    double norm = 0;
    for (int m = 1; m <= n_bin; ++m)
      for (int n = 1; n <= n_bin; ++n) norm = norm + qp(Br[i], m, n);
    double h1 = 0, h2 = 0;
    for (int m = 1; m <= n_bin; ++m)
      for (int n = 1; n <= n_bin; ++n) {
        double E = en_min + (m - 0.5) * dE;
        double V = v_min + (n - 0.5) * dV;
        double q = qp(Br[i], m, n) / norm;
        h1 = h1 + q * (E + p * V);
        h2 = h2 + q * ((E + p * V) * (E + p * V));
      }
    T_out[i] = Tr[i];
    cp_out[i] = (h2 - h1 * h1) / (k * (Tr[i] * Tr[i]));
  }
  return 0;
}

}  // extern "C"
