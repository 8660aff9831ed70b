"""GB300 parallel-tempering Monte Carlo engine — host-side mirror of the
ParallelTemperingMonteCarlo.jl API for the replica-cycle hot path.

Names, argument meaning and error behaviour follow the reference:
MCParams / TempGrid (src/InputParams.jl:35-95), SphericalBC / CubicBC
(src/BoundaryConditions.jl:44-80), Config (src/Configurations.jl:42),
NVT / NPT (src/Ensembles.jl:42-86), ELJPotential / ELJPotentialEven /
EmbeddedAtomPotential (src/EnergyEvaluation.jl:923-942, 1059-1073),
ptmc_run! (src/MCRun.jl:363-481, here `ptmc_run`), Output
(src/InputParams.jl:114-176), multihistogram_NVT / multihistogram_NPT
(src/multihist_NVT.jl:95, src/multihist_NPT.jl:113) and the checkpoint
directory of src/ReadSave.jl.

Every computation runs in libptmc_gb300.so on the GPU through its C ABI
(include/ptmc_gb300.h); this module only marshals arguments.  There is no CPU
fallback: without the built library or a usable GPU every call raises.
"""
import ctypes
import math
import os
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

from . import _capi
from ._capi import PTMCError

kB = 3.16681196e-6  # Hartree/K, src/InputParams.jl:19

__all__ = ["kB", "MCParams", "TempGrid", "SphericalBC", "CubicBC", "RectangularBC", "RhombicBC",
           "Config", "NVT", "NPT",
           "ELJPotential", "ELJPotentialEven", "ELJPotentialB", "LookupTablePotential",
           "read_lookuptable", "EmbeddedAtomPotential", "RuNNerPotential",
           "RuNNerPotential2Atom", "NNVT",
           "Output", "MCState", "PairSurrogate",
           "Engine", "ptmc_run", "multihistogram_NVT", "multihistogram_NPT", "read_checkpoint",
           "multihistogram", "postprocess",
           "distance2", "get_distance2_mat", "get_volume", "get_r_cut", "PTMCError"]


# ------------------------------------------------------------------ parameters
@dataclass
class MCParams:
    """MCParams (src/InputParams.jl:35-63)."""
    mc_cycles: int
    eq_cycles: int
    mc_sample: int
    n_traj: int
    n_atoms: int
    n_adjust: int = 100
    n_bin: int = 100
    min_acc: float = 0.4
    max_acc: float = 0.6

    @classmethod
    def new(cls, cycles, n_traj, n_atoms, eq_percentage=0.2, mc_sample=1, n_adjust=100,
            n_bin=100, min_acc=0.4, max_acc=0.6):
        cycles = int(cycles)
        return cls(cycles, int(round(eq_percentage * cycles)), mc_sample, n_traj, n_atoms,
                   n_adjust, n_bin, min_acc, max_acc)


def _mcparams(cycles, n_traj, n_atoms, **kw):
    return MCParams.new(cycles, n_traj, n_atoms, **kw)


class TempGrid:
    """TempGrid{N}(ti, tf; tdistr) (src/InputParams.jl:77-95)."""

    def __init__(self, ti, tf, N, tdistr="geometric"):
        if tdistr not in ("geometric", "equally_spaced"):
            raise ValueError("chosen temperature distribution %s does not exist" % tdistr)
        i = np.arange(N, dtype=np.float64)
        if N == 1:  # the reference's formulas divide 0 / 0 here (NaN); one temperature, ti
            self.t_grid = np.array([float(ti)])
        elif tdistr == "equally_spaced":
            delta = (tf - ti) / (N - 1)
            self.t_grid = ti + i * delta
        else:
            self.t_grid = np.array([ti * (tf / ti) ** (k / (N - 1)) for k in range(N)])
        self.beta_grid = 1.0 / (kB * self.t_grid)
        self.ti, self.tf, self.N, self.tdistr = float(ti), float(tf), N, tdistr

    def __len__(self):
        return self.N


@dataclass
class SphericalBC:
    """SphericalBC(radius) (src/BoundaryConditions.jl:44-49); stores radius^2."""
    radius: float

    @property
    def radius2(self):
        return self.radius * self.radius


@dataclass
class CubicBC:
    """CubicBC(side_length) (src/BoundaryConditions.jl:72-78)."""
    box_length: float


@dataclass
class RectangularBC:
    """RectangularBC(box_length, box_height) (src/BoundaryConditions.jl:80-92):
    square side box_length in x and y, box_height in z."""
    box_length: float
    box_height: float


@dataclass
class RhombicBC:
    """RhombicBC(box_length, box_height) (src/BoundaryConditions.jl:95-116): a
    rhombus of side box_length (60 degrees) in the xy plane, box_height in z."""
    box_length: float
    box_height: float


SQRT3 = 1.7320508075688772  # 3^0.5


class Config:
    """Config(positions, boundary_condition) (src/Configurations.jl:42-56)."""

    def __init__(self, positions, boundary_condition):
        self.positions = np.array(positions, dtype=np.float64).reshape(-1, 3)
        self.boundary_condition = boundary_condition

    def __len__(self):
        return len(self.positions)


def distance2(a, b, bc=None):
    """distance2 (src/Configurations.jl:101-126) with the minimum image of
    CubicBC, RectangularBC and RhombicBC."""
    a, b = np.asarray(a, float), np.asarray(b, float)
    if isinstance(bc, CubicBC):
        L = bc.box_length
        b = b + L * np.round((a - b) / L)
    elif isinstance(bc, RectangularBC):
        L, H = bc.box_length, bc.box_height
        b = b + np.array([L, L, H]) * np.round((a - b) / np.array([L, L, H]))
    elif isinstance(bc, RhombicBC):
        L, H = bc.box_length, bc.box_height
        hy = SQRT3 / 2 * L
        by = b[1] + hy * np.round((a[1] - b[1]) / hy)
        bx = (b[0] - b[1] / SQRT3 + L * np.round(((a[0] - b[0]) - 1 / SQRT3 * (a[1] - b[1])) / L)
              + 1 / SQRT3 * by)
        bz = b[2] + H * np.round((a[2] - b[2]) / H)
        b = np.array([bx, by, bz])
    d = a - b
    return float((d[0] * d[0] + d[1] * d[1]) + d[2] * d[2])


def get_distance2_mat(config):
    """get_distance2_mat (src/Configurations.jl:135-162)."""
    n = len(config)
    m = np.zeros((n, n))
    for i in range(n):
        for j in range(i + 1, n):
            m[i, j] = m[j, i] = distance2(config.positions[i], config.positions[j],
                                          config.boundary_condition)
    return m


def get_volume(bc):
    """get_volume (src/Configurations.jl:246-256)."""
    if isinstance(bc, CubicBC):
        return bc.box_length ** 3
    if isinstance(bc, RhombicBC):
        return bc.box_length * bc.box_length * bc.box_height * SQRT3 / 2
    if isinstance(bc, RectangularBC):
        return bc.box_length * bc.box_length * bc.box_height
    raise TypeError("get_volume is defined for periodic boxes")


def get_r_cut(bc):
    """get_r_cut (src/Ensembles.jl:118-155): the squared cut-off of a periodic box."""
    if isinstance(bc, CubicBC):
        return bc.box_length * bc.box_length / 4
    if isinstance(bc, RhombicBC):
        L, H = bc.box_length, bc.box_height
        return min(L * L * 3 / 16, H * H / 4)
    if isinstance(bc, RectangularBC):
        L, H = bc.box_length, bc.box_height
        return min(L * L / 4, H * H / 4)
    raise TypeError("get_r_cut is defined for periodic boxes")


def _bc_kind(bc):
    """(C ABI kind, box_length or radius, box_height) of a boundary condition."""
    if isinstance(bc, CubicBC):
        return _capi.BC_CUBIC, bc.box_length, bc.box_length
    if isinstance(bc, RectangularBC):
        return _capi.BC_RECTANGULAR, bc.box_length, bc.box_height
    if isinstance(bc, RhombicBC):
        return _capi.BC_RHOMBIC, bc.box_length, bc.box_height
    return _capi.BC_SPHERE, bc.radius, bc.radius


@dataclass
class NVT:
    """NVT(n_atoms) (src/Ensembles.jl:42-50)."""
    n_atoms: int

    @property
    def n_atom_moves(self):
        return self.n_atoms


@dataclass
class NPT:
    """NPT(n_atoms, pressure, separated_volume) (src/Ensembles.jl:75-86)."""
    n_atoms: int
    pressure: float
    separated_volume: bool = False


@dataclass
class NNVT:
    """NNVT(natoms; natomswaps=1) (src/Ensembles.jl:138-151): two species,
    natoms = [n1, n2], atoms 0..n1-1 of every configuration are species 1;
    N atom moves and natomswaps atom swaps per cycle."""
    natoms: tuple
    n_atom_swaps: int = 1

    @property
    def n_atoms(self):
        return int(self.natoms[0]) + int(self.natoms[1])

    @property
    def n_atom_moves(self):
        return self.n_atoms


@dataclass
class ELJPotential:
    """ELJPotential: V(r) = sum_i c_i r^-(5+i) (src/EnergyEvaluation.jl:923-932)."""
    coeff: list

    even = False


@dataclass
class ELJPotentialB:
    """ELJPotentialB(a, b, c) (src/EnergyEvaluation.jl:161-183): the extended
    Lennard-Jones dimer in a magnetic field; its energy depends on |tan| of
    the pair angle to z (dimer_energy, :943-958)."""
    coeff_a: list
    coeff_b: list
    coeff_c: list


@dataclass
class RuNNerPotential2Atom:
    """RuNNerPotential2Atom(nnp1, nnp2, radsymvec, angsymvec, n1, n2)
    (src/EnergyEvaluation.jl:1287-1314): rad [nrad, 10] rows {eta, r_cut,
    G_offset[4], G_norm[4]} (RadialType2a), ang [nang, 16] rows {eta, lambda,
    zeta, r_cut, tpz[6], G_offset[6]} (AngularType3a), the two species'
    networks w1, w2 (per layer W[n_in][n_out] then b) with nodes =
    [2 nrad + 3 nang, H1, H2, 1]; species 1 = the first n1 atoms."""
    rad: np.ndarray
    ang: np.ndarray
    w1: np.ndarray
    w2: np.ndarray
    nodes: list
    n1: int

    @staticmethod
    def radial(eta, r_cut, g_vals_a, g_vals_b):
        """RadialType2a{T}(eta, r_cut, type, G_vals_a, G_vals_b)
        (MachineLearningPotential/SymmFunc.jl:64-85): G_vals_x = [[max, min]
        of the species-1 neighbour row, [max, min] of the species-2 row]."""
        vals = [g_vals_a[0], g_vals_a[1], g_vals_b[0], g_vals_b[1]]
        norm = [1 / (v[0] - v[1]) for v in vals]
        off = [-v[1] * n for v, n in zip(vals, norm)]
        return [eta, r_cut] + off + norm

    @staticmethod
    def angular(eta, lam, zeta, r_cut, g_vals_a, g_vals_b):
        """AngularType3a{T}(eta, lambda, zeta, r_cut, type, G_valsa, G_valsb)
        (SymmFunc.jl:139-175): three [max, min] per centre species."""
        vals = list(g_vals_a) + list(g_vals_b)
        norm = [1 / (v[0] - v[1]) for v in vals]
        tpz = [2.0 ** (1 - zeta) * n for n in norm]
        off = [-v[1] * n for v, n in zip(vals, norm)]
        return [eta, lam, zeta, r_cut] + tpz + off


@dataclass
class LookupTablePotential:
    """LookupTablePotential (src/EnergyEvaluation.jl:210-260): table[angle,
    distance] (l_angle x l_dist) of dimer energies; LookupTablePotential(path)
    reads the reference's table format (read_lookuptable)."""
    table: np.ndarray
    start_dist: float
    start_angle: float
    l_dist: int
    l_angle: int
    d_dist: float
    d_angle: float
    c6coeff: float

    @classmethod
    def from_file(cls, path):
        return cls(*read_lookuptable(path))


def read_lookuptable(path):
    """read_lookuptable (src/EnergyEvaluation.jl:227-256): line 1 "l_dist,
    start_dist, d_dist", line 2 "l_angle, start_angle, d_angle" ('!' starts a
    comment), then l_angle x l_dist values, angle-major; c6coeff = the mean
    over angles of table[:, 1000] times (start_dist + 1000 d_dist)^6."""
    with open(path) as f:
        def line():
            return f.readline().split("!")[0]
        h = line().split(", ")
        l_dist, start_dist, d_dist = int(h[0]), float(h[1]), float(h[2])
        h = line().split(", ")
        l_angle, start_angle, d_angle = int(h[0]), float(h[1]), float(h[2])
        table = np.empty((l_angle, l_dist))
        for i in range(l_angle):
            for j in range(l_dist):
                table[i, j] = float(line())
    avg = 0.0
    for i in range(l_angle):
        avg += table[i, 999]
    avg /= l_angle
    c6 = avg * (start_dist + 1000 * d_dist) ** 6
    return table, start_dist, start_angle, l_dist, l_angle, d_dist, d_angle, c6


@dataclass
class ELJPotentialEven:
    """ELJPotentialEven: V(r) = sum_i c_i r^-(4+2i) (src/EnergyEvaluation.jl:934-942)."""
    coeff: list

    even = True


class EmbeddedAtomPotential:
    """EmbeddedAtomPotential(n, m, eps, C, a) (src/EnergyEvaluation.jl:1059-1073)."""

    def __init__(self, n, m, eps=None, C=None, a=None, *, ean=None, eCam=None):
        self.n, self.m = float(n), float(m)
        if ean is not None:
            self.ean, self.eCam = float(ean), float(eCam)
        else:
            self.ean = eps * a ** n / 2
            self.eCam = eps * C * a ** (m / 2)


class RuNNerPotential:
    """RuNNerPotential (src/EnergyEvaluation.jl:1182-1213): Behler-Parrinello
    symmetry functions + per-atom MLP {n_sf, H1, H2, 1} with tanh hidden layers
    (MachineLearningPotential/ForwardPass.jl:21-41).

    sf: rows {kind (0 radial, 1 angular), type, eta, lambda, zeta, r_cut,
    G_min, G_max}; weights: per layer W[n_in][n_out] (input-major), then the
    biases; boundary: hard-core distance (bohr), E = 100 below it
    (src/EnergyEvaluation.jl:1602-1606)."""

    def __init__(self, sf, weights, nodes=(88, 20, 20, 1), boundary=0.0):
        self.sf = np.ascontiguousarray(sf, dtype=np.float64).reshape(-1, 8)
        self.weights = np.ascontiguousarray(weights, dtype=np.float64)
        self.nodes = np.ascontiguousarray(nodes, dtype=np.int32)
        self.boundary = float(boundary)

    @staticmethod
    def sf_table(tables, r_cut=None):
        """The (n_sf, 8) table from the symmetry-function list of scripts/cu55.jl
        (as stored in tests/golden/nn_cu55.json), optionally with another cut-off."""
        rows = []
        for f in tables["sf"]:
            rows.append([f["kind"], f["type"], f["eta"], f["lambda"], f["zeta"],
                         r_cut if r_cut is not None else f["rcut"], f["gmin"], f["gmax"]])
        return np.array(rows)

    @staticmethod
    def random_weights(nodes, seed, out_scale=1.0):
        """FP32-valued weights and biases ~ U(-1/sqrt(fan_in), 1/sqrt(fan_in)),
        seeded; the last layer is multiplied by out_scale (sets the energy scale)."""
        rng = np.random.default_rng(seed)
        w = []
        for l in range(1, len(nodes)):
            ni, no = nodes[l - 1], nodes[l]
            lim = 1.0 / np.sqrt(ni)
            W = rng.uniform(-lim, lim, (ni, no)).astype(np.float32)
            bvec = rng.uniform(-lim, lim, no).astype(np.float32)
            if l == len(nodes) - 1:
                W = (W * out_scale).astype(np.float32)
                bvec = (bvec * out_scale).astype(np.float32)
            w.append(W.astype(np.float64).reshape(-1))
            w.append(bvec.astype(np.float64))
        return np.concatenate(w)


@dataclass
class Output:
    """Output{Float64} (src/InputParams.jl:114-176), one run."""
    n_bin: int
    en_min: float = 0.0
    en_max: float = 0.0
    v_min: float = 0.0
    v_max: float = 0.0
    delta_en_hist: float = 0.0
    delta_v_hist: float = 0.0
    delta_r2: float = 0.0
    max_displ: np.ndarray = None
    en_avg: np.ndarray = None
    heat_cap: np.ndarray = None
    en_histogram: np.ndarray = None
    ev_histogram: np.ndarray = None
    rdf: list = field(default_factory=list)
    count_stat_atom: np.ndarray = None
    count_stat_vol: np.ndarray = None
    count_stat_exc: np.ndarray = None


@dataclass
class MCState:
    """Slot-ordered replica state after a run (the host view of MCState,
    src/MCStates.jl:33-53)."""
    temp: float
    beta: float
    config: Config
    en_tot: float
    max_displ: np.ndarray
    count_atom: np.ndarray
    count_vol: np.ndarray
    count_exc: np.ndarray
    ham: np.ndarray
    count_vol_xy: np.ndarray = None   # separated volume moves (RectangularBC, RhombicBC)
    count_vol_z: np.ndarray = None


# ------------------------------------------------------------------ engine
def _fptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def _dptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class PairSurrogate:
    """Configuration of the learned pair surrogate of delayed-acceptance moves
    (no counterpart in the reference): 16 Gaussian radial features with centres
    evenly spaced on [r_lo, r_hi], width parameter gamma, cosine cut-off r_cut,
    MLP 16 -> 32 -> 32 -> 1 (tanh), output scale escale (0: set from the
    recorded energy changes at the first training)."""

    def __init__(self, r_lo=2.0, r_hi=12.0, gamma=None, r_cut=12.0, escale=0.0):
        self.r_lo, self.r_hi, self.r_cut, self.escale = float(r_lo), float(r_hi), float(r_cut), float(escale)
        dmu = (self.r_hi - self.r_lo) / 15.0
        self.gamma = float(gamma) if gamma is not None else 1.0 / (2.0 * dmu * dmu)

    def cfg(self):
        c = _capi.SurrogateCfg()
        c.r_lo, c.r_hi, c.gamma, c.r_cut, c.escale = self.r_lo, self.r_hi, self.gamma, self.r_cut, self.escale
        return c

    def as_array(self):
        return np.array([self.r_lo, self.r_hi, self.gamma, self.r_cut, self.escale])

    def eval(self, params, rows, device=0):
        """dE_s of move records (n, 128) on the GPU (tensor-core forward)."""
        L = _capi.load()
        rows = np.ascontiguousarray(rows, dtype=np.float32)
        P = np.ascontiguousarray(params, dtype=np.float32)
        out = np.zeros(rows.shape[0])
        c = self.cfg()
        _capi.check(L.ptmc_surrogate_eval(ctypes.byref(c), _fptr(P), _fptr(rows), rows.shape[0],
                                          _dptr(out), device))
        return out

    def loss_grad(self, params, rows, targets, device=0):
        """Huber loss of (dE_s - targets)/escale and its gradient, on the GPU."""
        L = _capi.load()
        rows = np.ascontiguousarray(rows, dtype=np.float32)
        y = np.ascontiguousarray(targets, dtype=np.float32)
        P = np.ascontiguousarray(params, dtype=np.float32)
        g = np.zeros(_capi.SUR_NPARAMS, dtype=np.float32)
        loss = ctypes.c_double()
        c = self.cfg()
        _capi.check(L.ptmc_surrogate_loss_grad(ctypes.byref(c), _fptr(P), _fptr(rows), _fptr(y),
                                               rows.shape[0], ctypes.byref(loss), _fptr(g), device))
        return loss.value, g


class Engine:
    """A batch of `n_runs` independent PT runs on the GPU (one ptmc_ctx).

    Every run shares the potential, the ensemble, the temperature grid and the
    MC parameters; each run gets its own start configurations (and may have its
    own atom count)."""

    def __init__(self, mc_params, temp, potential, ensemble, *, n_runs=1, precision="fp64",
                 resync_every=1000, exch_prob=0.1, seed=1234, cycles_per_launch=0, device=0,
                 rdfsave=False):
        self.L = _capi.load()
        self.rdfsave = bool(rdfsave)
        self.mc_params, self.temp, self.potential, self.ensemble = mc_params, temp, potential, ensemble
        p = _capi.Params()
        p.n_runs = n_runs
        p.n_traj = mc_params.n_traj
        p.mc_cycles = mc_params.mc_cycles
        p.eq_cycles = mc_params.eq_cycles
        p.mc_sample = mc_params.mc_sample
        p.n_adjust = mc_params.n_adjust
        p.n_bin = mc_params.n_bin
        p.min_acc = mc_params.min_acc
        p.max_acc = mc_params.max_acc
        p.ensemble = (_capi.NPT if isinstance(ensemble, NPT)
                      else _capi.NNVT if isinstance(ensemble, NNVT) else _capi.NVT)
        p.pressure = ensemble.pressure if isinstance(ensemble, NPT) else 0.0
        p.t_i, p.t_f = temp.ti, temp.tf
        p.tdistr = _capi.TLINEAR if temp.tdistr == "equally_spaced" else _capi.TGEOMETRIC
        p.exch_prob = exch_prob
        p.precision = {"fp64": _capi.FP64, "fp32": _capi.FP32_RESYNC,
                       "fp32_resync": _capi.FP32_RESYNC}[precision]
        p.resync_every = resync_every
        p.seed = seed
        p.cycles_per_launch = cycles_per_launch
        p.device = device
        self.params = p
        h = ctypes.c_void_p()
        _capi.check(self.L.ptmc_create(ctypes.byref(h), ctypes.byref(p)))
        self.h = h
        if self.rdfsave:
            self._ck(self.L.ptmc_set_rdf(h, 1))
        if isinstance(ensemble, NPT) and ensemble.separated_volume:
            self._ck(self.L.ptmc_set_separated_volume(h, 1))
        if isinstance(ensemble, NNVT):
            self._ck(self.L.ptmc_set_atom_swaps(h, int(ensemble.n_atom_swaps)))
        self.n_runs, self.R = n_runs, mc_params.n_traj
        self.N = {}
        self.bc = {}
        if isinstance(potential, (ELJPotential, ELJPotentialEven)):
            c = np.ascontiguousarray(potential.coeff, dtype=np.float64)
            self._ck(self.L.ptmc_set_potential_elj(h, _dptr(c), len(c), int(potential.even)))
        elif isinstance(potential, RuNNerPotential2Atom):
            if not isinstance(ensemble, NNVT) or int(ensemble.natoms[0]) != potential.n1:
                raise ValueError("RuNNerPotential2Atom runs in NNVT(natoms) with natoms[0] == n1")
            rad = np.ascontiguousarray(potential.rad, dtype=np.float64)
            ang = np.ascontiguousarray(potential.ang, dtype=np.float64).reshape(-1, 16)
            w1 = np.ascontiguousarray(potential.w1, dtype=np.float64)
            w2 = np.ascontiguousarray(potential.w2, dtype=np.float64)
            nodes = np.ascontiguousarray(potential.nodes, dtype=np.int32)
            self._ck(self.L.ptmc_set_potential_nn2(
                h, _dptr(rad), len(rad), _dptr(ang), len(ang), _dptr(w1), _dptr(w2), len(w1),
                nodes.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), len(nodes), potential.n1))
        elif isinstance(potential, ELJPotentialB):
            a, b, c = (np.ascontiguousarray(v, dtype=np.float64)
                       for v in (potential.coeff_a, potential.coeff_b, potential.coeff_c))
            self._ck(self.L.ptmc_set_potential_eljb(h, _dptr(a), _dptr(b), _dptr(c), len(c)))
        elif isinstance(potential, LookupTablePotential):
            t = np.asarray(potential.table, dtype=np.float64)
            flat = np.ascontiguousarray(t.reshape(-1, order="F"))  # Julia's column-major
            self._ck(self.L.ptmc_set_potential_lookup(
                h, _dptr(flat), t.shape[0], t.shape[1], potential.start_dist,
                potential.start_angle, potential.d_dist, potential.d_angle, potential.c6coeff))
        elif isinstance(potential, EmbeddedAtomPotential):
            self._ck(self.L.ptmc_set_potential_eam(h, potential.n, potential.m, potential.ean,
                                                   potential.eCam))
        elif isinstance(potential, RuNNerPotential):
            self._ck(self.L.ptmc_set_potential_nn(
                h, _dptr(potential.sf), potential.sf.shape[0], _dptr(potential.weights),
                len(potential.weights), potential.nodes.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                len(potential.nodes), potential.boundary))
        else:
            raise TypeError("unsupported potential %r" % type(potential))

    def _ck(self, rc):
        return _capi.check(rc, self.h)

    def set_configs(self, run, configs, max_displ=None):
        """Start configurations of `run` (one Config or a sequence; replica i
        starts from configs[i mod len], src/Initialization.jl:88-96)."""
        if isinstance(configs, Config):
            configs = [configs]
        bc = configs[0].boundary_condition
        N = len(configs[0])
        xyz = np.ascontiguousarray(np.stack([c.positions for c in configs]), dtype=np.float64)
        kind, par, height = _bc_kind(bc)
        self._ck(self.L.ptmc_set_run_configs_box(self.h, run, _dptr(xyz), N, len(configs), kind,
                                                 par, height))
        self.N[run], self.bc[run] = N, bc
        if max_displ is not None:  # per slot: [atom], [atom, volume] or [atom, volume, xy, z]
            md = np.ascontiguousarray(max_displ, dtype=np.float64).reshape(self.R, -1)
            if md.shape[1] == 1:
                md = np.concatenate([md, np.full((self.R, 1), 0.1)], 1)
            self._ck(self.L.ptmc_set_max_displ(self.h, run, _dptr(np.ascontiguousarray(md[:, :2]))))
            if md.shape[1] == 4:
                self._ck(self.L.ptmc_set_max_displ_sep(
                    self.h, run, _dptr(np.ascontiguousarray(md[:, 2:]))))

    def set_configs_batch(self, xyz, bc, first=0):
        """One start configuration per run for runs first .. first + len(xyz) - 1
        in one call: xyz [n_runs, N, 3] (bohr), one boundary condition for all."""
        x = np.ascontiguousarray(xyz, dtype=np.float64)
        if x.ndim != 3 or x.shape[2] != 3:
            raise ValueError("xyz: [n_runs, N, 3]")
        n, N = x.shape[0], x.shape[1]
        kind, par, height = _bc_kind(bc)
        self._ck(self.L.ptmc_set_runs_configs(self.h, int(first), n, _dptr(x), N, kind, par, height))
        for r in range(first, first + n):
            self.N[r], self.bc[r] = N, bc

    def init(self):
        self._ck(self.L.ptmc_init(self.h))

    def equilibrate(self):
        self._ck(self.L.ptmc_equilibrate(self.h))

    def run_cycles(self, n):
        self._ck(self.L.ptmc_run_cycles(self.h, int(n)))

    def cycles_nosample(self, n):
        self._ck(self.L.ptmc_cycles_nosample(self.h, int(n)))

    def resync(self):
        self._ck(self.L.ptmc_resync(self.h))

    # ---- launch shapes (FP32 form)
    def set_launch_shape(self, N, ctas_per_run, lanes_per_walker=32):
        """Runs with N atoms: spread over a cluster of `ctas_per_run` CTAs, with
        `lanes_per_walker` lanes (32, or 16 = two walkers per warp) per walker."""
        self._ck(self.L.ptmc_set_launch_shape(self.h, int(N), int(ctas_per_run),
                                              int(lanes_per_walker)))

    def autotune(self, trial_cycles=20, cache=None):
        """Pick (CTAs per run, lanes per walker) for every atom count by timed
        trials (the chain is restored after each); returns {N: (C, L)}."""
        out = np.zeros(2 * self.n_runs, dtype=np.int32)
        path = None if cache is None else os.fsencode(cache)
        self._ck(self.L.ptmc_autotune(self.h, int(trial_cycles), path,
                                      out.ctypes.data_as(ctypes.POINTER(ctypes.c_int))))
        return {int(self.N[r]): (int(out[2 * r]), int(out[2 * r + 1])) for r in range(self.n_runs)}

    def occupancy(self, N, ctas_per_run=1, lanes_per_walker=32):
        """Resident CTAs per SM of the cycle kernel for runs of N atoms with the
        launch shape (C, L) (FP32 form; the plain form ignores the shape)."""
        n = ctypes.c_int()
        self._ck(self.L.ptmc_occupancy(self.h, int(N), int(ctas_per_run), int(lanes_per_walker),
                                       ctypes.byref(n)))
        return n.value

    # ---- bounded device waits
    def set_wait_test(self, clocks=0, never_set=False):
        """Exchange-partner wait limit of the FP32 form in clocks (0 = the
        default 2^33) and the test switch that makes every such wait target a
        flag value nobody writes (the failure path, without a fault)."""
        self._ck(self.L.ptmc_set_wait_test(self.h, int(clocks), int(bool(never_set))))

    def walker_status(self, run=0):
        """Status word of every walker of `run` (walker order): 0 running,
        1 out of the sphere, 2 tensor-core wait ran out, 3 exchange wait ran out."""
        st = np.zeros(self.R, dtype=np.int32)
        self._ck(self.L.ptmc_get_walker_status(self.h, int(run),
                                               st.ctypes.data_as(ctypes.POINTER(ctypes.c_int))))
        return st

    # ---- delayed acceptance with the learned pair surrogate (NN potential)
    def surrogate_set(self, surrogate, capacity=100000, record_every=1, params=None):
        """Attach a PairSurrogate (configuration and, unless `params` is given,
        seeded initial weights) with a ring of `capacity` training records."""
        cfg = surrogate.cfg()
        p = None if params is None else _fptr(np.ascontiguousarray(params, dtype=np.float32))
        self._ck(self.L.ptmc_surrogate_set(self.h, ctypes.byref(cfg), p, int(capacity),
                                           int(record_every)))

    def surrogate_record(self, on=True):
        self._ck(self.L.ptmc_surrogate_record(self.h, int(bool(on))))

    def surrogate_train(self, steps, batch=512, lr=1e-3):
        """Adam on the GPU over minibatches of the captured records; returns the
        mean minibatch loss of the last 10 % of steps."""
        loss = ctypes.c_double()
        self._ck(self.L.ptmc_surrogate_train(self.h, int(steps), int(batch), float(lr),
                                             ctypes.byref(loss)))
        return loss.value

    def surrogate_enable(self, on=True):
        self._ck(self.L.ptmc_surrogate_enable(self.h, int(bool(on))))

    def surrogate_calibrate(self, cost_ratio=0.0, timing_cycles=20):
        """Per-temperature screening strength kappa (returned, one per slot),
        chosen from the captured records; cost_ratio <= 0 measures the cost of
        a surrogate stage relative to an exact evaluation by timing
        `timing_cycles` plain cycles without and with screening."""
        k = np.zeros(self.R)
        self._ck(self.L.ptmc_surrogate_calibrate(self.h, float(cost_ratio), int(timing_cycles),
                                                 _dptr(k)))
        return k

    def surrogate_set_kappa(self, kappa):
        """Screening strength per temperature slot (R values in [0, 1])."""
        k = np.ascontiguousarray(kappa, dtype=np.float64)
        if k.shape != (self.R,):
            raise ValueError("kappa: one value per temperature slot")
        self._ck(self.L.ptmc_surrogate_set_kappa(self.h, _dptr(k)))

    def surrogate_state(self):
        """(parameters, PairSurrogate config, stats dict)."""
        P = np.zeros(_capi.SUR_NPARAMS, dtype=np.float32)
        cfg = _capi.SurrogateCfg()
        st = np.zeros(4, dtype=np.int64)
        self._ck(self.L.ptmc_surrogate_get(self.h, _fptr(P), ctypes.byref(cfg),
                                           st.ctypes.data_as(ctypes.POINTER(ctypes.c_longlong))))
        sur = PairSurrogate(cfg.r_lo, cfg.r_hi, cfg.gamma, cfg.r_cut, cfg.escale)
        return P, sur, dict(records=int(st[0]), stage1_rejects=int(st[1]), exact_evals=int(st[2]))

    def surrogate_records(self, max_n=None):
        _, _, st = self.surrogate_state()
        n = st["records"] if max_n is None else max_n
        n = max(0, int(n))
        rows = np.zeros((max(n, 1), 128), dtype=np.float32)
        y = np.zeros(max(n, 1), dtype=np.float32)
        got = ctypes.c_int()
        self._ck(self.L.ptmc_surrogate_records(self.h, _fptr(rows), _fptr(y), n, ctypes.byref(got)))
        return rows[:got.value], y[:got.value]

    def states(self, run=0):
        """Slot-ordered (xyz [R,N,3], en_tot [R], box [R], max_displ [R,2],
        counts [R,6], ham [R,2])."""
        R, N = self.R, self.N[run]
        xyz = np.zeros((R, N, 3))
        en, box = np.zeros(R), np.zeros(R)
        md, ham = np.zeros((R, 2)), np.zeros((R, 2))
        cnt = np.zeros((R, 6), dtype=np.int64)
        self._ck(self.L.ptmc_get_states(self.h, run, _dptr(xyz), _dptr(en), _dptr(box), _dptr(md),
                                        cnt.ctypes.data_as(ctypes.POINTER(ctypes.c_longlong)),
                                        _dptr(ham)))
        return dict(xyz=xyz, en_tot=en, box=box, max_displ=md, counts=cnt, ham=ham)

    def swaps(self, run=0):
        """Accepted atom swaps of `run` so far (NNVT)."""
        n = ctypes.c_longlong()
        self._ck(self.L.ptmc_get_swaps(self.h, run, ctypes.byref(n)))
        return n.value

    def energies(self):
        """Slot-ordered energies of every run, [n_runs, R], in one read."""
        out = np.zeros((self.n_runs, self.R))
        self._ck(self.L.ptmc_get_energies(self.h, _dptr(out)))
        return out

    def box_states(self, run=0):
        """Slot-ordered box state of RectangularBC / RhombicBC runs: box_height
        [R], max_displ_sep [R,2] (max_displ[3:4]), counts_sep [R,4]
        (count_vol_xy[1:2], count_vol_z[1:2])."""
        R = self.R
        h, md = np.zeros(R), np.zeros((R, 2))
        cnt = np.zeros((R, 4), dtype=np.int64)
        self._ck(self.L.ptmc_get_box_states(self.h, run, _dptr(h), _dptr(md),
                                            cnt.ctypes.data_as(ctypes.POINTER(ctypes.c_longlong))))
        return dict(box_height=h, max_displ_sep=md, counts_sep=cnt)

    def output(self, run=0):
        R, nb = self.R, self.mc_params.n_bin + 2
        npt = isinstance(self.ensemble, NPT)
        arrs = dict(en_avg=np.zeros(R), heat_cap=np.zeros(R), count_stat_atom=np.zeros(R),
                    count_stat_vol=np.zeros(R), count_stat_exc=np.zeros(R),
                    max_displ=np.zeros((R, 2)))
        eh = np.zeros((R, nb))
        ev = np.zeros((R, nb, nb)) if npt else np.zeros(1)
        o = _capi.Output()
        for k, v in arrs.items():
            setattr(o, k, _dptr(v))
        o.en_histogram = _dptr(eh)
        o.ev_histogram = _dptr(ev)
        rdf = np.zeros((R, 5 * self.mc_params.n_bin)) if self.rdfsave else None
        if rdf is not None:
            o.rdf = _dptr(rdf)
        self._ck(self.L.ptmc_get_output(self.h, run, ctypes.byref(o)))
        hp = list(o.hist_params)
        return Output(n_bin=self.mc_params.n_bin, en_min=hp[0], en_max=hp[1], v_min=hp[2],
                      v_max=hp[3], delta_en_hist=hp[4], delta_v_hist=hp[5],
                      delta_r2=o.delta_r2, rdf=list(rdf) if rdf is not None else [],
                      max_displ=arrs["max_displ"], en_avg=arrs["en_avg"],
                      heat_cap=arrs["heat_cap"], en_histogram=eh,
                      ev_histogram=ev if npt else None,
                      count_stat_atom=arrs["count_stat_atom"],
                      count_stat_vol=arrs["count_stat_vol"],
                      count_stat_exc=arrs["count_stat_exc"])

    def stats(self):
        s = _capi.Stats()
        self._ck(self.L.ptmc_get_stats(self.h, ctypes.byref(s)))
        return {k: getattr(s, k) for k, _ in _capi.Stats._fields_}

    def checkpoint(self, directory):
        self._ck(self.L.ptmc_checkpoint(self.h, os.fsencode(directory)))

    def restore(self, directory):
        self._ck(self.L.ptmc_restore(self.h, os.fsencode(directory)))

    def mc_states(self, run=0):
        s = self.states(run)
        bc = self.bc[run]
        boxed = isinstance(bc, (RectangularBC, RhombicBC))
        b = self.box_states(run) if boxed else None
        out = []
        for i in range(self.R):
            if boxed:
                bci = type(bc)(s["box"][i], b["box_height"][i])
                md = np.concatenate([s["max_displ"][i], b["max_displ_sep"][i]])
            else:
                bci = CubicBC(s["box"][i]) if isinstance(bc, CubicBC) else SphericalBC(s["box"][i])
                md = s["max_displ"][i]
            out.append(MCState(self.temp.t_grid[i], self.temp.beta_grid[i],
                               Config(s["xyz"][i], bci), s["en_tot"][i], md,
                               s["counts"][i, 0:2], s["counts"][i, 2:4], s["counts"][i, 4:6],
                               s["ham"][i],
                               b["counts_sep"][i, 0:2] if boxed else None,
                               b["counts_sep"][i, 2:4] if boxed else None))
        return out

    def close(self):
        if getattr(self, "h", None):
            self.L.ptmc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def ptmc_run(mc_params, temp=None, start_config=None, potential=None, ensemble=None, *,
             rdfsave=False, restart=False, save=False, saveconfigs=False,
             configsname="configuration", workingdirectory=None, precision="fp64",
             resync_every=1000, exch_prob=0.1, seed=1234, max_displ=None, eq_cycles=0.2):
    """ptmc_run! (src/MCRun.jl:363-432): initialise, equilibrate, run
    mc_params.mc_cycles production cycles with optional checkpoints every
    `save` cycles into <workingdirectory>/checkpoint, finalise.

    ptmc_run(True, ...) is the reference's resume method (src/MCRun.jl:435-481):
    parameters, ensemble and potential come from checkpoint/params.data, the
    states from the checkpoint (the engine's own engine.bin, exact; or the text
    files a reference run wrote, rebuilt as rebuild_states does), and the run
    continues to mc_cycles.

    Returns (mc_states, results) with slot-ordered states and an Output; with
    rdfsave the radial distribution (Output.rdf) is sampled every 1000th
    production cycle (src/Sampling.jl:341-345)."""
    wd = workingdirectory or os.getcwd()
    ckdir = os.path.join(wd, "checkpoint")
    if isinstance(mc_params, bool):  # ptmc_run!(restart::Bool; ...)
        if not mc_params:
            raise ValueError("ptmc_run(False) has no meaning: pass the run's parameters")
        restart = True
        mc_params, temp, ensemble, potential = read_params(ckdir, eq_cycles)
        ck = read_checkpoint(ckdir)
        start_config = ck["configs"][0]["config"]
    eng = Engine(mc_params, temp, potential, ensemble, precision=precision,
                 resync_every=resync_every, exch_prob=exch_prob, seed=seed, rdfsave=rdfsave)
    try:
        eng.set_configs(0, start_config, max_displ)
        eng.init()
        if restart:
            eng.restore(ckdir)
            done = _restored_index(ckdir)
            if not os.path.exists(os.path.join(ckdir, "engine.bin")):
                # a reference checkpoint: its loop resumes at the saved index,
                # so cycle `index` runs again (src/MCRun.jl:455)
                done -= 1
        else:
            eng.equilibrate()
            done = 0
        total = mc_params.mc_cycles
        marks = set()
        if save:
            marks.update(range(save, total + 1, save))
        if saveconfigs:
            marks.update(range(saveconfigs, total + 1, saveconfigs))
        for m in sorted(x for x in marks if x > done):
            eng.run_cycles(m - done)
            done = m
            if save and m % save == 0:
                eng.checkpoint(ckdir)
            if saveconfigs and m % saveconfigs == 0:
                _save_configs(eng, ckdir, "%s%d" % (configsname, m))
        if done < total:
            eng.run_cycles(total - done)
        if save and total % save != 0:
            eng.checkpoint(ckdir)
        results = eng.output(0)
        states = eng.mc_states(0)
        return states, results
    finally:
        eng.close()


def read_params(ckdir, eq_cycles=0.2):
    """read_init (src/ReadSave.jl:330-345) of checkpoint/params.data: MCParams
    (with eq_cycles = floor(eq_cycles * cycles) as on restart, :310-320),
    TempGrid, the ensemble and the potential (ELJ, ELJEven, EAM, ELJB)."""
    with open(os.path.join(ckdir, "params.data")) as f:
        rows = [ln.split() for ln in f.read().strip().split("\n")]
    pv = [float(x) for x in rows[1]]
    mp = MCParams(int(pv[0]), int(math.floor(eq_cycles * pv[0])), int(pv[1]), int(pv[2]),
                  int(pv[3]), int(pv[4]), int(pv[5]), pv[6], pv[7])
    temp = TempGrid(pv[8], pv[9], int(pv[2]))
    ens = rows[3]
    if ens[0] == "NVT":
        ensemble = NVT(int(ens[1]))
    elif ens[0].startswith("NPT"):
        ensemble = NPT(int(ens[1]), float(ens[5]), ens[6] == "true")
    else:
        raise ValueError("params.data: ensemble %s cannot be rebuilt here" % ens[0])
    pot = rows[4]
    # "ELJPotentialEven{6, Float64} c1 ... c6": the type's tokens are not numbers
    coeff = [float(x) for x in pot[1:] if _is_number(x)]
    if pot[0].startswith("ELJPotentialEven"):
        potential = ELJPotentialEven(coeff)
    elif pot[0].startswith("ELJPotential"):
        potential = ELJPotential(coeff)
    elif pot[0] == "EAM:":
        n, m, ean, ecam = (float(x) for x in pot[1:5])
        potential = EmbeddedAtomPotential(n, m, ean=ean, eCam=ecam)
    elif pot[0] == "ELJB":
        a = [float(x) for x in rows[5]]
        b = [float(x) for x in rows[6]]
        c = [float(x) for x in rows[7]]
        potential = ELJPotentialB(a, b, c)
    else:
        raise ValueError("params.data: potential %s cannot be rebuilt here" % pot[0])
    return mp, temp, ensemble, potential


def _is_number(t):
    try:
        float(t)
        return True
    except ValueError:
        return False


def _restored_index(ckdir):
    with open(os.path.join(ckdir, "index.txt")) as f:
        return int(float(f.read().split()[0]))


def _save_configs(eng, ckdir, name):
    """save_configs (src/ReadSave.jl:160-170) in the xyz format of checkpoint_config."""
    os.makedirs(ckdir, exist_ok=True)
    for i, st in enumerate(eng.mc_states(0)):
        with open(os.path.join(ckdir, "%sT%d.xyz" % (name, i + 1)), "w") as f:
            f.write("%d\n" % len(st.config))
            bc = st.config.boundary_condition
            if isinstance(bc, SphericalBC):
                hdr = "SphericalBC{Float64} r2: %s" % _jl(bc.radius2)
            elif isinstance(bc, CubicBC):
                hdr = "CubicBC{Float64} box_length: %s" % _jl(bc.box_length)
            else:  # bc_info (src/ReadSave.jl:133-135)
                hdr = "%s{Float64} box_dims: %s, %s" % (type(bc).__name__, _jl(bc.box_length),
                                                        _jl(bc.box_height))
            md3 = st.max_displ[2] if len(st.max_displ) > 2 else 0.1
            f.write("%s %s %s %s %d %d\n" % (hdr, _jl(st.max_displ[0]), _jl(st.max_displ[1]),
                                             _jl(md3), st.count_atom[0], st.count_vol[0]))
            for x in st.config.positions:
                f.write("1  %s %s %s \n" % (_jl(x[0]), _jl(x[1]), _jl(x[2])))


# ------------------------------------------------------------------ analysis
def multihistogram_NVT(ensemble, temp, results, conv_threshold, readfile=False, debug=False):
    """multihistogram_NVT (src/multihist_NVT.jl:95-221) on the GPU; returns
    Cv on TempGrid{10R}(t_1, t_R)."""
    T, cv, _ = multihist_nvt_arrays(results.en_histogram, temp.t_grid, temp.beta_grid,
                                    results.en_min, results.en_max, conv_threshold)
    return cv


def multihistogram_NPT(ensemble, temp, results, conv_threshold, readfile=False, debug=False):
    """multihistogram_NPT (src/multihist_NPT.jl:113-338) on the GPU; returns
    (T, Cp) on TempGrid{10R}(t_1, t_R)."""
    T, cp, _ = multihist_npt_arrays(results.ev_histogram, temp.t_grid, temp.beta_grid,
                                    results.en_min, results.en_max, results.v_min,
                                    results.v_max, ensemble.pressure, conv_threshold)
    return T, cp


def multihist_nvt_arrays(hist, t_grid, beta, en_min, en_max, thr):
    L = _capi.load()
    h = np.ascontiguousarray(hist, dtype=np.float64)
    R, nb = h.shape
    t, b = np.ascontiguousarray(t_grid, float), np.ascontiguousarray(beta, float)
    T, cv, it = np.zeros(10 * R), np.zeros(10 * R), ctypes.c_int()
    _capi.check(L.ptmc_multihist_nvt(R, nb - 2, _dptr(h), _dptr(t), _dptr(b), en_min, en_max,
                                     thr, _dptr(T), _dptr(cv), ctypes.byref(it)))
    return T, cv, it.value


def multihist_npt_arrays(hist, t_grid, beta, en_min, en_max, v_min, v_max, p, thr):
    L = _capi.load()
    h = np.ascontiguousarray(hist, dtype=np.float64)
    R, nb = h.shape[0], h.shape[1]
    t, b = np.ascontiguousarray(t_grid, float), np.ascontiguousarray(beta, float)
    T, cp, it = np.zeros(10 * R), np.zeros(10 * R), ctypes.c_int()
    _capi.check(L.ptmc_multihist_npt(R, nb - 2, _dptr(h), _dptr(t), _dptr(b), en_min, en_max,
                                     v_min, v_max, p, thr, _dptr(T), _dptr(cp), ctypes.byref(it)))
    return T, cp, it.value


# ------------------------------------------------------------------ checkpoints
def multihist_linear_arrays(hist, beta, en_min, en_max, npoints=1000):
    """The linear-solve multihistogram on the GPU (ptmc_multihist_linear)."""
    L = _capi.load()
    h = np.ascontiguousarray(hist, dtype=np.float64)
    R, nb = h.shape
    n_bin = nb - 2
    b = np.ascontiguousarray(beta, dtype=np.float64)
    E, S, al = np.zeros(n_bin), np.zeros(n_bin), np.zeros(R)
    nk = ctypes.c_int()
    out = {k: np.zeros(npoints) for k in ("T", "Z", "U", "Cv", "dCv", "S_T")}
    _capi.check(L.ptmc_multihist_linear(R, n_bin, _dptr(h), _dptr(b), en_min, en_max, int(npoints),
                                        _dptr(E), _dptr(S), ctypes.byref(nk), _dptr(al),
                                        _dptr(out["T"]), _dptr(out["Z"]), _dptr(out["U"]),
                                        _dptr(out["Cv"]), _dptr(out["dCv"]), _dptr(out["S_T"])))
    k = nk.value
    out.update(energies=E[:k], S_E=S[:k], alpha=al)
    return out


def _jl(x):
    """A float as Julia prints it ("0.1", "100.0", "1.0e-5", "-5.6e7")."""
    x = float(x)
    if x == 0:
        return "-0.0" if math.copysign(1, x) < 0 else "0.0"
    if not math.isfinite(x):
        return "NaN" if x != x else ("Inf" if x > 0 else "-Inf")
    r = repr(abs(x))  # shortest round-trip digits
    if "e" in r:
        mant, ex = r.split("e")
        ex = int(ex)
    else:
        mant, ex = r, 0
        if "." in mant:
            ip, fp = mant.split(".")
        else:
            ip, fp = mant, ""
        # normalise to d.ddd x 10^ex
        if ip.strip("0"):
            ex = len(ip.lstrip("0")) - 1
            digits = (ip.lstrip("0") + fp).rstrip("0") or "0"
        else:
            lead = len(fp) - len(fp.lstrip("0"))
            ex = -lead - 1
            digits = fp.lstrip("0").rstrip("0") or "0"
        mant = digits[0] + ("." + digits[1:] if len(digits) > 1 else "")
    digits = mant.replace(".", "").rstrip("0") or "0"
    if -4 <= ex < 6:  # Julia: 0.0001 fixed, 1.0e-5 and 1.0e6 scientific
        if ex >= 0:
            ip = digits[:ex + 1].ljust(ex + 1, "0")
            fp = digits[ex + 1:] or "0"
            txt = ip + "." + fp
        else:
            txt = "0." + "0" * (-ex - 1) + digits
    else:
        txt = digits[0] + "." + (digits[1:] or "0") + "e" + str(ex)
    return ("-" if x < 0 else "") + txt


def multihistogram(output, temp, outdir=None, npoints=1000):
    """multihistogram(output, Tvec; outdir, NPoints) (src/multihist.jl:437-455):
    the linear-solve multihistogram on the GPU.  Writes histograms.data, Sol.X,
    S.data and analysis.NVT (T, Z, Cv, dCv, U(T)) into `outdir` (default: the
    current directory) and returns the arrays (dict)."""
    res = multihist_linear_arrays(output.en_histogram, temp.beta_grid, output.en_min,
                                  output.en_max, npoints)
    h = np.asarray(output.en_histogram, dtype=float)[:, 1:-1] / output.n_bin
    h = h[:, h.sum(axis=0) != 0]
    res["histograms"] = h
    d = outdir or os.getcwd()
    os.makedirs(d, exist_ok=True)

    def row(v):
        return "\t".join(_jl(x) for x in v) + "\n"
    with open(os.path.join(d, "histograms.data"), "w") as f:
        f.write(row(res["energies"]))
        for r in h:
            f.write(row(r))
    with open(os.path.join(d, "Sol.X"), "w") as f:
        f.write("alpha\n" + row(res["alpha"]))
    with open(os.path.join(d, "S.data"), "w") as f:
        f.write("E\tEntropy\n")
        for e, s_ in zip(res["energies"], res["S_E"]):
            f.write(row((e, s_)))
    with open(os.path.join(d, "analysis.NVT"), "w") as f:
        f.write("T\tZ\tCv\tdCv\tU(T)\n")
        for k in range(npoints):
            f.write(row((res["T"][k], res["Z"][k], res["Cv"][k], res["dCv"][k], res["U"][k])))
    return res


def postprocess(xdir=None, npoints=1000):
    """postprocess(; xdir) (src/multihist.jl:457-485): the linear-solve
    multihistogram of the run whose checkpoint is <xdir>/checkpoint (its
    histograms and temperature grid); the four output files are written into
    xdir, the checkpoint is left as it is.  Returns (energies, histogramdata,
    T, Z, Cv, dCv, U) as the reference (its last column is U(T))."""
    d = xdir or os.getcwd()
    ck = read_checkpoint(os.path.join(d, "checkpoint"))
    p = ck["params"]
    R, n_bin = int(p[2]), int(p[5])
    temp = TempGrid(p[8], p[9], R)
    hi = ck["hist_info"]
    out = Output(n_bin=n_bin, en_min=hi[0], en_max=hi[1], en_histogram=ck["histograms"][:R])
    res = multihistogram(out, temp, outdir=d, npoints=npoints)
    return (res["energies"], list(res["histograms"]), res["T"], res["Z"], res["Cv"], res["dCv"],
            res["U"])


def read_checkpoint(directory):
    """Read a reference checkpoint directory (src/ReadSave.jl:330-481):
    params.data, hist_info.data, histograms.data, [volume_hist.data],
    index.txt and configT<i>.xyz or config.<i>.  Returns a dict."""
    def rows(path):
        with open(path) as f:
            return [ln.split() for ln in f.read().strip().split("\n")]

    out = {}
    p = rows(os.path.join(directory, "params.data"))
    out["params"] = [float(x) for x in p[1]]
    out["ensemble"] = p[3]
    out["potential"] = p[4]
    hi = rows(os.path.join(directory, "hist_info.data"))
    out["hist_info"] = [float(x) for x in hi[1]]
    out["histograms"] = np.array([[float(x) for x in r] for r in
                                  rows(os.path.join(directory, "histograms.data"))])
    vp = os.path.join(directory, "volume_hist.data")
    if os.path.exists(vp):
        v = np.array([[float(x) for x in r] for r in rows(vp)])
        nb = int(round(math.sqrt(v.shape[1])))
        out["volume_hist"] = v.reshape(v.shape[0], nb, nb).transpose(0, 2, 1)
    ip = os.path.join(directory, "index.txt")
    if os.path.exists(ip):
        out["index"] = int(float(open(ip).read().split()[0]))
    # one file per replica; the count is taken from the files present (the
    # reference's own fixture holds 25 files for n_traj = 24)
    configs = []
    i = 0
    while True:
        i += 1
        names = [n for n in ("configT%d.xyz" % i, "config.%d" % i)
                 if os.path.exists(os.path.join(directory, n))]
        if not names:
            break
        for name in names:
            path = os.path.join(directory, name)
            if os.path.exists(path):
                r = rows(path)
                n = int(r[0][0])
                hdr = r[1]
                xyz = np.array([[float(x) for x in ln[1:4]] for ln in r[2:2 + n]])
                if hdr[0].startswith("SphericalBC"):
                    bc = SphericalBC(math.sqrt(float(hdr[2])))
                    md = [float(x) for x in hdr[3:6]]
                    counts = [int(float(x)) for x in hdr[6:8]]
                elif hdr[0].startswith(("RhombicBC", "RectangularBC")):
                    # bc_info "box_dims: L, H" (src/ReadSave.jl:133-135)
                    cls = RhombicBC if hdr[0].startswith("RhombicBC") else RectangularBC
                    bc = cls(float(hdr[2].rstrip(",")), float(hdr[3]))
                    md = [float(x) for x in hdr[4:7]]
                    counts = [int(float(x)) for x in hdr[7:9]]
                else:
                    bc = CubicBC(float(hdr[2]))
                    md = [float(x) for x in hdr[3:6]]
                    counts = [int(float(x)) for x in hdr[6:8]]
                configs.append(dict(config=Config(xyz, bc), max_displ=md, counts=counts))
                break
    out["configs"] = configs
    return out
