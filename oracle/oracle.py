"""ctypes binding of the CPU oracle (oracle/ptmc_oracle.cpp).

TEST INFRASTRUCTURE ONLY: the checker for the GPU engine and the timed CPU
baseline.  Nothing in the product imports this module.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "libptmc_oracle.so")
SRC = os.path.join(HERE, "ptmc_oracle.cpp")

POT_ELJ, POT_ELJEVEN, POT_EAM, POT_NN = 0, 1, 2, 3
BC_SPHERE, BC_CUBIC, BC_RECT, BC_RHOMBIC = 0, 1, 2, 3
POT_ELJB, POT_LUT = 4, 5
NVT, NPT, NNVT = 0, 1, 2

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_lp = ctypes.POINTER(ctypes.c_long)


def build(force=False):
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < max(
            os.path.getmtime(SRC), os.path.getmtime(os.path.join(HERE, "ptmc_oracle.h"))):
        cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared",
               "-o", LIB + ".tmp", SRC]
        subprocess.run(cmd, check=True)
        os.replace(LIB + ".tmp", LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        L.orc_create.restype = ctypes.c_void_p
        L.orc_create.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                 ctypes.c_int, ctypes.c_double, _dp, _dp, _dp, ctypes.c_int,
                                 ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                 ctypes.c_double, ctypes.c_uint64, ctypes.c_int]
        L.orc_destroy.argtypes = [ctypes.c_void_p]
        L.orc_last_error.restype = ctypes.c_char_p
        L.orc_set_pot_elj.argtypes = [ctypes.c_void_p, _dp, ctypes.c_int, ctypes.c_int]
        L.orc_set_pot_eam.argtypes = [ctypes.c_void_p] + [ctypes.c_double] * 4
        L.orc_set_pot_nn.argtypes = [ctypes.c_void_p, _dp, ctypes.c_int, _dp, ctypes.c_int,
                                     _ip, ctypes.c_int, ctypes.c_double]
        L.orc_init.argtypes = [ctypes.c_void_p]
        L.orc_equilibrate.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.orc_production.argtypes = [ctypes.c_void_p, ctypes.c_long, ctypes.c_long]
        L.orc_cycles.argtypes = [ctypes.c_void_p, ctypes.c_long, ctypes.c_long]
        L.orc_get_walkers.argtypes = [ctypes.c_void_p, _dp, _dp, _dp]
        L.orc_get_slots.argtypes = [ctypes.c_void_p, _ip, _dp, _lp, _lp, _lp, _dp]
        L.orc_get_hist.argtypes = [ctypes.c_void_p, _dp, _dp, _dp]
        L.orc_finalise.argtypes = [ctypes.c_void_p, ctypes.c_long, ctypes.c_int, _dp, _dp, _dp, _dp]
        L.orc_get_nn_state.argtypes = [ctypes.c_void_p, ctypes.c_int, _dp, _dp]
        L.orc_dimer_energy.restype = ctypes.c_double
        L.orc_dimer_energy.argtypes = [ctypes.c_int, _dp, ctypes.c_int, ctypes.c_double]
        L.orc_distance2.restype = ctypes.c_double
        L.orc_distance2.argtypes = [_dp, _dp, ctypes.c_int, ctypes.c_double]
        L.orc_lrc.restype = ctypes.c_double
        L.orc_lrc.argtypes = [ctypes.c_int, ctypes.c_double, _dp, ctypes.c_int]
        L.orc_distance2_box.restype = ctypes.c_double
        L.orc_distance2_box.argtypes = [_dp, _dp, ctypes.c_int, ctypes.c_double, ctypes.c_double]
        L.orc_box_rcut.restype = ctypes.c_double
        L.orc_box_rcut.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_double]
        L.orc_box_volume.restype = ctypes.c_double
        L.orc_box_volume.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_double]
        L.orc_elj_config_energy_box.restype = ctypes.c_double
        L.orc_elj_config_energy_box.argtypes = [_dp, ctypes.c_int, ctypes.c_int, _dp, ctypes.c_int,
                                                ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                                ctypes.c_int]
        L.orc_get_tan.restype = ctypes.c_double
        L.orc_get_tan.argtypes = [_dp, _dp, ctypes.c_int, ctypes.c_double, ctypes.c_double]
        L.orc_eljb_energy.restype = ctypes.c_double
        L.orc_eljb_energy.argtypes = [_dp, _dp, _dp, ctypes.c_int, ctypes.c_double, ctypes.c_double]
        L.orc_lut_energy.restype = ctypes.c_double
        L.orc_lut_energy.argtypes = [_dp, ctypes.c_int, ctypes.c_int] + [ctypes.c_double] * 6
        L.orc_set_pot_eljb.argtypes = [ctypes.c_void_p, _dp, _dp, _dp, ctypes.c_int]
        L.orc_set_pot_lut.argtypes = [ctypes.c_void_p, _dp, ctypes.c_int, ctypes.c_int] + \
            [ctypes.c_double] * 5
        L.orc_set_pot_nn2.argtypes = [ctypes.c_void_p, _dp, ctypes.c_int, _dp, ctypes.c_int, _dp,
                                      _dp, ctypes.c_int, _ip, ctypes.c_int, ctypes.c_int,
                                      ctypes.c_int]
        L.orc_get_swaps.restype = ctypes.c_long
        L.orc_get_swaps.argtypes = [ctypes.c_void_p]
        L.orc_set_box.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_int, _dp]
        L.orc_get_box.argtypes = [ctypes.c_void_p, _dp, _dp, _lp, _lp]
        L.orc_eam_config_energy.restype = ctypes.c_double
        L.orc_eam_config_energy.argtypes = [_dp, ctypes.c_int] + [ctypes.c_double] * 4
        L.orc_elj_config_energy.restype = ctypes.c_double
        L.orc_elj_config_energy.argtypes = [_dp, ctypes.c_int, ctypes.c_int, _dp, ctypes.c_int,
                                            ctypes.c_int, ctypes.c_double, ctypes.c_double]
        L.orc_tempgrid.argtypes = [ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_int, _dp, _dp]
        L.orc_u01.restype = ctypes.c_double
        L.orc_u01.argtypes = [ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint64]
        L.orc_philox4x32.argtypes = [ctypes.POINTER(ctypes.c_uint32)] * 3
        L.orc_mlp_forward.argtypes = [_dp, ctypes.c_int, ctypes.c_int, _dp, ctypes.c_int, _ip,
                                      ctypes.c_int, _dp]
        L.orc_multihist_nvt.argtypes = [ctypes.c_int, ctypes.c_int, _dp, _dp, _dp, ctypes.c_double,
                                        ctypes.c_double, ctypes.c_double, _dp, _dp, _ip]
        L.orc_multihist_npt.argtypes = [ctypes.c_int, ctypes.c_int, _dp, _dp, _dp, ctypes.c_double,
                                        ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                        ctypes.c_double, ctypes.c_double, _dp, _dp, _ip]
        L.orc_multihist_linear.argtypes = [ctypes.c_int, ctypes.c_int, _dp, _dp, ctypes.c_double,
                                           ctypes.c_double, ctypes.c_int, _dp, _dp, _ip, _dp, _dp,
                                           _dp, _dp, _dp, _dp, _dp]
        L.orc_set_rdf.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.orc_get_rdf.argtypes = [ctypes.c_void_p, _dp, _dp]
        _fp = ctypes.POINTER(ctypes.c_float)
        L.orc_sur_nparams.restype = ctypes.c_int
        L.orc_sur_forward.argtypes = [_dp, _dp, _fp, ctypes.c_int, ctypes.c_int, _dp]
        L.orc_sur_loss_grad.argtypes = [_dp, _dp, _fp, _fp, ctypes.c_int, ctypes.c_int, _dp, _dp]
        L.orc_set_surrogate.argtypes = [ctypes.c_void_p, _dp, _dp, ctypes.c_int]
        L.orc_get_sur_stats.argtypes = [ctypes.c_void_p, _lp]
        _lib = L
    return _lib


def _d(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def P(a):
    return a.ctypes.data_as(_dp)


def _check(rc):
    if rc != 0:
        raise RuntimeError("oracle: " + lib().orc_last_error().decode())


def dimer_energy(kind, c, r2):
    c = _d(c)
    return lib().orc_dimer_energy(kind, P(c), len(c), float(r2))


def distance2(a, b, bc=BC_SPHERE, L=0.0):
    a, b = _d(a), _d(b)
    return lib().orc_distance2(P(a), P(b), bc, float(L))


def distance2_box(a, b, bc, L, H):
    """distance2 for a box of length L and height H (RectangularBC, RhombicBC)."""
    a, b = _d(a), _d(b)
    return lib().orc_distance2_box(P(a), P(b), bc, float(L), float(H))


def box_rcut(bc, L, H):
    return lib().orc_box_rcut(bc, float(L), float(H))


def box_volume(bc, L, H):
    return lib().orc_box_volume(bc, float(L), float(H))


def elj_config_energy_box(xyz, kind, c, bc, L, H, cut=True):
    x, c = _d(xyz), _d(c)
    return lib().orc_elj_config_energy_box(P(x), len(x), kind, P(c), len(c), bc, float(L),
                                           float(H), int(bool(cut)))


def get_tan(a, b, bc=BC_SPHERE, L=0.0, H=None):
    """get_tan (src/Configurations.jl:181-215)."""
    a, b = _d(a), _d(b)
    return lib().orc_get_tan(P(a), P(b), bc, float(L), float(L if H is None else H))


def eljb_energy(a, b, c, r2, tn):
    a, b, c = _d(a), _d(b), _d(c)
    return lib().orc_eljb_energy(P(a), P(b), P(c), len(c), float(r2), float(tn))


def lut_energy(lut, r2, tn):
    """lut: dict(table [l_angle, l_dist], start_dist, d_dist, d_angle, c6coeff)."""
    t = np.asfortranarray(lut["table"], dtype=np.float64)
    flat = np.ascontiguousarray(t.reshape(-1, order="F"))
    la, ld = t.shape
    return lib().orc_lut_energy(P(flat), la, ld, lut["start_dist"], lut["d_dist"], lut["d_angle"],
                                lut["c6coeff"], float(r2), float(tn))


def lrc(N, rc2, c):
    c = _d(c)
    return lib().orc_lrc(N, float(rc2), P(c), len(c))


def eam_config_energy(xyz, n, m, ean, ecam):
    x = _d(xyz)
    return lib().orc_eam_config_energy(P(x), len(x), n, m, ean, ecam)


def elj_config_energy(xyz, kind, c, bc=BC_SPHERE, L=0.0, rc2=0.0):
    x, c = _d(xyz), _d(c)
    return lib().orc_elj_config_energy(P(x), len(x), kind, P(c), len(c), bc, L, rc2)


def tempgrid(ti, tf, R, tdistr=0):
    T, B = np.zeros(R), np.zeros(R)
    lib().orc_tempgrid(ti, tf, R, tdistr, P(T), P(B))
    return T, B


def u01(seed, stream, run, idx):
    return lib().orc_u01(seed, stream, run, idx)


def philox4x32(ctr, key):
    c = np.ascontiguousarray(ctr, dtype=np.uint32)
    k = np.ascontiguousarray(key, dtype=np.uint32)
    o = np.zeros(4, dtype=np.uint32)
    u = ctypes.POINTER(ctypes.c_uint32)
    lib().orc_philox4x32(c.ctypes.data_as(u), k.ctypes.data_as(u), o.ctypes.data_as(u))
    return o


def mlp_forward(x, weights, nodes):
    x = _d(x)
    w = _d(weights)
    nd = np.ascontiguousarray(nodes, dtype=np.int32)
    out = np.zeros(x.shape[0])
    _check(lib().orc_mlp_forward(P(x), x.shape[1], x.shape[0], P(w), len(w),
                                 nd.ctypes.data_as(_ip), len(nd), P(out)))
    return out


def multihist_nvt(hist, t_grid, beta, en_min, en_max, thr):
    h = _d(hist)
    R, nb = h.shape
    T, cv, it = np.zeros(10 * R), np.zeros(10 * R), ctypes.c_int()
    _check(lib().orc_multihist_nvt(R, nb - 2, P(h), P(_d(t_grid)), P(_d(beta)), en_min, en_max,
                                   thr, P(T), P(cv), ctypes.byref(it)))
    return T, cv, it.value


def multihist_npt(hist, t_grid, beta, en_min, en_max, v_min, v_max, p, thr):
    h = _d(hist)
    R, nb = h.shape[0], h.shape[1]
    T, cp, it = np.zeros(10 * R), np.zeros(10 * R), ctypes.c_int()
    _check(lib().orc_multihist_npt(R, nb - 2, P(h), P(_d(t_grid)), P(_d(beta)), en_min, en_max,
                                   v_min, v_max, p, thr, P(T), P(cp), ctypes.byref(it)))
    return T, cp, it.value


class Run:
    """One PT run on the CPU oracle (walker/slot formulation, Philox draws)."""

    def __init__(self, N, R, xyz, T, ensemble=NVT, pressure=0.0, bc=BC_SPHERE, bc_param=10.0,
                 max_displ=None, n_bin=100, n_adjust=100, mc_sample=1, min_acc=0.4, max_acc=0.6,
                 exch_prob=0.1, seed=1234, run_index=0):
        self.N, self.R, self.ens = N, R, ensemble
        xyz = _d(xyz).reshape(R, N, 3)
        T = _d(T)
        md = _d(max_displ if max_displ is not None else np.full(2 * R, 0.1))
        self.n_bin = n_bin
        h = lib().orc_create(N, R, ensemble, pressure, bc, bc_param, P(xyz), P(T), P(md), n_bin,
                             n_adjust, mc_sample, min_acc, max_acc, exch_prob, seed, run_index)
        if not h:
            raise RuntimeError("oracle: " + lib().orc_last_error().decode())
        self.h = h

    def set_box(self, height, separated=False, max_displ_sep=None):
        """RectangularBC / RhombicBC: box height (bc_param is the length),
        NPT separated volume moves, initial max_displ[3:4] (2 per slot)."""
        md = None if max_displ_sep is None else _d(max_displ_sep)
        self._mds = md
        _check(lib().orc_set_box(self.h, float(height), int(bool(separated)),
                                 None if md is None else P(md)))

    def box(self):
        """walker heights [R]; per slot max_displ[3:4] [R,2], count_vol_xy [R,2], count_vol_z [R,2]"""
        R = self.R
        h, md = np.zeros(R), np.zeros(2 * R)
        cxy, cz = np.zeros(2 * R, dtype=np.int64), np.zeros(2 * R, dtype=np.int64)
        lp = lambda a: a.ctypes.data_as(_lp)
        _check(lib().orc_get_box(self.h, P(h), P(md), lp(cxy), lp(cz)))
        return dict(height=h, max_displ_sep=md.reshape(R, 2), count_xy=cxy.reshape(R, 2),
                    count_z=cz.reshape(R, 2))

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_destroy(self.h)
            self.h = None

    def set_elj(self, c, even):
        c = _d(c)
        _check(lib().orc_set_pot_elj(self.h, P(c), len(c), int(even)))

    def set_eljb(self, a, b, c):
        self._eljb = (_d(a), _d(b), _d(c))
        _check(lib().orc_set_pot_eljb(self.h, *(P(x) for x in self._eljb), len(self._eljb[2])))

    def set_lut(self, lut):
        """lut: dict(table [l_angle, l_dist], start_dist, start_angle, d_dist, d_angle, c6coeff)."""
        t = np.asarray(lut["table"], dtype=np.float64)
        self._lut = np.ascontiguousarray(t.reshape(-1, order="F"))
        la, ld = t.shape
        _check(lib().orc_set_pot_lut(self.h, P(self._lut), la, ld, lut["start_dist"],
                                     lut.get("start_angle", 0.0), lut["d_dist"], lut["d_angle"],
                                     lut["c6coeff"]))

    def set_nn2(self, rad, ang, w1, w2, nodes, n1, n_swaps=1):
        """RuNNerPotential2Atom in the NNVT ensemble: rad [nrad, 10], ang [nang, 16]."""
        self._nn2 = (_d(rad), _d(ang), _d(w1), _d(w2),
                     np.ascontiguousarray(nodes, dtype=np.int32))
        rd, an, a, b, nd = self._nn2
        _check(lib().orc_set_pot_nn2(self.h, P(rd), rd.shape[0], P(an), an.shape[0] if an.size else 0,
                                     P(a), P(b), len(a), nd.ctypes.data_as(_ip), len(nd), n1,
                                     n_swaps))

    def swaps(self):
        return lib().orc_get_swaps(self.h)

    def set_eam(self, n, m, ean, ecam):
        _check(lib().orc_set_pot_eam(self.h, n, m, ean, ecam))

    def set_nn(self, sf, weights, nodes, boundary=0.0):
        sf, w = _d(sf), _d(weights)
        nd = np.ascontiguousarray(nodes, dtype=np.int32)
        _check(lib().orc_set_pot_nn(self.h, P(sf), sf.shape[0], P(w), len(w),
                                    nd.ctypes.data_as(_ip), len(nd), boundary))

    def init(self):
        _check(lib().orc_init(self.h))

    def equilibrate(self, eq):
        _check(lib().orc_equilibrate(self.h, eq))

    def production(self, first, n):
        _check(lib().orc_production(self.h, first, n))

    def cycles(self, first, n):
        _check(lib().orc_cycles(self.h, first, n))

    def walkers(self):
        x = np.zeros((self.R, self.N, 3))
        e, b = np.zeros(self.R), np.zeros(self.R)
        lib().orc_get_walkers(self.h, P(x), P(e), P(b))
        return x, e, b

    def slots(self):
        R = self.R
        wos = np.zeros(R, dtype=np.int32)
        md = np.zeros(2 * R)
        ca, cv, ce = (np.zeros(2 * R, dtype=np.int64) for _ in range(3))
        ham = np.zeros(2 * R)
        lp = lambda a: a.ctypes.data_as(_lp)
        lib().orc_get_slots(self.h, wos.ctypes.data_as(_ip), P(md), lp(ca), lp(cv), lp(ce), P(ham))
        return dict(wos=wos, max_displ=md.reshape(R, 2), count_atom=ca.reshape(R, 2),
                    count_vol=cv.reshape(R, 2), count_exc=ce.reshape(R, 2), ham=ham.reshape(R, 2))

    def slot_states(self):
        """(xyz, en, box) in slot order, like the engine's ptmc_get_states."""
        x, e, b = self.walkers()
        wos = self.slots()["wos"]
        return x[wos], e[wos], b[wos]

    def hist(self):
        nb = self.n_bin + 2
        eh = np.zeros((self.R, nb))
        ev = np.zeros((self.R, nb, nb)) if self.ens == NPT else np.zeros(1)
        hp = np.zeros(6)
        lib().orc_get_hist(self.h, P(eh), P(ev), P(hp))
        return eh, ev, hp

    def finalise(self, mc_cycles, mc_sample=1):
        R = self.R
        a, b, c, d = (np.zeros(R) for _ in range(4))
        lib().orc_finalise(self.h, mc_cycles, mc_sample, P(a), P(b), P(c), P(d))
        return dict(en_avg=a, heat_cap=b, count_stat_atom=c, count_stat_exc=d)

    def set_rdf(self, on=True):
        _check(lib().orc_set_rdf(self.h, int(bool(on))))

    def rdf(self):
        out = np.zeros((self.R, 5 * self.n_bin))
        dr2 = np.zeros(1)
        _check(lib().orc_get_rdf(self.h, P(out), P(dr2)))
        return out, float(dr2[0])

    def set_surrogate(self, cfg, params, bf16=True):
        """Delayed-acceptance atom moves with the pair surrogate (None: off)."""
        if params is None:
            _check(lib().orc_set_surrogate(self.h, None, None, 0))
            return
        self._sur = (_d(cfg), _d(params))
        _check(lib().orc_set_surrogate(self.h, P(self._sur[0]), P(self._sur[1]), int(bf16)))

    def sur_stats(self):
        out = (ctypes.c_long * 2)()
        lib().orc_get_sur_stats(self.h, out)
        return dict(stage1_rejects=out[0], exact_evals=out[1])

    def nn_state(self, w, nsf):
        G = np.zeros((nsf, self.N))
        ea = np.zeros(self.N)
        _check(lib().orc_get_nn_state(self.h, w, P(G), P(ea)))
        return G, ea


# ---------------------------------------------------------------- surrogate
def _f(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _fptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def sur_nparams():
    return lib().orc_sur_nparams()


def sur_forward(cfg, params, rows, bf16=True):
    """dE_s of every record (rows: (n, 128) distances, negative = no pair)."""
    cfg, params, rows = _d(cfg), _d(params), _f(rows)
    out = np.zeros(rows.shape[0])
    _check(lib().orc_sur_forward(P(cfg), P(params), _fptr(rows), rows.shape[0], int(bf16), P(out)))
    return out


def sur_loss_grad(cfg, params, rows, targets, bf16=True):
    cfg, params, rows, targets = _d(cfg), _d(params), _f(rows), _f(targets)
    loss = np.zeros(1)
    g = np.zeros(sur_nparams())
    _check(lib().orc_sur_loss_grad(P(cfg), P(params), _fptr(rows), _fptr(targets), rows.shape[0],
                                   int(bf16), P(loss), P(g)))
    return float(loss[0]), g


def multihist_linear(en_hist, beta, en_min, en_max, npoints=1000):
    """Linear-solve multihistogram (src/multihist.jl); returns a dict."""
    h = _d(en_hist)
    R, nb = h.shape
    n_bin = nb - 2
    beta = _d(beta)
    E, S = np.zeros(n_bin), np.zeros(n_bin)
    nk = (ctypes.c_int * 1)()
    al = np.zeros(R)
    out = {k: np.zeros(npoints) for k in ("T", "Z", "U", "Cv", "dCv", "S_T")}
    _check(lib().orc_multihist_linear(R, n_bin, P(h), P(beta), en_min, en_max, npoints, P(E), P(S),
                                      ctypes.cast(nk, _ip), P(al), P(out["T"]), P(out["Z"]),
                                      P(out["U"]), P(out["Cv"]), P(out["dCv"]), P(out["S_T"])))
    k = nk[0]
    out.update(energies=E[:k], S_E=S[:k], alpha=al)
    return out
