"""GPU tests of the FP32_RESYNC form (FP32 move rows, FP64 running total,
periodic FP64 resync) against the FP64 plain form and the oracle.

The FP32 form is a different Markov chain realisation (FP32 pair terms, its own
draw stream, fixed-point positions), so it is compared statistically:
  * its running energy stays within a small drift of an FP64 recomputation of
    the same positions (tolerance 1e-6 relative, set by FP32 rounding of the
    pair terms over the resync interval);
  * after a run, the engine's energies equal the oracle's FP64 energy of the
    returned positions to 1e-7 relative (right after a resync: 1e-12);
  * per-temperature mean energies and heat capacities agree with the FP64
    form within 4 combined standard errors over independent runs.
"""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

C_NE = [-10.5097942564988, 989.725135614556, -101383.865938807, 3918846.12841668,
        -56234083.4334278, 288738837.441765]
CU_EAM = dict(n=8.482, m=4.692, eps=0.0367493 * 0.0370, C=27.561, a=0.25 * 18.8973)


def cu55_ico():
    d = json.load(open(os.path.join(GOLDEN, "nn_cu55.json")))
    return np.array(d["ico55_nm"]) * (d["cu_lattice_nm"] * d["nm_to_bohr"])


def engine(pk, *, N, R, starts, T, pot, bc, precision, resync=200, n_runs=1, seed=1,
           ens=None, eq=0, cycles=1000):
    mp = pk.MCParams(mc_cycles=cycles, eq_cycles=eq, mc_sample=1, n_traj=R, n_atoms=N)
    e = pk.Engine(mp, pk.TempGrid(T[0], T[1], R), pot, ens or pk.NVT(N), n_runs=n_runs,
                  precision=precision, resync_every=resync, exch_prob=1.0, seed=seed)
    for r in range(n_runs):
        e.set_configs(r, pk.Config(starts[r % len(starts)], bc))
    e.init()
    return e


def test_eam_fp32_energy_tracks_fp64(pk, orc):
    pot = pk.EmbeddedAtomPotential(**CU_EAM)
    e = engine(pk, N=55, R=8, starts=[cu55_ico()], T=(200.0, 1000.0), pot=pot,
               bc=pk.SphericalBC(14.0), precision="fp32", resync=100)
    e.cycles_nosample(350)           # resyncs at 100, 200, 300; 50 cycles of FP32 drift
    st = e.states(0)
    drift = e.stats()["max_drift"]
    ref = np.array([orc.eam_config_energy(x, pot.n, pot.m, pot.ean, pot.eCam) for x in st["xyz"]])
    assert np.all(np.abs(st["en_tot"] - ref) <= 1e-6 * np.abs(ref))
    assert 0 < drift <= 1e-6 * np.abs(ref).max()
    assert np.all(np.sum(st["xyz"] ** 2, axis=2) <= 14.0 ** 2 * (1 + 1e-6))
    e.resync()
    st = e.states(0)
    np.testing.assert_allclose(st["en_tot"], ref, rtol=1e-12)
    acc = st["counts"][:, 0] / (350 * 55)
    assert np.all(acc > 0.05) and np.all(acc < 0.95)
    e.close()


def test_npt_fp32_energy_tracks_fp64(pk, orc):
    import ptmc_gb300.starts as S
    p = 101325 * 3.398928944382626e-14
    x0 = S.fcc_box(3, 8.4, 0.05, 7)
    e = engine(pk, N=108, R=4, starts=[x0], T=(10.0, 40.0), pot=pk.ELJPotentialEven(C_NE),
               bc=pk.CubicBC(25.2), precision="fp32", resync=50, ens=pk.NPT(108, p))
    e.cycles_nosample(120)
    st = e.states(0)
    assert st["counts"][:, 2].sum() > 0, "volume moves accepted"
    ref = np.array([orc.elj_config_energy(x, orc.POT_ELJEVEN, C_NE, orc.BC_CUBIC, L, L * L / 4)
                    for x, L in zip(st["xyz"], st["box"])])
    np.testing.assert_allclose(st["en_tot"], ref, rtol=1e-6)
    e.close()


def _means(pk, precision, n_runs, cycles, eq, seed):
    import ptmc_gb300.starts as S
    starts = [S.sphere_start(13, 8.0, 4.5, 40 + k) for k in range(n_runs)]
    e = engine(pk, N=13, R=8, starts=starts, T=(4.0, 16.0), pot=pk.ELJPotentialEven(C_NE),
               bc=pk.SphericalBC(11.0), precision=precision, n_runs=n_runs, seed=seed,
               eq=eq, cycles=cycles)
    e.equilibrate()
    e.run_cycles(cycles)
    outs = [e.output(r) for r in range(n_runs)]
    e.close()
    E = np.array([o.en_avg for o in outs])
    C = np.array([o.heat_cap for o in outs])
    return E, C


def test_fp32_matches_fp64_statistically(pk):
    E32, C32 = _means(pk, "fp32", 16, 3000, 2000, 5)
    E64, C64 = _means(pk, "fp64", 16, 3000, 2000, 6)
    n = E32.shape[0]
    for a, b in ((E32, E64), (C32, C64)):
        se = np.sqrt(a.var(0, ddof=1) / n + b.var(0, ddof=1) / n)
        z = np.abs(a.mean(0) - b.mean(0)) / se
        assert np.all(z < 4.0), z


def _abs_pair_sum(x):
    """sum over pairs of |V(r_ij)| for the ELJEven neon coefficients"""
    d = x[:, None, :] - x[None, :, :]
    r2 = np.sum(d * d, axis=2)[np.triu_indices(len(x), 1)]
    inv = 1.0 / r2
    v = sum(c * inv ** (3 + k) for k, c in enumerate(C_NE))
    return float(np.sum(np.abs(v)))


def test_n147_cluster8_energy_tracks_fp64(pk, orc):
    """The largest atom count of the batched workload (147 atoms, 16 replicas)
    under the cluster shape the autotuner picks for it (8 CTAs per run, 2
    walkers each): the running FP32 energy stays within 1e-6 of the oracle's
    FP64 energy of the returned positions, across resyncs, relative to the sum
    of the pair terms' magnitudes (the scale of an FP32 pair sum's error: the
    dilute start clusters' net energy is a small difference of large terms)."""
    import ptmc_gb300.starts as S
    n = 147
    rad = 0.9 * n ** (1 / 3) * 3
    starts = [S.sphere_start(n, rad, 4.3, 700 + r) for r in range(2)]
    e = engine(pk, N=n, R=16, starts=starts, T=(4.0, 16.0), pot=pk.ELJPotentialEven(C_NE),
               bc=pk.SphericalBC(rad + 3.0), precision="fp32", resync=50, n_runs=2, seed=17)
    e.set_launch_shape(n, 8, 32)
    e.cycles_nosample(130)          # resyncs at 50 and 100, then 30 cycles of FP32 drift
    for r in range(2):
        st = e.states(r)
        ref = np.array([orc.elj_config_energy(x, orc.POT_ELJEVEN, C_NE) for x in st["xyz"]])
        scale = np.array([_abs_pair_sum(x) for x in st["xyz"]])
        assert np.all(np.abs(st["en_tot"] - ref) <= 1e-6 * scale), r
        assert st["counts"][:, 0].sum() > 0 and st["counts"][:, 5].sum() > 0
    assert 0 < e.stats()["max_drift"]
    e.close()


def test_large_n_fp32_spreads_over_a_cluster(pk, orc):
    """300 atoms x 32 replicas exceed one CTA's shared memory in the FP32 form:
    the run is spread over a cluster (C = 2 by default); the running energy
    tracks the oracle's FP64 energy of the returned positions."""
    import ptmc_gb300.starts as S
    n = 300
    rad = 0.9 * n ** (1 / 3) * 3
    e = engine(pk, N=n, R=32, starts=[S.sphere_start(n, rad, 4.3, 301)], T=(4.0, 16.0),
               pot=pk.ELJPotentialEven(C_NE), bc=pk.SphericalBC(rad + 3.0), precision="fp32",
               resync=20, seed=31)
    e.cycles_nosample(30)
    st = e.states(0)
    ref = np.array([orc.elj_config_energy(x, orc.POT_ELJEVEN, C_NE) for x in st["xyz"]])
    scale = np.array([_abs_pair_sum(x) for x in st["xyz"]])
    assert np.all(np.abs(st["en_tot"] - ref) <= 1e-6 * scale)
    assert st["counts"][:, 0].sum() > 0
    e.close()
