"""Launch shapes of the FP32 form: a run spread over a thread-block cluster of
C CTAs (walkers split across SMs, exchange/adaptation/sampling on the gathered
walkers via distributed shared memory) must give bit-identical results for
every C, and the autotuner must leave the chain where it found it.  With 8 or
4 lanes per walker (several walkers per warp, ptmc_cycles32n.cu) the draw
streams are the same: a 3-atom cluster, whose two pair terms add alike in any
order, gives the 32-lane chain bit for bit.
"""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

C_NE = [-10.5097942564988, 989.725135614556, -101383.865938807, 3918846.12841668,
        -56234083.4334278, 288738837.441765]


def engine(pk, pot, ens, starts, bc, R, T, seed):
    N = len(starts[0])
    mp = pk.MCParams(mc_cycles=200, eq_cycles=100, mc_sample=1, n_traj=R, n_atoms=N)
    eng = pk.Engine(mp, pk.TempGrid(T[0], T[1], R), pot, ens, n_runs=len(starts),
                    precision="fp32", exch_prob=1.0, seed=seed, resync_every=40)
    for r, x in enumerate(starts):
        eng.set_configs(r, pk.Config(x, bc))
    eng.init()
    return eng


def snapshot(eng):
    out = []
    for r in range(eng.n_runs):
        st = eng.states(r)
        o = eng.output(r)
        out.append((st["xyz"], st["en_tot"], st["box"], st["counts"], st["ham"], st["max_displ"],
                    o.en_histogram, o.ev_histogram))
    return out


def assert_identical(a, b):
    for ra, rb in zip(a, b):
        for x, y in zip(ra, rb):
            assert np.array_equal(x, y)


def protocol(eng):
    eng.equilibrate()
    eng.run_cycles(120)
    return snapshot(eng)


@pytest.mark.parametrize("ctas,lanes", [(2, 32), (4, 32), (8, 32), (1, 16)])
def test_cluster_split_ne13_bit_identical(pk, ctas, lanes):
    """The default shape (one CTA per run, a warp per walker) ends a cycle with
    the pairwise exchange handshake; clusters and half-warp walkers end it with
    CTA (cluster) barriers: the chains must agree bit for bit."""
    import ptmc_gb300.starts as S
    starts = [S.sphere_start(13, 8.0, 4.5, 40 + r) for r in range(3)]
    args = (pk, pk.ELJPotentialEven(C_NE), pk.NVT(13), starts, pk.SphericalBC(11.0), 16, (4.0, 16.0), 5)
    ref = engine(*args)
    a = protocol(ref)
    ref.close()
    eng = engine(*args)
    eng.set_launch_shape(13, ctas, lanes)
    b = protocol(eng)
    eng.close()
    assert_identical(a, b)
    assert a[0][3][:, 0].sum() > 0


def test_cluster_split_eam_and_npt_bit_identical(pk):
    d = json.load(open(os.path.join(GOLDEN, "nn_cu55.json")))
    x0 = np.array(d["ico55_nm"]) * (d["cu_lattice_nm"] * d["nm_to_bohr"])
    eam = pk.EmbeddedAtomPotential(8.482, 4.692, 0.0367493 * 0.0370, 27.561, 0.25 * 18.8973)
    args = (pk, eam, pk.NVT(55), [x0, x0], pk.SphericalBC(14.0), 8, (200.0, 1000.0), 6)
    ref = engine(*args)
    a = protocol(ref)
    ref.close()
    eng = engine(*args)
    eng.set_launch_shape(55, 4)
    b = protocol(eng)
    eng.close()
    assert_identical(a, b)
    import ptmc_gb300.starts as S
    x = S.fcc_box(2, 8.4, 0.05, 3)
    n = len(x)
    nargs = (pk, pk.ELJPotentialEven(C_NE), pk.NPT(n, 101325 * 3.398928944382626e-14), [x, x],
             pk.CubicBC(16.8), 8, (10.0, 40.0), 7)
    ref = engine(*nargs)
    a = protocol(ref)
    ref.close()
    eng = engine(*nargs)
    eng.set_launch_shape(n, 2)
    b = protocol(eng)
    eng.close()
    assert_identical(a, b)
    assert a[0][3][:, 2].sum() > 0  # volume moves accepted


def test_autotune_uneven_batch_restores_chain(pk, tmp_path):
    """Autotuning an uneven batch picks a valid shape per atom count, caches it,
    and leaves the whole device state (positions, energies, draw counters,
    counters, histograms) as it found it: with the default shape set back, the
    chain continues bit for bit like an untuned one."""
    import ptmc_gb300.starts as S
    sizes = [13, 38, 55, 101, 147] * 2
    starts = [S.sphere_start(n, 0.9 * n ** (1 / 3) * 3, 4.3, 500 + k) for k, n in enumerate(sizes)]

    def make(seed):
        mp = pk.MCParams(mc_cycles=100, eq_cycles=0, mc_sample=1, n_traj=16, n_atoms=13)
        eng = pk.Engine(mp, pk.TempGrid(4.0, 16.0, 16), pk.ELJPotentialEven(C_NE), pk.NVT(13),
                        n_runs=len(sizes), precision="fp32", exch_prob=1.0, seed=seed)
        for r, (n, x) in enumerate(zip(sizes, starts)):
            eng.set_configs(r, pk.Config(x, pk.SphericalBC(0.9 * n ** (1 / 3) * 3 + 3.0)))
        eng.init()
        return eng

    cache = str(tmp_path / "tune.json")
    eng = make(9)
    shapes = eng.autotune(trial_cycles=5, cache=cache)
    assert set(shapes) == set(sizes)
    assert all(c in (1, 2, 4, 8) and l in (4, 8, 16, 32) for c, l in shapes.values())
    assert all(c == 1 for c, l in shapes.values() if l <= 8)
    for n in set(sizes):  # back to one full warp per walker: the chain must continue bit for bit
        eng.set_launch_shape(n, 1, 32)
    eng.cycles_nosample(30)
    a = snapshot(eng)
    eng.close()
    ref = make(9)
    ref.cycles_nosample(30)
    b = snapshot(ref)
    ref.close()
    assert_identical(a, b)
    # a cache hit gives the same shapes without trials
    eng = make(9)
    assert eng.autotune(trial_cycles=5, cache=cache) == shapes
    eng.close()
    assert len(open(cache).read().strip().split("\n")) == 1


def test_half_warp_walkers(pk, orc):
    """16 lanes per walker (two walkers per warp): the running FP32 energy tracks
    the oracle's FP64 energy of the positions; the result does not depend on the
    cluster size at L = 16 (bit for bit); per-temperature mean energies agree
    with the 32-lane layout within 5 combined standard errors."""
    import ptmc_gb300.starts as S
    pot = pk.ELJPotentialEven(C_NE)
    starts = [S.sphere_start(13, 8.0, 4.5, 40 + r) for r in range(3)]
    args = (pk, pot, pk.NVT(13), starts, pk.SphericalBC(11.0), 16, (4.0, 16.0), 5)
    ref = engine(*args)
    ref.set_launch_shape(13, 1, 16)
    a = protocol(ref)
    for r in range(3):
        st = ref.states(r)
        e64 = np.array([orc.elj_config_energy(x, orc.POT_ELJEVEN, C_NE) for x in st["xyz"]])
        assert np.all(np.abs(st["en_tot"] - e64) <= 1e-6 * np.abs(e64))
    ref.close()
    eng = engine(*args)
    eng.set_launch_shape(13, 2, 16)
    b = protocol(eng)
    eng.close()
    assert_identical(a, b)
    # statistics against the 32-lane layout: 16 independent runs each
    st16 = [S.sphere_start(13, 8.0, 4.5, 60 + r) for r in range(16)]

    def means(lanes, seed):
        e = engine(pk, pot, pk.NVT(13), st16, pk.SphericalBC(11.0), 16, (4.0, 16.0), seed)
        e.set_launch_shape(13, 1, lanes)
        e.cycles_nosample(2000)
        m = []
        for _ in range(20):
            e.cycles_nosample(100)
            m.append([e.states(r)["en_tot"] for r in range(16)])
        e.close()
        return np.array(m).mean(axis=0)  # [runs, R]
    m16, m32 = means(16, 71), means(32, 72)
    se = np.sqrt(m16.var(axis=0, ddof=1) / 16 + m32.var(axis=0, ddof=1) / 16)
    z = np.abs(m16.mean(axis=0) - m32.mean(axis=0)) / se
    assert np.all(z < 5), z


def _three_atom(pk, pot, bc, lanes, seed):
    x = np.array([[0.0, 0.0, 0.0], [5.6, 0.3, -0.2], [2.1, 4.9, 0.4]]) - 2.5
    if pot == "eam":
        p = pk.EmbeddedAtomPotential(8.482, 4.692, 0.0367493 * 0.0370, 27.561, 0.25 * 18.8973)
        x = x * 0.88
    else:
        p = pk.ELJPotentialEven(C_NE)
    mp = pk.MCParams(mc_cycles=400, eq_cycles=200, mc_sample=1, n_traj=16, n_atoms=3)
    eng = pk.Engine(mp, pk.TempGrid(4.0, 60.0, 16), p, pk.NVT(3), n_runs=3, precision="fp32",
                    exch_prob=1.0, seed=seed, resync_every=0)
    for r in range(3):
        eng.set_configs(r, pk.Config(x + 0.1 * r, bc))
    eng.init()
    if lanes != 32:
        eng.set_launch_shape(3, 1, lanes)
    return eng


@pytest.mark.parametrize("lanes", [8, 4])
@pytest.mark.parametrize("pot,cube", [("elj", False), ("eam", False), ("elj", True)])
def test_narrow_walkers_same_streams(pk, lanes, pot, cube):
    """8 and 4 lanes per walker consume the 32-lane form's draw streams and
    make its exchange, adaptation and sampling: with two pair terms per move
    (3 atoms) every sum is order-free, so the chains agree bit for bit
    (positions, energies, counters, step sizes, E/E^2 sums, histograms)."""
    bc = pk.CubicBC(9.0) if cube else pk.SphericalBC(6.0)
    a_eng = _three_atom(pk, pot, bc, 32, 13)
    a = protocol(a_eng)
    a_eng.close()
    b_eng = _three_atom(pk, pot, bc, lanes, 13)
    b = protocol(b_eng)
    b_eng.close()
    assert_identical(a, b)
    assert a[0][3][:, 0].sum() > 0 and a[0][3][:, 5].sum() > 0


@pytest.mark.parametrize("lanes", [8, 4])
def test_narrow_walkers_cu55_tracks_fp64(pk, orc, lanes):
    """Cu55 EAM with 8 / 4 lanes per walker: after 350 cycles (last resync at
    300) every running energy is within 1e-6 relative of the oracle's FP64
    energy of the returned positions, the drift record is set, and an explicit
    resync lands on the FP64 value."""
    d = json.load(open(os.path.join(GOLDEN, "nn_cu55.json")))
    x0 = np.array(d["ico55_nm"]) * (d["cu_lattice_nm"] * d["nm_to_bohr"])
    pot = pk.EmbeddedAtomPotential(8.482, 4.692, 0.0367493 * 0.0370, 27.561, 0.25 * 18.8973)
    mp = pk.MCParams(mc_cycles=400, eq_cycles=0, mc_sample=1, n_traj=32, n_atoms=55)
    e = pk.Engine(mp, pk.TempGrid(200.0, 1000.0, 32), pot, pk.NVT(55), n_runs=2, precision="fp32",
                  exch_prob=1.0, seed=3, resync_every=100)
    for r in range(2):
        e.set_configs(r, pk.Config(x0, pk.SphericalBC(14.0)))
    e.init()
    e.set_launch_shape(55, 1, lanes)
    e.cycles_nosample(350)
    for r in range(2):
        st = e.states(r)
        ref = np.array([orc.eam_config_energy(x, pot.n, pot.m, pot.ean, pot.eCam) for x in st["xyz"]])
        assert np.all(np.abs(st["en_tot"] - ref) <= 1e-6 * np.abs(ref)), r
        acc = st["counts"][:, 0] / (350 * 55)
        assert np.all(acc > 0.05) and np.all(acc < 0.95)
        assert np.all(np.sum(st["xyz"] ** 2, axis=2) <= 14.0 ** 2 * (1 + 1e-6))
    assert 0 < e.stats()["max_drift"] <= 1e-6 * 10.0
    e.resync()
    st = e.states(0)
    ref = np.array([orc.eam_config_energy(x, pot.n, pot.m, pot.ean, pot.eCam) for x in st["xyz"]])
    np.testing.assert_allclose(st["en_tot"], ref, rtol=1e-12)
    e.close()


def test_narrow_walkers_statistics_ne13(pk, orc):
    """Ne13 with 4 lanes per walker: the FP32 running energy tracks the oracle's
    FP64 energy; per-temperature mean energies agree with the 32-lane layout
    within 5 combined standard errors over 16 independent runs."""
    import ptmc_gb300.starts as S
    pot = pk.ELJPotentialEven(C_NE)
    st16 = [S.sphere_start(13, 8.0, 4.5, 60 + r) for r in range(16)]

    def means(lanes, seed):
        e = engine(pk, pot, pk.NVT(13), st16, pk.SphericalBC(11.0), 16, (4.0, 16.0), seed)
        e.set_launch_shape(13, 1, lanes)
        e.cycles_nosample(2000)
        m = []
        for _ in range(20):
            e.cycles_nosample(100)
            m.append([e.states(r)["en_tot"] for r in range(16)])
        st = e.states(0)
        e64 = np.array([orc.elj_config_energy(x, orc.POT_ELJEVEN, C_NE) for x in st["xyz"]])
        assert np.all(np.abs(st["en_tot"] - e64) <= 1e-6 * np.abs(e64))
        e.close()
        return np.array(m).mean(axis=0)  # [runs, R]
    m4, m32 = means(4, 81), means(32, 82)
    se = np.sqrt(m4.var(axis=0, ddof=1) / 16 + m32.var(axis=0, ddof=1) / 16)
    z = np.abs(m4.mean(axis=0) - m32.mean(axis=0)) / se
    assert np.all(z < 5), z


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_occupancy_query_keeps_launch_limits(pk, precision):
    """ptmc_occupancy sizes whole-wave batches; a query for a small atom count
    must leave every later launch of the same kernel with more atoms (more
    shared memory) launchable, before and after the 48 KB opt-in."""
    import ptmc_gb300.starts as S
    mp = pk.MCParams(mc_cycles=10, eq_cycles=0, mc_sample=1, n_traj=16, n_atoms=13)
    probe = pk.Engine(mp, pk.TempGrid(4.0, 16.0, 16), pk.ELJPotentialEven(C_NE), pk.NVT(13),
                      precision=precision)
    probe.set_configs(0, pk.Config(S.sphere_start(13, 8.0, 4.5, 1), pk.SphericalBC(11.0)))
    shapes = [(1, 32)] if precision == "fp64" else [(1, 32), (1, 16), (1, 8), (1, 4)]
    for c, l in shapes:
        assert probe.occupancy(13, c, l) >= 1
    probe.close()
    for n in (38, 101, 147):
        x = S.sphere_start(n, 0.9 * n ** (1 / 3) * 3, 4.3, n)
        mp = pk.MCParams(mc_cycles=10, eq_cycles=0, mc_sample=1, n_traj=16, n_atoms=n)
        e = pk.Engine(mp, pk.TempGrid(4.0, 16.0, 16), pk.ELJPotentialEven(C_NE), pk.NVT(n),
                      precision=precision, exch_prob=1.0)
        e.set_configs(0, pk.Config(x, pk.SphericalBC(0.9 * n ** (1 / 3) * 3 + 3.0)))
        e.init()
        assert e.occupancy(n) >= 1
        e.cycles_nosample(3)
        assert e.states(0)["counts"][:, 0].sum() > 0
        e.close()


def test_r64_fp32_cluster_shapes(pk, orc):
    """64 replicas in the FP32 form: by default a cluster of 2 CTAs of 32
    walkers; the chains are bit-identical for clusters of 2, 4 and 8 CTAs and
    track the oracle's FP64 energy of the returned positions."""
    import ptmc_gb300.starts as S
    starts = [S.sphere_start(13, 8.0, 4.5, 90 + r) for r in range(2)]
    args = (pk, pk.ELJPotentialEven(C_NE), pk.NVT(13), starts, pk.SphericalBC(11.0), 64,
            (4.0, 40.0), 9)
    ref = engine(*args)
    a = protocol(ref)
    for r in range(2):
        st = ref.states(r)
        e64 = np.array([orc.elj_config_energy(x, orc.POT_ELJEVEN, C_NE) for x in st["xyz"]])
        assert np.all(np.abs(st["en_tot"] - e64) <= 1e-6 * np.abs(e64))
        assert st["counts"][:, 5].sum() > 0
    ref.close()
    for c in (4, 8):
        eng = engine(*args)
        eng.set_launch_shape(13, c, 32)
        b = protocol(eng)
        eng.close()
        assert_identical(a, b)
    with pytest.raises(pk.PTMCError):  # 64 walkers do not fit one CTA
        eng = engine(*args)
        try:
            eng.set_launch_shape(13, 1, 32)
        finally:
            eng.close()
