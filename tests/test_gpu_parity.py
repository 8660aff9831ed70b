"""GPU parity tests: the CUDA engine through its C ABI against the CPU oracle.

Both consume the same Philox draw streams in the reference's draw order, so the
plain FP64 form must reproduce the oracle's accept/reject sequence exactly:
accept counters, exchange counters, step sizes, walker permutation, positions
and histograms are compared for equality, energies to 1e-10 relative (the
tolerance north of FP64 rounding differences between the GPU's and the host's
exp/log/pow and between warp-tree and sequential sums).
"""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _pkg(pk):
    return pk

C_NE = [-10.5097942564988, 989.725135614556, -101383.865938807, 3918846.12841668,
        -56234083.4334278, 288738837.441765]  # examples/ne13.jl:24-31
REL = 1e-10


def sphere_start(N, radius, min_sep, seed):
    import ptmc_gb300.starts as st
    return st.sphere_start(N, radius, min_sep, seed)


def fcc(ncell, a, jitter, seed):
    import ptmc_gb300.starts as st
    return st.fcc_box(ncell, a, jitter, seed)


def cu55_ico():
    d = json.load(open(os.path.join(GOLDEN, "nn_cu55.json")))
    return np.array(d["ico55_nm"]) * (d["cu_lattice_nm"] * d["nm_to_bohr"])


CU_EAM = dict(n=8.482, m=4.692, eps=0.0367493 * 0.0370, C=27.561, a=0.25 * 18.8973)  # scripts/cu55.jl:39-48


def pair(pk, orc, *, N, R, x0, T0, T1, pot, ens="nvt", bc_param, exch_prob, seed, n_runs=1,
         starts=None, cycles_per_launch=0, pressure=0.0, eq=0, rdfsave=False, precision="fp64"):
    """An engine and matching oracle runs (one per engine run)."""
    mp = pk.MCParams(mc_cycles=1000, eq_cycles=eq, mc_sample=1, n_traj=R, n_atoms=N)
    temp = pk.TempGrid(T0, T1, R)
    ensemble = pk.NPT(N, pressure) if ens == "npt" else pk.NVT(N)
    bc = pk.CubicBC(bc_param) if ens == "npt" or ens == "nvt_cubic" else pk.SphericalBC(bc_param)
    eng = pk.Engine(mp, temp, pot, ensemble, n_runs=n_runs, exch_prob=exch_prob, seed=seed,
                    cycles_per_launch=cycles_per_launch, rdfsave=rdfsave, precision=precision)
    oracles = []
    for r in range(n_runs):
        xr = x0 if starts is None else starts[r]
        eng.set_configs(r, pk.Config(xr, bc))
        o = orc.Run(len(xr), R, np.stack([xr] * R), temp.t_grid,
                    ensemble=orc.NPT if ens == "npt" else orc.NVT, pressure=pressure,
                    bc=orc.BC_CUBIC if isinstance(bc, pk.CubicBC) else orc.BC_SPHERE,
                    bc_param=bc_param, exch_prob=exch_prob, seed=seed, run_index=r)
        if isinstance(pot, pk.EmbeddedAtomPotential):
            o.set_eam(pot.n, pot.m, pot.ean, pot.eCam)
        else:
            o.set_elj(pot.coeff, pot.even)
        if rdfsave:
            o.set_rdf(True)
        o.init()
        oracles.append(o)
    eng.init()
    return eng, oracles


def compare(eng, o, run=0, rel=REL, positions_exact=True):
    g = eng.states(run)
    xo, eo, bo = o.slot_states()
    s = o.slots()
    assert np.array_equal(g["counts"][:, 0:2], s["count_atom"]), "atom accept counters"
    assert np.array_equal(g["counts"][:, 2:4], s["count_vol"]), "volume accept counters"
    assert np.array_equal(g["counts"][:, 4:6], s["count_exc"]), "exchange counters"
    assert np.array_equal(g["max_displ"], s["max_displ"]), "step sizes"
    if positions_exact:
        assert np.array_equal(g["xyz"], xo), "positions (bitwise)"
    else:
        np.testing.assert_allclose(g["xyz"], xo, rtol=0, atol=1e-9)
    np.testing.assert_allclose(g["box"], bo, rtol=1e-14)
    np.testing.assert_allclose(g["en_tot"], eo, rtol=rel, atol=0)
    np.testing.assert_allclose(g["ham"], s["ham"], rtol=rel, atol=1e-300)
    return g


def test_ne13_nvt_fp64_parity(pk, orc):
    """Ne13 in a sphere of 11 bohr, 16 replicas 4-16 K (the Ne13 workload at
    reduced cycle count): equilibration, production, sampling, exchange p = 0.1."""
    x0 = sphere_start(13, 8.0, 4.5, 1234)
    eng, (o,) = pair(pk, orc, N=13, R=16, x0=x0, T0=4.0, T1=16.0, pot=pk.ELJPotentialEven(C_NE),
                     bc_param=11.0, exch_prob=0.1, seed=1234, eq=400)
    eng.equilibrate()
    o.equilibrate(400)
    eng.run_cycles(600)
    o.production(1, 600)
    compare(eng, o)
    out = eng.output(0)
    eh, _, hp = o.hist()
    # histogram bounds come from final equilibration energies (1e-10 relative)
    assert out.en_min == pytest.approx(hp[0], rel=REL) and out.en_max == pytest.approx(hp[1], rel=REL)
    assert np.array_equal(out.en_histogram, eh), "energy histograms"
    eng.close()


def test_ne13_exchange_every_cycle(pk, orc):
    x0 = sphere_start(13, 8.0, 4.5, 77)
    eng, (o,) = pair(pk, orc, N=13, R=8, x0=x0, T0=4.0, T1=16.0, pot=pk.ELJPotentialEven(C_NE),
                     bc_param=11.0, exch_prob=1.0, seed=42)
    eng.cycles_nosample(500)
    o.cycles(1, 500)
    g = compare(eng, o)
    assert g["counts"][:, 5].sum() > 0, "some exchanges accepted"
    eng.close()


def test_elj_all_powers_parity(pk, orc):
    x0 = sphere_start(13, 8.0, 4.5, 5)
    c = C_NE[:3] + [0.0, 1.0e5]
    eng, (o,) = pair(pk, orc, N=13, R=4, x0=x0, T0=4.0, T1=16.0, pot=pk.ELJPotential(c),
                     bc_param=11.0, exch_prob=1.0, seed=3)
    eng.cycles_nosample(200)
    o.cycles(1, 200)
    compare(eng, o)
    eng.close()


def test_cu55_eam_fp64_parity(pk, orc):
    """Cu55 Sutton-Chen EAM (scripts/cu55.jl:39-48), icosahedral start, sphere 14 bohr."""
    pot = pk.EmbeddedAtomPotential(**CU_EAM)
    eng, (o,) = pair(pk, orc, N=55, R=8, x0=cu55_ico(), T0=200.0, T1=1000.0, pot=pot,
                     bc_param=14.0, exch_prob=1.0, seed=11)
    eng.cycles_nosample(60)
    o.cycles(1, 60)
    compare(eng, o)
    eng.close()


def test_npt_fp64_parity(pk, orc):
    """Bulk Ne NPT, fcc start with jitter, cubic box, cut-off L/2 + lrc, volume moves."""
    x0 = fcc(2, 8.4, 0.05, 2)
    p = 101325 * 3.398928944382626e-14  # test/test_states.jl:64
    eng, (o,) = pair(pk, orc, N=32, R=4, x0=x0, T0=10.0, T1=40.0, pot=pk.ELJPotentialEven(C_NE),
                     ens="npt", bc_param=16.8, exch_prob=1.0, seed=8, pressure=p, eq=40)
    eng.equilibrate()
    o.equilibrate(40)
    eng.run_cycles(80)
    o.production(1, 80)
    # the volume scale exp(...)^(1/3) comes from the device's exp/pow and the
    # host's: they may round 1 ulp apart, so positions agree to ~1e-15 here
    g = compare(eng, o, positions_exact=False)
    assert g["counts"][:, 2].sum() > 0, "some volume moves accepted"
    out = eng.output(0)
    _, ev, hp = o.hist()
    assert np.array_equal(out.ev_histogram, ev)
    eng.close()


def test_nvt_cubic_parity(pk, orc):
    x0 = fcc(2, 8.4, 0.05, 4)
    eng, (o,) = pair(pk, orc, N=32, R=4, x0=x0, T0=10.0, T1=40.0, pot=pk.ELJPotentialEven(C_NE),
                     ens="nvt_cubic", bc_param=16.8, exch_prob=1.0, seed=6)
    eng.cycles_nosample(60)
    o.cycles(1, 60)
    # the NVT periodic form recomputes old distances from positions; the
    # reference stores them, so ties in the minimum image may round 1 ulp apart
    compare(eng, o, positions_exact=True)
    eng.close()


def test_batched_uneven_runs(pk, orc):
    """Several independent runs of different N in one context (grouped launches)."""
    sizes = [13, 38, 13, 20]
    starts = [sphere_start(n, 0.9 * n ** (1 / 3) * 3, 4.3, 100 + k) for k, n in enumerate(sizes)]
    radius = max(0.9 * n ** (1 / 3) * 3 for n in sizes) + 3
    eng, os_ = pair(pk, orc, N=13, R=4, x0=None, T0=4.0, T1=16.0, pot=pk.ELJPotentialEven(C_NE),
                    bc_param=radius, exch_prob=1.0, seed=21, n_runs=len(sizes), starts=starts,
                    cycles_per_launch=7)
    eng.cycles_nosample(50)
    en_all = eng.energies()  # ptmc_get_energies: every run in one read
    for r, o in enumerate(os_):
        o.cycles(1, 50)
        compare(eng, o, run=r)
        assert np.array_equal(en_all[r], eng.states(r)["en_tot"])
    st = eng.stats()
    assert st["kernel_launches"] >= 8
    eng.close()


def test_graph_replay_matches_direct(pk, orc):
    """CUDA-graph-replayed chunks give the same chain as the oracle."""
    x0 = sphere_start(13, 8.0, 4.5, 9)
    eng, (o,) = pair(pk, orc, N=13, R=4, x0=x0, T0=4.0, T1=16.0, pot=pk.ELJPotentialEven(C_NE),
                     bc_param=11.0, exch_prob=1.0, seed=17, cycles_per_launch=5)
    eng.cycles_nosample(5 * 8 * 3 + 7)   # 3 graph replays of 8 chunks + a remainder
    o.cycles(1, 5 * 8 * 3 + 7)
    compare(eng, o)
    assert eng.stats()["graph_launches"] == 3
    eng.close()


def test_checkpoint_exact_resume(pk, orc, tmp_path):
    x0 = sphere_start(13, 8.0, 4.5, 31)
    kw = dict(N=13, R=4, x0=x0, T0=4.0, T1=16.0, pot=pk.ELJPotentialEven(C_NE), bc_param=11.0,
              exch_prob=0.5, seed=5, eq=100)
    a, _ = pair(pk, orc, **kw)
    a.equilibrate()
    a.run_cycles(300)
    b, _ = pair(pk, orc, **kw)
    b.equilibrate()
    b.run_cycles(150)
    b.checkpoint(str(tmp_path / "ck"))
    b.close()
    c, _ = pair(pk, orc, **kw)
    c.restore(str(tmp_path / "ck"))
    c.run_cycles(150)
    sa, sc = a.states(0), c.states(0)
    for k in sa:
        assert np.array_equal(sa[k], sc[k]), k
    assert np.array_equal(a.output(0).en_histogram, c.output(0).en_histogram)
    # the reference-format files are readable by the reference-format reader
    r = pk.read_checkpoint(str(tmp_path / "ck"))
    assert r["index"] == 150 and len(r["configs"]) == 4
    assert r["histograms"].shape == (4, 102)
    assert r["histograms"].sum() == 4 * 150
    a.close()
    c.close()


def test_sphere_error_is_reported(pk):
    """An atom that cannot move back inside the sphere: 100 retries -> error
    (src/MCMoves.jl:132), reported through the status word, no fault."""
    x0 = sphere_start(13, 8.0, 4.5, 1) * 3.0   # every atom far outside radius 2
    mp = pk.MCParams(mc_cycles=10, eq_cycles=0, mc_sample=1, n_traj=2, n_atoms=13)
    eng = pk.Engine(mp, pk.TempGrid(4, 16, 2), pk.ELJPotentialEven(C_NE), pk.NVT(13))
    eng.set_configs(0, pk.Config(x0, pk.SphericalBC(2.0)))
    eng.init()
    with pytest.raises(pk.PTMCError) as ei:
        eng.cycles_nosample(2)
    assert ei.value.code == -4
    eng.close()


@pytest.mark.parametrize("name", ["multihist_nvt", "multihist_npt"])
def test_gpu_multihist_golden(pk, name):
    """GPU WHAM against the reference's golden values (test/multihist_test.jl)."""
    d = json.load(open(os.path.join(GOLDEN, name + ".json")))
    temp = pk.TempGrid(d["t_i"], d["t_f"], d["R"])
    if name == "multihist_nvt":
        T, cv, it = pk.multihist_nvt_arrays(np.array(d["en_histogram"]), temp.t_grid,
                                            temp.beta_grid, d["en_min"], d["en_max"], d["thr"])
    else:
        T, cv, it = pk.multihist_npt_arrays(np.array(d["ev_histogram"]), temp.t_grid,
                                            temp.beta_grid, d["en_min"], d["en_max"], d["v_min"],
                                            d["v_max"], d["pressure"], d["thr"])
    for k, v in d["expected"].items():
        assert cv[int(k) - 1] == pytest.approx(v, rel=1e-9), k


def test_gpu_multihist_matches_oracle(pk, orc):
    d = json.load(open(os.path.join(GOLDEN, "checkpoint_ne13.json")))
    h = np.array(d["histograms"])
    p = d["params"]
    temp = pk.TempGrid(p[8], p[9], h.shape[0])
    T, cv, it = pk.multihist_nvt_arrays(h, temp.t_grid, temp.beta_grid, d["hist_info"][0],
                                        d["hist_info"][1], 1e-3)
    To, cvo, ito = orc.multihist_nvt(h, temp.t_grid, temp.beta_grid, d["hist_info"][0],
                                     d["hist_info"][1], 1e-3)
    assert it == ito
    np.testing.assert_allclose(cv, cvo, rtol=1e-9)
    np.testing.assert_allclose(T, To, rtol=1e-15)


def test_rdf_sampler_parity(pk, orc, tmp_path):
    """rdfsave (update_rdf!, src/Sampling.jl:282-345): every 1000th production
    cycle each slot's configuration adds its pair distances.  FP64 sphere: the
    histograms equal the oracle's exactly (the distances are recomputed from
    positions that are bitwise identical).  NPT reads the scaled distance matrix;
    positions agree to ~1 ulp there, so a few pairs may fall in a neighbouring
    bin.  The FP32 form samples the same number of pairs."""
    x0 = sphere_start(13, 8.0, 4.5, 1234)
    args = dict(N=13, R=8, x0=x0, T0=4.0, T1=16.0, pot=pk.ELJPotentialEven(C_NE), bc_param=11.0,
                exch_prob=1.0, seed=21, eq=400, rdfsave=True)
    eng, (o,) = pair(pk, orc, **args)
    eng.equilibrate()
    o.equilibrate(400)
    eng.run_cycles(3000)
    o.production(1, 3000)
    out = eng.output(0)
    ro, dr2 = o.rdf()
    assert out.delta_r2 == dr2 == 4 * 11.0 ** 2 / 100 / 5
    g = np.array(out.rdf)
    assert np.array_equal(g, ro), "radial distribution histograms"
    assert g.sum() == 3 * 8 * 13 * 12 / 2
    ck = str(tmp_path / "ck")  # the reference's rdf.data: one row per replica
    eng.checkpoint(ck)
    np.testing.assert_array_equal(np.loadtxt(os.path.join(ck, "rdf.data")), ro)
    assert float(open(os.path.join(ck, "hist_info.data")).read().split("\n")[1].split()[6]) == dr2
    eng.close()
    e32, _ = pair(pk, orc, **dict(args, precision="fp32"))
    e32.equilibrate()
    e32.run_cycles(3000)
    assert np.array(e32.output(0).rdf).sum() == 3 * 8 * 13 * 12 / 2
    e32.close()
    p = 101325 * 3.398928944382626e-14
    eng, (o,) = pair(pk, orc, N=32, R=4, x0=fcc(2, 8.4, 0.05, 2), T0=10.0, T1=40.0,
                     pot=pk.ELJPotentialEven(C_NE), ens="npt", bc_param=16.8, exch_prob=1.0, seed=8,
                     pressure=p, eq=40, rdfsave=True)
    eng.equilibrate()
    o.equilibrate(40)
    eng.run_cycles(2000)
    o.production(1, 2000)
    g = np.array(eng.output(0).rdf)
    ro, _ = o.rdf()
    assert ro.sum() > 0 and abs(g.sum() - ro.sum()) <= 2
    assert np.abs(g - ro).sum() <= 0.001 * ro.sum() + 4
    eng.close()


def test_gpu_linear_multihistogram(pk, orc, tmp_path):
    """The linear-solve multihistogram (src/multihist.jl) on the GPU against the
    oracle's restatement (same gauge alpha[R-1] = 0) on the reference's golden
    NVT histograms; postprocess() of a checkpoint directory writes the
    reference's four files."""
    d = json.load(open(os.path.join(GOLDEN, "multihist_nvt.json")))
    h = np.array(d["en_histogram"])
    temp = pk.TempGrid(d["t_i"], d["t_f"], d["R"])
    g = pk.multihist_linear_arrays(h, temp.beta_grid, d["en_min"], d["en_max"])
    o = orc.multihist_linear(h, temp.beta_grid, d["en_min"], d["en_max"])
    assert np.array_equal(g["energies"], o["energies"])
    np.testing.assert_allclose(g["alpha"], o["alpha"], rtol=1e-9, atol=1e-9 * np.abs(o["alpha"]).max())
    np.testing.assert_allclose(g["S_E"], o["S_E"], rtol=1e-9, atol=1e-12)
    for k in ("T", "U", "Cv", "dCv", "Z", "S_T"):
        np.testing.assert_allclose(g[k], o[k], rtol=1e-8, err_msg=k)
    # postprocess of a checkpoint written by ptmc_run
    x0 = sphere_start(13, 8.0, 4.5, 1234)
    mp = pk.MCParams.new(2000, 8, 13, eq_percentage=0.5)
    pk.ptmc_run(mp, pk.TempGrid(4.0, 16.0, 8), pk.Config(x0, pk.SphericalBC(11.0)),
                pk.ELJPotentialEven(C_NE), pk.NVT(13), save=2000, exch_prob=1.0,
                workingdirectory=str(tmp_path))
    wd = str(tmp_path)
    ck_hist = open(os.path.join(wd, "checkpoint", "histograms.data")).read()
    E, hd, T, Z, Cv, dCv, U = pk.postprocess(wd, npoints=200)
    for f in ("histograms.data", "Sol.X", "S.data", "analysis.NVT"):
        assert os.path.exists(os.path.join(wd, f))
    assert open(os.path.join(wd, "checkpoint", "histograms.data")).read() == ck_hist
    a = np.loadtxt(os.path.join(wd, "analysis.NVT"), skiprows=1)
    np.testing.assert_allclose(a[:, 2], Cv, rtol=1e-12)
    assert np.all(np.isfinite(Cv)) and Cv.max() > 0 and len(hd) == 8


# ------------------------------------------------------------------
# The benchmarked configurations at their benched sizes (plain FP64 form)

def test_batched_uneven_benched_sizes(pk, orc):
    """The batched uneven-N workload's atom counts N in {13, 38, 55, 101, 147}
    (2 runs each, R = 16, sphere starts of radius 0.9 N^(1/3) 3 bohr in a
    container 3 bohr wider), in one context: one launch group per N on forked
    streams, chunks of 3 cycles replayed from a CUDA graph (8 chunks per
    replay).  N = 101 and 147 need the shared-memory opt-in of the FP64 form."""
    sizes = [13, 38, 55, 101, 147] * 2
    R = 16
    starts = [sphere_start(n, 0.9 * n ** (1 / 3) * 3, 4.3, 500 + k) for k, n in enumerate(sizes)]
    radii = [0.9 * n ** (1 / 3) * 3 + 3.0 for n in sizes]
    mp = pk.MCParams(mc_cycles=1000, eq_cycles=0, mc_sample=1, n_traj=R, n_atoms=13)
    temp = pk.TempGrid(4.0, 16.0, R)
    pot = pk.ELJPotentialEven(C_NE)
    eng = pk.Engine(mp, temp, pot, pk.NVT(13), n_runs=len(sizes), exch_prob=1.0, seed=77,
                    cycles_per_launch=3)
    os_ = []
    for r, (x, rad) in enumerate(zip(starts, radii)):
        eng.set_configs(r, pk.Config(x, pk.SphericalBC(rad)))
        o = orc.Run(len(x), R, np.stack([x] * R), temp.t_grid, bc=orc.BC_SPHERE, bc_param=rad,
                    exch_prob=1.0, seed=77, run_index=r)
        o.set_elj(C_NE, True)
        o.init()
        os_.append(o)
    eng.init()
    n = 3 * 8 * 2 + 5          # two graph replays and a remainder of 5 cycles
    eng.cycles_nosample(n)
    assert eng.stats()["graph_launches"] == 2
    for r, o in enumerate(os_):
        o.cycles(1, n)
        g = compare(eng, o, run=r)
        assert g["counts"][:, 0].sum() > 0
    eng.close()


def test_cu55_eam_fp64_parity_r32(pk, orc):
    """Cu55 EAM with the benched replica count, R = 32 over 200-1000 K, one
    exchange attempted every cycle."""
    pot = pk.EmbeddedAtomPotential(**CU_EAM)
    eng, (o,) = pair(pk, orc, N=55, R=32, x0=cu55_ico(), T0=200.0, T1=1000.0, pot=pot,
                     bc_param=14.0, exch_prob=1.0, seed=12)
    eng.cycles_nosample(40)
    o.cycles(1, 40)
    g = compare(eng, o)
    assert g["counts"][:, 5].sum() > 0, "some exchanges accepted"
    eng.close()


def test_ne108_npt_fp64_parity(pk, orc):
    """Bulk Ne NPT at the benched size: 108 atoms (fcc 3x3x3, a = 8.4 bohr,
    0.05 bohr jitter) in CubicBC(25.2), R = 32 over 10-40 K, 1 atm; volume moves
    (one slot in N + 1), equilibration and production with the E x V histogram."""
    x0 = fcc(3, 8.4, 0.05, 7)
    p = 101325 * 3.398928944382626e-14
    eng, (o,) = pair(pk, orc, N=108, R=32, x0=x0, T0=10.0, T1=40.0, pot=pk.ELJPotentialEven(C_NE),
                     ens="npt", bc_param=25.2, exch_prob=1.0, seed=9, pressure=p, eq=20)
    eng.equilibrate()
    o.equilibrate(20)
    eng.run_cycles(30)
    o.production(1, 30)
    g = compare(eng, o, positions_exact=False)
    assert g["counts"][:, 2].sum() > 0, "some volume moves accepted"
    out = eng.output(0)
    _, ev, hp = o.hist()
    assert np.array_equal(out.ev_histogram, ev)
    eng.close()


# ------------------------------------------------------------------
# More than 32 replicas per run (MCParams.n_traj has no bound in the reference)

def test_ne13_r64_fp64_parity(pk, orc):
    """64 replicas of Ne13: the plain form's warps each make the moves of two
    walkers in turn; same chain as the oracle (positions bitwise)."""
    x0 = sphere_start(13, 8.0, 4.5, 64)
    eng, (o,) = pair(pk, orc, N=13, R=64, x0=x0, T0=4.0, T1=40.0, pot=pk.ELJPotentialEven(C_NE),
                     bc_param=11.0, exch_prob=1.0, seed=64, eq=100)
    eng.equilibrate()
    o.equilibrate(100)
    eng.run_cycles(150)
    o.production(1, 150)
    g = compare(eng, o)
    assert g["counts"][:, 5].sum() > 0
    out = eng.output(0)
    eh, _, _ = o.hist()
    assert np.array_equal(out.en_histogram, eh)
    eng.close()


def test_cu55_eam_r64_and_npt_r48_fp64_parity(pk, orc):
    """Cu55 EAM with 64 replicas (the pair cache, two walkers per warp) and
    Ne32 NPT with 48 replicas (warps serving one or two walkers)."""
    pot = pk.EmbeddedAtomPotential(**CU_EAM)
    eng, (o,) = pair(pk, orc, N=55, R=64, x0=cu55_ico(), T0=200.0, T1=1000.0, pot=pot,
                     bc_param=14.0, exch_prob=1.0, seed=65)
    eng.cycles_nosample(25)
    o.cycles(1, 25)
    compare(eng, o)
    eng.close()
    x0 = fcc(2, 8.4, 0.05, 48)
    p = 101325 * 3.398928944382626e-14
    eng, (o,) = pair(pk, orc, N=32, R=48, x0=x0, T0=10.0, T1=40.0, pot=pk.ELJPotentialEven(C_NE),
                     ens="npt", bc_param=16.8, exch_prob=1.0, seed=66, pressure=p)
    eng.cycles_nosample(40)
    o.cycles(1, 40)
    g = compare(eng, o, positions_exact=False)
    assert g["counts"][:, 2].sum() > 0
    eng.close()


# ------------------------------------------------------------------
# Replica state beyond a CTA's shared memory (the reference has no size limit)

def test_large_n_hbm_state_fp64_parity(pk, orc):
    """32 replicas of 300 (ELJ) and 200 (EAM) atoms and of a 256-atom NPT box
    need more than 227 KB of per-atom state per run: the plain form keeps
    positions, EAM components and trial rows in HBM; same chain as the oracle."""
    n = 300
    rad = 0.9 * n ** (1 / 3) * 3
    x0 = sphere_start(n, rad, 4.3, 300)
    eng, (o,) = pair(pk, orc, N=n, R=32, x0=x0, T0=4.0, T1=16.0, pot=pk.ELJPotentialEven(C_NE),
                     bc_param=rad + 3.0, exch_prob=1.0, seed=300)
    eng.cycles_nosample(6)
    o.cycles(1, 6)
    g = compare(eng, o)
    assert g["counts"][:, 0].sum() > 0
    eng.close()
    n = 200
    x0 = sphere_start(n, 0.9 * n ** (1 / 3) * 3, 3.5, 200)
    pot = pk.EmbeddedAtomPotential(**CU_EAM)
    eng, (o,) = pair(pk, orc, N=n, R=32, x0=x0, T0=200.0, T1=1000.0, pot=pot,
                     bc_param=0.9 * n ** (1 / 3) * 3 + 3.0, exch_prob=1.0, seed=201)
    eng.cycles_nosample(4)
    o.cycles(1, 4)
    compare(eng, o)
    eng.close()
    x0 = fcc(4, 8.4, 0.05, 256)
    p = 101325 * 3.398928944382626e-14
    eng, (o,) = pair(pk, orc, N=256, R=32, x0=x0, T0=10.0, T1=40.0, pot=pk.ELJPotentialEven(C_NE),
                     ens="npt", bc_param=33.6, exch_prob=1.0, seed=256, pressure=p)
    eng.cycles_nosample(5)
    o.cycles(1, 5)
    compare(eng, o, positions_exact=False)
    eng.close()


def test_set_configs_batch_equals_per_run(pk):
    """ptmc_set_runs_configs (one configuration for each of many runs in one call)
    gives the same engine state as one ptmc_set_run_configs call per run; a run
    range beyond n_runs and a wrong array shape are refused."""
    import ptmc_gb300.starts as S
    C = [-10.5097942564988, 989.725135614556, -101383.865938807, 3918846.12841668,
         -56234083.4334278, 288738837.441765]
    B, N, R = 5, 13, 4
    xs = np.stack([S.sphere_start(N, 8.0, 4.5, 40 + r) for r in range(B)])

    def engine(batch):
        mp = pk.MCParams(mc_cycles=100, eq_cycles=20, mc_sample=1, n_traj=R, n_atoms=N)
        e = pk.Engine(mp, pk.TempGrid(4.0, 16.0, R), pk.ELJPotentialEven(C), pk.NVT(N),
                      n_runs=B, precision="fp32", exch_prob=1.0, seed=3)
        if batch:
            with pytest.raises(pk.PTMCError, match="run range"):
                e.set_configs_batch(xs, pk.SphericalBC(11.0), first=1)
            with pytest.raises(ValueError):
                e.set_configs_batch(xs[:, :, :2], pk.SphericalBC(11.0))
            e.set_configs_batch(xs, pk.SphericalBC(11.0))
        else:
            for r in range(B):
                e.set_configs(r, pk.Config(xs[r], pk.SphericalBC(11.0)))
        e.init()
        e.equilibrate()
        e.run_cycles(30)
        return e

    a, b = engine(True), engine(False)
    for r in range(B):
        sa, sb = a.states(r), b.states(r)
        assert np.array_equal(sa["xyz"], sb["xyz"])
        assert np.array_equal(sa["en_tot"], sb["en_tot"])
        assert np.array_equal(a.output(r).en_histogram, b.output(r).en_histogram)
    a.close()
    b.close()


@pytest.mark.parametrize("R", [1, 3])
def test_one_replica_and_two_atoms(pk, orc, R):
    """Edge cases against the oracle (plain FP64 form): one replica, where the
    exchange step has no partner (the reference's rand(1:n_traj - 1) has nothing to
    draw; engine and oracle skip the step and its draws), and the smallest
    configuration, two atoms (one pair); equilibration, then production with
    histograms.  The FP32 form runs the same cases."""
    for N, x0 in ((2, np.array([[0.0, 0.0, 0.0], [5.5, 0.0, 0.0]])), (13, sphere_start(13, 8.0, 4.5, 3))):
        eng, (o,) = pair(pk, orc, N=N, R=R, x0=x0, T0=4.0, T1=16.0, pot=pk.ELJPotentialEven(C_NE),
                         bc_param=11.0, exch_prob=1.0, seed=5, eq=40)
        eng.equilibrate()
        o.equilibrate(40)
        eng.run_cycles(100)
        o.production(1, 100)
        g = compare(eng, o)
        assert g["counts"][:, 0].sum() > 0
        if R == 1:
            assert g["counts"][:, 4].sum() == 0  # no exchange attempted
        eh, _, _ = o.hist()
        assert np.array_equal(eng.output(0).en_histogram, eh)
        eng.close()
        e32, _ = pair(pk, orc, N=N, R=R, x0=x0, T0=4.0, T1=16.0, pot=pk.ELJPotentialEven(C_NE),
                      bc_param=11.0, exch_prob=1.0, seed=5, eq=40, precision="fp32")
        e32.equilibrate()
        e32.run_cycles(100)
        s32 = e32.states(0)
        assert np.all(np.isfinite(s32["en_tot"])) and s32["counts"][:, 0].sum() > 0
        e32.close()
