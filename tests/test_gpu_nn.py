"""GPU tests of the neural-network (RuNNer) potential path.

The FP64 instantiation of the NN kernels consumes the same Philox streams as the
oracle's FP64 restatement (oracle/ptmc_oracle.cpp: G2/G4 symmetry functions,
their incremental update, per-atom MLP), so a short chain must match exactly:
accept counters, positions bitwise, energies to 1e-10 relative.  The FP32
instantiation must reproduce the FP64 energies to 1e-5 relative.
The symmetry-function table is the one of scripts/cu55.jl (88 functions, 31
active for one element) with the G scaling of scripts/data/scaling.data.
"""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def nn_potential(pk, r_cut=12.0, seed=3, out_scale=0.01):
    tables = json.load(open(os.path.join(GOLDEN, "nn_cu55.json")))
    sf = pk.RuNNerPotential.sf_table(tables, r_cut)
    nodes = [88, 20, 20, 1]
    w = pk.RuNNerPotential.random_weights(nodes, seed, out_scale)
    return pk.RuNNerPotential(sf, w, nodes), tables


def cu55(tables):
    return np.array(tables["ico55_nm"]) * (tables["cu_lattice_nm"] * tables["nm_to_bohr"])


def setup(pk, orc, pot, x0, R, precision, radius, T=(300.0, 900.0), seed=7):
    N = len(x0)
    mp = pk.MCParams(mc_cycles=100, eq_cycles=0, mc_sample=1, n_traj=R, n_atoms=N)
    temp = pk.TempGrid(T[0], T[1], R)
    eng = pk.Engine(mp, temp, pot, pk.NVT(N), precision=precision, exch_prob=1.0, seed=seed)
    eng.set_configs(0, pk.Config(x0, pk.SphericalBC(radius)))
    eng.init()
    o = orc.Run(N, R, np.stack([x0] * R), temp.t_grid, bc=orc.BC_SPHERE, bc_param=radius,
                exch_prob=1.0, seed=seed, max_displ=np.full(2 * R, 0.1))
    o.set_nn(pot.sf, pot.weights, pot.nodes, pot.boundary)
    o.init()
    return eng, o


def test_nn_fp64_chain_matches_oracle(pk, orc):
    import ptmc_gb300.starts as S
    pot, tables = nn_potential(pk)
    x0 = S.sphere_start(13, 7.0, 4.0, 11)
    eng, o = setup(pk, orc, pot, x0, 4, "fp64", 10.0)
    g0 = eng.states(0)
    _, e0, _ = o.slot_states()
    np.testing.assert_allclose(g0["en_tot"], e0, rtol=1e-12)
    eng.cycles_nosample(12)
    o.cycles(1, 12)
    g = eng.states(0)
    xo, eo, _ = o.slot_states()
    s = o.slots()
    assert np.array_equal(g["counts"][:, 0:2], s["count_atom"])
    assert np.array_equal(g["counts"][:, 4:6], s["count_exc"])
    assert g["counts"][:, 0].sum() > 0
    assert np.array_equal(g["xyz"], xo)
    np.testing.assert_allclose(g["en_tot"], eo, rtol=1e-10)
    eng.close()


def test_nn_cu55_initial_energy_fp32_vs_fp64(pk, orc):
    pot, tables = nn_potential(pk)
    x0 = cu55(tables)
    e64, o = setup(pk, orc, pot, x0, 2, "fp64", 14.0)
    e32, _ = setup(pk, orc, pot, x0, 2, "fp32", 14.0)
    _, eo, _ = o.slot_states()
    a, b = e64.states(0)["en_tot"], e32.states(0)["en_tot"]
    np.testing.assert_allclose(a, eo, rtol=1e-12)
    np.testing.assert_allclose(b, eo, rtol=1e-5)
    # a few FP32 cycles, then an FP64 recomputation of the same positions
    e32.cycles_nosample(3)
    run_e = e32.states(0)["en_tot"].copy()
    e32.resync()
    st = e32.states(0)
    np.testing.assert_allclose(run_e, st["en_tot"], rtol=1e-5)
    assert st["counts"][:, 0].sum() > 0
    e64.close()
    e32.close()


def _pin_clusters():
    import symm_restatement as SR
    rng = np.random.default_rng(7)
    x = [np.zeros(3)]
    while len(x) < 5:                      # a scalene 5-atom cluster, r >= 3.6 bohr
        p = rng.uniform(-6.0, 6.0, 3)
        if np.linalg.norm(np.array(x) - p, axis=1).min() > 3.6:
            x.append(p)
    return {"tetra": SR.tetrahedron(4.8), "right+far": SR.right_triangle_plus_far(4.8, 20.0),
            "scalene5": np.array(x)}


@pytest.mark.parametrize("precision,rtol,table", [("fp64", 1e-12, "cu55"), ("fp32", 1e-5, "cu55"),
                                                   ("fp32", 1e-5, "generic")])
@pytest.mark.parametrize("name", ["tetra", "right+far", "scalene5"])
def test_nn_energy_pinned_by_restatement(pk, orc, precision, rtol, table, name):
    """The engine's initial energies against the independent numpy restatement of
    SymmFunc.jl (tests/symm_restatement.py: hand-checked closed forms on the
    tetrahedron and the right triangle), not against the oracle; then a short
    chain, and the running energies against the restatement's energies of the
    engine's own final positions.  "cu55": the table of scripts/cu55.jl, whose
    26 angular functions run the table-specialised FP32 kernel; "generic": the
    same table with one angular function switched off (type 100), which runs
    the generic FP32 angular loop."""
    import symm_restatement as SR
    pot, _ = nn_potential(pk)
    if table == "generic":
        sf = pot.sf.copy()
        sf[np.flatnonzero((sf[:, 0] == 1) & (sf[:, 1] == 111))[7], 1] = 100
        pot = pk.RuNNerPotential(sf, pot.weights, pot.nodes, pot.boundary)
    x = _pin_clusters()[name]
    eng, _ = setup(pk, orc, pot, x, 2, precision, 30.0)
    ea = SR.mlp(SR.g_matrix(x, pot.sf), pot.weights, pot.nodes)
    tol = rtol * np.abs(ea).sum()
    np.testing.assert_allclose(eng.states(0)["en_tot"], ea.sum(), rtol=0, atol=tol)
    eng.cycles_nosample(20)
    st = eng.states(0)
    assert st["counts"][:, 0].sum() > 0
    for s in range(2):
        e = SR.energy(st["xyz"][s], pot.sf, pot.weights, pot.nodes)
        assert abs(st["en_tot"][s] - e) <= (1e-10 if precision == "fp64" else 1e-4) * np.abs(ea).sum()
    eng.close()
