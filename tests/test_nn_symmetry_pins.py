"""Pins of the NN symmetry functions that do not go through the closed
forward-pass library: closed forms derived by hand for symmetric 3- and 4-atom
clusters, an independent numpy restatement of the reference's G2/G4 formulas
(tests/symm_restatement.py), and the oracle's from-scratch (nn_full, nn2_G) and
incremental (energy_update! of DeltaMatrix.jl) symmetry matrices checked
against both, for the one-species RuNNerPotential (table of scripts/cu55.jl)
and the two-species RuNNerPotential2Atom (tests/nn2_synth.py)."""
import json
import os

import numpy as np
import pytest

import nn2_synth
import symm_restatement as SR
from conftest import GOLDEN

A = 4.8     # Cu nearest-neighbour distance in bohr, about
RC = 11.338


def _sf(pk, rc=None):
    tables = json.load(open(os.path.join(GOLDEN, "nn_cu55.json")))
    return pk.RuNNerPotential.sf_table(tables, rc)


def _active(sf):
    rad = [s for s, f in enumerate(sf) if f[0] == 0 and f[1] == 11]
    ang = [s for s, f in enumerate(sf) if f[0] == 1 and f[1] == 111]
    return rad, ang


def _norm(f):
    n = 1.0 / (f[7] - f[6])
    return n, -f[6] * n, 2.0 ** (1 - f[4]) * n


def test_restatement_closed_forms(pk):
    """G2 and G4 written out by hand from SymmFunc.jl:184-312 for three clusters:
    a regular tetrahedron (all r = a, all cos t = 1/2), an equilateral triangle
    with a fourth atom beyond the cut-off, and a right isosceles triangle
    (r = a, a, a sqrt 2; cos t = 0 at the right angle, 1/sqrt 2 at the others)."""
    sf = _sf(pk)
    rad, ang = _active(sf)
    assert len(rad) == 5 and len(ang) == 26
    fa, fb = SR.fc1(A, RC), SR.fc1(A * np.sqrt(2), RC)

    G = SR.g_matrix(SR.tetrahedron(A), sf)
    for s in rad:
        n, o, _ = _norm(sf[s])
        eta = sf[s][2]
        np.testing.assert_allclose(G[s], 3 * fa * np.exp(-eta * A * A) * n + o, rtol=1e-13)
    for s in ang:
        n, o, tpz = _norm(sf[s])
        eta, lam, zeta = sf[s][2:5]
        want = 3 * np.exp(-3 * eta * A * A) * fa ** 3 * (1 + lam / 2) ** zeta * tpz + o
        np.testing.assert_allclose(G[s], want, rtol=1e-13, atol=1e-15)
    inactive = [s for s in range(len(sf)) if s not in rad and s not in ang]
    assert np.all(G[inactive] == 0.0)          # zeros(N), no offset

    x = SR.tetrahedron(A)
    x[3] = [0.0, 0.0, 40.0]                    # beyond the cut-off from the triangle
    G = SR.g_matrix(x, sf)
    for s in rad:
        n, o, _ = _norm(sf[s])
        np.testing.assert_allclose(G[s, :3], 2 * fa * np.exp(-sf[s][2] * A * A) * n + o, rtol=1e-13)
        assert G[s, 3] == pytest.approx(o, abs=1e-15)
    for s in ang:
        n, o, tpz = _norm(sf[s])
        eta, lam, zeta = sf[s][2:5]
        want = np.exp(-3 * eta * A * A) * fa ** 3 * (1 + lam / 2) ** zeta * tpz + o
        np.testing.assert_allclose(G[s, :3], want, rtol=1e-13, atol=1e-15)
        assert G[s, 3] == pytest.approx(o, abs=1e-15)

    G = SR.g_matrix(SR.right_triangle_plus_far(A, 30.0), sf)
    for s in rad:
        n, o, _ = _norm(sf[s])
        eta = sf[s][2]
        va, vb = fa * np.exp(-eta * A * A), fb * np.exp(-2 * eta * A * A)
        np.testing.assert_allclose(G[s, :3], np.array([2 * va, va + vb, va + vb]) * n + o, rtol=1e-13)
    for s in ang:
        n, o, tpz = _norm(sf[s])
        eta, lam, zeta = sf[s][2:5]
        e = np.exp(-eta * 4 * A * A) * fa * fa * fb
        want = np.array([1.0, (1 + lam / np.sqrt(2)) ** zeta, (1 + lam / np.sqrt(2)) ** zeta]) * e * tpz + o
        np.testing.assert_allclose(G[s, :3], want, rtol=1e-12, atol=1e-15)


def test_restatement2_closed_forms():
    """Two species on a regular tetrahedron, atoms 0, 1 of species 1 and 2, 3 of
    species 2 (SymmFunc.jl:318-478): for a species-1 atom one species-1 and two
    species-2 neighbours, neighbour pairs with 0 / 1 / 2 species-2 atoms 0 / 2 / 1
    times; for a species-2 atom two species-1 and one species-2 neighbours, and
    1 / 2 / 0 such pairs."""
    rad, ang, *_ = nn2_synth.potential()
    G = SR.g_matrix2(SR.tetrahedron(A), rad, ang, 2)
    fa = SR.fc1(A, nn2_synth.RCUT)
    nr = len(rad)
    for k, q in enumerate(rad):
        v = fa * np.exp(-q[0] * A * A)
        off, norm = q[2:6], q[6:10]
        for a, c in ((0, 0), (1, 0), (2, 1), (3, 1)):
            cnt = (1, 2) if c == 0 else (2, 1)
            for row in (0, 1):
                np.testing.assert_allclose(G[2 * k + row, a], cnt[row] * v * norm[2 * c + row] + off[2 * c + row], rtol=1e-13)
    for k, q in enumerate(ang):
        eta, lam, zeta, tpz, off = q[0], q[1], q[2], q[4:10], q[10:16]
        t = np.exp(-3 * eta * A * A) * fa ** 3 * (1 + lam / 2) ** zeta
        for a, c in ((0, 0), (1, 0), (2, 1), (3, 1)):
            cnt = (0, 2, 1) if c == 0 else (1, 2, 0)
            for m in range(3):
                np.testing.assert_allclose(G[2 * nr + 3 * k + m, a], cnt[m] * t * tpz[3 * c + m] + off[3 * c + m],
                                           rtol=1e-13, atol=1e-15)


def _scalene(n, seed, lo=3.6, hi=9.5):
    rng = np.random.default_rng(seed)
    x = [np.zeros(3)]
    while len(x) < n:
        p = rng.uniform(-hi / 1.5, hi / 1.5, 3)
        r = np.linalg.norm(np.array(x) - p, axis=1)
        if r.min() > lo:
            x.append(p)
    return np.array(x)


def _oracle_nn(orc, pk, x, sf, weights, nodes, R=2, seed=5, radius=25.0):
    T, _ = orc.tempgrid(300.0, 900.0, R)
    o = orc.Run(len(x), R, np.stack([x] * R), T, bc=orc.BC_SPHERE, bc_param=radius,
                exch_prob=1.0, seed=seed, max_displ=np.full(2 * R, 0.4))
    o.set_nn(sf, weights, nodes, 0.0)
    o.init()
    return o


@pytest.mark.parametrize("name", ["tetra", "triangle+far", "right", "scalene4", "scalene4_rc9"])
def test_oracle_nn_full_against_restatement(orc, pk, name):
    """The oracle's from-scratch symmetry matrix (nn_full) and energy against the
    restatement, the three closed-form clusters and two scalene 4-atom ones (one
    with r_c = 9 bohr so that some pairs and triangles fall outside)."""
    rc = 9.0 if name.endswith("rc9") else None
    sf = _sf(pk, rc)
    x = {"tetra": SR.tetrahedron(A),
         "triangle+far": np.vstack([SR.tetrahedron(A)[:3], [[0, 0, 40.0]]]),
         "right": SR.right_triangle_plus_far(A, 30.0)}.get(name, None)
    if x is None:
        x = _scalene(4, 11 if rc else 7, hi=12.0 if rc else 9.5)
    nodes = [len(sf), 20, 20, 1]
    w = pk.RuNNerPotential.random_weights(nodes, 3, 0.01)
    o = _oracle_nn(orc, pk, x, sf, w, nodes)
    want = SR.g_matrix(x, sf)
    if rc:
        r = np.linalg.norm(x[:, None] - x[None], axis=2)
        assert np.any(r[np.triu_indices(4, 1)] > rc)
    for wk in range(2):
        G, ea = o.nn_state(wk, len(sf))
        np.testing.assert_allclose(G, want, rtol=1e-12, atol=1e-14)
        np.testing.assert_allclose(ea, SR.mlp(want, w, nodes), rtol=1e-12, atol=1e-14)
    np.testing.assert_allclose(o.walkers()[1], SR.energy(x, sf, w, nodes), rtol=1e-12)


def test_oracle_nn_delta_update_against_restatement(orc, pk):
    """After a chain of accepted and rejected atom moves (and exchanges) the
    oracle's incrementally updated symmetry matrices (total_thr_symm!,
    DeltaMatrix.jl:794-975) equal the restatement's from-scratch ones of the
    final positions, and the running energies the restatement's."""
    import ptmc_gb300.starts as st
    sf = _sf(pk)
    nodes = [len(sf), 20, 20, 1]
    w = pk.RuNNerPotential.random_weights(nodes, 3, 0.01)
    x0 = st.sphere_start(6, 5.0, 4.0, 3)
    R = 3
    T, _ = orc.tempgrid(300.0, 900.0, R)
    o = orc.Run(6, R, np.stack([x0] * R), T, bc=orc.BC_SPHERE, bc_param=8.0,
                exch_prob=1.0, seed=9, max_displ=np.full(2 * R, 0.5))
    o.set_nn(sf, w, nodes, 0.0)
    o.init()
    o.cycles(1, 80)
    assert o.slots()["count_atom"].sum() > 50
    x, e, _ = o.walkers()
    for wk in range(R):
        G, ea = o.nn_state(wk, len(sf))
        want = SR.g_matrix(x[wk], sf)
        assert np.abs(G - want).max() < 1e-11
        np.testing.assert_allclose(e[wk], SR.energy(x[wk], sf, w, nodes), rtol=1e-10)


def _oracle_nn2(orc, x, n1, R=2, seed=4, radius=25.0, n_swaps=1, md=0.4):
    rad, ang, w1, w2, nodes = nn2_synth.potential()
    T, _ = orc.tempgrid(300.0, 900.0, R)
    o = orc.Run(len(x), R, np.stack([x] * R), T, ensemble=orc.NNVT, bc=orc.BC_SPHERE,
                bc_param=radius, exch_prob=1.0, seed=seed, max_displ=np.full(2 * R, md))
    o.set_nn2(rad, ang, w1, w2, nodes, n1, n_swaps=n_swaps)
    o.init()
    return o, (rad, ang, w1, w2, nodes)


@pytest.mark.parametrize("name,n1", [("tetra", 2), ("tetra", 1), ("scalene5", 3)])
def test_oracle_nn2_full_against_restatement(orc, name, n1):
    x = SR.tetrahedron(A) if name == "tetra" else _scalene(5, 21)
    o, (rad, ang, w1, w2, nodes) = _oracle_nn2(orc, x, n1)
    want = SR.g_matrix2(x, rad, ang, n1)
    for wk in range(2):
        G, _ = o.nn_state(wk, len(want))
        np.testing.assert_allclose(G, want, rtol=1e-12, atol=1e-14)
    np.testing.assert_allclose(o.walkers()[1], SR.energy2(x, rad, ang, w1, w2, nodes, n1), rtol=1e-12)


def test_oracle_nn2_delta_update_against_restatement(orc):
    """Atom moves and species swaps (NNVT) update the oracle's two-species
    symmetry matrices incrementally; they equal the restatement's of the final
    positions (atoms keep their species, swaps exchange positions)."""
    import ptmc_gb300.starts as st
    x0 = st.sphere_start(8, 5.5, 4.2, 6)
    o, (rad, ang, w1, w2, nodes) = _oracle_nn2(orc, x0, 5, R=3, seed=8, radius=8.0,
                                               n_swaps=2, md=0.5)
    o.cycles(1, 60)
    assert o.swaps() > 0 and o.slots()["count_atom"].sum() > 50
    x, e, _ = o.walkers()
    for wk in range(3):
        G, _ = o.nn_state(wk, 2 * len(rad) + 3 * len(ang))
        assert np.abs(G - SR.g_matrix2(x[wk], rad, ang, 5)).max() < 1e-11
        np.testing.assert_allclose(e[wk], SR.energy2(x[wk], rad, ang, w1, w2, nodes, 5), rtol=1e-10)
