"""CPU tests: the oracle against the reference's own known answers.

Each test cites the reference test it restates (paths inside the reference
package).  These pin the oracle before it is trusted as the GPU checker.
"""
import json
import math
import os

import numpy as np
import pytest

from conftest import GOLDEN

C_NE = [-10.5097942564988, 989.725135614556, -101383.865938807, 3918846.12841668,
        -56234083.4334278, 288738837.441765]  # examples/ne13.jl:24-31


def test_philox_known_answers(orc):
    # Random123 published KAT vectors for philox4x32_10
    assert list(orc.philox4x32([0, 0, 0, 0], [0, 0])) == [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]
    assert list(orc.philox4x32([0xffffffff] * 4, [0xffffffff] * 2)) == [
        0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd]
    assert list(orc.philox4x32([0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344],
                               [0xa4093822, 0x299f31d0])) == [0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1]


def test_u01_stream_layout(orc):
    # draw k = half (k & 1) of Philox block k >> 1, 53 bits, in [0, 1)
    blk = orc.philox4x32([3, 0, 5, 2], [0x1234, 0])
    u0 = ((int(blk[0]) << 21) | (int(blk[1]) >> 11)) * 2.0 ** -53
    u1 = ((int(blk[2]) << 21) | (int(blk[3]) >> 11)) * 2.0 ** -53
    assert orc.u01(0x1234, 5, 2, 6) == u0
    assert orc.u01(0x1234, 5, 2, 7) == u1
    us = [orc.u01(1, 0, 0, k) for k in range(2000)]
    assert 0.0 <= min(us) and max(us) < 1.0
    assert abs(np.mean(us) - 0.5) < 0.03


def test_elj_closed_forms(orc):
    # test/test_potentials.jl:3-16
    assert orc.dimer_energy(orc.POT_ELJ, [-2.0, 0.0, 1.0], 1.0) == -1.0
    assert orc.dimer_energy(orc.POT_ELJEVEN, [-2.0, 1.0], 1.0) == -1.0
    assert orc.dimer_energy(orc.POT_ELJEVEN, [-2.0, 1.0], 2.0) == orc.dimer_energy(orc.POT_ELJ, [-2.0, 0.0, 1.0], 2.0)
    c = [-1.0, 2.0, 3.0, -4.0, 5.0]
    assert orc.dimer_energy(orc.POT_ELJ, c, 1.0) == sum(c)


def test_elj_config_consistency(orc):
    # test/test_potentials.jl:17-39: three atoms, pair sum, cut-off sum
    x = np.array([[1.0, 2.0, 3.0], [2.0, 4.0, 6.0], [0.0, 1.0, 0.0]])
    c = [-1.0, 2.0, 3.0, -4.0, 5.0]
    e = orc.elj_config_energy(x, orc.POT_ELJ, c)
    d = [orc.distance2(x[i], x[j]) for i, j in ((0, 1), (0, 2), (1, 2))]
    ref = 0.0
    for r2 in d:
        ref += orc.dimer_energy(orc.POT_ELJ, c, r2)
    assert e == ref
    assert e < 0 or e > 0
    # r_cut^2 = 4 excludes all three pairs (d2 = 14, 11, 49) and lrc(r_cut<=50) = 0
    # (a box of 100 leaves the distances unchanged; only the cut-off acts)
    assert orc.elj_config_energy(x, orc.POT_ELJEVEN, [-2.0, 1.0], orc.BC_CUBIC, 100.0, 4.0) == 0.0


def test_eam_known_answer(orc):
    # test/test_potentials.jl:41-56: n = m = eps = C = a = 1 -> ean = 0.5, eCam = 1
    x = np.array([[1.0, 2.0, 3.0], [2.0, 4.0, 6.0], [0.0, 1.0, 0.0]])
    e = orc.eam_config_energy(x, 1.0, 1.0, 0.5, 1.0)
    assert e == pytest.approx(-1.3495549581716526, rel=1e-15)


def test_distances_and_min_image(orc):
    # test/runtests.jl:87-125, test/configurations.jl
    v1, v2, v3 = [1.0, 2.0, 3.0], [2.0, 4.0, 6.0], [0.0, 1.0, 0.0]
    assert orc.distance2(v1, v2) == 14.0
    assert orc.distance2(v1, v3) == 11.0
    assert orc.distance2(v1, v2, orc.BC_CUBIC, 10.0) == 14.0
    w3 = [3.0, 6.0, 9.0]
    assert orc.distance2(v1, w3) == 56.0
    assert orc.distance2(v1, w3, orc.BC_CUBIC, 10.0) == 36.0


def test_tempgrid(orc, pk):
    # test/runtests.jl:216-235
    T, B = orc.tempgrid(2.0, 16.0, 31)
    assert len(T) == 31 and T.min() == 2.0 and T.max() == 16.0
    T, B = orc.tempgrid(2.0, 16.0, 32)
    assert 1.0 / (T[0] * B[0]) == pytest.approx(3.16681196e-6)
    T1, _ = orc.tempgrid(2.0, 16.0, 32, 1)
    assert (T1[1] - T1[0]) == pytest.approx(T1[-1] - T1[-2])
    g = pk.TempGrid(2, 16, 31)
    assert np.array_equal(g.t_grid, orc.tempgrid(2.0, 16.0, 31)[0])
    with pytest.raises(ValueError):
        pk.TempGrid(2, 16, 256, tdistr="test")


def test_lrc_matches_formula(orc):
    # lrc (src/EnergyEvaluation.jl:968-982), written out independently
    rc2, N = (25.2 * 25.2) / 4, 108
    rcs = math.sqrt(rc2)
    rc3 = rc2 * rcs
    e = 0.0
    for i, c in enumerate(C_NE, start=1):
        e += c / rc3 / (2 * i + 1)
        rc3 *= rc2
    e *= math.pi * N * N / 4 / (rcs ** 3)
    assert orc.lrc(N, rc2, C_NE) == pytest.approx(e, rel=1e-14)
    assert orc.lrc(N, 50.0, C_NE) == 0.0


def test_mlp_all_ones(orc):
    # test/test_runner_forward.jl:44-75: 88-20-20-1, all parameters and inputs 1 -> 21
    nodes = [88, 20, 20, 1]
    npar = sum(nodes[i - 1] * nodes[i] + nodes[i] for i in range(1, 4))
    assert npar == 2221
    out = orc.mlp_forward(np.ones((2, 88)), np.ones(npar), nodes)
    assert list(out) == [21.0, 21.0]


@pytest.mark.parametrize("name", ["multihist_nvt", "multihist_npt"])
def test_multihist_golden(orc, name):
    # test/multihist_test.jl:4-32 (golden Cv / Cp values of the reference)
    d = json.load(open(os.path.join(GOLDEN, name + ".json")))
    T, B = orc.tempgrid(d["t_i"], d["t_f"], d["R"])
    if name == "multihist_nvt":
        Tout, cv, it = orc.multihist_nvt(np.array(d["en_histogram"]), T, B, d["en_min"],
                                         d["en_max"], d["thr"])
        assert len(cv) == 320
    else:
        Tout, cv, it = orc.multihist_npt(np.array(d["ev_histogram"]), T, B, d["en_min"],
                                         d["en_max"], d["v_min"], d["v_max"], d["pressure"],
                                         d["thr"])
        assert len(cv) == 30
    for k, v in d["expected"].items():
        assert cv[int(k) - 1] == pytest.approx(v, rel=1e-12), k
    assert 1 <= it < 1000


def test_checkpoint_fixture_wham(orc):
    # test/testing_data/checkpoint: Ne13, 25 replicas, 102-bin histograms
    d = json.load(open(os.path.join(GOLDEN, "checkpoint_ne13.json")))
    p = d["params"]
    h = np.array(d["histograms"])
    # the fixture holds 25 histogram rows although params.data says n_traj = 24
    assert int(p[2]) == 24 and h.shape == (25, 102)
    R = h.shape[0]
    T, B = orc.tempgrid(p[8], p[9], R)
    Tout, cv, it = orc.multihist_nvt(h, T, B, d["hist_info"][0], d["hist_info"][1], 1e-3)
    assert np.all(np.isfinite(cv)) and np.all(cv > 0)
    assert Tout[0] == pytest.approx(p[8]) and Tout[-1] == pytest.approx(p[9])


def _ne13_start(seed=1234):
    rng = np.random.default_rng(seed)
    pos = []
    while len(pos) < 13:
        v = rng.uniform(-8, 8, 3)
        if np.linalg.norm(v) < 8.0 and all(np.linalg.norm(v - q) > 4.5 for q in pos):
            pos.append(v)
    return np.array(pos)


def test_oracle_run_invariants(orc):
    """A short Ne13 PT run: detailed bookkeeping invariants of the restatement."""
    N, R = 13, 8
    x0 = _ne13_start()
    T, _ = orc.tempgrid(4.0, 16.0, R)
    run = orc.Run(N, R, np.stack([x0] * R), T, bc_param=11.0, exch_prob=1.0, seed=5)
    run.set_elj(C_NE, True)
    run.init()
    run.equilibrate(200)
    run.production(1, 300)
    x, e, _ = run.slot_states()
    s = run.slots()
    # energies equal a fresh recomputation from the positions
    for i in range(R):
        assert e[i] == pytest.approx(orc.elj_config_energy(x[i], orc.POT_ELJEVEN, C_NE), rel=1e-12)
        assert np.all(np.sum(x[i] ** 2, 1) <= 121.0)  # inside the sphere
    eh, _, hp = run.hist()
    assert eh.sum() == R * 300  # one histogram entry per slot per cycle
    assert np.all(s["count_exc"][:, 1] <= s["count_exc"][:, 0])
    assert sorted(s["wos"]) == list(range(R))
    fin = run.finalise(300)
    assert np.all(fin["heat_cap"] >= 0)


def test_oracle_npt_invariants(orc):
    N, R = 32, 4
    a = 8.4
    cells = [(i, j, k) for i in range(2) for j in range(2) for k in range(2)]
    basis = [(0, 0, 0), (0.5, 0.5, 0), (0.5, 0, 0.5), (0, 0.5, 0.5)]
    x0 = np.array([[(c[d] + b[d]) * a for d in range(3)] for c in cells for b in basis]) - a
    L = 2 * a
    T, _ = orc.tempgrid(10.0, 40.0, R)
    run = orc.Run(N, R, np.stack([x0] * R), T, ensemble=orc.NPT, pressure=3.4439647528956955e-9,
                  bc=orc.BC_CUBIC, bc_param=L, exch_prob=1.0, seed=9)
    run.set_elj(C_NE, True)
    run.init()
    run.equilibrate(40)
    run.production(1, 60)
    x, e, box = run.slot_states()
    s = run.slots()
    assert s["count_vol"][:, 0].sum() > 0
    for i in range(R):
        rc2 = box[i] * box[i] / 4
        assert e[i] == pytest.approx(orc.elj_config_energy(x[i], orc.POT_ELJEVEN, C_NE, orc.BC_CUBIC,
                                                           box[i], rc2), rel=1e-9)
    _, ev, hp = run.hist()
    assert ev.sum() == R * 60


def test_rhombic_box_known_answers(orc):
    """test/runtests.jl:119-129, 186-215: rhombic distances (minimum image across
    the sheared face), get_r_cut and get_volume, bit for bit."""
    s3 = 3 ** 0.5
    bc = orc.BC_RHOMBIC
    v1, v2, v3 = [1.0, 2.0, 3.0], [2.0, 4.0, 6.0], [3.0, 6.0, 9.0]
    assert orc.distance2_box(v1, v2, bc, 10.0, 10.0) == 14.0
    assert orc.distance2(v1, v3) == 56.0
    assert orc.distance2_box(v1, v3, bc, 10.0, 10.0) == 36.0
    assert orc.distance2_box(v1, [15.0, 5.0 * s3, 2.0], bc, 10.0, 10.0) == 6.0
    assert orc.box_rcut(bc, 10.0, 10.0) == 10.0 ** 2 * 3 / 16
    assert orc.box_rcut(bc, 10.0, 5.0) == 5.0 ** 2 / 4
    assert orc.box_volume(bc, 10.0, 10.0) == s3 / 2 * 1000.0
    assert orc.box_volume(orc.BC_CUBIC, 10.0, 10.0) == 1000.0
    # rectangular: min(L^2/4, H^2/4), L^2 H, per-axis minimum image
    assert orc.box_rcut(orc.BC_RECT, 10.0, 6.0) == 9.0
    assert orc.box_volume(orc.BC_RECT, 10.0, 6.0) == 600.0
    assert orc.distance2_box([0.0, 0.0, 0.0], [9.0, 1.0, 5.0], orc.BC_RECT, 10.0, 6.0) == 3.0


def rhombic_hcp(n, m, a):
    """n x n triangular layers (side a) stacked ABAB in z (spacing a sqrt(2/3))
    inside RhombicBC(n a, m c): x - y/sqrt(3) in [0, L), y in [0, L sqrt(3)/2)."""
    s3 = 3 ** 0.5
    c = a * (2.0 / 3.0) ** 0.5
    pts = []
    for k in range(m):
        ox, oy = (a / 2, a / (2 * s3)) if k % 2 else (0.0, 0.0)
        for j in range(n):
            for i in range(n):
                pts.append((i * a + j * a / 2 + ox, j * a * s3 / 2 + oy, k * c + 0.25 * c))
    return np.array(pts), n * a, m * c


def test_oracle_separated_volume_rhombic(orc):
    """NPT with separated volume moves in a RhombicBC (volume_change_separated,
    src/MCMoves.jl:298-343): xy, z and uniform moves are all accepted, the box
    aspect changes, every walker's energy equals dimer_energy_config with the
    rhombic cut-off and long-range correction, and atoms stay in the cell."""
    x0, L, H = rhombic_hcp(3, 4, 5.9)
    N, R = len(x0), 4
    T, _ = orc.tempgrid(10.0, 30.0, R)
    run = orc.Run(N, R, np.stack([x0] * R), T, ensemble=orc.NPT, pressure=3.4439647528956955e-9,
                  bc=orc.BC_RHOMBIC, bc_param=L, exch_prob=1.0, seed=21)
    run.set_box(H, separated=True)
    run.set_elj(C_NE, True)
    run.init()
    run.equilibrate(100)
    run.production(1, 200)
    x, e, Lw = run.slot_states()
    b = run.box()
    wos = run.slots()["wos"]
    Hw = b["height"][wos]
    s = run.slots()
    assert s["count_vol"][:, 0].sum() > 0
    assert b["count_xy"][:, 0].sum() > 0 and b["count_z"][:, 0].sum() > 0
    assert np.any(np.abs(Lw / Hw - L / H) > 1e-6)
    s3 = 3 ** 0.5
    for i in range(R):
        ref = orc.elj_config_energy_box(x[i], orc.POT_ELJEVEN, C_NE, orc.BC_RHOMBIC, Lw[i], Hw[i])
        assert e[i] == pytest.approx(ref, rel=1e-9)
        u = x[i][:, 0] - x[i][:, 1] / s3
        assert np.all(u > -0.6 * Lw[i]) and np.all(u < 1.6 * Lw[i])
        assert np.all(x[i][:, 2] > -0.6 * Hw[i]) and np.all(x[i][:, 2] < 1.6 * Hw[i])
    _, ev, hp = run.hist()
    assert ev.sum() == R * 200


def test_oracle_rectangular_uniform_npt(orc):
    """RectangularBC with uniform volume moves: L and H scale together (the
    aspect is kept to rounding), energies follow dimer_energy_config."""
    a = 8.4
    cells = [(i, j, k) for i in range(2) for j in range(2) for k in range(3)]
    basis = [(0, 0, 0), (0.5, 0.5, 0), (0.5, 0, 0.5), (0, 0.5, 0.5)]
    x0 = np.array([[(c[d] + b[d]) * a for d in range(3)] for c in cells for b in basis])
    x0 -= np.array([a, a, 1.5 * a])
    N, R = len(x0), 3
    T, _ = orc.tempgrid(10.0, 30.0, R)
    run = orc.Run(N, R, np.stack([x0] * R), T, ensemble=orc.NPT, pressure=3.4439647528956955e-9,
                  bc=orc.BC_RECT, bc_param=2 * a, exch_prob=1.0, seed=5)
    run.set_box(3 * a)
    run.set_elj(C_NE, True)
    run.init()
    run.cycles(1, 150)
    x, e, Lw = run.slot_states()
    Hw = run.box()["height"][run.slots()["wos"]]
    assert run.slots()["count_vol"][:, 0].sum() > 0
    np.testing.assert_allclose(Lw / Hw, 2.0 / 3.0, rtol=1e-12)
    assert np.any(Lw != 2 * a)
    for i in range(R):
        ref = orc.elj_config_energy_box(x[i], orc.POT_ELJEVEN, C_NE, orc.BC_RECT, Lw[i], Hw[i])
        assert e[i] == pytest.approx(ref, rel=1e-9)


def test_tangent_and_eljb_known_answers(orc):
    """get_tan (test/runtests.jl:217-239) and ELJPotentialB in a rhombic NPT
    state (test/separated_v_test.jl:95-114): tan_mat[1,2], tan_mat[1,3] and
    en_tot == -0.00016263185592172208 (pair terms under the rhombic cut-off
    plus the box-scaled ELJB long-range correction), bit for bit."""
    from lut_synth import ELJB_A, ELJB_B, ELJB_C
    v1, v2, v3 = [5.0, 0.0, 0.0], [-3.0, 0.0, 4.0], [-2.0, 0.0, -3.0]
    assert orc.get_tan(v1, v3) == 7 / 3 and orc.get_tan(v2, v3) == 1 / 7
    assert orc.get_tan(v1, v3, orc.BC_CUBIC, 10.0) == 1.0
    assert orc.get_tan(v1, v2, orc.BC_RHOMBIC, 5.0, 5.0) == 2.0
    assert orc.get_tan(v2, v3, orc.BC_RHOMBIC, 5.0, 5.0) == 0.5
    x = np.array([[1.0, 2.0, 3.0], [2.0, 4.0, 6.0], [0.0, 1.0, 0.0]])
    assert orc.get_tan(x[0], x[1], orc.BC_RHOMBIC, 10.0, 10.0) == pytest.approx(0.7453559924999299)
    assert orc.get_tan(x[0], x[2], orc.BC_RHOMBIC, 10.0, 10.0) == pytest.approx(0.47140452079103173)
    T, _ = orc.tempgrid(10.0, 15.0, 2)
    run = orc.Run(3, 2, np.stack([x] * 2), T, ensemble=orc.NPT,
                  pressure=101325 * 3.398928944382626e-14, bc=orc.BC_RHOMBIC, bc_param=10.0)
    run.set_box(10.0, separated=True)
    run.set_eljb(ELJB_A, ELJB_B, ELJB_C)
    run.init()
    assert run.walkers()[1][0] == -0.00016263185592172208


def test_lookup_table_reference_header():
    """The reference's look-up_table-2.txt read by read_lookuptable gives the
    known answers of test/test_potentials.jl:58-64 (fixture made by
    tests/golden/make_golden.py)."""
    d = json.load(open(os.path.join(GOLDEN, "lookup_table_2.json")))
    assert d["samples"][0][2] == 282.19449125205114
    assert d["start_dist"] == 0.1 and d["start_angle"] == 0
    assert (d["l_angle"], d["l_dist"], d["d_dist"], d["d_angle"]) == (91, 1491, 0.01, 1.0)


def test_lookup_parser_and_oracle_energy(orc, pk, tmp_path):
    """read_lookuptable on a table in the reference's format, and the oracle's
    lookup (src/EnergyEvaluation.jl:277-298) against a numpy restatement over
    the hard-core, table and c6-tail ranges and all angle bands."""
    from lut_synth import write_lut, lut_energy_np
    t, sd, sa, ld, la, dd, da, c6 = pk.read_lookuptable(write_lut(str(tmp_path / "t.txt")))
    assert t.shape == (91, 1491) and (sd, sa, ld, la, dd, da) == (0.1, 0.0, 1491, 91, 0.01, 1.0)
    assert c6 == pytest.approx(np.mean(t[:, 999]) * (0.1 + 1000 * 0.01) ** 6, rel=1e-14)
    lut = dict(table=t, start_dist=sd, d_dist=dd, d_angle=da, c6coeff=c6)
    rng = np.random.default_rng(4)
    r = np.concatenate([rng.uniform(0.05, 0.2, 50), rng.uniform(0.2, 15.0, 400),
                        rng.uniform(15.0, 20.0, 50)])
    tn = np.concatenate([[0.0, 0.001, 0.5, 114.0, 200.0, np.inf], rng.exponential(2.0, 494)])
    for ri, ti in zip(r, tn):
        assert orc.lut_energy(lut, ri * ri, ti) == lut_energy_np(t, sd, dd, da, c6, ri * ri, ti)


def test_nnvt_oracle_chain_is_self_consistent(orc):
    """NNVT with the two-species RuNNer potential on the oracle: after atom moves
    and atom swaps the running energies equal a from-scratch evaluation of the
    final configurations, swaps are accepted, and a swap keeps the species
    composition (positions are exchanged, atoms keep their species)."""
    import ptmc_gb300.starts as st
    import nn2_synth as S
    rad, ang, w1, w2, nodes = S.potential()
    N, n1, R = 10, 6, 3
    x0 = st.sphere_start(N, 6.5, 4.5, 4)
    T, _ = orc.tempgrid(300.0, 900.0, R)
    run = orc.Run(N, R, np.stack([x0] * R), T, ensemble=orc.NNVT, bc=orc.BC_SPHERE,
                  bc_param=10.0, exch_prob=1.0, seed=2)
    run.set_nn2(rad, ang, w1, w2, nodes, n1, n_swaps=2)
    run.init()
    run.cycles(1, 150)
    x, e, _ = run.walkers()
    assert run.swaps() > 0
    fresh = orc.Run(N, R, x, T, ensemble=orc.NNVT, bc=orc.BC_SPHERE, bc_param=10.0, seed=2)
    fresh.set_nn2(rad, ang, w1, w2, nodes, n1, n_swaps=2)
    fresh.init()
    np.testing.assert_allclose(fresh.walkers()[1], e, rtol=1e-12)


def test_runner2atom_normalisations(pk):
    """RadialType2a / AngularType3a constructors (SymmFunc.jl:64-85, 139-175)."""
    r = pk.RuNNerPotential2Atom.radial(0.01, 12.0, [[3.0, 1.0], [2.0, 0.0]], [[5.0, 1.0], [4.0, 2.0]])
    assert r[:2] == [0.01, 12.0]
    assert r[6:] == [0.5, 0.5, 0.25, 0.5]  # G_norm = 1 / (max - min)
    assert r[2:6] == [-0.5, -0.0, -0.25, -1.0]  # G_offset = -min G_norm
    a = pk.RuNNerPotential2Atom.angular(0.001, -1.0, 4.0, 12.0, [[2.0, 0.0]] * 3, [[1.0, 0.5]] * 3)
    assert a[:4] == [0.001, -1.0, 4.0, 12.0]
    assert a[4:10] == [2.0 ** -3 * 0.5] * 3 + [2.0 ** -3 * 2.0] * 3  # tpz = 2^(1-zeta) G_norm
    assert a[10:] == [-0.0] * 3 + [-1.0] * 3


# ---------------------------------------------------------------- surrogate oracle
SUR_CFG = [2.0, 12.0, 1.125, 12.0, 0.02]


def _sur_case(orc, n=6, seed=0):
    rng = np.random.default_rng(seed)
    P = rng.normal(0, 0.3, orc.sur_nparams())
    rows = rng.uniform(3.0, 14.0, (n, 128)).astype(np.float32)
    rows[:, 50:64] = -1.0
    rows[:, 114:128] = -1.0
    y = rng.normal(0, 0.02, n).astype(np.float32)
    return P, rows, y


def test_surrogate_oracle_gradient_finite_differences(orc):
    """The oracle's analytic gradient of the Huber loss (FP64, no BF16 rounding)
    against central differences, on every parameter block."""
    P, rows, y = _sur_case(orc)
    L, g = orc.sur_loss_grad(SUR_CFG, P, rows, y, bf16=False)
    h = 1e-6
    idx = np.r_[0:5, 511, 512, 540, 544, 1000, 1567, 1568, 1599, 1600, 1631, 1632]
    for k in idx:
        Pp, Pm = P.copy(), P.copy()
        Pp[k] += h
        Pm[k] -= h
        fd = (orc.sur_loss_grad(SUR_CFG, Pp, rows, y, bf16=False)[0] -
              orc.sur_loss_grad(SUR_CFG, Pm, rows, y, bf16=False)[0]) / (2 * h)
        assert abs(fd - g[k]) <= 1e-6 * np.abs(g).max() + 1e-9, (k, fd, g[k])


def test_surrogate_oracle_antisymmetry_and_bf16(orc):
    """dE_s of the reverse move (new and old rows swapped) is -dE_s; BF16
    rounding of the matrix operands changes dE_s by a small relative amount."""
    P, rows, _ = _sur_case(orc, n=10, seed=1)
    rev = np.concatenate([rows[:, 64:], rows[:, :64]], axis=1)
    for bf in (False, True):
        a = orc.sur_forward(SUR_CFG, P, rows, bf16=bf)
        b = orc.sur_forward(SUR_CFG, P, rev, bf16=bf)
        np.testing.assert_allclose(a, -b, rtol=1e-12, atol=1e-15)
    a = orc.sur_forward(SUR_CFG, P, rows, bf16=False)
    b = orc.sur_forward(SUR_CFG, P, rows, bf16=True)
    assert np.max(np.abs(a - b)) < 0.05 * np.max(np.abs(a)) and np.max(np.abs(a - b)) > 0


def test_oracle_delayed_acceptance_zero_surrogate_is_exact_chain(orc):
    """With dE_s = 0 the first stage always passes; the chain makes the same
    accept decisions as the plain chain but consumes one more draw per move,
    so it is a valid, different chain with the same statistics."""
    import json
    tables = json.load(open(os.path.join(GOLDEN, "nn_cu55.json")))
    rows = []
    for f in tables["sf"]:
        rows.append([f["kind"], f["type"], f["eta"], f["lambda"], f["zeta"], 12.0, f["gmin"], f["gmax"]])
    sf = np.array(rows)
    rng = np.random.default_rng(3)
    nodes = [88, 20, 20, 1]
    w = []
    for l in range(1, 4):
        lim = 1 / np.sqrt(nodes[l - 1])
        w += [rng.uniform(-lim, lim, nodes[l - 1] * nodes[l]), rng.uniform(-lim, lim, nodes[l])]
    w = np.concatenate(w) * 0.01
    N, R = 6, 2
    x0 = np.array([[0, 0, 0], [4.5, 0, 0], [0, 4.5, 0], [0, 0, 4.5], [4.5, 4.5, 0], [0, 4.5, 4.5]], float)
    T, _ = orc.tempgrid(300.0, 900.0, R)
    run = orc.Run(N, R, np.stack([x0] * R), T, bc=orc.BC_SPHERE, bc_param=10.0, exch_prob=1.0, seed=4)
    run.set_nn(sf, w, nodes, 0.0)
    run.init()
    run.set_surrogate(SUR_CFG, np.zeros(orc.sur_nparams()))
    run.cycles(1, 5)
    st = run.sur_stats()
    assert st["stage1_rejects"] == 0 and st["exact_evals"] == 5 * N * R


def _ref_linear_cv(h, beta, en_min, en_max, npoints=1000):
    """src/multihist.jl restated in numpy with the singular A alpha = b solved by
    least squares (minimum norm): another choice of the free constant."""
    kB = 3.16681196e-6
    R, nb = h.shape
    n_bin = nb - 2
    de = (en_max - en_min) / (n_bin - 1)
    E = np.arange(n_bin) * de + en_min
    H = h[:, 1:-1] / n_bin
    keep = H.sum(axis=0) != 0
    H, E = H[:, keep], E[keep]
    nsum = H.sum(axis=0)
    with np.errstate(divide="ignore", invalid="ignore"):
        bmat = np.where(H == 0, 0.0, H * (np.log(H) + beta[:, None] * E[None, :]))
    b = (bmat - H * bmat.sum(axis=0) / nsum).sum(axis=1)
    A = -(H / nsum) @ H.T + np.diag(H.sum(axis=1))
    alpha = np.linalg.lstsq(A, b, rcond=None)[0]
    S = (bmat - H * alpha[:, None]).sum(axis=0) / nsum
    T0, T1 = 1 / (kB * beta[0]), 1 / (kB * beta[-1])
    T = np.arange(npoints) * ((T1 - T0) / npoints) + T0
    y = S[None, :] - E[None, :] / (T[:, None] * kB)
    y -= y.max(axis=1, keepdims=True)
    w = np.exp(y)
    w /= w.sum(axis=1, keepdims=True)
    U = (w * E).sum(axis=1)
    U2 = (w * E * E).sum(axis=1)
    return T, U, (U2 - U * U) / kB / T ** 2


def test_linear_multihistogram_gauge(orc):
    """The linear-solve multihistogram (src/multihist.jl) has a singular system;
    the oracle fixes alpha[R-1] = 0, a least-squares solve picks another constant:
    U(T) and Cv(T) must agree (they do not depend on the constant)."""
    d = json.load(open(os.path.join(GOLDEN, "multihist_nvt.json")))
    h = np.array(d["en_histogram"])
    _, beta = orc.tempgrid(d["t_i"], d["t_f"], d["R"])
    r = orc.multihist_linear(h, beta, d["en_min"], d["en_max"])
    T, U, Cv = _ref_linear_cv(h, beta, d["en_min"], d["en_max"])
    np.testing.assert_allclose(r["T"], T, rtol=1e-13)
    np.testing.assert_allclose(r["U"], U, rtol=1e-9)
    np.testing.assert_allclose(r["Cv"], Cv, rtol=1e-6)
    assert abs(r["alpha"][-1]) == 0.0
    assert len(r["energies"]) == int((h[:, 1:-1].sum(axis=0) != 0).sum())
