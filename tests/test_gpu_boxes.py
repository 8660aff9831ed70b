"""GPU parity of the RectangularBC / RhombicBC boxes and the NPT separated
volume moves (src/MCMoves.jl:66-98, 180-343; src/Configurations.jl:110-126,
246-256; src/Ensembles.jl:118-155; src/Exchange.jl:197-246;
src/Sampling.jl:64-130, 196-245) against the oracle.

Both sides draw the same Philox streams in the same order (move slot,
displacements, acceptance; volume move: rand(1:6) when separated, the scale
draw, the acceptance draw), so the plain FP64 form must make the same
decisions: accept counters of atom, uniform, xy and z volume moves, exchange
counters and step sizes are compared for equality, energies to 1e-10
relative.  The volume scale exp(...)^(1/3) or ^(1/2) comes from the device's
exp/pow and the host's, which may round 1 ulp apart, so positions and box
dimensions agree to ~1e-14 in NPT runs and bit for bit in NVT runs.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

C_NE = [-10.5097942564988, 989.725135614556, -101383.865938807, 3918846.12841668,
        -56234083.4334278, 288738837.441765]  # examples/ne13.jl:24-31
P_ATM = 101325 * 3.398928944382626e-14     # test/test_states.jl:64
REL = 1e-10


def rhombic_hcp(n, m, a, jitter=0.0, seed=0):
    """n x n triangular layers (side a) stacked ABAB in z (spacing a sqrt(2/3))
    in a RhombicBC(n a, m c) cell."""
    s3 = 3 ** 0.5
    c = a * (2.0 / 3.0) ** 0.5
    pts = []
    for k in range(m):
        ox, oy = (a / 2, a / (2 * s3)) if k % 2 else (0.0, 0.0)
        for j in range(n):
            for i in range(n):
                pts.append((i * a + j * a / 2 + ox, j * a * s3 / 2 + oy, k * c + 0.25 * c))
    x = np.array(pts)
    if jitter:
        x += np.random.default_rng(seed).uniform(-jitter, jitter, x.shape)
    return x, n * a, m * c


def fcc_rect(nx, nz, a, jitter=0.0, seed=0):
    """fcc block of nx x nx x nz cells in RectangularBC(nx a, nz a), centred."""
    basis = [(0, 0, 0), (0.5, 0.5, 0), (0.5, 0, 0.5), (0, 0.5, 0.5)]
    cells = [(i, j, k) for i in range(nx) for j in range(nx) for k in range(nz)]
    x = np.array([[(c[d] + b[d]) * a for d in range(3)] for c in cells for b in basis])
    x -= np.array([nx * a / 2, nx * a / 2, nz * a / 2])
    if jitter:
        x += np.random.default_rng(seed).uniform(-jitter, jitter, x.shape)
    return x, nx * a, nz * a


def box_pair(pk, orc, *, x0, L, H, kind, R, T, pot, ens, seed, separated=False, eq=0,
             exch_prob=1.0, rdfsave=False, mc_cycles=1000):
    N = len(x0)
    mp = pk.MCParams(mc_cycles=mc_cycles, eq_cycles=eq, mc_sample=1, n_traj=R, n_atoms=N)
    temp = pk.TempGrid(T[0], T[1], R)
    ensemble = pk.NPT(N, P_ATM, separated) if ens == "npt" else pk.NVT(N)
    bc = pk.RhombicBC(L, H) if kind == "rhombic" else pk.RectangularBC(L, H)
    eng = pk.Engine(mp, temp, pot, ensemble, exch_prob=exch_prob, seed=seed, rdfsave=rdfsave)
    eng.set_configs(0, pk.Config(x0, bc))
    o = orc.Run(N, R, np.stack([x0] * R), temp.t_grid,
                ensemble=orc.NPT if ens == "npt" else orc.NVT, pressure=P_ATM if ens == "npt" else 0.0,
                bc=orc.BC_RHOMBIC if kind == "rhombic" else orc.BC_RECT, bc_param=L,
                exch_prob=exch_prob, seed=seed)
    o.set_box(H, separated=separated)
    o.set_elj(pot.coeff, pot.even)
    if rdfsave:
        o.set_rdf(True)
    o.init()
    eng.init()
    return eng, o


def compare_box(eng, o, exact):
    g = eng.states(0)
    b = eng.box_states(0)
    xo, eo, Lo = o.slot_states()
    s = o.slots()
    ob = o.box()
    assert np.array_equal(g["counts"][:, 0:2], s["count_atom"]), "atom accept counters"
    assert np.array_equal(g["counts"][:, 2:4], s["count_vol"]), "uniform volume counters"
    assert np.array_equal(b["counts_sep"][:, 0:2], ob["count_xy"]), "xy volume counters"
    assert np.array_equal(b["counts_sep"][:, 2:4], ob["count_z"]), "z volume counters"
    assert np.array_equal(g["counts"][:, 4:6], s["count_exc"]), "exchange counters"
    assert np.array_equal(g["max_displ"], s["max_displ"]), "step sizes"
    assert np.array_equal(b["max_displ_sep"], ob["max_displ_sep"]), "xy / z step sizes"
    Ho = ob["height"][s["wos"]]
    if exact:
        assert np.array_equal(g["xyz"], xo), "positions (bitwise)"
        assert np.array_equal(g["box"], Lo) and np.array_equal(b["box_height"], Ho)
    else:
        np.testing.assert_allclose(g["xyz"], xo, rtol=0, atol=1e-9)
        np.testing.assert_allclose(g["box"], Lo, rtol=1e-14)
        np.testing.assert_allclose(b["box_height"], Ho, rtol=1e-14)
    np.testing.assert_allclose(g["en_tot"], eo, rtol=REL, atol=0)
    np.testing.assert_allclose(g["ham"], s["ham"], rtol=REL, atol=1e-300)
    return g, b


def test_rhombic_npt_separated_parity(pk, orc):
    """NPT, RhombicBC, separated volume moves: z, xy and uniform moves all
    accepted; E x V histograms (with the reference's rhombic volume index)
    identical."""
    x0, L, H = rhombic_hcp(3, 4, 5.9, jitter=0.05, seed=3)
    eng, o = box_pair(pk, orc, x0=x0, L=L, H=H, kind="rhombic", R=4, T=(10.0, 30.0),
                      pot=pk.ELJPotentialEven(C_NE), ens="npt", seed=21, separated=True, eq=100)
    eng.equilibrate()
    o.equilibrate(100)
    eng.run_cycles(200)
    o.production(1, 200)
    g, b = compare_box(eng, o, exact=False)
    assert g["counts"][:, 2].sum() > 0
    assert b["counts_sep"][:, 0].sum() > 0 and b["counts_sep"][:, 2].sum() > 0
    assert np.any(np.abs(g["box"] / b["box_height"] - L / H) > 1e-6), "aspect ratio moved"
    out = eng.output(0)
    _, ev, hp = o.hist()
    # en_min/en_max are energies (1e-10); delta_en_hist is their difference / (n_bin - 1)
    np.testing.assert_allclose([out.en_min, out.en_max, out.v_min, out.v_max, out.delta_en_hist,
                                out.delta_v_hist], hp, rtol=REL)
    assert np.array_equal(out.ev_histogram, ev)
    # energies equal dimer_energy_config of the returned boxes (rhombic cut-off, scaled lrc)
    for i in range(4):
        ref = orc.elj_config_energy_box(g["xyz"][i], orc.POT_ELJEVEN, C_NE, orc.BC_RHOMBIC,
                                        g["box"][i], b["box_height"][i])
        assert g["en_tot"][i] == pytest.approx(ref, rel=1e-10)
    eng.close()


def test_rectangular_npt_uniform_parity(pk, orc):
    """NPT, RectangularBC, uniform volume moves (L and H scale together)."""
    x0, L, H = fcc_rect(2, 3, 8.4, jitter=0.05, seed=4)
    eng, o = box_pair(pk, orc, x0=x0, L=L, H=H, kind="rect", R=3, T=(10.0, 30.0),
                      pot=pk.ELJPotentialEven(C_NE), ens="npt", seed=5, eq=60)
    eng.equilibrate()
    o.equilibrate(60)
    eng.run_cycles(120)
    o.production(1, 120)
    g, b = compare_box(eng, o, exact=False)
    assert g["counts"][:, 2].sum() > 0
    np.testing.assert_allclose(g["box"] / b["box_height"], L / H, rtol=1e-12)
    out = eng.output(0)
    _, ev, _ = o.hist()
    assert np.array_equal(out.ev_histogram, ev)
    eng.close()


def test_rectangular_npt_separated_parity(pk, orc):
    """NPT, RectangularBC, separated volume moves."""
    x0, L, H = fcc_rect(2, 3, 8.4, jitter=0.05, seed=6)
    eng, o = box_pair(pk, orc, x0=x0, L=L, H=H, kind="rect", R=4, T=(10.0, 30.0),
                      pot=pk.ELJPotentialEven(C_NE), ens="npt", seed=7, separated=True, eq=60)
    eng.equilibrate()
    o.equilibrate(60)
    eng.run_cycles(150)
    o.production(1, 150)
    g, b = compare_box(eng, o, exact=False)
    assert b["counts_sep"][:, 0].sum() > 0 and b["counts_sep"][:, 2].sum() > 0
    eng.close()


@pytest.mark.parametrize("kind", ["rhombic", "rect"])
def test_box_nvt_parity_with_rdf(pk, orc, kind):
    """NVT in the periodic boxes with the all-powers ELJ potential: the
    minimum image, the wrap of moved atoms and the RDF bins (delta_r2 from the
    box, src/Sampling.jl:210, 240) bit for bit."""
    if kind == "rhombic":
        x0, L, H = rhombic_hcp(3, 2, 5.9, jitter=0.1, seed=8)
    else:
        x0, L, H = fcc_rect(2, 2, 8.4, jitter=0.1, seed=8)
        H = 1.25 * H
    eng, o = box_pair(pk, orc, x0=x0, L=L, H=H, kind=kind, R=4, T=(10.0, 40.0),
                      pot=pk.ELJPotential(C_NE), ens="nvt", seed=9, eq=40, rdfsave=True)
    eng.equilibrate()
    o.equilibrate(40)
    eng.run_cycles(1000)
    o.production(1, 1000)
    compare_box(eng, o, exact=True)
    out = eng.output(0)
    rdf_o, dr2_o = o.rdf()
    assert out.delta_r2 == dr2_o
    rdf_g = np.array(out.rdf)
    assert np.array_equal(rdf_g, rdf_o) and rdf_g.sum() > 0
    eh, _, _ = o.hist()
    assert np.array_equal(out.en_histogram, eh)
    eng.close()


def test_rhombic_checkpoint_resume(pk, orc, tmp_path):
    """A separated-volume rhombic run checkpointed and restored continues as the
    uninterrupted run (box heights, xy/z step sizes and counters included)."""
    x0, L, H = rhombic_hcp(3, 4, 5.9, jitter=0.05, seed=11)
    kw = dict(x0=x0, L=L, H=H, kind="rhombic", R=4, T=(10.0, 30.0),
              pot=pk.ELJPotentialEven(C_NE), ens="npt", seed=12, separated=True, eq=40)
    a, _ = box_pair(pk, orc, **kw)
    a.equilibrate()
    a.run_cycles(60)
    a.checkpoint(str(tmp_path))
    a.run_cycles(40)
    b, _ = box_pair(pk, orc, **kw)
    b.restore(str(tmp_path))
    b.run_cycles(40)
    for k in ("xyz", "en_tot", "box", "max_displ", "counts", "ham"):
        assert np.array_equal(a.states(0)[k], b.states(0)[k]), k
    for k in ("box_height", "max_displ_sep", "counts_sep"):
        assert np.array_equal(a.box_states(0)[k], b.box_states(0)[k]), k
    ck = pk.read_checkpoint(str(tmp_path))
    assert isinstance(ck["configs"][0]["config"].boundary_condition, pk.RhombicBC)
    a.close()
    b.close()


def test_box_argument_errors(pk):
    """The boxes run in the plain FP64 form with the ELJ potentials; separated
    volume moves need NPT with one of them."""
    x0, L, H = rhombic_hcp(3, 2, 5.9)
    N = len(x0)
    mp = pk.MCParams(mc_cycles=10, eq_cycles=0, mc_sample=1, n_traj=2, n_atoms=N)
    temp = pk.TempGrid(10.0, 20.0, 2)
    e = pk.Engine(mp, temp, pk.ELJPotentialEven(C_NE), pk.NVT(N), precision="fp32")
    e.set_configs(0, pk.Config(x0, pk.RhombicBC(L, H)))
    with pytest.raises(pk.PTMCError, match="FP64"):
        e.init()
    e.close()
    e = pk.Engine(mp, temp, pk.ELJPotentialEven(C_NE), pk.NPT(N, P_ATM, True))
    e.set_configs(0, pk.Config(x0, pk.CubicBC(L)))
    with pytest.raises(pk.PTMCError, match="separated"):
        e.init()
    e.close()
