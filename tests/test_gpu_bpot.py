"""GPU parity of the angle-dependent dimer potentials, ELJPotentialB and
LookupTablePotential (src/EnergyEvaluation.jl:161-298, 476-780, 797-880,
983-1009, 1508-1564; src/Configurations.jl:181-240; src/swap_config.jl:196-206),
in the plain FP64 form against the oracle.

Both keep the distance and the tangent matrix of every walker (the reference's
dist2_mat and tan_mat) and update them with the same values, so NVT runs agree
bit for bit in positions and counters, energies to 1e-10 relative; NPT runs
agree in counters and step sizes, positions to 1e-9 (the volume scale comes
from the device's and the host's exp/pow).  The lookup table is synthetic, in
the reference's file format (tests/lut_synth.py): the ELJB energy sampled on
the table grid.  Lengths are in angstrom, the unit of these coefficients.
"""
import numpy as np
import pytest

from lut_synth import ELJB_A, ELJB_B, ELJB_C, write_lut

pytestmark = pytest.mark.gpu

P_ATM = 101325 * 3.398928944382626e-14
REL = 1e-10


def sphere13(seed):
    import ptmc_gb300.starts as st
    return st.sphere_start(13, 3.4, 2.7, seed)


def fcc(nx, nz, a, jitter, seed):
    basis = [(0, 0, 0), (0.5, 0.5, 0), (0.5, 0, 0.5), (0, 0.5, 0.5)]
    cells = [(i, j, k) for i in range(nx) for j in range(nx) for k in range(nz)]
    x = np.array([[(c[d] + b[d]) * a for d in range(3)] for c in cells for b in basis])
    x -= np.array([nx * a / 2, nx * a / 2, nz * a / 2])
    return x + np.random.default_rng(seed).uniform(-jitter, jitter, x.shape), nx * a, nz * a


def rhombic_hcp(n, m, a, jitter, seed):
    s3 = 3 ** 0.5
    c = a * (2.0 / 3.0) ** 0.5
    pts = []
    for k in range(m):
        ox, oy = (a / 2, a / (2 * s3)) if k % 2 else (0.0, 0.0)
        for j in range(n):
            for i in range(n):
                pts.append((i * a + j * a / 2 + ox, j * a * s3 / 2 + oy, k * c + 0.25 * c))
    x = np.array(pts) + np.random.default_rng(seed).uniform(-jitter, jitter, (len(pts), 3))
    return x, n * a, m * c


@pytest.fixture(scope="module")
def lut(pk, tmp_path_factory):
    path = write_lut(str(tmp_path_factory.mktemp("lut") / "table.txt"))
    return pk.LookupTablePotential.from_file(path)


def run_pair(pk, orc, *, pot, x0, bc, R, T, ens="nvt", seed, separated=False, eq=0,
             rdfsave=False):
    N = len(x0)
    mp = pk.MCParams(mc_cycles=1000, eq_cycles=eq, mc_sample=1, n_traj=R, n_atoms=N)
    temp = pk.TempGrid(T[0], T[1], R)
    ensemble = pk.NPT(N, P_ATM, separated) if ens == "npt" else pk.NVT(N)
    eng = pk.Engine(mp, temp, pot, ensemble, exch_prob=1.0, seed=seed, rdfsave=rdfsave)
    eng.set_configs(0, pk.Config(x0, bc))
    if isinstance(bc, pk.SphericalBC):
        kind, L, H = orc.BC_SPHERE, bc.radius, bc.radius
    elif isinstance(bc, pk.CubicBC):
        kind, L, H = orc.BC_CUBIC, bc.box_length, bc.box_length
    else:
        kind = orc.BC_RHOMBIC if isinstance(bc, pk.RhombicBC) else orc.BC_RECT
        L, H = bc.box_length, bc.box_height
    o = orc.Run(N, R, np.stack([x0] * R), temp.t_grid, ensemble=orc.NPT if ens == "npt" else orc.NVT,
                pressure=P_ATM if ens == "npt" else 0.0, bc=kind, bc_param=L, exch_prob=1.0,
                seed=seed)
    if kind in (orc.BC_RECT, orc.BC_RHOMBIC):
        o.set_box(H, separated=separated)
    if isinstance(pot, pk.ELJPotentialB):
        o.set_eljb(pot.coeff_a, pot.coeff_b, pot.coeff_c)
    else:
        o.set_lut(dict(table=pot.table, start_dist=pot.start_dist, start_angle=pot.start_angle,
                       d_dist=pot.d_dist, d_angle=pot.d_angle, c6coeff=pot.c6coeff))
    if rdfsave:
        o.set_rdf(True)
    o.init()
    eng.init()
    return eng, o


def compare(eng, o, exact, boxes=False):
    g = eng.states(0)
    xo, eo, bo = o.slot_states()
    s = o.slots()
    assert np.array_equal(g["counts"], np.concatenate([s["count_atom"], s["count_vol"],
                                                       s["count_exc"]], 1)), "counters"
    assert np.array_equal(g["max_displ"], s["max_displ"]), "step sizes"
    if boxes:
        b, ob = eng.box_states(0), o.box()
        assert np.array_equal(b["counts_sep"], np.concatenate([ob["count_xy"], ob["count_z"]], 1))
        assert np.array_equal(b["max_displ_sep"], ob["max_displ_sep"])
    if exact:
        assert np.array_equal(g["xyz"], xo), "positions (bitwise)"
        assert np.array_equal(g["box"], bo)
    else:
        np.testing.assert_allclose(g["xyz"], xo, rtol=0, atol=1e-9)
        np.testing.assert_allclose(g["box"], bo, rtol=1e-14)
    np.testing.assert_allclose(g["en_tot"], eo, rtol=REL, atol=0)
    np.testing.assert_allclose(g["ham"], s["ham"], rtol=REL, atol=1e-300)
    return g


def test_eljb_nvt_sphere_parity(pk, orc):
    pot = pk.ELJPotentialB(ELJB_A, ELJB_B, ELJB_C)
    eng, o = run_pair(pk, orc, pot=pot, x0=sphere13(5), bc=pk.SphericalBC(5.32), R=8,
                      T=(4.0, 16.0), seed=3, eq=200, rdfsave=True)
    eng.equilibrate()
    o.equilibrate(200)
    eng.run_cycles(1000)
    o.production(1, 1000)
    compare(eng, o, exact=True)
    out = eng.output(0)
    eh, _, _ = o.hist()
    assert np.array_equal(out.en_histogram, eh)
    rdf_o, _ = o.rdf()
    assert np.array_equal(np.array(out.rdf), rdf_o)
    eng.close()


def test_eljb_nvt_cube_parity(pk, orc):
    x0, L, _ = fcc(2, 2, 4.4, 0.05, 7)
    eng, o = run_pair(pk, orc, pot=pk.ELJPotentialB(ELJB_A, ELJB_B, ELJB_C), x0=x0,
                      bc=pk.CubicBC(L), R=4, T=(5.0, 20.0), seed=8)
    eng.cycles_nosample(300)
    o.cycles(1, 300)
    g = compare(eng, o, exact=True)
    assert g["counts"][:, 0].sum() > 0
    eng.close()


def test_eljb_npt_rhombic_separated_parity(pk, orc):
    x0, L, H = rhombic_hcp(3, 4, 3.1, 0.03, 9)
    eng, o = run_pair(pk, orc, pot=pk.ELJPotentialB(ELJB_A, ELJB_B, ELJB_C), x0=x0,
                      bc=pk.RhombicBC(L, H), R=4, T=(10.0, 30.0), ens="npt", seed=10,
                      separated=True, eq=60)
    eng.equilibrate()
    o.equilibrate(60)
    eng.run_cycles(150)
    o.production(1, 150)
    g = compare(eng, o, exact=False, boxes=True)
    b = eng.box_states(0)
    assert g["counts"][:, 2].sum() + b["counts_sep"][:, 0].sum() + b["counts_sep"][:, 2].sum() > 0
    out = eng.output(0)
    _, ev, _ = o.hist()
    assert np.array_equal(out.ev_histogram, ev)
    eng.close()


def test_eljb_npt_rect_uniform_parity(pk, orc):
    x0, L, H = fcc(2, 3, 4.4, 0.03, 11)
    eng, o = run_pair(pk, orc, pot=pk.ELJPotentialB(ELJB_A, ELJB_B, ELJB_C), x0=x0,
                      bc=pk.RectangularBC(L, H), R=3, T=(10.0, 30.0), ens="npt", seed=12, eq=40)
    eng.equilibrate()
    o.equilibrate(40)
    eng.run_cycles(120)
    o.production(1, 120)
    g = compare(eng, o, exact=False, boxes=True)
    assert g["counts"][:, 2].sum() > 0
    eng.close()


def test_lookup_nvt_sphere_parity(pk, orc, lut):
    eng, o = run_pair(pk, orc, pot=lut, x0=sphere13(6), bc=pk.SphericalBC(5.32), R=8,
                      T=(4.0, 16.0), seed=13, eq=200)
    eng.equilibrate()
    o.equilibrate(200)
    eng.run_cycles(600)
    o.production(1, 600)
    compare(eng, o, exact=True)
    out = eng.output(0)
    eh, _, _ = o.hist()
    assert np.array_equal(out.en_histogram, eh)
    eng.close()


def test_lookup_npt_cube_parity(pk, orc, lut):
    x0, L, _ = fcc(2, 2, 4.4, 0.03, 14)
    eng, o = run_pair(pk, orc, pot=lut, x0=x0, bc=pk.CubicBC(L), R=4, T=(10.0, 30.0),
                      ens="npt", seed=15, eq=40)
    eng.equilibrate()
    o.equilibrate(40)
    eng.run_cycles(100)
    o.production(1, 100)
    g = compare(eng, o, exact=False)
    assert g["counts"][:, 2].sum() > 0
    eng.close()


def test_eljb_checkpoint_resume(pk, orc, tmp_path):
    """The tangent matrices travel in engine.bin; params.data carries the
    reference's ELJB potential block (src/ReadSave.jl:71-77)."""
    x0, L, _ = fcc(2, 2, 4.4, 0.05, 16)
    kw = dict(pot=pk.ELJPotentialB(ELJB_A, ELJB_B, ELJB_C), x0=x0, bc=pk.CubicBC(L), R=4,
              T=(10.0, 30.0), ens="npt", seed=17, eq=20)
    a, _ = run_pair(pk, orc, **kw)
    a.equilibrate()
    a.run_cycles(50)
    a.checkpoint(str(tmp_path))
    a.run_cycles(30)
    b, _ = run_pair(pk, orc, **kw)
    b.restore(str(tmp_path))
    b.run_cycles(30)
    for k in ("xyz", "en_tot", "box", "max_displ", "counts", "ham"):
        assert np.array_equal(a.states(0)[k], b.states(0)[k]), k
    lines = open(str(tmp_path / "params.data")).read().split("\n")
    i = lines.index("ELJB 6 ")
    assert [float(v) for v in lines[i + 3].split("\t")] == ELJB_C
    a.close()
    b.close()


def test_bpot_argument_errors(pk, lut):
    x0 = sphere13(1)
    mp = pk.MCParams(mc_cycles=10, eq_cycles=0, mc_sample=1, n_traj=2, n_atoms=13)
    temp = pk.TempGrid(4.0, 8.0, 2)
    e = pk.Engine(mp, temp, lut, pk.NVT(13), precision="fp32")
    e.set_configs(0, pk.Config(x0, pk.SphericalBC(5.32)))
    with pytest.raises(pk.PTMCError, match="FP64"):
        e.init()
    e.close()
