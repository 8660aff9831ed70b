"""GPU parity of the NNVT ensemble with the two-species RuNNer potential
(RuNNerPotential2Atom, src/EnergyEvaluation.jl:1276-1448; MachineLearningPotential/
SymmFunc.jl:326-541; NNVT and atom swaps, src/Ensembles.jl:138-151,
src/MCMoves.jl:363-370, src/swap_config.jl:237-276) against the oracle.

Both draw the same Philox streams in the same order (move index over N + n_swaps
moves; a displacement's three draws or a swap's two atom draws; the acceptance
draw) and build the same symmetry matrices (every pair and triangle term formed
alike; only the order in which terms are added differs), so the plain FP64 form
makes the same decisions: positions, atom-move, exchange and swap counters and
histograms agree exactly, energies to 1e-10 relative.  The potential is
synthetic (tests/nn2_synth.py): no trained two-species potential is available,
and the reference's known answer for this potential (test/test_potentials.jl:86)
goes through a closed library, so parity is against the oracle only.
"""
import numpy as np
import pytest

import nn2_synth as S

pytestmark = pytest.mark.gpu
REL = 1e-10


def pair(pk, orc, *, N, n1, R, seed, n_swaps=1, eq=0, T=(300.0, 900.0), radius=10.0,
         start_radius=7.0):
    import ptmc_gb300.starts as st
    rad, ang, w1, w2, nodes = S.potential()
    x0 = st.sphere_start(N, start_radius, 4.5, seed)
    mp = pk.MCParams(mc_cycles=1000, eq_cycles=eq, mc_sample=1, n_traj=R, n_atoms=N)
    temp = pk.TempGrid(T[0], T[1], R)
    pot = pk.RuNNerPotential2Atom(rad, ang, w1, w2, nodes, n1)
    eng = pk.Engine(mp, temp, pot, pk.NNVT((n1, N - n1), n_swaps), exch_prob=1.0, seed=seed)
    eng.set_configs(0, pk.Config(x0, pk.SphericalBC(radius)))
    eng.init()
    o = orc.Run(N, R, np.stack([x0] * R), temp.t_grid, ensemble=orc.NNVT, bc=orc.BC_SPHERE,
                bc_param=radius, exch_prob=1.0, seed=seed)
    o.set_nn2(rad, ang, w1, w2, nodes, n1, n_swaps=n_swaps)
    o.init()
    return eng, o


def compare(eng, o):
    g = eng.states(0)
    xo, eo, _ = o.slot_states()
    s = o.slots()
    assert np.array_equal(g["counts"][:, 0:2], s["count_atom"]), "atom accept counters"
    assert np.array_equal(g["counts"][:, 4:6], s["count_exc"]), "exchange counters"
    assert np.array_equal(g["max_displ"], s["max_displ"]), "step sizes"
    assert np.array_equal(g["xyz"], xo), "positions (bitwise)"
    np.testing.assert_allclose(g["en_tot"], eo, rtol=REL, atol=0)
    np.testing.assert_allclose(g["ham"], s["ham"], rtol=REL, atol=1e-300)
    assert eng.swaps(0) == o.swaps(), "accepted swaps"
    return g


def test_nnvt_initial_energies(pk, orc):
    eng, o = pair(pk, orc, N=12, n1=7, R=4, seed=3)
    np.testing.assert_allclose(eng.states(0)["en_tot"], o.slot_states()[1], rtol=1e-12)
    eng.close()


def test_nnvt_parity(pk, orc):
    """Atom moves, one swap per cycle, exchange every cycle, production with
    histograms: 12 atoms (7 + 5), 4 replicas."""
    eng, o = pair(pk, orc, N=12, n1=7, R=4, seed=5, eq=100)
    eng.equilibrate()
    o.equilibrate(100)
    eng.run_cycles(300)
    o.production(1, 300)
    g = compare(eng, o)
    assert g["counts"][:, 0].sum() > 0 and eng.swaps(0) > 0
    out = eng.output(0)
    eh, _, _ = o.hist()
    assert np.array_equal(out.en_histogram, eh)
    eng.close()


def test_nnvt_parity_two_swaps(pk, orc):
    """20 atoms (12 + 8), two swaps per cycle, 3 replicas."""
    eng, o = pair(pk, orc, N=20, n1=12, R=3, seed=9, n_swaps=2, start_radius=8.5, radius=11.0)
    eng.cycles_nosample(120)
    o.cycles(1, 120)
    compare(eng, o)
    eng.close()


def test_nnvt_running_energy_is_the_configuration_energy(pk, orc):
    eng, o = pair(pk, orc, N=12, n1=6, R=4, seed=11)
    eng.cycles_nosample(200)
    before = eng.states(0)["en_tot"].copy()
    eng.resync()  # recompute from the positions
    np.testing.assert_allclose(eng.states(0)["en_tot"], before, rtol=1e-12)
    eng.close()


def test_nnvt_argument_errors(pk):
    import ptmc_gb300.starts as st
    rad, ang, w1, w2, nodes = S.potential()
    x0 = st.sphere_start(12, 7.0, 4.5, 1)
    mp = pk.MCParams(mc_cycles=10, eq_cycles=0, mc_sample=1, n_traj=2, n_atoms=12)
    temp = pk.TempGrid(300.0, 600.0, 2)
    pot = pk.RuNNerPotential2Atom(rad, ang, w1, w2, nodes, 7)
    e = pk.Engine(mp, temp, pot, pk.NNVT((7, 5)), precision="fp32")
    e.set_configs(0, pk.Config(x0, pk.SphericalBC(10.0)))
    with pytest.raises(pk.PTMCError, match="FP64"):
        e.init()
    e.close()
    with pytest.raises(ValueError, match="NNVT"):
        pk.Engine(mp, temp, pot, pk.NVT(12))


@pytest.mark.parametrize("N,n1", [(4, 2), (4, 1), (9, 5)])
def test_nnvt_energy_pinned_by_restatement(pk, orc, N, n1):
    """Initial and running energies against the independent numpy restatement of
    the two-species symmetry functions (tests/symm_restatement.py; SymmFunc.jl:
    318-541) instead of the oracle: the regular tetrahedron (closed form) and a
    9-atom cluster, before and after a chain with atom moves and swaps."""
    import symm_restatement as SR
    import ptmc_gb300.starts as st
    rad, ang, w1, w2, nodes = S.potential()
    x0 = SR.tetrahedron(4.8) if N == 4 else st.sphere_start(N, 6.0, 4.2, 3)
    mp = pk.MCParams(mc_cycles=100, eq_cycles=0, mc_sample=1, n_traj=3, n_atoms=N)
    temp = pk.TempGrid(300.0, 900.0, 3)
    pot = pk.RuNNerPotential2Atom(rad, ang, w1, w2, nodes, n1)
    eng = pk.Engine(mp, temp, pot, pk.NNVT((n1, N - n1), 1), exch_prob=1.0, seed=4)
    eng.set_configs(0, pk.Config(x0, pk.SphericalBC(9.0)))
    eng.init()
    e0 = SR.energy2(x0, rad, ang, w1, w2, nodes, n1)
    np.testing.assert_allclose(eng.states(0)["en_tot"], e0, rtol=1e-12)
    eng.cycles_nosample(60)
    g = eng.states(0)
    assert g["counts"][:, 0].sum() > 0 and eng.swaps(0) > 0
    for s in range(3):
        np.testing.assert_allclose(g["en_tot"][s], SR.energy2(g["xyz"][s], rad, ang, w1, w2, nodes, n1),
                                   rtol=1e-10)
    eng.close()
