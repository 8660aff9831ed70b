"""Bounded device waits: the failure path runs out without a fault.

The FP32 form's exchange handshake (one CTA per run, a warp per walker) has
the two walkers of the drawn pair wait for each other on flags in shared
memory.  Every such wait is bounded; when one runs out the walker stops with
status 3, neither walker of the pair swaps, and the host call returns
PTMC_ERR_CUDA naming the wait.  A test switch (ptmc_set_wait_test) shortens the
bound to 10^5 clocks and makes every partner wait target a flag value that no
walker writes, so the limit is reached on purpose: no trap, no fault, the
kernel returns by itself and the process's CUDA context stays usable.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

C_NE = [-10.5097942564988, 989.725135614556, -101383.865938807, 3918846.12841668,
        -56234083.4334278, 288738837.441765]


def _engine(pk, seed):
    import ptmc_gb300.starts as S
    R = 8
    mp = pk.MCParams(mc_cycles=1000, eq_cycles=0, mc_sample=1, n_traj=R, n_atoms=13)
    eng = pk.Engine(mp, pk.TempGrid(4.0, 16.0, R), pk.ELJPotentialEven(C_NE), pk.NVT(13),
                    precision="fp32", exch_prob=1.0, seed=seed, cycles_per_launch=4)
    eng.set_configs(0, pk.Config(S.sphere_start(13, 8.0, 4.5, seed), pk.SphericalBC(11.0)))
    eng.init()
    return eng


def test_exchange_partner_wait_runs_out(pk):
    eng = _engine(pk, 5)
    eng.cycles_nosample(8)                      # healthy cycles first
    assert np.all(eng.walker_status(0) == 0)
    before = eng.states(0)
    eng.set_wait_test(clocks=100000, never_set=True)
    with pytest.raises(pk.PTMCError) as ei:
        eng.cycles_nosample(4)
    assert ei.value.code == -3
    assert "exchange partner" in str(ei.value)
    st = eng.walker_status(0)
    assert (st == 3).sum() >= 2, st             # at least the walkers of the first drawn pair
    assert set(st.tolist()) <= {0, 3}, st
    after = eng.states(0)
    # no exchange was counted after the failure began, and the walker <-> slot
    # table is still a permutation (no two slots show one configuration)
    assert np.array_equal(after["counts"][:, 4], before["counts"][:, 4])
    flat = after["xyz"].reshape(8, -1)
    assert len({row.tobytes() for row in flat}) == 8
    eng.close()
    # the CUDA context of the process is healthy: a new engine runs normally
    eng = _engine(pk, 6)
    eng.cycles_nosample(40)
    assert np.all(eng.walker_status(0) == 0)
    assert eng.states(0)["counts"][:, 5].sum() > 0, "exchanges accepted"
    eng.close()


def test_wait_limit_restored(pk):
    """Limit 0 restores the default bound; a generous test limit changes no chain."""
    a, b = _engine(pk, 9), _engine(pk, 9)
    b.set_wait_test(clocks=1 << 30, never_set=False)
    a.cycles_nosample(40)
    b.cycles_nosample(40)
    sa, sb = a.states(0), b.states(0)
    for k in sa:
        assert np.array_equal(sa[k], sb[k]), k
    b.set_wait_test(0, False)
    b.cycles_nosample(4)
    a.close()
    b.close()
