"""GPU tests of the delayed-acceptance pair surrogate (no counterpart in the
reference; the model is restated in the oracle, oracle/ptmc_oracle.cpp
`sur_row` / `sur_loss_grad`).

* the tensor-core forward pass (BF16 operands, FP32 accumulation) against the
  oracle's FP64 forward with the same BF16 rounding of the matrix operands;
* the GPU loss and gradient against the oracle's analytic gradient (itself
  checked against central finite differences in tests/test_oracle_kats.py);
* the two-stage chain with a zero surrogate against the oracle's two-stage
  chain, bit for bit (draw order: proposal, stage-1 draw, stage-2 draw);
* a surrogate trained on the GPU from the exact chain's own moves: what it
  gains (exact evaluations avoided) and that the chain stays exact (per-
  temperature mean energies equal to the exact chain's within errors).
"""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

NP = 1633


def random_params(seed, scale=1.0):
    rng = np.random.default_rng(seed)
    P = np.zeros(NP, dtype=np.float32)
    P[0:512] = rng.uniform(-1, 1, 512) / 4.0 * scale
    P[512:544] = rng.uniform(-0.2, 0.2, 32)
    P[544:1568] = rng.uniform(-1, 1, 1024) / np.sqrt(32) * scale
    P[1568:1600] = rng.uniform(-0.2, 0.2, 32)
    P[1600:1632] = rng.uniform(-1, 1, 32) / np.sqrt(32)
    P[1632] = 0.1
    return P


def random_records(n, seed, N=55):
    """n move records: N-1 valid new and old distances, the other rows empty."""
    rng = np.random.default_rng(seed)
    rows = np.full((n, 128), -1.0, dtype=np.float32)
    for b in range(n):
        i = rng.integers(0, N)
        for j in range(N):
            if j == i:
                continue
            rows[b, j] = rng.uniform(3.0, 15.0)
            rows[b, 64 + j] = rng.uniform(3.0, 15.0)
    return rows


def test_surrogate_forward_matches_oracle(pk, orc):
    sur = pk.PairSurrogate(2.0, 12.0, None, 12.0, 0.02)
    P = random_params(1)
    rows = random_records(300, 2)
    g = sur.eval(P, rows)
    o = orc.sur_forward(sur.as_array(), P.astype(np.float64), rows, bf16=True)
    err = np.abs(g - o)
    # FP32 accumulation vs FP64; a rare BF16 rounding tie of a feature may
    # round the other way on the two sides (one operand off by 2^-8 relative)
    assert np.max(err) < 5e-3 * sur.escale, np.max(err)
    assert np.mean(err) < 2e-4 * sur.escale, np.mean(err)
    # and not trivially zero
    assert np.std(o) > 0.1 * sur.escale


def test_surrogate_gradient_matches_oracle(pk, orc):
    sur = pk.PairSurrogate(2.0, 12.0, None, 12.0, 0.02)
    P = random_params(3)
    rows = random_records(64, 4)
    y = (orc.sur_forward(sur.as_array(), P.astype(np.float64), rows, bf16=False)
         + np.random.default_rng(5).normal(0, 0.03, 64)).astype(np.float32)
    lg, gg = sur.loss_grad(P, rows, y)
    lo, go = orc.sur_loss_grad(sur.as_array(), P.astype(np.float64), rows, y, bf16=True)
    assert abs(lg - lo) <= 1e-3 * abs(lo), (lg, lo)
    rel = np.linalg.norm(gg - go) / np.linalg.norm(go)
    assert rel < 2e-3, rel
    # every parameter block carries gradient
    for a, b in [(0, 512), (512, 544), (544, 1568), (1568, 1600), (1600, 1632)]:
        assert np.linalg.norm(go[a:b]) > 0
        np.testing.assert_allclose(gg[a:b], go[a:b], atol=5e-3 * np.abs(go[a:b]).max() + 1e-12)


def nn_potential(pk, r_cut=12.0, seed=3, out_scale=0.01):
    tables = json.load(open(os.path.join(GOLDEN, "nn_cu55.json")))
    sf = pk.RuNNerPotential.sf_table(tables, r_cut)
    nodes = [88, 20, 20, 1]
    return pk.RuNNerPotential(sf, pk.RuNNerPotential.random_weights(nodes, seed, out_scale), nodes)


def test_da_zero_surrogate_chain_matches_oracle(pk, orc):
    """FP64 form, a surrogate with all parameters zero (dE_s = 0): the stage-1
    draw is consumed and always passes, stage 2 is the exact Metropolis test.
    The GPU chain must equal the oracle's two-stage chain bit for bit."""
    import ptmc_gb300.starts as S
    pot = nn_potential(pk)
    N, R = 13, 4
    x0 = S.sphere_start(N, 7.0, 4.0, 11)
    mp = pk.MCParams(mc_cycles=100, eq_cycles=0, mc_sample=1, n_traj=R, n_atoms=N)
    temp = pk.TempGrid(300.0, 900.0, R)
    eng = pk.Engine(mp, temp, pot, pk.NVT(N), precision="fp64", exch_prob=1.0, seed=21)
    eng.set_configs(0, pk.Config(x0, pk.SphericalBC(10.0)))
    eng.init()
    sur = pk.PairSurrogate(2.0, 12.0, None, 12.0, 1.0)
    zero = np.zeros(NP, dtype=np.float32)
    eng.surrogate_set(sur, capacity=16, params=zero)
    eng.surrogate_enable(True)
    eng.cycles_nosample(10)
    g = eng.states(0)
    _, _, st = eng.surrogate_state()
    o = orc.Run(N, R, np.stack([x0] * R), temp.t_grid, bc=orc.BC_SPHERE, bc_param=10.0,
                exch_prob=1.0, seed=21, max_displ=np.full(2 * R, 0.1))
    o.set_nn(pot.sf, pot.weights, pot.nodes, pot.boundary)
    o.init()
    o.set_surrogate(sur.as_array(), zero.astype(np.float64))
    o.cycles(1, 10)
    xo, eo, _ = o.slot_states()
    so = o.slots()
    ost = o.sur_stats()
    eng.close()
    assert st["stage1_rejects"] == 0 and ost["stage1_rejects"] == 0
    assert st["exact_evals"] == ost["exact_evals"] == 10 * N * R
    assert np.array_equal(g["counts"][:, 0:2], so["count_atom"])
    assert np.array_equal(g["counts"][:, 4:6], so["count_exc"])
    assert np.array_equal(g["xyz"], xo)
    np.testing.assert_allclose(g["en_tot"], eo, rtol=1e-10)


def _nn13_engine(pk, pot, n_runs, seed, R=8):
    import ptmc_gb300.starts as S
    N = 13
    mp = pk.MCParams(mc_cycles=1000, eq_cycles=0, mc_sample=1, n_traj=R, n_atoms=N)
    temp = pk.TempGrid(300.0, 900.0, R)
    eng = pk.Engine(mp, temp, pot, pk.NVT(N), precision="fp32", exch_prob=1.0, seed=seed,
                    n_runs=n_runs)
    for r in range(n_runs):
        eng.set_configs(r, pk.Config(S.sphere_start(N, 7.0, 4.0, 100 + r), pk.SphericalBC(10.0)))
    eng.init()
    return eng, temp


def _accepted(eng, runs):
    return sum(int(eng.states(r)["counts"][:, 0].sum()) for r in range(runs))


def test_trained_surrogate_gain_and_exactness(pk):
    """Two engines with the same protocol (600 cycles of step-size adaptation,
    300 more cycles, then a measured window of 200 cycles) differ only in the
    measured window: exact moves in one, delayed-acceptance moves with a
    surrogate trained on the GPU from the second engine's own 300 cycles in the
    other.  Energy scale: random NN weights with output layer x0.3 and a 3-bohr
    hard core, so that the exact chain accepts ~40 % of the moves at 300-900 K.
    Gain: the trained network predicts held-out dE (corr > 0.9, the untrained one
    does not) and rejects a large share of proposals without an exact
    evaluation, at fewer exact evaluations per accepted move than the exact
    chain.  Exactness: per-temperature mean energies of the measured windows
    (fixed screening strength 1, then the per-temperature strengths chosen by
    ptmc_surrogate_calibrate) agree with the exact chain's within 5 combined
    standard errors (independent runs as samples)."""
    pot = nn_potential(pk, out_scale=0.3)
    pot.boundary = 3.0
    runs, N, R = 24, 13, 8

    def window(eng):
        e, a0 = [], _accepted(eng, runs)
        for _ in range(20):
            eng.cycles_nosample(10)
            e.append([eng.states(r)["en_tot"] for r in range(runs)])
        return np.array(e), _accepted(eng, runs) - a0

    ref, _ = _nn13_engine(pk, pot, runs, 1, R)
    ref.cycles_nosample(900)
    e_ref, acc_ref = window(ref)
    ref.close()

    eng, _ = _nn13_engine(pk, pot, runs, 2, R)
    eng.cycles_nosample(600)
    eng.surrogate_set(pk.PairSurrogate(2.0, 12.0, None, 12.0, 0.0), capacity=40000, record_every=2)
    eng.surrogate_record(True)
    eng.cycles_nosample(300)
    eng.surrogate_record(False)
    rows, y = eng.surrogate_records()
    assert len(y) > 20000
    P0, _, _ = eng.surrogate_state()
    eng.surrogate_train(4000, batch=512, lr=2e-3)
    P1, sur1, _ = eng.surrogate_state()
    held = slice(-5000, None)
    corr = np.corrcoef(sur1.eval(P1, rows[held]), y[held])[0, 1]
    corr0 = np.corrcoef(sur1.eval(P0, rows[held]), y[held])[0, 1]
    assert corr > 0.9 and corr > corr0 + 0.5, (corr, corr0)
    eng.surrogate_enable(True)
    e_da, acc_da = window(eng)
    _, _, st = eng.surrogate_state()
    # per-temperature screening strength from the records, then a second window
    kappa = eng.surrogate_calibrate(0.05)
    assert kappa.shape == (R,) and np.all((kappa >= 0) & (kappa <= 1))
    assert np.all(np.abs(kappa * 16 - np.round(kappa * 16)) < 1e-9)
    e_cal, acc_cal = window(eng)
    eng.close()

    moves = 200 * N * R * runs
    assert st["stage1_rejects"] + st["exact_evals"] == moves
    assert st["stage1_rejects"] / moves > 0.15, st
    # exact evaluations per accepted move: every move for the exact chain
    assert st["exact_evals"] / acc_da < moves / acc_ref, (st, acc_da, acc_ref)
    m_ref = e_ref.mean(axis=(0, 1))
    se_ref = e_ref.mean(axis=0).std(axis=0, ddof=1) / np.sqrt(runs)
    for e_x in (e_da, e_cal):
        m_x = e_x.mean(axis=(0, 1))
        se_x = e_x.mean(axis=0).std(axis=0, ddof=1) / np.sqrt(runs)
        z = np.abs(m_ref - m_x) / np.sqrt(se_ref ** 2 + se_x ** 2)
        assert np.all(z < 5), z


def test_set_kappa_zero_is_the_exact_chain(pk):
    """ptmc_surrogate_set_kappa: screening strength 0 on every slot skips the
    first stage (no draw), so the delayed-acceptance chain is the exact chain
    bit for bit (FP64 form, same seed); strengths outside [0, 1] and a wrong
    count are refused."""
    import ptmc_gb300.starts as S
    pot = nn_potential(pk)
    N, R = 13, 4
    x0 = S.sphere_start(N, 7.0, 4.0, 11)

    def engine():
        mp = pk.MCParams(mc_cycles=100, eq_cycles=0, mc_sample=1, n_traj=R, n_atoms=N)
        e = pk.Engine(mp, pk.TempGrid(300.0, 900.0, R), pot, pk.NVT(N), precision="fp64",
                      exch_prob=1.0, seed=5)
        e.set_configs(0, pk.Config(x0, pk.SphericalBC(10.0)))
        e.init()
        return e

    ref = engine()
    ref.cycles_nosample(8)
    g_ref = ref.states(0)
    ref.close()
    eng = engine()
    rng = np.random.default_rng(1)
    eng.surrogate_set(pk.PairSurrogate(2.0, 12.0, None, 12.0, 1.0), capacity=16,
                      params=(rng.standard_normal(NP) * 0.1).astype(np.float32))
    with pytest.raises(pk.PTMCError, match="kappa"):
        eng.surrogate_set_kappa(np.full(R, 1.5))
    with pytest.raises(ValueError):
        eng.surrogate_set_kappa(np.zeros(R + 1))
    eng.surrogate_set_kappa(np.zeros(R))
    eng.surrogate_enable(True)
    eng.cycles_nosample(8)
    g = eng.states(0)
    _, _, st = eng.surrogate_state()
    eng.close()
    assert st["stage1_rejects"] == 0 and st["exact_evals"] == 8 * N * R
    assert np.array_equal(g["xyz"], g_ref["xyz"])
    assert np.array_equal(g["counts"], g_ref["counts"])
    np.testing.assert_array_equal(g["en_tot"], g_ref["en_tot"])
