"""Resuming from a checkpoint directory the reference wrote.

The reference resumes with ptmc_run!(true; ...) (src/MCRun.jl:435-481): read_init
reads params.data, rebuild_states (src/ReadSave.jl:436-481) rebuilds every state
from configT<i>.xyz (configuration, box, max_displ, accepted-move totals) and the
results from hist_info.data / histograms.data, every configuration is recentred,
and the production loop resumes at the index in index.txt.  Without an
engine.bin the engine's ptmc_restore does the same from those text files.

The directory is made from the reference's own checkpoint fixture
(test/testing_data/checkpoint, kept as tests/golden/checkpoint_ne13.json): 25
Ne13 configurations with their comment lines, the 25 x 102 energy histograms
and the histogram parameters, index 1000.  Its params.data header claims 24
replicas of 55 atoms; the files hold 25 of 13, so params.data is written with
the counts the files have (and a short cycle count).
"""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def _reference_checkpoint(root, cycles):
    d = json.load(open(os.path.join(GOLDEN, "checkpoint_ne13.json")))
    ck = os.path.join(root, "checkpoint")
    os.makedirs(ck, exist_ok=True)
    R, N = len(d["configs"]), len(d["configs"][0]["xyz"])
    p = d["params"]
    with open(os.path.join(ck, "params.data"), "w") as f:
        f.write("cycles: sample_rate: n_traj: n_atoms: n_adjust n_bins min_acc: max_acc t_i: t_f\n")
        f.write(" ".join(repr(float(v)) for v in [cycles, p[1], R, N] + p[4:]) + "\n")
        f.write("ensemble n_atom_moves n_atom_swaps\n")
        f.write("NVT %d %d 0\n" % (N, N))
        f.write(" ".join(d["potential"]) + "\n")
    with open(os.path.join(ck, "hist_info.data"), "w") as f:
        f.write("e_min e_max v_min v_max Δ_E Δ_V Δ_r2\n")
        f.write(" ".join(repr(v) for v in d["hist_info"]) + "\n")
    with open(os.path.join(ck, "histograms.data"), "w") as f:
        for row in d["histograms"]:
            f.write("\t".join(repr(float(v)) for v in row) + "\n")
    with open(os.path.join(ck, "index.txt"), "w") as f:
        f.write("%d\n" % d["index"])
    for i, c in enumerate(d["configs"]):
        with open(os.path.join(ck, "configT%d.xyz" % (i + 1)), "w") as f:
            f.write("%d\n%s\n" % (N, " ".join(c["header"])))
            for x in c["xyz"]:
                f.write("1  %r %r %r \n" % tuple(x))
    return d, ck


def test_restore_reference_checkpoint(pk, orc, tmp_path):
    d, ck = _reference_checkpoint(str(tmp_path), 1500)
    mp, temp, ens, pot = pk.read_params(ck)
    assert (mp.n_traj, mp.n_atoms, mp.mc_cycles) == (25, 13, 1500)
    c0 = pk.read_checkpoint(ck)["configs"][0]["config"]
    eng = pk.Engine(mp, temp, pot, ens, exch_prob=0.1, seed=7)
    eng.set_configs(0, c0)
    eng.init()
    eng.restore(ck)                      # no engine.bin: the reference's text files
    st, out = eng.states(0), eng.output(0)
    R = 25
    for s in range(R):
        hdr = d["configs"][s]["header"]
        x = np.array(d["configs"][s]["xyz"])
        np.testing.assert_allclose(st["xyz"][s], x - x.mean(axis=0), rtol=0, atol=1e-12)  # recentre!
        assert st["max_displ"][s, 0] == float(hdr[3]) and st["max_displ"][s, 1] == float(hdr[4])
        assert st["counts"][s, 0] == int(hdr[6]) and st["counts"][s, 1] == 0
        assert st["box"][s] == pytest.approx(np.sqrt(float(hdr[2])), rel=1e-15)
    assert np.array_equal(out.en_histogram, np.array(d["histograms"]))
    assert (out.en_min, out.en_max) == (d["hist_info"][0], d["hist_info"][1])
    assert np.all(st["ham"] == 0)       # rebuild_states starts the sums afresh
    e64 = np.array([orc.elj_config_energy(x, orc.POT_ELJEVEN, pot.coeff) for x in st["xyz"]])
    np.testing.assert_allclose(st["en_tot"], e64, rtol=1e-12)
    eng.run_cycles(50)                   # and the chains go on from there
    st = eng.states(0)
    assert st["counts"][:, 1].sum() > 0
    assert eng.output(0).en_histogram.sum() == np.sum(d["histograms"]) + 50 * R
    eng.close()


def test_ptmc_run_resumes_reference_checkpoint(pk, tmp_path):
    """ptmc_run(True) (the reference's ptmc_run!(restart::Bool)) reads
    params.data, rebuilds the states and runs cycles index .. mc_cycles (the
    reference's loop repeats the saved index), checkpointing on the way."""
    d, ck = _reference_checkpoint(str(tmp_path), 1200)
    states, results = pk.ptmc_run(True, save=100, workingdirectory=str(tmp_path))
    R = len(states)
    assert R == 25
    ran = 1200 - d["index"] + 1
    assert results.en_histogram.sum() == np.sum(d["histograms"]) + ran * R
    r = pk.read_checkpoint(ck)
    assert os.path.exists(os.path.join(ck, "engine.bin"))   # the engine's own checkpoint now
    assert r["index"] == 1200 and len(r["configs"]) == R
