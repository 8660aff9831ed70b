"""CPU tests of the C-ABI library and the host-side mirror (no GPU needed).

- libptmc_gb300.so loads and exports every symbol include/ptmc_gb300.h declares;
- argument validation happens before any device work and reports the
  reference's error messages;
- without a usable GPU the engine fails loudly (no CPU fallback);
- host logic: MCParams, TempGrid, reference checkpoint reading.
"""
import ctypes
import json
import os
import re

import numpy as np
import pytest

from conftest import GOLDEN, ROOT

HEADER = os.path.join(ROOT, "include", "ptmc_gb300.h")


def _declared():
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"\b(ptmc_[a-z_0-9]+)\s*\(", txt)))


def test_header_symbols_exported(pk):
    L = pk._capi.load()
    names = _declared()
    assert len(names) >= 20
    for n in names:
        assert hasattr(L, n), n
    assert set(names) == set(pk._capi.SIGNATURES), "ctypes signatures cover the header"
    assert L.ptmc_version().decode().startswith("ptmc-gb300")


def _params(pk, **kw):
    p = pk._capi.Params()
    p.n_runs, p.n_traj, p.mc_cycles, p.eq_cycles = 1, 4, 100, 20
    p.mc_sample, p.n_adjust, p.n_bin = 1, 100, 100
    p.min_acc, p.max_acc, p.ensemble = 0.4, 0.6, 0
    p.t_i, p.t_f, p.tdistr, p.exch_prob, p.precision, p.seed = 4.0, 16.0, 0, 0.1, 0, 1
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def _create(pk, p):
    L = pk._capi.load()
    h = ctypes.c_void_p()
    rc = L.ptmc_create(ctypes.byref(h), ctypes.byref(p))
    return rc, h, L.ptmc_last_error(None).decode()


def test_argument_validation(pk):
    rc, h, msg = _create(pk, _params(pk, n_traj=1025))
    assert rc == -6 and "1024 replicas" in msg
    rc, h, msg = _create(pk, _params(pk, tdistr=7))
    assert rc == -1 and "temperature distribution" in msg
    rc, h, msg = _create(pk, _params(pk, n_runs=0))
    assert rc == -1


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(_has_gpu(), reason="checks the no-GPU failure path")
def test_no_gpu_fails_loudly(pk):
    rc, h, msg = _create(pk, _params(pk))
    assert rc == -3 and "CUDA" in msg.upper()
    mp = pk.MCParams.new(10, 2, 13)
    with pytest.raises(pk.PTMCError):
        pk.Engine(mp, pk.TempGrid(4, 16, 2), pk.ELJPotentialEven([-1.0, 1.0]), pk.NVT(13))
    h = np.ones((2, 12))
    with pytest.raises(pk.PTMCError):
        pk.multihist_nvt_arrays(h, [4.0, 8.0], [1.0, 2.0], -1.0, 0.0, 1e-3)


def test_mcparams_and_grid(pk):
    # MCParams (src/InputParams.jl:47-63): eq = round(eq_percentage * cycles)
    mp = pk.MCParams.new(1000, 16, 13)
    assert (mp.mc_cycles, mp.eq_cycles, mp.n_adjust, mp.n_bin) == (1000, 200, 100, 100)
    assert pk.MCParams.new(10 ** 6, 16, 13, eq_percentage=0.1).eq_cycles == 100000
    t = pk.TempGrid(4, 16, 16)
    assert t.t_grid[0] == 4.0 and t.t_grid[-1] == pytest.approx(16.0)
    assert 1.0 / (t.t_grid[3] * t.beta_grid[3]) == pytest.approx(pk.kB)
    assert pk.SphericalBC(2.0).radius2 == 4.0
    assert pk.get_volume(pk.CubicBC(10.0)) == 1000.0
    assert pk.distance2([1.0, 2.0, 3.0], [3.0, 6.0, 9.0], pk.CubicBC(10.0)) == 36.0


def test_read_reference_checkpoint(pk, tmp_path):
    """read_checkpoint parses the reference's on-disk format (src/ReadSave.jl);
    the files are re-created from the Ne13 fixture test/testing_data/checkpoint."""
    d = json.load(open(os.path.join(GOLDEN, "checkpoint_ne13.json")))
    ck = tmp_path / "checkpoint"
    ck.mkdir()
    hdr = "cycles: sample_rate: n_traj: n_atoms: n_adjust n_bins min_acc: max_acc t_i: t_f\n"
    (ck / "params.data").write_text(hdr + " ".join(repr(x) for x in d["params"]) + "\n" +
                                    "ensemble n_atom_moves n_atom_swaps\n" +
                                    " ".join(d["ensemble"]) + "\n" + " ".join(d["potential"]) + "\n")
    (ck / "hist_info.data").write_text("e_min e_max v_min v_max dE dV dr2\n" +
                                       " ".join(repr(x) for x in d["hist_info"]) + "\n")
    (ck / "histograms.data").write_text("\n".join("\t".join(repr(x) for x in r)
                                                  for r in d["histograms"]) + "\n")
    (ck / "index.txt").write_text("%d\n" % d["index"])
    for i, c in enumerate(d["configs"], start=1):
        lines = ["%d" % len(c["xyz"]), " ".join(c["header"])]
        lines += ["1  %r %r %r " % tuple(x) for x in c["xyz"]]
        (ck / ("config.%d" % i)).write_text("\n".join(lines) + "\n")
    r = pk.read_checkpoint(str(ck))
    assert r["index"] == 1000
    assert len(r["configs"]) == 25
    assert r["histograms"].shape == (25, 102)
    c0 = r["configs"][0]
    assert isinstance(c0["config"].boundary_condition, pk.SphericalBC)
    assert c0["config"].boundary_condition.radius2 == pytest.approx(101.06969058367278)
    assert c0["max_displ"][0] == pytest.approx(0.3138428376721002)
    assert c0["counts"] == [9758, 0]
    assert len(c0["config"]) == 13


def test_julia_float_text(pk):
    """Floats in checkpoint and multihistogram files are printed as Julia prints
    them (writedlm / print): fixed notation from 1e-4 to below 1e6."""
    cases = {0.1: "0.1", 100.0: "100.0", 1e6: "1.0e6", 1e-5: "1.0e-5", 1e-4: "0.0001",
             -5.62340834334278e7: "-5.62340834334278e7", 123456.5: "123456.5", 0.0: "0.0",
             3.166811429e-6: "3.166811429e-6", -0.00123: "-0.00123"}
    for x, t in cases.items():
        assert pk._jl(x) == t, (x, pk._jl(x), t)


def test_read_params_of_a_reference_checkpoint(pk, tmp_path):
    """read_init's params.data (src/ReadSave.jl:280-345): MCParams with the
    restart's eq_cycles = floor(0.2 cycles), TempGrid, ensemble, potential."""
    ck = tmp_path / "checkpoint"
    ck.mkdir()
    (ck / "params.data").write_text(
        "cycles: sample_rate: n_traj: n_atoms: n_adjust n_bins min_acc: max_acc t_i: t_f\n"
        "1.0e6 1.0 24.0 55.0 100.0 100.0 0.4 0.6 6.0 20.0\n"
        "ensemble n_atom_moves n_atom_swaps\n"
        "NVT 55 55 0\n"
        "ELJPotentialEven{6, Float64} -10.5097942564988 989.725135614556 -101383.865938807 "
        "3.91884612841668e6 -5.62340834334278e7 2.88738837441765e8\n")
    mp, temp, ens, pot = pk.read_params(str(ck))
    assert (mp.mc_cycles, mp.eq_cycles, mp.n_traj, mp.n_atoms, mp.n_bin) == (10 ** 6, 200000, 24, 55, 100)
    assert temp.t_grid[0] == 6.0 and temp.t_grid[-1] == pytest.approx(20.0, rel=1e-15)
    assert isinstance(ens, pk.NVT) and ens.n_atoms == 55
    assert isinstance(pot, pk.ELJPotentialEven) and pot.coeff[3] == 3.91884612841668e6
    (ck / "params.data").write_text(
        "cycles: sample_rate: n_traj: n_atoms: n_adjust n_bins min_acc: max_acc t_i: t_f\n"
        "1000.0 1.0 8.0 32.0 100.0 50.0 0.4 0.6 10.0 40.0\n"
        "ensemble n_atom_moves n_volume_moves n_atom_swaps pressure separated_volume\n"
        "NPT 32 32 1 0 3.4439647528956955e-9 false\n"
        "EAM: 8.482 4.692 1.23 4.56 \n")
    mp, temp, ens, pot = pk.read_params(str(ck))
    assert isinstance(ens, pk.NPT) and ens.pressure == 3.4439647528956955e-9
    assert not ens.separated_volume and mp.n_bin == 50
    assert isinstance(pot, pk.EmbeddedAtomPotential) and (pot.n, pot.ean, pot.eCam) == (8.482, 1.23, 4.56)
