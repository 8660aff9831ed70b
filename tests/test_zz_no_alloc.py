"""The allocation-free multihistogram entry point (ptmc_multihist_nvt_noalloc).

It serves callers that cannot allocate device memory (CUDA.jl-owned pools,
stream capture, pre-reserved services): they pass their own device buffers and
the WHAM scratch lives in a fixed device array inside the library.  This test
owns its device buffers through torch (any allocator would do), calls the
entry point twice in a row on different histograms, and checks both results
against the allocating entry point ptmc_multihist_nvt to 1e-9 relative (the
two differ only in where the output temperature grid is computed).  The file
sorts last so that a run stopping at the first failure has run everything else.
"""
import ctypes
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def test_noalloc_matches_allocating_entry_point(pk):
    import torch
    L = pk._capi.load()
    d = json.load(open(os.path.join(GOLDEN, "multihist_nvt.json")))
    temp = pk.TempGrid(d["t_i"], d["t_f"], d["R"])
    h1 = np.array(d["en_histogram"], dtype=np.float64)
    h2 = np.floor(h1 * 1.5) + (h1 > 0)      # a second, different input of the same shape
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    R, nb = h1.shape
    assert R == d["R"] and h2.shape == h1.shape
    for h, (emin, emax) in ((h1, (d["en_min"], d["en_max"])),
                            (h2, (d["en_min"], d["en_max"] * 1.01))):
        T_ref, cv_ref, it_ref = pk.multihist_nvt_arrays(h, temp.t_grid, temp.beta_grid, emin, emax, 1e-3)
        dh = torch.from_numpy(np.ascontiguousarray(h)).to(dev)
        dt = torch.from_numpy(temp.t_grid.copy()).to(dev)
        db = torch.from_numpy(temp.beta_grid.copy()).to(dev)
        dT = torch.full((10 * R,), float("nan"), dtype=torch.float64, device=dev)
        dcv = torch.full((10 * R,), float("nan"), dtype=torch.float64, device=dev)
        dit = torch.zeros(1, dtype=torch.int32, device=dev)
        torch.cuda.synchronize(dev)
        rc = L.ptmc_multihist_nvt_noalloc(R, nb - 2, dh.data_ptr(), dt.data_ptr(), db.data_ptr(),
                                          emin, emax, 1e-3, dT.data_ptr(), dcv.data_ptr(),
                                          dit.data_ptr(), ctypes.c_void_p(stream.cuda_stream))
        assert rc == 0
        torch.cuda.synchronize(dev)
        assert int(dit.item()) == it_ref
        np.testing.assert_allclose(dT.cpu().numpy(), T_ref, rtol=1e-13)
        np.testing.assert_allclose(dcv.cpu().numpy(), cv_ref, rtol=1e-9)


def test_noalloc_rejects_sizes_beyond_the_scratch(pk):
    L = pk._capi.load()
    # 3R + 3 n_bin + 20R + 2 > 16384 doubles
    rc = L.ptmc_multihist_nvt_noalloc(32, 6000, 1, 1, 1, -1.0, 0.0, 1e-3, 1, 1, 1, None)
    assert rc == -6
    msg = L.ptmc_last_error(None).decode()
    assert "ptmc_multihist_nvt_noalloc" in msg and "16384" in msg, msg
    rc = L.ptmc_multihist_nvt_noalloc(0, 100, 1, 1, 1, -1.0, 0.0, 1e-3, 1, 1, 1, None)
    assert rc == -1
    assert "ptmc_multihist_nvt_noalloc" in L.ptmc_last_error(None).decode()
