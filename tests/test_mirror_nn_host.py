"""CPU tests of the host helpers that build NN potentials for the engine:
RuNNerPotential.sf_table (the symmetry-function table of scripts/cu55.jl) and
RuNNerPotential.random_weights (seeded FP32-valued weights, layer order
W1, b1, W2, b2, ...)."""
import json
import os

import numpy as np

from conftest import GOLDEN


def test_sf_table_rows_and_cutoff(pk):
    tables = json.load(open(os.path.join(GOLDEN, "nn_cu55.json")))
    t = pk.RuNNerPotential.sf_table(tables)
    assert t.shape == (len(tables["sf"]), 8)
    assert np.array_equal(t[:, 5], [f["rcut"] for f in tables["sf"]])
    t12 = pk.RuNNerPotential.sf_table(tables, 12.0)
    assert np.all(t12[:, 5] == 12.0)
    assert np.array_equal(np.delete(t12, 5, axis=1), np.delete(t, 5, axis=1))


def test_random_weights_layout_and_scale(pk):
    nodes = [88, 20, 20, 1]
    w = pk.RuNNerPotential.random_weights(nodes, 3)
    assert len(w) == sum((a + 1) * b for a, b in zip(nodes[:-1], nodes[1:]))
    assert np.array_equal(w, w.astype(np.float32).astype(np.float64))  # FP32-valued
    off = 0
    for a, b in zip(nodes[:-1], nodes[1:]):  # every entry within its layer's U(-1/sqrt(a), 1/sqrt(a))
        blk = w[off:off + (a + 1) * b]
        assert np.all(np.abs(blk) <= 1 / np.sqrt(a))
        off += (a + 1) * b
    ws = pk.RuNNerPotential.random_weights(nodes, 3, 0.3)
    last = (nodes[-2] + 1) * nodes[-1]
    assert np.array_equal(ws[:-last], w[:-last])  # only the output layer is scaled
    np.testing.assert_allclose(ws[-last:], w[-last:] * 0.3, rtol=1e-6)
    assert np.array_equal(pk.RuNNerPotential.random_weights(nodes, 3), w)  # seeded
