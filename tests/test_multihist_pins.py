"""Known answers for the linear-solve multihistogram (src/multihist.jl), which
the reference ships without a test or golden output.

With histograms that are the exact expected counts of a known discrete
density of states g(E_b) at each replica's temperature,
    h_k(E_b) = n_k g(E_b) exp(-beta_k E_b) / Z_k,
the linear system's equations are consistent, so the method must recover
S(E_b) = ln g(E_b) + const exactly and, from it, the exact U(T) and Cv(T) of the
spectrum on its output temperature grid:
    Cv(T) = (<E^2> - <E>^2) / (kB T^2),  weights g(E_b) exp(-E_b / (kB T)).
Spectra: n two-level units (g = C(n, b), E_b = b eps) and a power-law density
(g = (b + 1)^2).  Checked for the oracle restatement (CPU) and the engine's
GPU solve (ptmc_multihist_linear).
"""
from math import comb

import numpy as np
import pytest

KB = 3.16681196e-6  # Hartree/K (src/InputParams.jl:19)


def _spectrum(kind, n=40):
    b = np.arange(n + 1)
    g = np.array([comb(n, k) for k in b], dtype=np.float64) if kind == "two_level" else (b + 1.0) ** 2
    return b, g


def _case(kind, eps=2.0e-5, R=8, t=(2.0, 20.0), counts=1.0e6):
    b, g = _spectrum(kind)
    E = b * eps
    T = t[0] * (t[1] / t[0]) ** (np.arange(R) / (R - 1))  # geometric grid, as TempGrid
    beta = 1.0 / (KB * T)
    lw = np.log(g)[None, :] - beta[:, None] * E[None, :]
    lw -= lw.max(axis=1, keepdims=True)
    w = np.exp(lw)
    h = np.zeros((R, len(E) + 2))  # under- and overflow bins empty
    h[:, 1:-1] = counts * w / w.sum(axis=1, keepdims=True)
    return h, beta, E, g


def _exact(E, g, T):
    lw = np.log(g)[None, :] - E[None, :] / (KB * T[:, None])
    lw -= lw.max(axis=1, keepdims=True)
    w = np.exp(lw)
    w /= w.sum(axis=1, keepdims=True)
    U = (w * E).sum(axis=1)
    return U, ((w * E * E).sum(axis=1) - U * U) / (KB * T ** 2)


def _check(r, E, g):
    assert len(r["energies"]) == len(E)  # no bin dropped
    np.testing.assert_allclose(r["energies"], E, rtol=1e-13, atol=1e-18)
    S = np.asarray(r["S_E"])
    np.testing.assert_allclose(S - S[0], np.log(g) - np.log(g[0]), rtol=0, atol=1e-8)
    U, Cv = _exact(E, g, np.asarray(r["T"]))
    np.testing.assert_allclose(r["U"], U, rtol=1e-9)
    np.testing.assert_allclose(r["Cv"], Cv, rtol=1e-7)


@pytest.mark.parametrize("kind", ["two_level", "power_law"])
def test_oracle_linear_multihistogram_exact_spectrum(orc, kind):
    h, beta, E, g = _case(kind)
    r = orc.multihist_linear(h, beta, E[0], E[-1], npoints=200)
    _check(r, E, g)


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["two_level", "power_law"])
def test_gpu_linear_multihistogram_exact_spectrum(pk, kind):
    h, beta, E, g = _case(kind)
    r = pk.multihist_linear_arrays(h, beta, E[0], E[-1], npoints=200)
    _check(r, E, g)
