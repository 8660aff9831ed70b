"""A synthetic two-species RuNNer potential (RuNNerPotential2Atom,
src/EnergyEvaluation.jl:1287-1314) for the NNVT tests: four radial
(RadialType2a) and three angular (AngularType3a) symmetry functions with
normalisations of the reference's form (G_norm = 1 / (G_max - G_min),
G_offset = -G_min G_norm, tpz = 2^(1 - zeta) G_norm), and seeded random MLP
weights 29-12-12-1 for each species (no trained potential is available)."""
import numpy as np

RCUT = 12.0
RAD_ETA = [0.002, 0.01, 0.03, 0.08]
ANG = [(0.001, 1.0, 1.0), (0.001, -1.0, 1.0), (0.004, 1.0, 4.0)]


def symmetry_functions():
    """rad [4, 10]: eta, r_cut, G_offset[4], G_norm[4]; ang [3, 16]: eta,
    lambda, zeta, r_cut, tpz[6], G_offset[6]."""
    rad = []
    for k, eta in enumerate(RAD_ETA):
        gmax = [4.0 / (1 + 20 * eta) * f for f in (1.0, 0.7, 0.8, 1.1)]
        gmin = [0.1 * g for g in gmax]
        norm = [1 / (a - b) for a, b in zip(gmax, gmin)]
        off = [-b * n for b, n in zip(gmin, norm)]
        rad.append([eta, RCUT] + off + norm)
    ang = []
    for eta, lam, zeta in ANG:
        gmax = [2.0, 1.5, 1.0, 1.2, 1.6, 2.2]
        gmin = [0.0] * 6
        norm = [1 / (a - b) for a, b in zip(gmax, gmin)]
        tpz = [2.0 ** (1 - zeta) * n for n in norm]
        off = [-b * n for b, n in zip(gmin, norm)]
        ang.append([eta, lam, zeta, RCUT] + tpz + off)
    return np.array(rad), np.array(ang)


def mlp_weights(nodes, seed, out_scale=0.3):
    """Per layer W[n_in][n_out] (input-major) then b[n_out]."""
    rng = np.random.default_rng(seed)
    w = []
    for l in range(1, len(nodes)):
        ni, no = nodes[l - 1], nodes[l]
        lim = np.sqrt(3.0 / ni)
        W = rng.uniform(-lim, lim, (ni, no))
        b = rng.uniform(-lim, lim, no)
        if l == len(nodes) - 1:
            W, b = W * out_scale, b * out_scale
        w += [W.reshape(-1), b]
    return np.concatenate(w)


def potential(seed=3):
    rad, ang = symmetry_functions()
    nodes = [2 * len(rad) + 3 * len(ang), 12, 12, 1]
    return rad, ang, mlp_weights(nodes, seed), mlp_weights(nodes, seed + 1), nodes
