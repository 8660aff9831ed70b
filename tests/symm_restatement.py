"""Independent numpy restatement of the RuNNer symmetry functions and the
per-atom network, written from the formulas of the reference's open Julia code
and not from the oracle's loops, so that the oracle's G matrices (and through
the energies the engine's) can be pinned without the closed forward-pass
library.

Formulas (MachineLearningPotential/SymmFunc.jl, Cutoff.jl):
  fc(r)  = (cos(pi r / r_c) + 1) / 2 for r < r_c, else 0          (Cutoff.jl:77-86)
  G2_i   = G_norm sum_{j != i} fc_ij exp(-eta r_ij^2) + G_offset   (SymmFunc.jl:225-278)
           (a pair term is 0 when fc is exactly 0 or 1,            SymmFunc.jl:225-227)
  G4_i   = tpz sum_{j<k; j,k != i} (1 + lambda cos t_jik)^zeta
                exp(-eta (r_ij^2 + r_ik^2 + r_jk^2)) fc_ij fc_ik fc_jk + G_offset
           cos t_jik = (x_i - x_j).(x_i - x_k) / (r_ij r_ik)         (SymmFunc.jl:184-312,
                                                                     Cutoff.jl:27,48-58)
  G_norm = 1 / (G_max - G_min), G_offset = -G_min G_norm,
  tpz    = 2^(1 - zeta) G_norm                                     (SymmFunc.jl:37-44, 104-112)
Rows of a type other than 11 (radial) or 111 (angular) are zero
(SymmFunc.jl:275-277, 309-311).

Two species (RuNNerPotential2Atom; species 1 = atoms 0..n1-1,
SymmFunc.jl:318-478, 511-541): radial function k fills rows 2k (neighbours of
species 1) and 2k+1 (neighbours of species 2); angular function k fills rows
2 nrad + 3k + m with m = the number of species-2 atoms among the two
neighbours.  Each row is scaled per centre species: radial g G_norm[s] +
G_offset[s] (s = 2 c + row, c = 0 for species 1, 1 for species 2), angular
g tpz[3 c + m] + G_offset[3 c + m].

The per-atom network: tanh hidden layers, linear output, weights per layer
W[n_in][n_out] (input-major) then the biases (the network form of
MachineLearningPotential/ForwardPass.jl:21-41).
"""
import numpy as np


def _geometry(x):
    x = np.asarray(x, dtype=np.float64)
    d = x[:, None, :] - x[None, :, :]          # d[i, j] = x_i - x_j
    r2 = np.einsum("ijc,ijc->ij", d, d)
    return d, r2


def cutoff(r, rc):
    return np.where(r < rc, 0.5 * (np.cos(np.pi * r / rc) + 1.0), 0.0)


def _pair_weights(r2, rc, eta):
    fc = cutoff(np.sqrt(r2), rc)
    v = fc * np.exp(-eta * r2)
    v[(fc == 0.0) | (fc == 1.0)] = 0.0         # includes the diagonal (r = 0, fc = 1)
    return v


def _triplets(d, r2, rc, eta, lam, zeta):
    """T[i, j, k] = (1 + lam cos t_jik)^zeta exp(-eta (r_ij^2 + r_ik^2 + r_jk^2))
    fc_ij fc_ik fc_jk for distinct i, j, k (0 elsewhere)."""
    N = len(r2)
    r = np.sqrt(r2)
    fc = cutoff(r, rc)
    dot = np.einsum("ijc,ikc->ijk", d, d)
    with np.errstate(divide="ignore", invalid="ignore"):
        cos = dot / (r[:, :, None] * r[:, None, :])
    i, j, k = np.indices((N, N, N))
    distinct = (i != j) & (i != k) & (j != k)
    cos = np.where(distinct, cos, 0.0)
    ang = (1.0 + lam * cos) ** zeta
    rad = np.exp(-eta * (r2[:, :, None] + r2[:, None, :] + r2[None, :, :]))
    f3 = fc[:, :, None] * fc[:, None, :] * fc[None, :, :]
    return np.where(distinct, ang * rad * f3, 0.0)


def g_matrix(x, sf):
    """[n_sf, N] symmetry matrix of one configuration.  sf: rows {kind, type,
    eta, lambda, zeta, r_c, G_min, G_max}."""
    d, r2 = _geometry(x)
    N = len(r2)
    G = np.zeros((len(sf), N))
    for s, (kind, typ, eta, lam, zeta, rc, gmin, gmax) in enumerate(np.asarray(sf, float)):
        norm = 1.0 / (gmax - gmin)
        off = -gmin * norm
        if kind == 0:
            if int(typ) != 11:
                continue
            G[s] = _pair_weights(r2, rc, eta).sum(axis=1) * norm + off
        else:
            if int(typ) != 111:
                continue
            T = _triplets(d, r2, rc, eta, lam, zeta)
            # each unordered neighbour pair {j, k} once: half of the ordered sum
            G[s] = 0.5 * T.sum(axis=(1, 2)) * (2.0 ** (1 - zeta) * norm) + off
    return G


def g_matrix2(x, rad, ang, n1):
    """[2 nrad + 3 nang, N] symmetry matrix of a two-species configuration.
    rad rows {eta, r_c, G_offset[4], G_norm[4]}; ang rows {eta, lambda, zeta,
    r_c, tpz[6], G_offset[6]}; the cut-off is the first radial function's."""
    d, r2 = _geometry(x)
    N = len(r2)
    rc = float(rad[0][1])
    sp2 = (np.arange(N) >= n1).astype(int)      # 1 for species-2 atoms
    c = sp2
    nr, na = len(rad), len(ang)
    G = np.zeros((2 * nr + 3 * na, N))
    for k, q in enumerate(np.asarray(rad, float)):
        eta, off, norm = q[0], q[2:6], q[6:10]
        v = _pair_weights(r2, rc, eta)
        for row in (0, 1):
            g = (v * (sp2[None, :] == row)).sum(axis=1)
            G[2 * k + row] = g * norm[2 * c + row] + off[2 * c + row]
    for k, q in enumerate(np.asarray(ang, float)):
        eta, lam, zeta, tpz, off = q[0], q[1], q[2], q[4:10], q[10:16]
        T = _triplets(d, r2, rc, eta, lam, zeta)
        m = sp2[None, :, None] + sp2[None, None, :]   # species-2 neighbours of the pair
        for row in (0, 1, 2):
            g = 0.5 * (T * (m == row)).sum(axis=(1, 2))
            G[2 * nr + 3 * k + row] = g * tpz[3 * c + row] + off[3 * c + row]
    return G


def mlp(G, weights, nodes):
    """Per-atom energies of the [n_in, N] input matrix."""
    h = np.asarray(G, float).T
    off = 0
    L = len(nodes)
    for l in range(1, L):
        ni, no = int(nodes[l - 1]), int(nodes[l])
        W = np.asarray(weights[off:off + ni * no]).reshape(ni, no)
        b = np.asarray(weights[off + ni * no:off + ni * no + no])
        off += ni * no + no
        h = h @ W + b
        if l < L - 1:
            h = np.tanh(h)
    return h[:, 0]


def energy(x, sf, weights, nodes):
    return float(mlp(g_matrix(x, sf), weights, nodes).sum())


def energy2(x, rad, ang, w1, w2, nodes, n1):
    G = g_matrix2(x, rad, ang, n1)
    e = np.concatenate([mlp(G[:, :n1], w1, nodes), mlp(G[:, n1:], w2, nodes)])
    return float(e.sum())


# ------------------------------------------------------------ closed forms
def tetrahedron(a):
    """Regular tetrahedron of edge a centred on the origin."""
    s = a / np.sqrt(8.0)
    return s * np.array([[1, 1, 1], [1, -1, -1], [-1, 1, -1], [-1, -1, 1]], float)


def right_triangle_plus_far(a, far):
    """Atoms O, (a,0,0), (0,a,0) and one at (0,0,far) (beyond the cut-off)."""
    return np.array([[0, 0, 0], [a, 0, 0], [0, a, 0], [0, 0, far]], float)


def fc1(r, rc):
    return 0.5 * (np.cos(np.pi * r / rc) + 1.0) if r < rc else 0.0
