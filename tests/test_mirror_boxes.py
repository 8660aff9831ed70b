"""CPU tests of the host mirror's box geometry against the oracle (whose
rhombic distances, cut-offs and volumes are pinned to the reference's own known
answers in test_oracle_kats.py): distance2 / get_distance2_mat
(src/Configurations.jl:101-162), get_volume (src/Configurations.jl:246-256) and
get_r_cut (src/Ensembles.jl:118-155) for every boundary condition, with
positions spread over several box images so that every minimum-image branch
is taken."""
import numpy as np
import pytest


def cases(pk, orc):
    return [
        (pk.SphericalBC(9.0), orc.BC_SPHERE, 9.0, 0.0),
        (pk.CubicBC(10.0), orc.BC_CUBIC, 10.0, 10.0),
        (pk.RectangularBC(9.0, 13.5), orc.BC_RECT, 9.0, 13.5),
        (pk.RhombicBC(8.5, 11.0), orc.BC_RHOMBIC, 8.5, 11.0),
    ]


def oracle_d2(orc, a, b, kind, L, H):
    if kind in (orc.BC_RECT, orc.BC_RHOMBIC):
        return orc.distance2_box(a, b, kind, L, H)
    return orc.distance2(a, b, kind, L)


@pytest.mark.parametrize("which", range(4))
def test_distance2_mat_matches_oracle(pk, orc, which):
    bc, kind, L, H = cases(pk, orc)[which]
    rng = np.random.default_rng(11 + which)
    x = rng.uniform(-1.7 * max(L, H), 1.7 * max(L, H), size=(14, 3))
    m = pk.get_distance2_mat(pk.Config(x, bc))
    ref = np.zeros_like(m)
    for i in range(len(x)):
        for j in range(len(x)):
            if i != j:
                ref[i, j] = oracle_d2(orc, x[i], x[j], kind, L, H)
    np.testing.assert_allclose(m, ref, rtol=1e-12, atol=1e-12)
    assert np.array_equal(m, m.T) and np.all(np.diag(m) == 0)
    if kind != orc.BC_SPHERE:  # minimum images are no farther than the box allows
        assert np.all(m <= 3 * max(L, H) ** 2)


@pytest.mark.parametrize("which", range(1, 4))
def test_volume_and_cutoff_match_oracle(pk, orc, which):
    bc, kind, L, H = cases(pk, orc)[which]
    np.testing.assert_allclose(pk.get_volume(bc), orc.box_volume(kind, L, H), rtol=1e-15)
    np.testing.assert_allclose(pk.get_r_cut(bc), orc.box_rcut(kind, L, H), rtol=1e-15)


def test_volume_needs_a_periodic_box(pk):
    with pytest.raises(TypeError):
        pk.get_volume(pk.SphericalBC(5.0))
