"""Known-answer tests of the oracle's perfect-magnetic-conductor walls (kinds 3 E and 4 B of
oracle.walls) against entries of the reference's tables (pmc_bc_e/b_2d_odd/even,
source/emf/boundary/os-emf-pmc.f90:159-260, 640-760), restated as the conducting-wall image rule
with the signs of E and B exchanged.  Indices are the reference's 1-based cell indices."""
import numpy as np
import pytest

NX = [8, 7]


def _grid(oracle, order):
    return oracle.Grid(NX, order, [0.1, 0.1])


def _at(g, f, c, i1, i2):
    return f[i2 - 1 + g.gcl[1], i1 - 1 + g.gcl[0], c - 1]


def _apply(oracle, g, f, kind, mask):
    out = f.copy()
    oracle.walls(g, "f64", out, kind, mask)
    return out


@pytest.mark.parametrize("i2", [1, 3, 7])
def test_e_odd_lower_x1(oracle, i2):
    g = _grid(oracle, 1)
    f0 = np.random.default_rng(1).standard_normal(g.shape)
    f = _apply(oracle, g, f0, 3, 1)
    for i1 in range(1 - g.gcl[0], 1):
        assert _at(g, f, 1, i1, i2) == -_at(g, f0, 1, 1 - i1, i2)
        assert _at(g, f, 2, i1, i2) == _at(g, f0, 2, 2 - i1, i2)
        assert _at(g, f, 3, i1, i2) == _at(g, f0, 3, 2 - i1, i2)


@pytest.mark.parametrize("i1", [1, 4, 8])
def test_e_odd_lower_x2(oracle, i1):
    g = _grid(oracle, 3)
    f0 = np.random.default_rng(2).standard_normal(g.shape)
    f = _apply(oracle, g, f0, 3, 2)
    for i2 in range(1 - g.gcl[1], 1):
        assert _at(g, f, 1, i1, i2) == _at(g, f0, 1, i1, 2 - i2)
        assert _at(g, f, 2, i1, i2) == -_at(g, f0, 2, i1, 1 - i2)
        assert _at(g, f, 3, i1, i2) == _at(g, f0, 3, i1, 2 - i2)


@pytest.mark.parametrize("i2", [1, 5])
def test_e_odd_upper_x1(oracle, i2):
    g = _grid(oracle, 1)
    n = NX[0]
    f0 = np.random.default_rng(3).standard_normal(g.shape)
    f = _apply(oracle, g, f0, 3, 1)
    for i in range(1, g.gcu[0] + 1):
        assert _at(g, f, 1, n + i, i2) == -_at(g, f0, 1, n + 1 - i, i2)
        assert _at(g, f, 2, n + i, i2) == _at(g, f0, 2, n + 2 - i, i2)


@pytest.mark.parametrize("i2", [2, 6])
def test_b_odd_lower_x1(oracle, i2):
    g = _grid(oracle, 1)
    f0 = np.random.default_rng(4).standard_normal(g.shape)
    f = _apply(oracle, g, f0, 4, 1)
    for i1 in range(1 - g.gcl[0], 1):
        assert _at(g, f, 1, i1, i2) == _at(g, f0, 1, 2 - i1, i2)
        assert _at(g, f, 2, i1, i2) == -_at(g, f0, 2, 1 - i1, i2)
        assert _at(g, f, 3, i1, i2) == -_at(g, f0, 3, 1 - i1, i2)


@pytest.mark.parametrize("i2", [1, 7])
def test_e_even_lower_x1(oracle, i2):
    g = _grid(oracle, 2)
    f0 = np.random.default_rng(5).standard_normal(g.shape)
    f = _apply(oracle, g, f0, 3, 1)
    for i1 in range(1 - g.gcl[0], 0):
        assert _at(g, f, 1, i1, i2) == -_at(g, f0, 1, -i1, i2)
    assert _at(g, f, 1, 0, i2) == 0
    for i1 in range(1 - g.gcl[0], 1):
        assert _at(g, f, 2, i1, i2) == _at(g, f0, 2, 1 - i1, i2)
        assert _at(g, f, 3, i1, i2) == _at(g, f0, 3, 1 - i1, i2)


@pytest.mark.parametrize("i2", [3])
def test_b_even_lower_x1(oracle, i2):
    g = _grid(oracle, 2)
    f0 = np.random.default_rng(6).standard_normal(g.shape)
    f = _apply(oracle, g, f0, 4, 1)
    for i1 in range(1 - g.gcl[0], 1):
        assert _at(g, f, 1, i1, i2) == _at(g, f0, 1, 1 - i1, i2)
    for i1 in range(1 - g.gcl[0], 0):
        assert _at(g, f, 2, i1, i2) == -_at(g, f0, 2, -i1, i2)
        assert _at(g, f, 3, i1, i2) == -_at(g, f0, 3, -i1, i2)
    assert _at(g, f, 2, 0, i2) == 0 and _at(g, f, 3, 0, i2) == 0


def test_pmc_is_pec_with_e_and_b_signs_exchanged(oracle):
    """Away from the points a wall zeroes, the PMC image of E equals minus the PEC image."""
    g = _grid(oracle, 3)
    f0 = np.random.default_rng(7).standard_normal(g.shape)
    a, b = _apply(oracle, g, f0, 3, 1), _apply(oracle, g, f0, 0, 1)
    guard = a != f0
    assert np.allclose(a[guard], -b[guard])
