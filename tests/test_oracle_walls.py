"""Known-answer tests of the oracle's conducting walls against entries of the reference's
tables (pec_bc_e/b_2d_odd/even, source/emf/boundary/os-emf-pec.f90:131-1123; spec_bc_2d,
source/current/os-current-boundary.f03:204-618), restated in the oracle as one image rule, and
of specular particle reflection (source/spec/os-spec-boundary.f03:1293-1310).  Indices below
are the reference's 1-based cell indices along the walled axis.

Two table entries do not follow the rule and are not reproduced: the cubic lower-x2 current
(`jay(3,i1,3) = jay(3,i1,2) + jay(3,i1,-1)`, where every other entry adds into the point it
updates) and the odd-order upper-x1 B wall (it zeroes B2 at nx+1 where the lower wall zeroes
B1 at 1)."""
import numpy as np
import pytest

NX = [8, 7]


def _grid(oracle, order):
    return oracle.Grid(NX, order, [0.1, 0.1])


def _rand(g, seed):
    return np.random.default_rng(seed).standard_normal(g.shape)


def _at(g, f, c, i1, i2):
    """component c (1-based) at reference indices (i1, i2)"""
    return f[i2 - 1 + g.gcl[1], i1 - 1 + g.gcl[0], c - 1]


def _apply(oracle, g, f, kind, mask):
    out = f.copy()
    oracle.walls(g, "f64", out, kind, mask)
    return out


@pytest.mark.parametrize("i2", [1, 4, 7])
def test_current_linear_x1(oracle, i2):
    g = _grid(oracle, 1)
    j0 = _rand(g, 1)
    j = _apply(oracle, g, j0, 2, 1)
    n = NX[0]
    a = lambda f, c, i: _at(g, f, c, i, i2)
    assert a(j, 1, 1) == a(j0, 1, 1) - a(j0, 1, 0)
    assert a(j, 2, 1) == 2 * a(j0, 2, 1) and a(j, 3, 1) == 2 * a(j0, 3, 1)
    assert a(j, 2, 2) == a(j0, 2, 2) + a(j0, 2, 0) and a(j, 3, 2) == a(j0, 3, 2) + a(j0, 3, 0)
    assert a(j, 1, n) == a(j0, 1, n) - a(j0, 1, n + 1)
    assert a(j, 2, n) == a(j0, 2, n) + a(j0, 2, n + 2)
    assert a(j, 2, n + 1) == 2 * a(j0, 2, n + 1) and a(j, 3, n + 1) == 2 * a(j0, 3, n + 1)


@pytest.mark.parametrize("i1", [1, 5, 8])
def test_current_quadratic_x2(oracle, i1):
    g = _grid(oracle, 2)
    j0 = _rand(g, 2)
    j = _apply(oracle, g, j0, 2, 2)
    n = NX[1]
    a = lambda f, c, i: _at(g, f, c, i1, i)
    assert a(j, 2, 0) == 0
    assert a(j, 1, 1) == a(j0, 1, 1) + a(j0, 1, 0)
    assert a(j, 2, 1) == a(j0, 2, 1) - a(j0, 2, -1)
    assert a(j, 1, 2) == a(j0, 1, 2) + a(j0, 1, -1) and a(j, 3, 2) == a(j0, 3, 2) + a(j0, 3, -1)
    assert a(j, 1, n - 1) == a(j0, 1, n - 1) + a(j0, 1, n + 2)
    assert a(j, 2, n - 1) == a(j0, 2, n - 1) - a(j0, 2, n + 1)
    assert a(j, 2, n) == 0 and a(j, 3, n) == a(j0, 3, n) + a(j0, 3, n + 1)


def test_current_quartic_x1(oracle):
    g = _grid(oracle, 4)
    j0 = _rand(g, 3)
    j = _apply(oracle, g, j0, 2, 1)
    n = NX[0]
    a = lambda f, c, i: _at(g, f, c, i, 3)
    assert a(j, 1, 0) == 0 and a(j, 1, 2) == a(j0, 1, 2) - a(j0, 1, -2)
    assert a(j, 2, 3) == a(j0, 2, 3) + a(j0, 2, -2)
    assert a(j, 1, n - 2) == a(j0, 1, n - 2) - a(j0, 1, n + 2)
    assert a(j, 1, n) == 0 and a(j, 3, n) == a(j0, 3, n) + a(j0, 3, n + 1)


def test_pec_e_odd_and_even(oracle):
    g = _grid(oracle, 1)                         # linear: odd
    e0 = _rand(g, 4)
    e = _apply(oracle, g, e0, 0, 1)
    n = NX[0]
    a = lambda f, c, i: _at(g, f, c, i, 2)
    assert a(e, 1, 0) == a(e0, 1, 1) and a(e, 2, 0) == -a(e0, 2, 2) and a(e, 3, 0) == -a(e0, 3, 2)
    assert a(e, 2, 1) == 0 and a(e, 3, 1) == 0
    assert a(e, 1, n + 1) == a(e0, 1, n) and a(e, 2, n + 1) == 0
    assert a(e, 2, n + 2) == -a(e0, 2, n)
    g = _grid(oracle, 2)                         # quadratic: even
    e0 = _rand(g, 5)
    e = _apply(oracle, g, e0, 0, 2)
    n = NX[1]
    a = lambda f, c, i: _at(g, f, c, 3, i)
    for i in (0, -1):
        assert a(e, 1, i) == -a(e0, 1, 1 - i) and a(e, 2, i) == a(e0, 2, -i)
        assert a(e, 3, i) == -a(e0, 3, 1 - i)
    assert a(e, 2, n + 1) == a(e0, 2, n - 1) and a(e, 1, n + 1) == -a(e0, 1, n)


def test_pec_b_odd_and_even(oracle):
    g = _grid(oracle, 3)                         # cubic: odd
    b0 = _rand(g, 6)
    b = _apply(oracle, g, b0, 1, 2)
    n = NX[1]
    a = lambda f, c, i: _at(g, f, c, 4, i)
    for i in (0, -1):
        assert a(b, 1, i) == a(b0, 1, 1 - i) and a(b, 2, i) == -a(b0, 2, 2 - i)
        assert a(b, 3, i) == a(b0, 3, 1 - i)
    assert a(b, 2, 1) == 0 and a(b, 2, n + 1) == 0
    assert a(b, 1, n + 2) == a(b0, 1, n - 1) and a(b, 2, n + 2) == -a(b0, 2, n)
    g = _grid(oracle, 2)                         # quadratic: even
    b0 = _rand(g, 7)
    b = _apply(oracle, g, b0, 1, 1)
    n = NX[0]
    a = lambda f, c, i: _at(g, f, c, i, 5)
    for i in (0, -1):
        assert a(b, 1, i) == -a(b0, 1, 1 - i) and a(b, 2, i) == a(b0, 2, -i)
    assert a(b, 1, n + 1) == -a(b0, 1, n) and a(b, 3, n + 2) == a(b0, 3, n - 2)


def test_walled_step_keeps_particles_and_energy(oracle):
    """A thermal plasma between conducting walls along x1 (periodic x2), FP64: every particle
    stays inside, charges are kept, and the total energy drifts by less than 1% in 200 steps."""
    g = oracle.Grid([24, 16], 2, [0.1, 0.1])
    ix, x, u, q = oracle.load(oracle.mt_new(9), "f64", 2, [24, 16], [2, 2], [0.1, 0.1], -1.0,
                              [0.1] * 3, [0.0] * 3)
    sp = [dict(ix=ix, x=x, u=u, q=q, rqm=-1.0)]
    e, b, j = g.zeros("f64"), g.zeros("f64"), g.zeros("f64")
    dt = 0.05

    def energy(ene):
        fe = sum(oracle.field_energy(g, "f64", f).sum() for f in (e, b))
        return fe + (-1.0) * 0.01 * ene[0]

    w = []
    for _ in range(200):
        ene = oracle.step(g, "f64", e, b, j, sp, dt, walls=1)
        w.append(energy(ene))
    assert ix[:, 0].min() >= 1 and ix[:, 0].max() <= 24
    assert np.all(np.abs(x) <= 0.5)
    w = np.array(w)
    assert np.abs(w / w[0] - 1).max() < 1e-2
