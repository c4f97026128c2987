"""Known-answer tests of the current smoothing (source/vdf/os-vdf-smooth.f90): the filter
coefficients of every type (the oracle's restatement and the library's host function, which
keeps them in FP64), and the oracle's filter against the analytic transfer function of the
binomial filter."""
import numpy as np
import pytest
from math import comb


@pytest.fixture(scope="module")
def osg():
    import __graft_entry__ as g
    g.build_native()
    import osiris_gb300
    return osiris_gb300


@pytest.mark.parametrize("n", [1, 2, 3, 5])
def test_binomial_coefficients(oracle, n):
    m, c = oracle.smooth_coefficients(2, n)
    assert m == n
    want = [comb(2 * n, k) / 4.0 ** n for k in range(2 * n + 1)]
    assert np.allclose(c, want, rtol=0, atol=1e-16)


def test_compensated_and_fixed_kernels(oracle):
    _, c = oracle.smooth_coefficients(3, 2)
    assert np.allclose(c, np.array([-1, 4, 10, 4, -1]) / 16.0, rtol=0, atol=1e-16)
    for t, n in ((3, 3), (4, 5), (5, 3), (6, 4)):
        m, c = oracle.smooth_coefficients(t, n)
        assert len(c) == 2 * m + 1
        assert abs(sum(c) - 1.0) < 1e-15
        assert np.allclose(c, c[::-1], rtol=0, atol=1e-16)       # symmetric


@pytest.mark.parametrize("t,n", [(2, 1), (2, 3), (3, 2), (3, 4), (4, 5), (5, 3), (6, 4)])
def test_library_coefficients_match_oracle(osg, oracle, t, n):
    m, c = osg.smooth_coefficients(t, n)
    mo, co = oracle.smooth_coefficients(t, n)
    assert m == mo and np.array_equal(c, np.array(co))


@pytest.mark.parametrize("n", [1, 2])
def test_binomial_transfer_function(oracle, n):
    """A mode sin(k x1) comes out multiplied by cos^(2n)(k dx / 2) at every filtered point."""
    nx = [32, 8]
    g = oracle.Grid(nx, 2, [0.1, 0.1], guard=(n + 2, n + 3))
    f = g.zeros("f64")
    kdx = 2 * np.pi * 3 / nx[0]
    i1 = np.arange(g.size[0]) - g.gcl[0] + 1
    f[..., 0] = np.sin(kdx * i1)[None, :]
    ref = f.copy()
    oracle.smooth(g, "f64", f, [2, 0], [n, 0])
    inner = slice(n, g.size[0] - n)
    gain = np.cos(kdx / 2) ** (2 * n)
    assert np.abs(f[:, inner, 0] - gain * ref[:, inner, 0]).max() < 1e-14
    assert np.array_equal(f[:, :n, 0], ref[:, :n, 0])      # points near the ends are kept
