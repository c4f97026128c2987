"""The product's seeded lattice loader (host C++ in the native library) reproduces the
oracle's restatement of the OSIRIS load bit for bit, for both precisions, and shares one
generator across species like the reference."""
import numpy as np
import pytest


@pytest.fixture(scope="module")
def osg():
    import __graft_entry__ as g
    g.build_native()
    import osiris_gb300
    return osiris_gb300


@pytest.mark.parametrize("prec", [32, 64])
@pytest.mark.parametrize("dim", [2, 3])
def test_loader_matches_oracle(osg, oracle, prec, dim):
    nx = [6, 5, 4][:dim]
    ppc = [2, 3, 1][:dim]
    dx = [0.05, 0.07, 0.1][:dim]
    p = "f32" if prec == 32 else "f64"
    r_o = oracle.mt_new(5)
    r_p = osg.Rng(5)
    for rqm, uth, ufl, amp in ((-1.0, [0.1, 0.2, 0.3], [0.2, 0.0, -0.1], 1e-3),
                               (-1.0, [0.01] * 3, [-0.2, 0.0, 0.0], 0.0)):
        a = oracle.load(r_o, p, dim, nx, ppc, dx, rqm, uth, ufl, amp, 1.0)
        b = osg.load_lattice(r_p, prec, nx, ppc, dx, rqm, uth, ufl, amp, 1.0)
        for x, y in zip(a, b):
            assert x.dtype == y.dtype
            assert np.array_equal(x, y)


def test_loader_statistics(osg):
    r = osg.Rng(1)
    ix, x, u, q = osg.load_lattice(r, 64, [32, 32], [4, 4], [0.05, 0.05], -1.0, [0.1] * 3,
                                   [0.0] * 3)
    assert ix.min() == 1 and ix[:, 0].max() == 32
    assert abs(u.std() - 0.1) < 0.003
    assert np.allclose(q, -1.0 / 16)
    assert (x >= -0.5).all() and (x < 0.5).all()
