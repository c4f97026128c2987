"""The host side of the PML walls in the library (osg_pml_state_size, osg_pml_init_*: no device
work) against the oracle's: the state has the same size for every axis mask in 2D and 3D, the
walls start at zero, and the attenuation tables of every axis (setup_att_coeff,
source/emf/boundary/os-emf-vpml.f03:3586-3684, computed in double and stored in the field
precision) are the oracle's bit for bit; bad arguments are refused."""
import numpy as np
import pytest


@pytest.fixture(scope="module")
def osg():
    import __graft_entry__ as g
    g.build_native()
    import osiris_gb300
    return osiris_gb300


@pytest.mark.parametrize("dim,mask", [(2, 1), (2, 2), (2, 3), (3, 1), (3, 2), (3, 4), (3, 3),
                                      (3, 5), (3, 6), (3, 7)])
@pytest.mark.parametrize("order", [1, 2, 4])
@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_pml_state_matches_oracle(osg, oracle, dim, mask, order, prec):
    nx = [12, 10, 9][:dim]
    dx = [0.1, 0.12, 0.09][:dim]
    nb, dt = 7, 0.03
    g = oracle.Grid(nx, order, dx)
    ref = oracle.pml_state(g, prec, mask, nb, dt)
    nx_, gl, gu = g.args()
    got = osg.pml_state(dim, nx, gl, gu, mask, nb, dx, dt, ref.dtype)
    assert got.shape == ref.shape and got.dtype == ref.dtype
    assert np.array_equal(got, ref)
    ntab = 12 * dim * nb
    assert not got[:len(got) - ntab].any()
    assert (got[len(got) - ntab:] != 0).all()


@pytest.mark.parametrize("dim,mask,nb", [(2, 0, 8), (2, 4, 8), (3, 8, 8), (2, 1, 4), (1, 1, 8)])
def test_pml_state_refuses_bad_arguments(osg, dim, mask, nb):
    nx, gl, gu = [12] * max(dim, 1), [2] * max(dim, 1), [3] * max(dim, 1)
    with pytest.raises(osg.OsirisGB300Error):
        osg.pml_state(dim, nx, gl, gu, mask, nb, [0.1] * 3, 0.03, np.float64)


def test_pml_phase_refuses_a_short_state(osg):
    nx, gl, gu = [12, 10], [2, 2], [3, 3]
    st = osg.pml_state(2, nx, gl, gu, 1, 8, [0.1, 0.1], 0.03, np.float64)
    shape = (10 + 5, 12 + 5, 3)
    e, b = np.zeros(shape), np.zeros(shape)
    with pytest.raises(ValueError):
        osg.pml(2, nx, gl, gu, 1, 8, 1, e, b, st[:-1].copy(), [0.1, 0.1], 0.03)
