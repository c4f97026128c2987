"""Oracle tests of the thermal-bath particle boundary (p_bc_thermal,
source/spec/os-spec-boundary.f03:1315-1387; thermal_bath :972-1067, thermal_type "thermal").

Particles driven through a wall within one step are re-emitted at the edge cell: offset
between the edge and where they got to in the rest of the step, the normal momentum pointing
into the box with the half-Maxwellian distribution (mean uth sqrt(pi/2)), the other components
Gaussian with spread uth, and the fluid momentum added when all three of its components are
non-zero; the same counter gives the same particles, another step other ones."""
import numpy as np
import pytest


def _crossers(oracle, prec, n_side=32, u_in=-3.0, axis=0):
    nx = [8, n_side]
    g = oracle.Grid(nx, 2, [0.1, 0.1])
    n = n_side * 64
    dt_ = np.float32 if prec == "f32" else np.float64
    rng = np.random.default_rng(2)
    ix = np.ones((n, 2), np.int32)
    ix[:, 1] = rng.integers(1, n_side + 1, n)
    x = np.zeros((n, 2), dt_)
    x[:, 0] = -0.45
    x[:, 1] = rng.uniform(-0.5, 0.5, n)
    u = np.zeros((n, 3), dt_)
    u[:, 0] = u_in
    q = np.full(n, -0.01, dt_)
    if axis == 1:
        ix, x, u = ix[:, ::-1].copy(), x[:, ::-1].copy(), u[:, [1, 0, 2]].copy()
        nx = nx[::-1]
        g = oracle.Grid(nx, 2, [0.1, 0.1])
    return g, dict(ix=ix, x=x, u=u, q=q, rqm=-1.0)


def _step(oracle, g, prec, sp, dt, step, uth, ufl=(0.0, 0.0, 0.0), seed=5, mask=1):
    e, b, j = g.zeros(prec), g.zeros(prec), g.zeros(prec)
    oracle.step(g, prec, e, b, j, [sp], dt, walls=mask,
                thermal=dict(mask=mask, uth=uth, ufl=ufl, seed=seed, step=step))
    return j


@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_reemitted_particles_follow_the_bath(oracle, prec):
    g, sp = _crossers(oracle, prec)
    uth = [0.2, 0.3, 0.1]
    dt = 0.05
    _step(oracle, g, prec, sp, dt, 0, uth)
    u = sp["u"].astype(np.float64)
    assert np.all(sp["ix"][:, 0] == 1)
    assert np.all(u[:, 0] > 0)
    gam = np.sqrt(1 + (u ** 2).sum(1))
    vperp = u[:, 0] / gam * dt / 0.1
    x0 = sp["x"][:, 0].astype(np.float64)
    assert np.all(x0 >= -0.5 - 1e-7) and np.all(x0 <= -0.5 + vperp + 1e-7)
    n = len(u)
    assert abs(u[:, 0].mean() / (uth[0] * np.sqrt(np.pi / 2)) - 1) < 4 / np.sqrt(n)
    for c in (1, 2):
        assert abs(u[:, c].mean()) < 4 * uth[c] / np.sqrt(n)
        assert abs(u[:, c].std() / uth[c] - 1) < 5 / np.sqrt(n)


def test_upper_wall_and_axis_2(oracle):
    g, sp = _crossers(oracle, "f64", u_in=3.0, axis=1)
    sp["ix"][:, 1] = g.nx[1]
    sp["x"][:, 1] = 0.45
    _step(oracle, g, "f64", sp, 0.05, 3, [0.2, 0.2, 0.2], mask=2)
    assert np.all(sp["ix"][:, 1] == g.nx[1])
    assert np.all(sp["u"][:, 1] < 0)
    assert np.all(sp["x"][:, 1] < 0.5) and np.all(sp["x"][:, 1] > 0.0)


def test_fluid_momentum_only_with_all_three_components(oracle):
    out = []
    for ufl in ([0.5, 0.0, 0.0], [0.5, 0.1, 0.1]):
        g, sp = _crossers(oracle, "f64")
        _step(oracle, g, "f64", sp, 0.05, 0, [0.2, 0.2, 0.2], ufl=ufl)
        out.append(sp["u"].copy())
    g, sp = _crossers(oracle, "f64")
    _step(oracle, g, "f64", sp, 0.05, 0, [0.2, 0.2, 0.2])
    assert np.array_equal(out[0], sp["u"])          # one zero component: no fluid momentum
    assert abs(out[1][:, 1].mean() - sp["u"][:, 1].mean() - 0.1) < 0.02


def test_stream_is_keyed_by_counter(oracle):
    res = []
    for step, seed in ((0, 5), (0, 5), (1, 5), (0, 6)):
        g, sp = _crossers(oracle, "f64")
        j = _step(oracle, g, "f64", sp, 0.05, step, [0.2, 0.2, 0.2], seed=seed)
        res.append((sp["u"].copy(), j))
    assert np.array_equal(res[0][0], res[1][0]) and np.array_equal(res[0][1], res[1][1])
    assert not np.any(res[0][0] == res[2][0])
    assert not np.any(res[0][0] == res[3][0])


def test_waterbag_and_random_dir(oracle):
    uth = [0.4, 0.3, 0.2]
    g, sp = _crossers(oracle, "f64")
    e, b, j = g.zeros("f64"), g.zeros("f64"), g.zeros("f64")
    oracle.step(g, "f64", e, b, j, [sp], 0.05, walls=1,
                thermal=dict(mask=1, uth=uth, seed=1, step=0, type=2))
    u = sp["u"]
    assert np.all(u[:, 0] >= 0)
    for c in range(3):
        assert np.abs(u[:, c]).max() <= uth[c] / 2 + 1e-12
        assert np.abs(u[:, c]).max() > 0.45 * uth[c]
    g, sp = _crossers(oracle, "f64")
    oracle.step(g, "f64", e, b, j, [sp], 0.05, walls=1,
                thermal=dict(mask=1, uth=uth, seed=1, step=0, type=1))
    u = sp["u"]
    ut = np.sqrt(sum(v * v for v in uth))
    upar = u[:, 2] / ut
    assert np.all(upar >= -1) and np.all(upar <= 1) and np.all(u[:, 0] >= 0)
    # the reference's perpendicular radius sqrt(1 - upar) |uth|
    assert np.allclose(np.hypot(u[:, 0], u[:, 1]), np.sqrt(1 - upar) * ut, rtol=1e-12)
