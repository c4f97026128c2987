"""Known-answer tests of the oracle's Vay, Higuera-Cary, full-rotation and Euler-rotation
momentum updates (dudt_vay, source/spec/os-spec-push.f03:636-796; dudt_cary, :1104-1253;
dudt_fullrot, :83-231; dudt_euler, :235-352; dudt_cond_vay, :800-1100), restated from Fortran
that cannot be run here:
all keep |u| in a pure magnetic field; Vay and Higuera-Cary keep a particle at the E x B drift
velocity exactly for any step (their defining property); the two rotation pushers turn the
momentum by the exact gyration angle in a uniform magnetic field (Boris does not); all agree
with the exact pusher to O(dt^3) per step; the step-level push with them conserves charge; the
conditional Vay pusher is the Vay update above gamma 5 and the Fortran Boris loops below."""
import numpy as np
import pytest


def _run(oracle, pusher, e, b, u0, dt, steps=1, prec="f64"):
    dt_ = np.float32 if prec == "f32" else np.float64
    u = np.array(u0, dtype=dt_, copy=True)
    q = np.full(len(u), -1.0, dtype=dt_)
    e = np.ascontiguousarray(e, dtype=dt_)
    b = np.ascontiguousarray(b, dtype=dt_)
    for _ in range(steps):
        oracle.dudt(pusher, prec, e, b, u, q, -1.0, dt, 1e-12)
    return u.astype(np.float64)


@pytest.mark.parametrize("pusher", ["vay", "hc", "fullrot", "euler", "cond_vay"])
def test_pure_b_keeps_energy(oracle, pusher):
    rng = np.random.default_rng(1)
    u0 = rng.standard_normal((8, 3))
    b = rng.standard_normal((8, 3))
    u = _run(oracle, pusher, np.zeros_like(b), b, u0, 0.7, steps=50)
    assert np.abs((u ** 2).sum(1) / (u0 ** 2).sum(1) - 1).max() < 1e-13


@pytest.mark.parametrize("pusher", ["vay", "hc"])
def test_exb_drift_is_kept(oracle, pusher):
    e0, b0 = 0.6, 1.0                         # |E| < |B|: drift at v = E/B along x
    v = e0 / b0
    g = 1.0 / np.sqrt(1 - v * v)
    u0 = np.array([[g * v, 0.0, 0.0]])
    e = np.array([[0.0, e0, 0.0]])
    b = np.array([[0.0, 0.0, b0]])
    u = _run(oracle, pusher, e, b, u0, 0.9, steps=100)
    assert np.abs(u - u0).max() < 1e-12


@pytest.mark.parametrize("pusher", ["fullrot", "euler"])
def test_rotation_pushers_gyrate_by_the_exact_angle(oracle, pusher):
    # u perpendicular to a uniform B along z: per step the exact gyration angle is
    # |B| dt / (rqm gamma) (rqm = -1), which Boris only approximates (2 atan of half of it)
    b0, dt, n = 1.3, 0.4, 25
    u0 = np.array([[0.7, -0.2, 0.0]])
    g = np.sqrt(1.0 + (u0 ** 2).sum())
    b = np.array([[0.0, 0.0, b0]])
    u = _run(oracle, pusher, np.zeros_like(b), b, u0, dt, steps=n)
    th = n * (-(b0 * dt) / g)            # rotation u -> R(th) u  (u x B force for rqm = -1)
    want = np.array([[u0[0, 0] * np.cos(th) + u0[0, 1] * np.sin(th),
                      -u0[0, 0] * np.sin(th) + u0[0, 1] * np.cos(th), 0.0]])
    assert np.abs(u - want).max() < 1e-12
    # and not by the Boris angle 2 atan(theta / 2)
    tb = n * (-2.0 * np.arctan(0.5 * b0 * dt / g))
    boris = np.array([[u0[0, 0] * np.cos(tb) + u0[0, 1] * np.sin(tb),
                       -u0[0, 0] * np.sin(tb) + u0[0, 1] * np.cos(tb), 0.0]])
    assert np.abs(u - boris).max() > 1e-3


@pytest.mark.parametrize("pusher", ["vay", "hc", "fullrot", "euler", "cond_vay"])
def test_second_order_against_exact(oracle, pusher):
    rng = np.random.default_rng(4)
    e = rng.standard_normal((6, 3)) * 0.5
    b = rng.standard_normal((6, 3)) * 0.5
    u0 = rng.standard_normal((6, 3)) * 0.5
    errs = []
    for dt in (0.02, 0.01):
        ue = _run(oracle, "exact", e, b, u0, dt)
        up = _run(oracle, pusher, e, b, u0, dt)
        errs.append(np.abs(up - ue).max())
    assert errs[1] < errs[0] / 6        # local error O(dt^3)
    assert errs[0] < 1e-4


@pytest.mark.parametrize("pusher", ["vay", "hc", "fullrot", "euler", "cond_vay"])
def test_push_with_pusher_conserves_charge(oracle, pusher):
    dim, order, nx = 2, 2, [8, 7]
    g = oracle.Grid(nx, order, [0.1] * dim)
    ix, x, u, q = oracle.load(oracle.mt_new(3), "f64", dim, nx, [2] * dim, [0.1] * dim, -1.0,
                              [0.8] * 3, [0.0] * 3)
    rng = np.random.default_rng(1)
    e = rng.standard_normal(g.shape) * 0.5
    b = rng.standard_normal(g.shape) * 0.5
    oracle.periodic(g, "f64", e, 0)
    oracle.periodic(g, "f64", b, 0)
    dt = 0.05
    rho0 = oracle.deposit_rho(g, "f64", ix, x, q)
    oracle.periodic(g, "f64", rho0, 1)
    j = g.zeros("f64")
    oracle.push("f64", dim, order, ix, x, u, q, 1, len(q), -1.0, e, b, j, g.size, g.gcl,
                g.dx, dt, pusher=pusher)
    oracle.wrap(g, ix)
    oracle.periodic(g, "f64", j, 1)
    rho1 = oracle.deposit_rho(g, "f64", ix, x, q)
    oracle.periodic(g, "f64", rho1, 1)
    drho = (g.interior(rho1)[..., 0] - g.interior(rho0)[..., 0]) / dt
    assert np.abs(drho + oracle.div(g, "f64", j)).max() / np.abs(drho).max() < 1e-12


def _fortran_boris(e, b, u, q, tem):
    """The Boris loops of dudt_cond_vay (source/spec/os-spec-push.f03:1011-1094) in FP64, term
    by term as the Fortran evaluates them."""
    ep = e * tem
    ut = u + ep
    u2 = (ut[:, 0] ** 2 + ut[:, 1] ** 2) + ut[:, 2] ** 2
    gam = np.sqrt(u2 + 1)
    ene = (q * u2 / (gam + 1.0)).sum()
    bp = b * (tem / gam)[:, None]
    pn = np.empty_like(ut)
    pn[:, 0] = ut[:, 0] + ut[:, 1] * bp[:, 2]
    pn[:, 1] = ut[:, 1] + ut[:, 2] * bp[:, 0]
    pn[:, 2] = ut[:, 2] + ut[:, 0] * bp[:, 1]
    pn[:, 0] = pn[:, 0] - ut[:, 2] * bp[:, 1]
    pn[:, 1] = pn[:, 1] - ut[:, 0] * bp[:, 2]
    pn[:, 2] = pn[:, 2] - ut[:, 1] * bp[:, 0]
    otsq = 2.0 / (((1.0 + bp[:, 0] ** 2) + bp[:, 1] ** 2) + bp[:, 2] ** 2)
    bp = bp * otsq[:, None]
    ut[:, 0] = ut[:, 0] + pn[:, 1] * bp[:, 2]
    ut[:, 1] = ut[:, 1] + pn[:, 2] * bp[:, 0]
    ut[:, 2] = ut[:, 2] + pn[:, 0] * bp[:, 1]
    ut[:, 0] = ut[:, 0] - pn[:, 2] * bp[:, 1]
    ut[:, 1] = ut[:, 1] - pn[:, 0] * bp[:, 2]
    ut[:, 2] = ut[:, 2] - pn[:, 1] * bp[:, 0]
    return ut + ep, ene


def test_cond_vay_switches_at_gamma_5(oracle):
    rng = np.random.default_rng(8)
    n = 64
    u0 = rng.standard_normal((n, 3)) * 3.0
    e = rng.standard_normal((n, 3)) * 0.5
    b = rng.standard_normal((n, 3)) * 0.5
    dt = 0.3
    g0 = np.sqrt(((1.0 + u0[:, 0] ** 2) + u0[:, 1] ** 2) + u0[:, 2] ** 2)
    hot = g0 > 5
    assert 0 < hot.sum() < n
    uc = _run(oracle, "cond_vay", e, b, u0, dt)
    uv = _run(oracle, "vay", e, b, u0, dt)
    assert np.array_equal(uc[hot], uv[hot])
    tem = 0.5 * dt / -1.0
    ub, _ = _fortran_boris(e[~hot], b[~hot], u0[~hot].copy(), -np.ones((~hot).sum()), tem)
    assert np.array_equal(uc[~hot], ub)
    assert np.abs(uc[~hot] - uv[~hot]).max() > 1e-6
