"""Known-answer tests of the oracle's exact momentum update (push_type = "exact", dudt_exact,
source/spec/os-spec-extpush.f03:40-348).  The reference is Fortran and cannot be run here, so
the restatement is pinned against analytic orbits (uniform B gyration, uniform E acceleration)
and against a fine fourth-order Runge-Kutta integration of the Lorentz force for general,
light-like and weak fields."""
import numpy as np
import pytest


def _rk4(e, b, u, qm, dt, n=4000):
    """du/dt = qm (E + u x B / gamma), fixed fields, n RK4 steps (FP64 reference orbit)."""
    u = u.astype(np.float64).copy()
    e = e.astype(np.float64) * qm
    b = b.astype(np.float64) * qm
    h = dt / n

    def f(v):
        g = np.sqrt(1.0 + (v * v).sum(-1, keepdims=True))
        return e + np.cross(v / g, b)

    for _ in range(n):
        k1 = f(u)
        k2 = f(u + 0.5 * h * k1)
        k3 = f(u + 0.5 * h * k2)
        k4 = f(u + h * k3)
        u = u + (h / 6.0) * (k1 + 2 * k2 + 2 * k3 + k4)
    return u


def _run(oracle, prec, e, b, u, rqm, dt, tol):
    dt_ = np.float32 if prec == "f32" else np.float64
    uu = np.array(u, dtype=dt_, copy=True)
    q = np.full(len(u), -1.0, dtype=dt_)
    ene = oracle.dudt_exact(prec, np.ascontiguousarray(e, dtype=dt_),
                            np.ascontiguousarray(b, dtype=dt_), uu, q, rqm, dt, tol)
    return uu.astype(np.float64), ene


def test_uniform_b_gyration(oracle):
    """Pure B along z: |u| is kept and (u1, u2) turns by qm B0 dt / gamma exactly."""
    u0 = np.array([[0.5, 0.0, 0.3], [0.1, -0.7, 0.0], [2.0, 1.0, -1.0]])
    b0, rqm, dt = 0.8, -1.0, 0.3
    e = np.zeros_like(u0)
    b = np.tile([0.0, 0.0, b0], (3, 1))
    u, _ = _run(oracle, "f64", e, b, u0, rqm, dt, 1e-3)
    g = np.sqrt(1 + (u0 ** 2).sum(1))
    th = (1.0 / rqm) * b0 * dt / g
    ref = np.stack([u0[:, 0] * np.cos(th) + u0[:, 1] * np.sin(th),
                    -u0[:, 0] * np.sin(th) + u0[:, 1] * np.cos(th), u0[:, 2]], 1)
    assert np.abs(u - ref).max() < 1e-13


def test_uniform_e_from_rest(oracle):
    """Pure E from rest: u = (q/m) E dt exactly (hyperbolic motion, Newton to 1e-12)."""
    e = np.array([[0.7, 0.0, 0.0], [0.0, -2.0, 0.5]])
    rqm, dt = -1.0, 0.4
    u, ene = _run(oracle, "f64", e, np.zeros_like(e), np.zeros_like(e), rqm, dt, 1e-12)
    ref = (1.0 / rqm) * e * dt
    assert np.abs(u - ref).max() < 1e-12
    g = np.sqrt(1 + (ref ** 2).sum(1))
    assert abs(ene - (-1.0) * (g - 1).sum()) < 1e-12


@pytest.mark.parametrize("tol,bound", [(1e-12, 1e-10), (1e-6, 1e-7), (1e-3, 2e-4)])
def test_general_field_against_rk4(oracle, tol, bound):
    rng = np.random.default_rng(5)
    n = 16
    e = rng.standard_normal((n, 3)) * 0.8
    b = rng.standard_normal((n, 3)) * 1.2
    u0 = rng.standard_normal((n, 3)) * 0.9
    rqm, dt = -1.0, 0.25
    u, _ = _run(oracle, "f64", e, b, u0, rqm, dt, tol)
    ref = _rk4(e, b, u0, 1.0 / rqm, dt)
    assert np.abs(u - ref).max() / np.abs(ref).max() < bound


def test_light_like_crossed_field_against_rk4(oracle):
    """|E| = |B|, E perpendicular to B: both invariants vanish (the get_t_light branch)."""
    e = np.array([[0.0, 0.6, 0.0], [0.0, 0.0, -1.1]])
    b = np.array([[0.0, 0.0, 0.6], [0.0, 1.1, 0.0]])
    u0 = np.array([[0.3, -0.2, 0.1], [0.0, 0.5, 0.4]])
    rqm, dt = -1.0, 0.2
    u, _ = _run(oracle, "f64", e, b, u0, rqm, dt, 1e-12)
    ref = _rk4(e, b, u0, 1.0 / rqm, dt)
    assert np.abs(u - ref).max() / np.abs(ref).max() < 1e-10


def test_weak_field_leaves_momentum(oracle):
    e = np.full((2, 3), 1e-7)
    b = np.full((2, 3), -2e-7)
    u0 = np.array([[0.4, 0.1, -0.2], [0.0, 0.0, 0.0]])
    u, _ = _run(oracle, "f64", e, b, u0, -1.0, 0.5, 1e-3)
    assert np.array_equal(u, u0)


def test_single_precision_tracks_double(oracle):
    rng = np.random.default_rng(8)
    n = 64
    e = rng.standard_normal((n, 3)) * 0.3
    b = rng.standard_normal((n, 3)) * 0.5
    u0 = rng.standard_normal((n, 3)) * 0.4
    u32, _ = _run(oracle, "f32", e.astype(np.float32), b.astype(np.float32),
                  u0.astype(np.float32), -1.0, 0.05, 1e-3)
    u64, _ = _run(oracle, "f64", e.astype(np.float32).astype(np.float64),
                  b.astype(np.float32).astype(np.float64),
                  u0.astype(np.float32).astype(np.float64), -1.0, 0.05, 1e-3)
    assert np.abs(u32 - u64).max() / np.abs(u64).max() < 2e-6


@pytest.mark.parametrize("dim,order", [(2, 2), (3, 3)])
def test_exact_push_conserves_charge(oracle, dim, order):
    """The exact pusher changes only the momentum update: the split deposit still satisfies
    (rho(t+dt) - rho(t))/dt + div J = 0 to roundoff."""
    nx = [8, 7, 6][:dim]
    g = oracle.Grid(nx, order, [0.1] * dim)
    rng0 = oracle.mt_new(3)
    ix, x, u, q = oracle.load(rng0, "f64", dim, nx, [2] * dim, [0.1] * dim, -1.0, [0.8] * 3,
                              [0.0] * 3)
    rng = np.random.default_rng(1)
    e = rng.standard_normal(g.shape) * 0.5
    b = rng.standard_normal(g.shape) * 0.5
    oracle.periodic(g, "f64", e, 0)
    oracle.periodic(g, "f64", b, 0)
    dt = 0.05
    rho0 = oracle.deposit_rho(g, "f64", ix, x, q)
    oracle.periodic(g, "f64", rho0, 1)
    j = g.zeros("f64")
    u_before = u.copy()
    oracle.push("f64", dim, order, ix, x, u, q, 1, len(q), -1.0, e, b, j, g.size, g.gcl,
                g.dx, dt, pusher="exact")
    assert not np.array_equal(u, u_before)
    oracle.wrap(g, ix)
    oracle.periodic(g, "f64", j, 1)
    rho1 = oracle.deposit_rho(g, "f64", ix, x, q)
    oracle.periodic(g, "f64", rho1, 1)
    drho = (g.interior(rho1)[..., 0] - g.interior(rho0)[..., 0]) / dt
    divj = oracle.div(g, "f64", j)
    assert np.abs(drho + divj).max() / np.abs(drho).max() < 1e-12


def test_exact_and_boris_agree_for_small_steps(oracle):
    """Both pushers are second-order accurate: for a small step their momenta agree to
    O(dt^3) in the same interpolated fields."""
    dim, order = 2, 2
    nx = [8, 8]
    g = oracle.Grid(nx, order, [0.1] * dim)
    rng0 = oracle.mt_new(4)
    ix, x, u, q = oracle.load(rng0, "f64", dim, nx, [2, 2], [0.1] * dim, -1.0, [0.3] * 3,
                              [0.0] * 3)
    rng = np.random.default_rng(2)
    e = rng.standard_normal(g.shape) * 0.2
    b = rng.standard_normal(g.shape) * 0.2
    oracle.periodic(g, "f64", e, 0)
    oracle.periodic(g, "f64", b, 0)
    dt = 1e-3
    u_init = u.copy()
    st = [a.copy() for a in (ix, x, u)]
    oracle.push("f64", dim, order, ix, x, u, q, 1, len(q), -1.0, e, b, g.zeros("f64"), g.size,
                g.gcl, g.dx, dt, pusher="exact", iter_tol=1e-12)
    ix2, x2, u2 = st
    oracle.push("f64", dim, order, ix2, x2, u2, q, 1, len(q), -1.0, e, b, g.zeros("f64"),
                g.size, g.gcl, g.dx, dt)
    du = np.abs(u - u_init).max()
    assert np.abs(u - u2).max() < 1e-7
    assert du > 1e-5
