"""GPU parity of the exact pusher (push_type = "exact", dudt_exact) against the CPU oracle:
the drop-in entry point osg_advance_deposit_exact_* and the device-resident plain engine.

Tolerances (normwise max|a-b|/max|b|): FP64 particles and current 1e-12 (the device's and the
host's tan/tanh may differ in the last bit, and the current sums are atomic); FP32 momenta and
positions 1e-5, current 1e-5.  The exact pusher's momenta differ from Boris's by O(dt^3), far
above these tolerances, so the comparison pins the pusher, not only the deposit.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
TOL = {"f32": 1e-5, "f64": 1e-12}


@pytest.fixture(scope="module")
def osg():
    import __graft_entry__ as g
    g.build_native()
    import osiris_gb300
    if osiris_gb300.lib().osg_device_count() < 1:
        pytest.fail("no CUDA device visible")
    return osiris_gb300


def _nerr(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def _pos(ix, x):
    return ix.astype(np.float64) + x.astype(np.float64)


@pytest.mark.parametrize("prec", ["f32", "f64"])
@pytest.mark.parametrize("dim,order", [(1, 2), (2, 1), (2, 2), (2, 3), (3, 2), (3, 3)])
def test_gpu_exact_dropin_matches_oracle(osg, oracle, prec, dim, order):
    nx = [12, 10, 8][:dim]
    dx = [0.1, 0.12, 0.15][:dim]
    g = oracle.Grid(nx, order, dx)
    rng = np.random.default_rng(dim * 10 + order + 3)
    dt_ = np.float32 if prec == "f32" else np.float64
    r = oracle.mt_new(13)
    ix, x, u, q = oracle.load(r, prec, dim, nx, [2] * dim, dx, -1.0, [0.6] * 3, [0.2, 0.0, 0.0])
    e = (rng.standard_normal(g.shape) * 0.6).astype(dt_)
    b = (rng.standard_normal(g.shape) * 0.6).astype(dt_)
    dt = 0.04
    a = [v.copy() for v in (ix, x, u, q)]
    j_g = g.zeros(prec)
    ene_g = osg.vadvance_deposit(dim, order, *a, 1, len(q), -1.0, e, b, g.size, g.gcl, j_g,
                                 g.size, g.gcl, dx, dt, pusher=osg.PUSHER_EXACT)
    o = [v.copy() for v in (ix, x, u, q)]
    j_o = g.zeros(prec)
    ene_o = oracle.push(prec, dim, order, *o, 1, len(q), -1.0, e, b, j_o, g.size, g.gcl, dx, dt,
                        pusher="exact")
    assert _nerr(a[2], o[2]) <= TOL[prec]
    assert _nerr(_pos(a[0], a[1]), _pos(o[0], o[1])) <= TOL[prec]
    assert _nerr(j_g, j_o) <= TOL[prec]
    assert abs(ene_g - ene_o) <= 10 * TOL[prec] * abs(ene_o)
    # the exact update is not the Boris one
    ub = [v.copy() for v in (ix, x, u, q)]
    oracle.push(prec, dim, order, *ub, 1, len(q), -1.0, e, b, g.zeros(prec), g.size, g.gcl, dx,
                dt)
    assert _nerr(a[2], ub[2]) > (1e-10 if prec == "f64" else 1e-7)


@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_gpu_exact_sim_step_matches_oracle(osg, oracle, prec):
    """Two full device-resident steps (plain engine) with the exact pusher against the oracle's
    time step with the same pusher."""
    nx, dx, dt, order = [16, 12], [0.1, 0.1], 0.05, 2
    rng = np.random.default_rng(21)
    r = osg.Rng(5)
    p = 32 if prec == "f32" else 64
    sp = [osg.load_lattice(r, p, nx, [2, 2], dx, -1.0, [0.3] * 3, [0.2, 0.0, 0.0])]
    sim = osg.Simulation(nx, dx, dt, order=order, precision=p, engine=osg.ENGINE_PLAIN,
                         pusher=osg.PUSHER_EXACT)
    g = oracle.Grid(nx, order, dx)
    e = (rng.standard_normal(g.shape) * 0.3).astype(g.zeros(prec).dtype)
    b = (rng.standard_normal(g.shape) * 0.3).astype(e.dtype)
    sim.set_fields(e, b)
    for s in sp:
        sim.add_species(-1.0, *s)
    sim.step(2)
    e_g, b_g, _ = sim.fields()
    kin, _ = sim.energy()
    ora = [dict(ix=s[0].copy(), x=s[1].copy(), u=s[2].copy(), q=s[3].copy(), rqm=-1.0)
           for s in sp]
    e_o, b_o, j_o = e.copy(), b.copy(), g.zeros(prec)
    for _ in range(2):
        ene = oracle.step(g, prec, e_o, b_o, j_o, ora, dt, pusher="exact")
    tol = 1e-12 if prec == "f64" else 5e-5
    for a, o in ((e_g, e_o), (b_g, b_o)):
        assert _nerr(g.interior(a), g.interior(o)) <= tol
    ix, x, u, q = sim.species(0)      # the plain engine keeps the particle order
    assert _nerr(u, ora[0]["u"]) <= tol
    assert _nerr(_pos(ix, x), _pos(ora[0]["ix"], ora[0]["x"])) <= tol
    cell_dv = dx[0] * dx[1]
    assert abs(kin[0] - (-1.0) * cell_dv * ene[0]) <= 1e3 * tol * abs(kin[0])
    sim.close()
