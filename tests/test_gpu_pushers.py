"""GPU parity of the Vay, Higuera-Cary, full-rotation and Euler-rotation momentum updates
(push_type "vay", "cary", "fullrot", "euler", "cond_vay"; dudt_vay / dudt_cary / dudt_fullrot /
dudt_euler / dudt_cond_vay)
against the CPU oracle, through the drop-in entry point osg_advance_deposit_* and through both
engines of the device-resident time step.

Tolerances (normwise max|a-b|/max|b|) as for the Boris path: FP64 1e-12, FP32 1e-5 for one
call or step, 5e-5 over 10 steps.  The drop-in cases use fields of rms 5 and momenta of rms 2,
where each update differs from Boris's by more than the FP32 tolerance, so the comparison pins
the pusher and not only the deposit.
"""
import numpy as np
import pytest

from test_gpu_step import _compare

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


@pytest.mark.parametrize("pusher", ["vay", "hc", "fullrot", "euler", "cond_vay"])
@pytest.mark.parametrize("prec", ["f32", "f64"])
@pytest.mark.parametrize("dim,order", [(1, 2), (2, 1), (2, 2), (2, 3), (3, 2), (3, 4)])
def test_gpu_pusher_dropin_matches_oracle(osg, oracle, pusher, prec, dim, order):
    nx = [12, 10, 8][:dim]
    dx = [0.1, 0.12, 0.15][:dim]
    g = oracle.Grid(nx, order, dx)
    rng = np.random.default_rng(dim * 10 + order + 7)
    dt_ = np.float32 if prec == "f32" else np.float64
    r = oracle.mt_new(17)
    ix, x, u, q = oracle.load(r, prec, dim, nx, [2] * dim, dx, -1.0, [2.0] * 3, [0.2, 0.0, 0.0])
    e = (rng.standard_normal(g.shape) * 5.0).astype(dt_)
    b = (rng.standard_normal(g.shape) * 5.0).astype(dt_)
    dt = 0.04
    code = {"vay": osg.PUSHER_VAY, "hc": osg.PUSHER_HC, "fullrot": osg.PUSHER_FULLROT,
            "euler": osg.PUSHER_EULER, "cond_vay": osg.PUSHER_COND_VAY}[pusher]
    a = [v.copy() for v in (ix, x, u, q)]
    j_g = g.zeros(prec)
    ene_g = osg.vadvance_deposit(dim, order, *a, 1, len(q), -1.0, e, b, g.size, g.gcl, j_g,
                                 g.size, g.gcl, dx, dt, pusher=code)
    o = [v.copy() for v in (ix, x, u, q)]
    j_o = g.zeros(prec)
    ene_o = oracle.push(prec, dim, order, *o, 1, len(q), -1.0, e, b, j_o, g.size, g.gcl, dx, dt,
                        pusher=pusher)
    assert _nerr(a[2], o[2]) <= TOL[prec]
    assert _nerr(_pos(a[0], a[1]), _pos(o[0], o[1])) <= TOL[prec]
    assert _nerr(j_g, j_o) <= TOL[prec]
    assert abs(ene_g - ene_o) <= 10 * TOL[prec] * abs(ene_o)
    ub = [v.copy() for v in (ix, x, u, q)]
    oracle.push(prec, dim, order, *ub, 1, len(q), -1.0, e, b, g.zeros(prec), g.size, g.gcl, dx,
                dt)
    # not a silent Boris: (the conditional Vay differs from it only in its particles above
    # gamma 5, by O(dt^2))
    thr = 1e-10 if prec == "f64" else (1e-6 if pusher == "cond_vay" else TOL[prec])
    assert _nerr(a[2], ub[2]) > thr


@pytest.mark.parametrize("pusher", ["vay", "hc", "fullrot", "euler", "cond_vay"])
@pytest.mark.parametrize("steps", [1, 10])
@pytest.mark.parametrize("dim,order,nx", [(2, 2, [24, 20]), (3, 3, [10, 10, 10])])
def test_plain_fp64_pusher_matches_oracle(osg, oracle, pusher, dim, order, nx, steps):
    _compare(osg, oracle, 64, osg.ENGINE_PLAIN, dim, order, nx, [2] * dim, steps, 1e-12,
             pusher=pusher)


@pytest.mark.parametrize("pusher", ["vay", "hc", "fullrot", "euler", "cond_vay"])
@pytest.mark.parametrize("steps,tol", [(1, 1e-5), (10, 5e-5)])
@pytest.mark.parametrize("dim,order,nx,tile", [(2, 2, [32, 24], [8, 8]),
                                               (3, 2, [16, 8, 8], [4, 4, 4])])
def test_tiled_fp32_pusher_matches_oracle(osg, oracle, pusher, dim, order, nx, tile, steps, tol):
    _compare(osg, oracle, 32, osg.ENGINE_TILED, dim, order, nx, [2] * dim, steps, tol,
             tile=tile, pusher=pusher)


@pytest.mark.parametrize("prec,tol", [(64, 1e-12), (32, 5e-5)])
def test_cond_vay_hot_plasma_takes_both_branches(osg, oracle, prec, tol):
    """A plasma hot enough (u_th = 3) that part of it is above gamma 5 (Vay) and part below
    (Boris), 10 steps of the plain engine against the oracle."""
    from test_gpu_step import _setup
    nx = [20, 16]
    p, g, dx, dt, species, e, b = _setup(oracle, prec, 2, 2, nx, [2, 2], 9, uth=3.0, ufl=0.0)
    gam = np.sqrt(1 + (species[0]["u"].astype(np.float64) ** 2).sum(1))
    assert 0.05 < (gam > 5).mean() < 0.95
    sim = osg.Simulation(nx, dx, dt, order=2, precision=prec, engine=osg.ENGINE_PLAIN,
                         pusher=osg.PUSHER_COND_VAY)
    sim.set_fields(e, b)
    for s in species:
        sim.add_species(s["rqm"], s["ix"], s["x"], s["u"], s["q"])
    sim.step(10)
    eg, bg, jg = sim.fields()
    eo, bo, jo = e.copy(), b.copy(), g.zeros(p)
    for _ in range(10):
        oracle.step(g, p, eo, bo, jo, species, dt, pusher="cond_vay")
    assert _nerr(eg, eo) <= tol and _nerr(bg, bo) <= tol and _nerr(jg, jo) <= tol
    for k, s in enumerate(species):
        ix, x, u, q = sim.species(k)
        assert _nerr(_pos(ix, x), _pos(s["ix"], s["x"])) <= tol
        assert _nerr(u, s["u"]) <= tol
    sim.close()
