"""GPU parity of conducting walls (osg_config.walls, plain and tiled engines) against the
oracle's walled step: PEC field images after every partial field step, the current beyond a wall added back as
its image, specular particle reflection.  FP64 1e-12 and FP32 1e-5 (after 1 and 10 steps), for
walls along x1, x2 and both, odd and even interpolation orders.  Particles move fast enough
(momenta of rms 0.6) that many reflect."""
import numpy as np
import pytest

from test_gpu_step import _nerr, _setup

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def osg():
    import __graft_entry__ as g
    g.build_native()
    import osiris_gb300
    if osiris_gb300.lib().osg_device_count() < 1:
        pytest.fail("no CUDA device visible")
    return osiris_gb300


def _run(osg, oracle, prec, order, mask, steps):
    dim, nx = 2, [20, 16]
    p, g, dx, dt, species, e, b = _setup(oracle, prec, dim, order, nx, [2, 2], 11, uth=0.6,
                                         ufl=0.1)
    sim = osg.Simulation(nx, dx, dt, order=order, precision=prec, engine=osg.ENGINE_PLAIN,
                         walls=mask)
    sim.set_fields(e, b)
    for s in species:
        sim.add_species(s["rqm"], s["ix"], s["x"], s["u"], s["q"])
    sim.step(steps)
    eg, bg, jg = sim.fields()
    ora = [{k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in s.items()}
           for s in species]
    eo, bo, jo = e.copy(), b.copy(), g.zeros(p)
    for _ in range(steps):
        oracle.step(g, p, eo, bo, jo, ora, dt, walls=mask)
    errs = {"E": _nerr(g.interior(eg), g.interior(eo)), "B": _nerr(g.interior(bg), g.interior(bo)),
            "J": _nerr(g.interior(jg), g.interior(jo))}
    for k, s in enumerate(ora):
        ix, x, u, q = sim.species(k)          # the plain engine keeps the particle order
        errs[f"x{k}"] = _nerr(ix + x, s["ix"] + s["x"])
        errs[f"u{k}"] = _nerr(u, s["u"])
        assert ix.min() >= 1 and np.all(ix.max(axis=0) <= np.array(nx))
    sim.close()
    return errs


@pytest.mark.parametrize("mask", [1, 2, 3])
@pytest.mark.parametrize("order", [1, 2, 3])
@pytest.mark.parametrize("prec,steps,tol", [(64, 1, 1e-12), (64, 10, 1e-12), (32, 1, 1e-5),
                                            (32, 10, 5e-5)])
def test_walls_match_oracle(osg, oracle, prec, steps, tol, order, mask):
    errs = _run(osg, oracle, prec, order, mask, steps)
    bad = {k: v for k, v in errs.items() if not v <= tol}
    assert not bad, (bad, errs)


@pytest.mark.parametrize("mask", [1, 2, 3])
@pytest.mark.parametrize("order", [2, 3])
@pytest.mark.parametrize("steps,tol", [(1, 1e-5), (10, 5e-5)])
def test_tiled_walls_match_oracle(osg, oracle, steps, tol, order, mask):
    """The mixed-precision tiled engine between conducting walls (particles reflect in the tile
    push; the fields and current take the same images as the plain engine)."""
    dim, nx = 2, [32, 24]
    p, g, dx, dt, species, e, b = _setup(oracle, 32, dim, order, nx, [2, 2], 12, uth=0.6,
                                         ufl=0.1)
    sim = osg.Simulation(nx, dx, dt, order=order, precision=32, engine=osg.ENGINE_TILED,
                         tile=[8, 8], walls=mask)
    sim.set_fields(e, b)
    for s in species:
        sim.add_species(s["rqm"], s["ix"], s["x"], s["u"], s["q"])
    sim.step(steps)
    eg, bg, jg = sim.fields()
    ora = [{k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in s.items()}
           for s in species]
    eo, bo, jo = e.copy(), b.copy(), g.zeros(p)
    for _ in range(steps):
        oracle.step(g, p, eo, bo, jo, ora, dt, walls=mask)
    errs = {"E": _nerr(g.interior(eg), g.interior(eo)), "B": _nerr(g.interior(bg), g.interior(bo)),
            "J": _nerr(g.interior(jg), g.interior(jo))}
    for k, s in enumerate(ora):
        ix, x, u, q = sim.species(k)
        assert len(q) == len(s["q"])
        a, o = np.argsort(q, kind="stable"), np.argsort(s["q"], kind="stable")
        errs[f"x{k}"] = _nerr(ix[a] + x[a], s["ix"][o] + s["x"][o])
        errs[f"u{k}"] = _nerr(u[a], s["u"][o])
        assert ix.min() >= 1 and np.all(ix.max(axis=0) <= np.array(nx))
    sim.close()
    bad = {k: v for k, v in errs.items() if not v <= tol}
    assert not bad, (bad, errs)


@pytest.mark.parametrize("prec,order,kind,mask", [("f64", 1, 0, 1), ("f64", 2, 2, 3),
                                                  ("f32", 3, 1, 2), ("f32", 4, 2, 1)])
def test_host_array_walls_match_oracle(osg, oracle, prec, order, kind, mask):
    g = oracle.Grid([12, 10], order, [0.1, 0.1])
    dt_ = np.float32 if prec == "f32" else np.float64
    f0 = np.random.default_rng(order + kind).standard_normal(g.shape).astype(dt_)
    a, o = f0.copy(), f0.copy()
    osg.walls(2, g.nx, g.gcl, g.gcu, a, kind, mask, order)
    oracle.walls(g, prec, o, kind, mask)
    assert np.array_equal(a, o)


@pytest.mark.parametrize("prec,order,kind,mask", [("f64", 1, 3, 1), ("f64", 2, 4, 3),
                                                  ("f32", 3, 3, 2), ("f32", 4, 4, 1)])
def test_host_array_pmc_walls_match_oracle(osg, oracle, prec, order, kind, mask):
    g = oracle.Grid([12, 10], order, [0.1, 0.1])
    dt_ = np.float32 if prec == "f32" else np.float64
    f0 = np.random.default_rng(order + kind).standard_normal(g.shape).astype(dt_)
    a, o = f0.copy(), f0.copy()
    osg.walls(2, g.nx, g.gcl, g.gcu, a, kind, mask, order)
    oracle.walls(g, prec, o, kind, mask)
    assert np.array_equal(a, o)


@pytest.mark.parametrize("engine,prec,tol", [("plain", 64, 1e-12), ("plain", 32, 5e-5),
                                             ("tiled", 32, 5e-5)])
@pytest.mark.parametrize("walls,pmc", [(1, 1), (3, 2), (3, 3)])
def test_pmc_walls_match_oracle(osg, oracle, engine, prec, tol, walls, pmc):
    """Perfect magnetic conductor walls (osg_config.pmc) on some or all walled axes, 10 steps."""
    dim, nx, order = 2, [32, 24], 2
    p, g, dx, dt, species, e, b = _setup(oracle, prec, dim, order, nx, [2, 2], 13, uth=0.6,
                                         ufl=0.1)
    sim = osg.Simulation(nx, dx, dt, order=order, precision=prec,
                         engine=osg.ENGINE_PLAIN if engine == "plain" else osg.ENGINE_TILED,
                         tile=[8, 8] if engine == "tiled" else None, walls=walls, pmc=pmc)
    sim.set_fields(e, b)
    for s in species:
        sim.add_species(s["rqm"], s["ix"], s["x"], s["u"], s["q"])
    sim.step(10)
    eg, bg, jg = sim.fields()
    ora = [{k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in s.items()}
           for s in species]
    eo, bo, jo = e.copy(), b.copy(), g.zeros(p)
    for _ in range(10):
        oracle.step(g, p, eo, bo, jo, ora, dt, walls=walls, pmc=pmc)
    errs = {"E": _nerr(g.interior(eg), g.interior(eo)), "B": _nerr(g.interior(bg), g.interior(bo)),
            "J": _nerr(g.interior(jg), g.interior(jo))}
    for k, s in enumerate(ora):
        ix, x, u, q = sim.species(k)
        a, o = np.argsort(q, kind="stable"), np.argsort(s["q"], kind="stable")
        errs[f"x{k}"] = _nerr(ix[a] + x[a], s["ix"][o] + s["x"][o])
        errs[f"u{k}"] = _nerr(u[a], s["u"][o])
    sim.close()
    bad = {k: v for k, v in errs.items() if not v <= tol}
    assert not bad, (bad, errs)
