"""GPU parity of the current smoothing (osg_smooth_*, and inside the device-resident step)
against the oracle's restatement of filter_2d/3d (source/vdf/os-vdf-smooth.f90:639-1000).

The library keeps the coefficients and the sums in FP64 (for the FP32 field too); the oracle's
FP32 path follows the single-precision reference build (float coefficients and sums), so FP32
agrees to a few float roundings (2e-6 normwise) and FP64 to 1e-14.  Full steps with smoothing
after the current fold: plain FP64 engine 1e-12, tiled FP32 engine 1e-5 after 2 steps."""
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


@pytest.mark.parametrize("prec,tol", [("f64", 1e-14), ("f32", 2e-6)])
@pytest.mark.parametrize("dim,types,orders", [(2, [2, 2], [1, 1]), (2, [3, 2], [2, 3]),
                                              (2, [4, 5], [5, 3]), (3, [2, 6, 3], [2, 4, 2])])
def test_gpu_smooth_matches_oracle(osg, oracle, prec, tol, dim, types, orders):
    nx = [24, 20, 12][:dim]
    g = oracle.Grid(nx, 2, [0.1] * dim, guard=(6, 7))
    rng = np.random.default_rng(dim + sum(orders))
    f = rng.standard_normal(g.shape).astype(g.zeros(prec).dtype)
    a, o = f.copy(), f.copy()
    osg.smooth(dim, nx, g.gcl, g.gcu, a, types, orders)
    oracle.smooth(g, prec, o, types, orders)
    assert _nerr(a, o) <= tol
    assert _nerr(a, f) > 1e-3          # the filter did something


@pytest.mark.parametrize("prec,engine,tol", [(64, "plain", 1e-12), (32, "tiled", 1e-5)])
def test_gpu_step_with_smoothing_matches_oracle(osg, oracle, prec, engine, tol):
    nx, order, steps, st = [32, 24], 2, 2, (2, 3)     # 3 binomial passes: wider guards
    p, g0, dx, dt, species, e0, b0 = _setup(oracle, prec, 2, order, nx, [2, 2], seed=17)
    eng = osg.ENGINE_TILED if engine == "tiled" else osg.ENGINE_PLAIN
    sim = osg.Simulation(nx, dx, dt, order=order, precision=prec, engine=eng,
                         tile=[8, 8] if eng == osg.ENGINE_TILED else None,
                         smooth_type=st[0], smooth_order=st[1])
    g = oracle.Grid(nx, order, dx, guard=(sim.gcl[0], sim.gcu[0]))
    assert sim.gcl[0] == 3 and sim.gcu[0] == 4
    rng = np.random.default_rng(3)
    e = (rng.standard_normal(g.shape) * 0.02).astype(e0.dtype)
    b = (rng.standard_normal(g.shape) * 0.02).astype(e0.dtype)
    sim.set_fields(e, b)
    for s in species:
        sim.add_species(s["rqm"], s["ix"], s["x"], s["u"], s["q"])
    sim.step(steps)
    eg, bg, jg = sim.fields()
    sim.close()
    ora = [{k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in s.items()}
           for s in species]
    eo, bo, jo = e.copy(), b.copy(), g.zeros(p)
    for _ in range(steps):
        oracle.step(g, p, eo, bo, jo, ora, dt, smooth=st)
    for a, o in ((eg, eo), (bg, bo), (jg, jo)):
        assert _nerr(g.interior(a), g.interior(o)) <= tol
    # and it is not the unsmoothed step
    ora2 = [{k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in s.items()}
            for s in species]
    e2, b2, j2 = e.copy(), b.copy(), g.zeros(p)
    for _ in range(steps):
        oracle.step(g, p, e2, b2, j2, ora2, dt)
    assert _nerr(g.interior(j2), g.interior(jo)) > 1e-3


@pytest.mark.parametrize("prec,engine,tol", [(64, "plain", 1e-12), (32, "tiled", 5e-5)])
@pytest.mark.parametrize("dim,st", [(2, (2, 2)), (2, (3, 3)), (3, (2, 1))])
def test_gpu_step_with_field_smoothing_matches_oracle(osg, oracle, prec, engine, tol, dim, st):
    """The fields the particles see smoothed (the reference's e_part / b_part, smooth_type
    "stand", update_particle_fld_emf, source/emf/os-emf.f03:1065-1151): smoothed copies of E
    and B after their guard update feed the push; E and B themselves stay unsmoothed.  The
    field guards grow by the filter's order.  4 steps against the oracle's step(...,
    smooth_emf=...); the particles' momenta differ from an unsmoothed run."""
    nx, order, steps = ([32, 24] if dim == 2 else [16, 12, 12]), 2, 4
    p, g0, dx, dt, species, e0, b0 = _setup(oracle, prec, dim, order, nx, [2] * dim, seed=19)
    eng = osg.ENGINE_TILED if engine == "tiled" else osg.ENGINE_PLAIN
    sim = osg.Simulation(nx, dx, dt, order=order, precision=prec, engine=eng,
                         tile=[4] * dim if eng == osg.ENGINE_TILED else None,
                         emf_smooth_type=st[0], emf_smooth_order=st[1])
    g = oracle.Grid(nx, order, dx, guard=(sim.gcl[0], sim.gcu[0]))
    ne = st[1] if st[0] != 3 else max(2, st[1])
    assert sim.gcl[0] == order + ne and sim.gcu[0] == order + 1 + ne
    rng = np.random.default_rng(5)
    e = (rng.standard_normal(g.shape) * 0.05).astype(e0.dtype)
    b = (rng.standard_normal(g.shape) * 0.05).astype(e0.dtype)
    sim.set_fields(e, b)
    for s in species:
        sim.add_species(s["rqm"], s["ix"], s["x"], s["u"], s["q"])
    sim.step(steps)
    eg, bg, jg = sim.fields()
    spg = [sim.species(k) for k in range(2)]
    sim.close()
    ora = [{k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in s.items()}
           for s in species]
    eo, bo, jo = e.copy(), b.copy(), g.zeros(p)
    for _ in range(steps):
        oracle.step(g, p, eo, bo, jo, ora, dt, smooth_emf=st)
    for a, o in ((eg, eo), (bg, bo), (jg, jo)):
        assert _nerr(g.interior(a), g.interior(o)) <= tol
    for k in range(2):
        ix, x, u, q = spg[k]
        o, ro = np.argsort(q), np.argsort(ora[k]["q"])
        assert np.array_equal(q[o], ora[k]["q"][ro])
        assert _nerr(u[o], ora[k]["u"][ro]) <= tol
    # and it is not the unsmoothed step
    ora2 = [{k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in s.items()}
            for s in species]
    e2, b2, j2 = e.copy(), b.copy(), g.zeros(p)
    for _ in range(steps):
        oracle.step(g, p, e2, b2, j2, ora2, dt)
    assert _nerr(ora2[0]["u"], ora[0]["u"]) > 1e-4
