"""GPU parity of Lindman open boundaries (osg_config.open_fields) against the oracle's step:
first-order Mur update of the tangential E after the E step, the lower B buffer after each B
half step, the boundary planes restored by the guard update, no periodic fold of the current
along the open axis, particles absorbed at the open edges.  Whole arrays are compared, guard
cells included (the boundary planes live there).

* plain engine, 2D, FP64 1e-12 and FP32 1e-5 / 5e-5 (1 and 10 steps), orders 1-3, either axis;
  3D FP64 along x3;
* tiled engine (FP32, particles removed rather than kept with charge 0): fields and the live
  particles against the oracle, in 2D and, with walls or open edges, in 3D;
* a vacuum pulse leaves the box with less than 1e-4 of its energy left;
* checkpoint / restore keeps the Lindman state: 4 + 4 steps equal 8 steps to 1e-12 (FP64
  atomics) with the same particles absorbed.
"""
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


def _oracle_run(oracle, g, p, e, b, species, dt, axis, steps):
    ora = [{k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in s.items()}
           for s in species]
    eo, bo, jo = e.copy(), b.copy(), g.zeros(p)
    st = oracle.lindman_state(g, p, axis)
    for _ in range(steps):
        oracle.step(g, p, eo, bo, jo, ora, dt, open_fields=(axis, st))
    return eo, bo, jo, ora


def _plain(osg, oracle, prec, dim, order, axis, steps, nx, seed=11):
    p, g, dx, dt, species, e, b = _setup(oracle, prec, dim, order, nx, [2] * dim, seed,
                                         uth=0.6, ufl=0.1)
    sim = osg.Simulation(nx, dx, dt, order=order, precision=prec, engine=osg.ENGINE_PLAIN,
                         open_fields=1 << axis)
    sim.set_fields(e, b)
    for s in species:
        sim.add_species(s["rqm"], s["ix"], s["x"], s["u"], s["q"])
    sim.step(steps)
    eg, bg, jg = sim.fields()
    eo, bo, jo, ora = _oracle_run(oracle, g, p, e, b, species, dt, axis, steps)
    errs = {"E": _nerr(eg, eo), "B": _nerr(bg, bo), "J": _nerr(jg, jo)}
    absorbed = 0
    for k, s in enumerate(ora):
        ix, x, u, q = sim.species(k)          # the plain engine keeps the particle order
        errs[f"x{k}"] = _nerr(ix + x, s["ix"] + s["x"])
        errs[f"u{k}"] = _nerr(u, s["u"])
        assert np.array_equal(q == 0, s["q"] == 0)
        absorbed += int((q == 0).sum())
        assert ix.min() >= 1 and np.all(ix.max(axis=0) <= np.array(nx))
    sim.close()
    return errs, absorbed


@pytest.mark.parametrize("axis", [0, 1])
@pytest.mark.parametrize("order", [1, 2, 3])
@pytest.mark.parametrize("prec,steps,tol", [(64, 1, 1e-12), (64, 10, 1e-12), (32, 1, 1e-5),
                                            (32, 10, 5e-5)])
def test_open_plain_matches_oracle(osg, oracle, prec, steps, tol, order, axis):
    errs, absorbed = _plain(osg, oracle, prec, 2, order, axis, steps, [20, 16])
    bad = {k: v for k, v in errs.items() if not v <= tol}
    assert not bad, (bad, errs)
    if steps > 1:
        assert absorbed > 0


@pytest.mark.parametrize("axis", [0, 2])
def test_open_plain_3d_matches_oracle(osg, oracle, axis):
    errs, absorbed = _plain(osg, oracle, 64, 3, 2, axis, 6, [10, 9, 8])
    bad = {k: v for k, v in errs.items() if not v <= 1e-12}
    assert not bad, (bad, errs)
    assert absorbed > 0


@pytest.mark.parametrize("axis", [0, 1])
@pytest.mark.parametrize("order", [2, 3])
@pytest.mark.parametrize("steps,tol", [(1, 1e-5), (10, 5e-5)])
def test_open_tiled_matches_oracle(osg, oracle, steps, tol, order, axis):
    """The tiled engine drops absorbed particles; the oracle keeps them with charge 0."""
    dim, nx = 2, [32, 24]
    p, g, dx, dt, species, e, b = _setup(oracle, 32, dim, order, nx, [2, 2], 12, uth=0.6,
                                         ufl=0.1)
    sim = osg.Simulation(nx, dx, dt, order=order, precision=32, engine=osg.ENGINE_TILED,
                         tile=[8, 8], open_fields=1 << axis)
    sim.set_fields(e, b)
    for s in species:
        sim.add_species(s["rqm"], s["ix"], s["x"], s["u"], s["q"])
    sim.step(steps)
    eg, bg, jg = sim.fields()
    eo, bo, jo, ora = _oracle_run(oracle, g, p, e, b, species, dt, axis, steps)
    errs = {"E": _nerr(eg, eo), "B": _nerr(bg, bo), "J": _nerr(jg, jo)}
    for k, s in enumerate(ora):
        ix, x, u, q = sim.species(k)
        live = s["q"] != 0
        assert len(q) == int(live.sum())
        if steps > 1:
            assert len(q) < len(s["q"])
        a = np.argsort(q, kind="stable")
        o = np.flatnonzero(live)[np.argsort(s["q"][live], kind="stable")]
        errs[f"x{k}"] = _nerr(ix[a] + x[a], s["ix"][o] + s["x"][o])
        errs[f"u{k}"] = _nerr(u[a], s["u"][o])
        assert ix.min() >= 1 and np.all(ix.max(axis=0) <= np.array(nx))
    sim.close()
    bad = {k: v for k, v in errs.items() if not v <= tol}
    assert not bad, (bad, errs)


@pytest.mark.parametrize("engine,prec", [("plain", 64), ("tiled", 32)])
def test_vacuum_pulse_leaves_the_box(osg, engine, prec):
    nx, dx = [128, 16], [0.2, 0.2]
    dt = 0.9 / np.sqrt(sum(1 / d ** 2 for d in dx))
    sim = osg.Simulation(nx, dx, dt, order=2, precision=prec,
                         engine=osg.ENGINE_PLAIN if engine == "plain" else osg.ENGINE_TILED,
                         tile=[16, 8] if engine == "tiled" else None, open_fields=1)
    gl, gu = osg.GUARD[2]
    dtype = np.float32 if prec == 32 else np.float64
    shape = tuple(reversed([n + gl + gu for n in nx])) + (3,)
    e, b = np.zeros(shape, dtype), np.zeros(shape, dtype)
    L = nx[0] * dx[0]
    i1 = np.arange(shape[1]) - gl
    prof = lambda x: np.exp(-((x - 0.5 * L) / (0.08 * L)) ** 2)
    e[:, :, 1] = prof(i1 * dx[0])[None, :]
    b[:, :, 2] = prof((i1 + 0.5) * dx[0])[None, :]
    sim.set_fields(e, b)
    empty = np.zeros((0, 2), np.int32), np.zeros((0, 2), dtype), np.zeros((0, 3), dtype), \
        np.zeros(0, dtype)
    sim.add_species(-1.0, *empty)

    def energy(fe, fb):
        sl = (slice(gl, gl + nx[1]), slice(gl, gl + nx[0]))
        return float((fe[sl].astype(np.float64) ** 2).sum() + (fb[sl].astype(np.float64) ** 2).sum())

    w0 = energy(e, b)
    sim.step(int(L / dt))
    e1, b1, _ = sim.fields()
    assert energy(e1, b1) / w0 < 1e-4
    sim.close()


def test_checkpoint_keeps_the_lindman_state(osg, oracle, tmp_path):
    nx = [20, 16]
    p, g, dx, dt, species, e, b = _setup(oracle, 64, 2, 2, nx, [2, 2], 4, uth=0.6, ufl=0.1)

    def fresh():
        sim = osg.Simulation(nx, dx, dt, order=2, precision=64, engine=osg.ENGINE_PLAIN,
                             open_fields=1)
        sim.set_fields(e, b)
        for s in species:
            sim.add_species(s["rqm"], s["ix"], s["x"], s["u"], s["q"])
        return sim

    ref = fresh()
    ref.step(8)
    want = ref.fields()[:2], ref.species(0)
    ref.close()
    a = fresh()
    a.step(4)
    a.checkpoint(tmp_path / "open.ckpt")
    a.close()
    c = osg.Simulation.restore(tmp_path / "open.ckpt")
    assert c.cfg.open_fields == 1
    c.step(4)
    got = c.fields()[:2], c.species(0)
    c.close()
    # the FP64 current's atomic sums are the only difference between the runs; a lost state
    # would change the boundary planes at the size of the fields themselves
    for x, y in zip(got[0], want[0]):
        assert _nerr(x, y) <= 1e-12
    (ia, xa, ua, qa), (ib, xb, ub, qb) = got[1], want[1]
    assert np.array_equal(qa, qb)
    assert _nerr(ia + xa, ib + xb) <= 1e-12 and _nerr(ua, ub) <= 1e-12


@pytest.mark.parametrize("walls,open_fields", [(0, 4), (5, 0), (3, 0)])
def test_tiled_3d_bounded_matches_oracle(osg, oracle, walls, open_fields):
    """3D tiled engine (FP32) with Lindman open edges or conducting walls, 6 steps."""
    dim, nx = 3, [16, 8, 8]
    p, g, dx, dt, species, e, b = _setup(oracle, 32, dim, 2, nx, [2] * 3, 14, uth=0.6,
                                         ufl=0.1)
    sim = osg.Simulation(nx, dx, dt, order=2, precision=32, engine=osg.ENGINE_TILED,
                         tile=[4, 4, 4], walls=walls, open_fields=open_fields)
    sim.set_fields(e, b)
    for s in species:
        sim.add_species(s["rqm"], s["ix"], s["x"], s["u"], s["q"])
    steps = 6
    sim.step(steps)
    eg, bg, jg = sim.fields()
    ora = [{k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in s.items()}
           for s in species]
    eo, bo, jo = e.copy(), b.copy(), g.zeros(p)
    axis = open_fields.bit_length() - 1
    st = oracle.lindman_state(g, p, axis) if open_fields else None
    for _ in range(steps):
        oracle.step(g, p, eo, bo, jo, ora, dt, walls=walls,
                    open_fields=(axis, st) if open_fields else None)
    if open_fields:
        errs = {"E": _nerr(eg, eo), "B": _nerr(bg, bo), "J": _nerr(jg, jo)}
    else:
        errs = {"E": _nerr(g.interior(eg), g.interior(eo)),
                "B": _nerr(g.interior(bg), g.interior(bo)),
                "J": _nerr(g.interior(jg), g.interior(jo))}
    for k, s in enumerate(ora):
        ix, x, u, q = sim.species(k)
        live = s["q"] != 0
        assert len(q) == int(live.sum())
        a = np.argsort(q, kind="stable")
        o = np.flatnonzero(live)[np.argsort(s["q"][live], kind="stable")]
        errs[f"x{k}"] = _nerr(ix[a] + x[a], s["ix"][o] + s["x"][o])
        errs[f"u{k}"] = _nerr(u[a], s["u"][o])
        assert ix.min() >= 1 and np.all(ix.max(axis=0) <= np.array(nx))
    sim.close()
    bad = {k: v for k, v in errs.items() if not v <= 5e-5}
    assert not bad, (bad, errs)


def test_gauss_residual_refuses_open_edges(osg):
    sim = osg.Simulation([16, 16], [0.1, 0.1], 0.03, order=2, precision=64,
                         engine=osg.ENGINE_PLAIN, open_fields=2)
    with pytest.raises(osg.OsirisGB300Error):
        sim.gauss_residual()
    sim.close()


@pytest.mark.parametrize("prec,tol", [("f64", 1e-14), ("f32", 1e-6)])
@pytest.mark.parametrize("dim,axis", [(2, 0), (2, 1), (3, 1)])
@pytest.mark.parametrize("what", [0, 1, 2])
def test_host_array_lindman_matches_oracle(osg, oracle, prec, tol, dim, axis, what):
    """osg_lindman_* (one phase on host arrays) against the oracle's phase, from random fields
    and a random state."""
    nx = [12, 10] if dim == 2 else [8, 7, 6]
    dx = [0.1, 0.12, 0.09][:dim]
    g = oracle.Grid(nx, 2, dx)
    dt_ = np.float32 if prec == "f32" else np.float64
    rng = np.random.default_rng(10 * what + axis)
    e0 = rng.standard_normal(g.shape).astype(dt_)
    b0 = rng.standard_normal(g.shape).astype(dt_)
    s0 = rng.standard_normal(oracle.lindman_state(g, prec, axis).shape).astype(dt_)
    ea, ba, sa = e0.copy(), b0.copy(), s0.copy()
    eo, bo, so = e0.copy(), b0.copy(), s0.copy()
    dt = 0.03
    osg.lindman(dim, g.nx, g.gcl, g.gcu, axis, what, ea, ba, sa, dx, dt)
    oracle.lindman_phase(g, prec, axis, what, eo, bo, so, dt)
    for a, o, a0 in ((ea, eo, e0), (ba, bo, b0), (sa, so, s0)):
        assert _nerr(a, o) <= tol
    assert not (np.array_equal(ea, e0) and np.array_equal(ba, b0) and np.array_equal(sa, s0))
