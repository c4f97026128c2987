"""GPU parity of PML walls (osg_config.pml, Vay's split-field perfectly matched layer at both
edges of the axes in a mask of a 2D box; with both axes the x1 walls cover the corners) against
the oracle's step.  The walls advance their E after the
first B half step and their B after the E step, exchange the boundary points with the box
through the interfaces, and take their own periodic update along the other axis at the guard
update; the current is not folded along the PML axis and particles leaving through it are
absorbed.  Whole field arrays are compared, guard cells included (the interfaces write there).

* plain engine, FP64 1e-12 and FP32 1e-5 / 5e-5 (1 and 10 steps), orders 1-3, either axis and
  both (corners);
* tiled engine (FP32; absorbed particles removed rather than kept with charge 0): fields and
  the live particles against the oracle, either axis and both;
* a vacuum pulse travelling along the PML axis leaves the box with less than 1e-4 of its
  energy, in both engines; with both axes, a cylindrical pulse leaves less than 1e-4;
* 3D, any set of PML axes (the walls of a lower axis covering the edge regions of the higher
  ones): plain FP64 1e-12 and tiled FP32 5e-5 against the oracle after 6 steps; a plane pulse
  leaves less than 1e-4 of its energy, and with all three axes a divergence-free spherical
  pulse less than 1e-4;
* checkpoint / restore keeps the walls: 4 + 4 steps equal 8 steps to 1e-12;
* configurations the walls are not built for are refused.
"""
import numpy as np
import pytest

from test_gpu_step import _nerr, _setup

pytestmark = pytest.mark.gpu

NB = 8


@pytest.fixture(scope="module")
def osg():
    import __graft_entry__ as g
    g.build_native()
    import osiris_gb300
    if osiris_gb300.lib().osg_device_count() < 1:
        pytest.fail("no CUDA device visible")
    return osiris_gb300


def _oracle_run(oracle, g, p, e, b, species, dt, mask, steps, nb=NB):
    ora = [{k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in s.items()}
           for s in species]
    eo, bo, jo = e.copy(), b.copy(), g.zeros(p)
    st = oracle.pml_state(g, p, mask, nb, dt)
    for _ in range(steps):
        oracle.step(g, p, eo, bo, jo, ora, dt, pml=(mask, nb, st))
    return eo, bo, jo, ora


@pytest.mark.parametrize("mask", [1, 2, 3])
@pytest.mark.parametrize("order", [1, 2, 3])
@pytest.mark.parametrize("prec,steps,tol", [(64, 1, 1e-12), (64, 10, 1e-12), (32, 1, 1e-5),
                                            (32, 10, 5e-5)])
def test_pml_plain_matches_oracle(osg, oracle, prec, steps, tol, order, mask):
    nx = [20, 16]
    p, g, dx, dt, species, e, b = _setup(oracle, prec, 2, order, nx, [2, 2], 11, uth=0.6,
                                         ufl=0.1)
    sim = osg.Simulation(nx, dx, dt, order=order, precision=prec, engine=osg.ENGINE_PLAIN,
                         pml=mask, pml_cells=NB)
    sim.set_fields(e, b)
    for s in species:
        sim.add_species(s["rqm"], s["ix"], s["x"], s["u"], s["q"])
    sim.step(steps)
    eg, bg, jg = sim.fields()
    eo, bo, jo, ora = _oracle_run(oracle, g, p, e, b, species, dt, mask, steps)
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
    bad = {k: v for k, v in errs.items() if not v <= tol}
    assert not bad, (bad, errs)
    if steps > 1:
        assert absorbed > 0


@pytest.mark.parametrize("mask", [1, 2, 3])
@pytest.mark.parametrize("order", [2, 3])
@pytest.mark.parametrize("steps,tol", [(1, 1e-5), (10, 5e-5)])
def test_pml_tiled_matches_oracle(osg, oracle, steps, tol, order, mask):
    """The tiled engine drops absorbed particles; the oracle keeps them with charge 0."""
    nx = [32, 24]
    p, g, dx, dt, species, e, b = _setup(oracle, 32, 2, order, nx, [2, 2], 12, uth=0.6,
                                         ufl=0.1)
    sim = osg.Simulation(nx, dx, dt, order=order, precision=32, engine=osg.ENGINE_TILED,
                         tile=[8, 8], pml=mask, pml_cells=NB)
    sim.set_fields(e, b)
    for s in species:
        sim.add_species(s["rqm"], s["ix"], s["x"], s["u"], s["q"])
    sim.step(steps)
    eg, bg, jg = sim.fields()
    eo, bo, jo, ora = _oracle_run(oracle, g, p, e, b, species, dt, mask, steps)
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
@pytest.mark.parametrize("axis", [0, 1])
def test_vacuum_pulse_leaves_through_the_pml(osg, engine, prec, axis):
    nl, dx = 128, [0.2, 0.2]
    nx = [nl, 16] if axis == 0 else [16, nl]
    dt = 0.9 / np.sqrt(sum(1 / d ** 2 for d in dx))
    sim = osg.Simulation(nx, dx, dt, order=2, precision=prec,
                         engine=osg.ENGINE_PLAIN if engine == "plain" else osg.ENGINE_TILED,
                         tile=([16, 8] if axis == 0 else [8, 16]) if engine == "tiled" else None,
                         pml=1 << axis)
    gl, gu = osg.GUARD[2]
    dtype = np.float32 if prec == 32 else np.float64
    shape = tuple(reversed([n + gl + gu for n in nx])) + (3,)
    e, b = np.zeros(shape, dtype), np.zeros(shape, dtype)
    L = nl * dx[axis]
    i = np.arange(shape[1 - axis]) - gl
    prof = lambda x: np.exp(-((x - 0.5 * L) / (0.08 * L)) ** 2)
    if axis == 0:   # Ey, Bz travelling along +x1
        e[:, :, 1] = prof(i * dx[0])[None, :]
        b[:, :, 2] = prof((i + 0.5) * dx[0])[None, :]
    else:           # Ex, -Bz travelling along +x2
        e[:, :, 0] = prof(i * dx[1])[:, None]
        b[:, :, 2] = -prof((i + 0.5) * dx[1])[:, None]
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


@pytest.mark.parametrize("engine,prec", [("plain", 64), ("tiled", 32)])
def test_cylindrical_pulse_leaves_through_pml_on_both_axes(osg, engine, prec):
    nx, dx = [64, 48], [0.2, 0.2]
    dt = 0.9 / np.sqrt(sum(1 / d ** 2 for d in dx))
    sim = osg.Simulation(nx, dx, dt, order=2, precision=prec,
                         engine=osg.ENGINE_PLAIN if engine == "plain" else osg.ENGINE_TILED,
                         tile=[8, 8] if engine == "tiled" else None, pml=3)
    gl, gu = osg.GUARD[2]
    dtype = np.float32 if prec == 32 else np.float64
    shape = tuple(reversed([n + gl + gu for n in nx])) + (3,)
    e, b = np.zeros(shape, dtype), np.zeros(shape, dtype)
    y, x = np.meshgrid(np.arange(shape[0]), np.arange(shape[1]), indexing="ij")
    e[:, :, 2] = np.exp(-((x - shape[1] / 2) ** 2 + (y - shape[0] / 2) ** 2) / 8.0)
    sim.set_fields(e, b)
    empty = np.zeros((0, 2), np.int32), np.zeros((0, 2), dtype), np.zeros((0, 3), dtype), \
        np.zeros(0, dtype)
    sim.add_species(-1.0, *empty)
    sl = (slice(gl, gl + nx[1]), slice(gl, gl + nx[0]))
    w0 = float((e[sl].astype(np.float64) ** 2).sum())
    sim.step(int(3 * max(nx) * dx[0] / dt))
    e1, b1, _ = sim.fields()
    w1 = float((e1[sl].astype(np.float64) ** 2).sum() + (b1[sl].astype(np.float64) ** 2).sum())
    assert w1 / w0 < 1e-4
    sim.close()


def test_checkpoint_keeps_the_pml_walls(osg, oracle, tmp_path):
    nx = [20, 16]
    p, g, dx, dt, species, e, b = _setup(oracle, 64, 2, 2, nx, [2, 2], 4, uth=0.6, ufl=0.1)

    def fresh():
        sim = osg.Simulation(nx, dx, dt, order=2, precision=64, engine=osg.ENGINE_PLAIN,
                             pml=3)
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
    a.checkpoint(tmp_path / "pml.ckpt")
    a.close()
    c = osg.Simulation.restore(tmp_path / "pml.ckpt")
    assert c.cfg.pml == 3
    c.step(4)
    got = c.fields()[:2], c.species(0)
    c.close()
    for x, y in zip(got[0], want[0]):
        assert _nerr(x, y) <= 1e-12
    (ia, xa, ua, qa), (ib, xb, ub, qb) = got[1], want[1]
    assert np.array_equal(qa, qb)
    assert _nerr(ia + xa, ib + xb) <= 1e-12 and _nerr(ua, ub) <= 1e-12


@pytest.mark.parametrize("kw", [dict(pml=4), dict(pml=1, walls=2), dict(pml=1, open_fields=2),
                                dict(pml=1, pml_cells=4), dict(pml=1, smooth_type=2,
                                                               smooth_order=1)])
def test_pml_refuses_what_it_is_not_built_for(osg, kw):
    with pytest.raises(osg.OsirisGB300Error):
        osg.Simulation([16, 16], [0.1, 0.1], 0.03, order=2, precision=64,
                       engine=osg.ENGINE_PLAIN, **kw)


@pytest.mark.parametrize("mask", [1, 2, 4, 3, 5, 6, 7])
@pytest.mark.parametrize("order", [2, 3])
@pytest.mark.parametrize("engine,prec,tol", [("plain", 64, 1e-12), ("tiled", 32, 5e-5)])
def test_pml_3d_matches_oracle(osg, oracle, engine, prec, tol, order, mask):
    nx = [12, 8, 8]
    p, g, dx, dt, species, e, b = _setup(oracle, prec, 3, order, nx, [2, 2, 2], 21, uth=0.6,
                                         ufl=0.1)
    sim = osg.Simulation(nx, dx, dt, order=order, precision=prec,
                         engine=osg.ENGINE_PLAIN if engine == "plain" else osg.ENGINE_TILED,
                         tile=[4, 4, 4] if engine == "tiled" else None, pml=mask)
    sim.set_fields(e, b)
    for s_ in species:
        sim.add_species(s_["rqm"], s_["ix"], s_["x"], s_["u"], s_["q"])
    steps = 6
    sim.step(steps)
    eg, bg, jg = sim.fields()
    eo, bo, jo, ora = _oracle_run(oracle, g, p, e, b, species, dt, mask, steps)
    errs = {"E": _nerr(eg, eo), "B": _nerr(bg, bo), "J": _nerr(jg, jo)}
    for k, s_ in enumerate(ora):
        ix, x, u, q = sim.species(k)
        if engine == "plain":
            errs[f"x{k}"] = _nerr(ix + x, s_["ix"] + s_["x"])
            errs[f"u{k}"] = _nerr(u, s_["u"])
            assert np.array_equal(q == 0, s_["q"] == 0)
        else:
            live = s_["q"] != 0
            assert len(q) == int(live.sum())
            a = np.argsort(q, kind="stable")
            o = np.flatnonzero(live)[np.argsort(s_["q"][live], kind="stable")]
            errs[f"x{k}"] = _nerr(ix[a] + x[a], s_["ix"][o] + s_["x"][o])
            errs[f"u{k}"] = _nerr(u[a], s_["u"][o])
    sim.close()
    bad = {k: v for k, v in errs.items() if not v <= tol}
    assert not bad, (bad, errs)


@pytest.mark.parametrize("engine,prec", [("plain", 64), ("tiled", 32)])
def test_3d_spherical_pulse_leaves_through_pml_on_all_axes(osg, engine, prec):
    nx, dx = [24, 24, 16], [0.1] * 3
    dt = 0.9 / np.sqrt(sum(1 / d ** 2 for d in dx))
    sim = osg.Simulation(nx, dx, dt, order=2, precision=prec,
                         engine=osg.ENGINE_PLAIN if engine == "plain" else osg.ENGINE_TILED,
                         tile=[8, 8, 8] if engine == "tiled" else None, pml=7)
    gl, gu = osg.GUARD[2]
    dtype = np.float32 if prec == 32 else np.float64
    shape = tuple(reversed([n + gl + gu for n in nx])) + (3,)
    e, b = np.zeros(shape, dtype), np.zeros(shape, dtype)
    z, y, x = np.meshgrid(np.arange(shape[0]), np.arange(shape[1]), np.arange(shape[2]),
                          indexing="ij")
    az = np.exp(-((x - shape[2] / 2) ** 2 + (y - shape[1] / 2) ** 2 + (z - shape[0] / 2) ** 2) / 6.0)
    b[:, :-1, :, 0] = (az[:, 1:, :] - az[:, :-1, :]) / dx[1]
    b[:, :, :-1, 1] = -(az[:, :, 1:] - az[:, :, :-1]) / dx[0]
    sim.set_fields(e, b)
    empty = np.zeros((0, 3), np.int32), np.zeros((0, 3), dtype), np.zeros((0, 3), dtype), \
        np.zeros(0, dtype)
    sim.add_species(-1.0, *empty)
    sl = (slice(gl, gl + nx[2]), slice(gl, gl + nx[1]), slice(gl, gl + nx[0]))
    w0 = float((b[sl].astype(np.float64) ** 2).sum())
    sim.step(int(3 * max(nx) * dx[0] / dt))
    e1, b1, _ = sim.fields()
    w1 = float((e1[sl].astype(np.float64) ** 2).sum() + (b1[sl].astype(np.float64) ** 2).sum())
    assert w1 / w0 < 1e-4
    sim.close()


@pytest.mark.parametrize("axis", [0, 2])
def test_3d_plane_pulse_leaves_through_the_pml(osg, axis):
    nx = [8, 8, 8]
    nx[axis] = 96
    dx = [0.2] * 3
    dt = 0.9 / np.sqrt(sum(1 / d ** 2 for d in dx))
    sim = osg.Simulation(nx, dx, dt, order=2, precision=64, engine=osg.ENGINE_PLAIN,
                         pml=1 << axis)
    gl, gu = osg.GUARD[2]
    shape = tuple(reversed([n + gl + gu for n in nx])) + (3,)
    e, b = np.zeros(shape), np.zeros(shape)
    L = nx[axis] * dx[axis]
    i = np.arange(shape[2 - axis]) - gl
    prof = lambda x: np.exp(-((x - 0.5 * L) / (0.08 * L)) ** 2)
    shp = [1, 1, 1]
    shp[2 - axis] = shape[2 - axis]
    e[..., (axis + 1) % 3] = prof(i * dx[axis]).reshape(shp)
    b[..., (axis + 2) % 3] = prof((i + 0.5) * dx[axis]).reshape(shp)
    sim.set_fields(e, b)
    empty = np.zeros((0, 3), np.int32), np.zeros((0, 3)), np.zeros((0, 3)), np.zeros(0)
    sim.add_species(-1.0, *empty)
    sl = (slice(gl, gl + nx[2]), slice(gl, gl + nx[1]), slice(gl, gl + nx[0]))
    w0 = float((e[sl] ** 2).sum() + (b[sl] ** 2).sum())
    sim.step(int(L / dt))
    e1, b1, _ = sim.fields()
    assert float((e1[sl] ** 2).sum() + (b1[sl] ** 2).sum()) / w0 < 1e-4
    sim.close()


@pytest.mark.parametrize("dim,mask", [(2, 1), (2, 2), (2, 3), (3, 1), (3, 4), (3, 5), (3, 7)])
@pytest.mark.parametrize("what", [0, 1, 2])
@pytest.mark.parametrize("prec,tol", [(64, 1e-12), (32, 1e-6)])
def test_host_array_pml_phase_matches_oracle(osg, oracle, dim, mask, what, prec, tol):
    """One phase of osg_pml_* on host arrays against the oracle's phase, from random fields and
    random walls (the tables from the initialisation kept)."""
    nx = [10, 8] if dim == 2 else [8, 6, 7]
    g = oracle.Grid(nx, 2, [0.1, 0.12, 0.09][:dim])
    p = "f32" if prec == 32 else "f64"
    dt = 0.03
    rng = np.random.default_rng(7 + what + 3 * mask)
    st0 = oracle.pml_state(g, p, mask, NB, dt)
    nx_, gl, gu = g.args()
    st1 = osg.pml_state(dim, nx, gl, gu, mask, NB, g.dx, dt, st0.dtype)
    assert st1.shape == st0.shape
    assert _nerr(st1, st0) <= tol          # the same tables (computed in double)
    nwall = len(st0) - 12 * dim * NB
    st0[:nwall] = rng.standard_normal(nwall).astype(st0.dtype)
    st1[...] = st0
    e = rng.standard_normal(g.shape).astype(st0.dtype)
    b = rng.standard_normal(g.shape).astype(st0.dtype)
    eo, bo = e.copy(), b.copy()
    oracle.pml_phase(g, p, mask, NB, what, eo, bo, st0, dt)
    osg.pml(dim, nx, gl, gu, mask, NB, what, e, b, st1, g.dx, dt)
    errs = {"E": _nerr(e, eo), "B": _nerr(b, bo), "state": _nerr(st1, st0)}
    bad = {k: v for k, v in errs.items() if not v <= tol}
    assert not bad, (bad, errs)


@pytest.mark.parametrize("dim,mask,steps,tol", [(2, 2, 12, 1e-5), (2, 2, 24, 5e-5),
                                                (3, 6, 10, 5e-5)])
def test_window_with_transverse_pml_matches_oracle(osg, oracle, dim, mask, steps, tol):
    """Moving window along x1 with PML walls on the other axes, which shift with the fields on
    every move (move_window_vpml): tiled engine against the oracle's window and walls.  As in the
    window's own test, the cell-0 column the reference keeps one push longer and the band its
    current reaches are left out."""
    from test_gpu_configs import match_particles
    nx = [64, 16] if dim == 2 else [32, 8, 8]
    dx = [0.05] * dim
    dt = 0.035 if dim == 2 else 0.025
    edge = 24 if dim == 2 else 12
    ppc = [2] * dim
    L = nx[0] * dx[0]
    prof_x, prof_f = [0.5 * L, 0.8 * L, 1e6], [0.0, 1.0, 1.0]
    r = oracle.mt_new(7)
    ix, x, u, q = oracle.load(r, "f32", dim, nx, ppc, dx, -1.0, [0.05] * 3, [0.02, 0.0, 0.0])
    xg = (ix[:, 0].astype(np.float64) - 0.5 + x[:, 0]) * dx[0]
    den = np.interp(xg, prof_x, prof_f, left=0.0, right=1.0).astype(np.float32)
    keep = den > 0
    sp0 = dict(ix=np.ascontiguousarray(ix[keep]), x=np.ascontiguousarray(x[keep]),
               u=np.ascontiguousarray(u[keep]), q=np.ascontiguousarray(q[keep] * den[keep]),
               rqm=-1.0)
    g = oracle.Grid(nx, 2, dx)
    rng = np.random.default_rng(3)
    e0 = (rng.standard_normal(g.shape) * 0.02).astype(np.float32)
    b0 = (rng.standard_normal(g.shape) * 0.02).astype(np.float32)

    sim = osg.Simulation(nx, dx, dt, order=2, precision=32, engine=osg.ENGINE_TILED,
                         tile=[8] * dim, pml=mask)
    sim.set_fields(e0, b0)
    sim.add_species(-1.0, sp0["ix"], sp0["x"], sp0["u"], sp0["q"])
    sim.set_window(0, ppc, prof_x, prof_f)
    sim.step(steps)
    eg, bg, jg = sim.fields()
    gix, gx, gu, gq = sim.species(0)
    moves_gpu = sim.window_moves()
    sim.close()

    sp = [{k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in sp0.items()}]
    e, b, j = e0.copy(), b0.copy(), g.zeros("f32")
    st = oracle.pml_state(g, "f32", mask, NB, dt)
    win = oracle.Window(g, "f32", 0, ppc, prof_x, prof_f)
    for _ in range(steps):
        win.start_step(e, b, sp, dt, pml=(mask, NB, st))
        oracle.step(g, "f32", e, b, j, sp, dt, window=True, pml=(mask | 8, NB, st))
    win.start_step(e, b, sp, dt, pml=(mask, NB, st))
    assert win.moves == moves_gpu and moves_gpu > 0

    o = sp[0]
    live = (o["ix"][:, 0] != 0) & (o["q"] != 0)
    assert len(gq) == int(live.sum()), (len(gq), int(live.sum()))
    ref = (o["ix"][live], o["x"][live], o["u"][live])
    m, _ = match_particles(nx, ref, (gix, gx, gu))
    gix, gx, gu = gix[m], gx[m], gu[m]
    far = ref[0][:, 0] >= edge
    errs = {"x": _nerr((gix + gx)[far], (ref[0] + ref[1])[far]), "u": _nerr(gu[far], ref[2][far])}
    for name, a, c in (("E", eg, e), ("B", bg, b), ("J", jg, j)):
        ia, ic = g.interior(a), g.interior(c)
        errs[name] = _nerr(ia[..., edge - 1:, :], ic[..., edge - 1:, :])
    bad = {k: v for k, v in errs.items() if not v <= tol}
    assert not bad, (bad, errs)


@pytest.mark.parametrize("mask", [1, 2, 3])
@pytest.mark.parametrize("engine,prec,tol", [("plain", 64, 1e-12), ("tiled", 32, 5e-5)])
def test_pml_diffusion_matches_oracle(osg, oracle, engine, prec, tol, mask):
    """The walls' diffusion correction (pml_diffuse, 2D) against the oracle, 10 steps."""
    nx = [24, 16]
    p, g, dx, dt, species, e, b = _setup(oracle, prec, 2, 2, nx, [2, 2], 31, uth=0.6, ufl=0.1)
    sim = osg.Simulation(nx, dx, dt, order=2, precision=prec,
                         engine=osg.ENGINE_PLAIN if engine == "plain" else osg.ENGINE_TILED,
                         tile=[8, 8] if engine == "tiled" else None, pml=mask, pml_diffuse=mask)
    sim.set_fields(e, b)
    for s_ in species:
        sim.add_species(s_["rqm"], s_["ix"], s_["x"], s_["u"], s_["q"])
    sim.step(10)
    eg, bg, jg = sim.fields()
    sim.close()
    ora = [{k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in s_.items()}
           for s_ in species]
    eo, bo, jo = e.copy(), b.copy(), g.zeros(p)
    st = oracle.pml_state(g, p, mask, NB, dt)
    for _ in range(10):
        oracle.step(g, p, eo, bo, jo, ora, dt, pml=(mask | (mask << 4), NB, st))
    errs = {"E": _nerr(eg, eo), "B": _nerr(bg, bo), "J": _nerr(jg, jo)}
    bad = {k: v for k, v in errs.items() if not v <= tol}
    assert not bad, (bad, errs)
    # without the correction the fields differ
    sim = osg.Simulation(nx, dx, dt, order=2, precision=prec,
                         engine=osg.ENGINE_PLAIN if engine == "plain" else osg.ENGINE_TILED,
                         tile=[8, 8] if engine == "tiled" else None, pml=mask)
    sim.set_fields(e, b)
    for s_ in species:
        sim.add_species(s_["rqm"], s_["ix"], s_["x"], s_["u"], s_["q"])
    sim.step(10)
    assert _nerr(sim.fields()[1], bg) > 1e-8
    sim.close()
