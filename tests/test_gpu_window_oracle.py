"""Moving window of the tiled engine against the oracle's restatement of the reference's window
(move_boundary_space_global, move_window_vdf, move_window_species and the injection of
inject_std; the x1 guards of E, B and J left as the shift and the Yee update leave them; the
lower x1 edge absorbing and the upper one reflecting): a warm plasma behind a density ramp in
random initial fields, 2D quadratic, FP32, 12 and 24 steps (8 and 17 window moves).

The two differ in one documented way: after a move the reference keeps the particles of the
old first cell column at cell index 0 for one more push (whose current lands in the guard cells
and the first two cells) and absorbs them after it, while the tiled engine drops them at the
move.  So the comparison leaves out that column and a band of cells near the lower edge that
its current reaches (the fields and the particles with x1 cell >= EDGE, in window coordinates):
there fields are within 1e-5 (12 steps) / 5e-5 (24 steps) of the FP32 oracle, normwise, the
particles (matched by nearest neighbour) within the same tolerances, and the particle counts
agree once the oracle's cell-0 column is set aside.
"""
import numpy as np
import pytest

from test_gpu_configs import match_particles
from test_gpu_step import _nerr

pytestmark = pytest.mark.gpu

NX, DX, DT, ORDER = [64, 16], [0.05, 0.05], 0.035, 2
EDGE = 24


@pytest.fixture(scope="module")
def osg():
    import __graft_entry__ as g
    g.build_native()
    import osiris_gb300
    if osiris_gb300.lib().osg_device_count() < 1:
        pytest.fail("no CUDA device visible")
    return osiris_gb300


@pytest.mark.parametrize("steps,tol", [(12, 1e-5), (24, 5e-5)])
def test_window_matches_oracle(osg, oracle, steps, tol):
    L = NX[0] * DX[0]
    prof_x, prof_f = [0.5 * L, 0.8 * L, 1e6], [0.0, 1.0, 1.0]
    r = oracle.mt_new(7)
    ix, x, u, q = oracle.load(r, "f32", 2, NX, [2, 2], DX, -1.0, [0.05] * 3, [0.02, 0.0, 0.0])
    xg = (ix[:, 0].astype(np.float64) - 0.5 + x[:, 0]) * DX[0]
    den = np.interp(xg, prof_x, prof_f, left=0.0, right=1.0).astype(np.float32)
    keep = den > 0
    sp0 = dict(ix=np.ascontiguousarray(ix[keep]), x=np.ascontiguousarray(x[keep]),
               u=np.ascontiguousarray(u[keep]), q=np.ascontiguousarray(q[keep] * den[keep]),
               rqm=-1.0)
    g = oracle.Grid(NX, ORDER, DX)
    rng = np.random.default_rng(3)
    e0 = (rng.standard_normal(g.shape) * 0.02).astype(np.float32)
    b0 = (rng.standard_normal(g.shape) * 0.02).astype(np.float32)

    sim = osg.Simulation(NX, DX, DT, order=ORDER, precision=32, engine=osg.ENGINE_TILED,
                         tile=[8, 8])
    sim.set_fields(e0, b0)
    sim.add_species(-1.0, sp0["ix"], sp0["x"], sp0["u"], sp0["q"])
    sim.set_window(0, [2, 2], prof_x, prof_f)
    sim.step(steps)
    eg, bg, jg = sim.fields()
    gix, gx, gu, gq = sim.species(0)
    moves_gpu = sim.window_moves()
    sim.close()

    sp = [{k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in sp0.items()}]
    e, b, j = e0.copy(), b0.copy(), g.zeros("f32")
    win = oracle.Window(g, "f32", 0, [2, 2], prof_x, prof_f)
    for _ in range(steps):
        win.start_step(e, b, sp, DT)
        oracle.step(g, "f32", e, b, j, sp, DT, window=True)
    # the tiled engine applies the next step's move at the end of the last one
    win.start_step(e, b, sp, DT)
    assert win.moves == moves_gpu and moves_gpu > 0

    o = sp[0]
    at0 = o["ix"][:, 0] == 0
    assert len(gq) == int((~at0).sum()), (len(gq), len(o["q"]), int(at0.sum()))
    ref = (o["ix"][~at0], o["x"][~at0], o["u"][~at0])
    m, _ = match_particles(NX, ref, (gix, gx, gu))
    gix, gx, gu, gq = gix[m], gx[m], gu[m], gq[m]
    assert np.array_equal(gq, o["q"][~at0])
    far = ref[0][:, 0] >= EDGE
    errs = {"x": _nerr((gix + gx)[far], (ref[0] + ref[1])[far]), "u": _nerr(gu[far], ref[2][far])}
    for name, a, c in (("E", eg, e), ("B", bg, b), ("J", jg, j)):
        ia, ic = g.interior(a), g.interior(c)
        errs[name] = _nerr(ia[:, EDGE - 1:], ic[:, EDGE - 1:])
    print(steps, moves_gpu, errs)
    bad = {k: v for k, v in errs.items() if not v <= tol}
    assert not bad, (bad, errs)
