"""The oracle's moving window (pyoracle.Window with step(..., window=True)), on the CPU:

* the window moves one cell each time the accumulated dt reaches dx1 (dt added at the start of
  every step, as move_boundary_space_global);
* a cold plasma at rest in zero fields stays on the OSIRIS lattice: after k moves the particles
  fill global cells k + 1 .. k + nx (the column shifted to cell 0 is absorbed by the push that
  follows, the new last column injected), with the profile's charge;
* a move shifts E and B one cell down along x1, guard cells included, and zeroes the last
  plane;
* particles leaving through the upper x1 edge are reflected, those below cell 1 absorbed.
"""
import numpy as np


def _cold(oracle, nx, dx):
    r = oracle.mt_new(1)
    ix, x, u, q = oracle.load(r, "f64", 2, nx, [2, 2], dx, -1.0, [0.0] * 3, [0.0] * 3)
    return dict(ix=ix, x=x, u=u, q=q, rqm=-1.0)


def test_window_moves_and_keeps_the_lattice(oracle):
    nx, dx, dt = [16, 8], [0.05, 0.05], 0.035
    g = oracle.Grid(nx, 2, dx)
    sp = [_cold(oracle, nx, dx)]
    ix0, x0 = sp[0]["ix"].copy(), sp[0]["x"].copy()
    e, b, j = g.zeros("f64"), g.zeros("f64"), g.zeros("f64")
    win = oracle.Window(g, "f64", 0, [2, 2], [-1e6, 1e6], [1.0, 1.0])
    moves, xm = 0, 0.0
    for _ in range(20):
        xm += dt
        if xm >= dx[0]:
            xm -= dx[0]
            moves += 1
        win.start_step(e, b, sp, dt)
        oracle.step(g, "f64", e, b, j, sp, dt, window=True)
    assert win.moves == moves > 0
    got = sorted(zip((sp[0]["ix"][:, 0] + moves).tolist(), sp[0]["ix"][:, 1].tolist(),
                     sp[0]["x"][:, 0].tolist(), sp[0]["x"][:, 1].tolist()))
    want = sorted(zip((ix0[:, 0] + moves).tolist(), ix0[:, 1].tolist(), x0[:, 0].tolist(),
                      x0[:, 1].tolist()))
    assert got == want
    assert np.all(sp[0]["q"] == sp[0]["q"][0]) and not np.any(sp[0]["u"])
    assert not np.any(e) and not np.any(b)


def test_window_shift_of_the_fields(oracle):
    nx, dx = [12, 6], [0.05, 0.05]
    g = oracle.Grid(nx, 2, dx)
    rng = np.random.default_rng(0)
    e = rng.standard_normal(g.shape)
    b = rng.standard_normal(g.shape)
    e0, b0 = e.copy(), b.copy()
    win = oracle.Window(g, "f64", 0, [1, 1], [0.0, 1.0], [0.0, 0.0])
    sp = [dict(ix=np.zeros((0, 2), np.int32), x=np.zeros((0, 2)), u=np.zeros((0, 3)),
               q=np.zeros(0), rqm=-1.0)]
    assert not win.start_step(e, b, sp, 0.02)
    assert win.start_step(e, b, sp, 0.04)
    for f, f0 in ((e, e0), (b, b0)):
        assert np.array_equal(f[..., :-1, :], f0[..., 1:, :])
        assert not np.any(f[..., -1, :])


def test_window_particle_edges(oracle):
    nx, dx, dt = [8, 4], [0.1, 0.1], 0.05
    g = oracle.Grid(nx, 2, dx)
    sp = [dict(ix=np.array([[8, 2], [1, 3], [4, 2]], np.int32),
               x=np.array([[0.45, 0.0], [-0.45, 0.0], [0.0, 0.0]]),
               u=np.array([[5.0, 0.0, 0.0], [-5.0, 0.0, 0.0], [0.0, 0.0, 0.0]]),
               q=np.array([-0.1, -0.2, -0.3]), rqm=-1.0)]
    e, b, j = g.zeros("f64"), g.zeros("f64"), g.zeros("f64")
    oracle.step(g, "f64", e, b, j, sp, dt, window=True)
    # the second particle left below cell 1: absorbed; the first crossed nx: reflected
    assert len(sp[0]["q"]) == 2 and np.array_equal(sp[0]["q"], [-0.1, -0.3])
    # (it reached cell 9 at offset -0.06: back in cell 8 at +0.06, u1 reversed)
    assert sp[0]["ix"][0, 0] == 8 and sp[0]["u"][0, 0] < 0 and 0 < sp[0]["x"][0, 0] < 0.1
