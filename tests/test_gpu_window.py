"""GPU tests of the moving window (osg_sim_set_window, tiled engine) and of the laser launch
in a running simulation.

* a cold plasma in zero fields does not move: after the window has moved k cells, the particles
  sit exactly on the OSIRIS lattice of global cells k+1 .. k+nx (old columns dropped, new
  columns injected), the count and the charges are kept, the fields stay zero, and k follows
  the reference's rule (dt added per step, one cell per dx);
* injection into an empty box follows the piecewise-linear profile: the charge of every
  injected particle is sign(1/ppc) * den(global x1);
* a laser pulse in vacuum rides with a window moving at c: its envelope stays at the same
  window position (within 3 cells over 150 steps) and the field energy stays within 2%.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def osg():
    import __graft_entry__ as g
    g.build_native()
    import osiris_gb300
    if osiris_gb300.lib().osg_device_count() < 1:
        pytest.fail("no CUDA device visible")
    return osiris_gb300


def _expected_moves(dt, dx, steps):
    xm, k = dt, 0
    for _ in range(steps):
        xm += dt
        if xm >= dx:
            xm -= dx
            k += 1
    return k


def test_window_shifts_cold_plasma_exactly(osg):
    nx, dx, dt = [64, 16], [0.05, 0.05], 0.035
    sim = osg.Simulation(nx, dx, dt, order=2, precision=32, engine=osg.ENGINE_TILED, tile=[8, 8])
    r = osg.Rng(1)
    ix, x, u, q = osg.load_lattice(r, 32, nx, [2, 2], dx, -1.0, [0.0] * 3, [0.0] * 3)
    sim.add_species(-1.0, ix, x, u, q)
    sim.set_window(0, [2, 2], [-1e6, 1e6], [1.0, 1.0])
    steps = 20
    sim.step(steps)
    k = sim.window_moves()
    assert k == _expected_moves(dt, dx[0], steps) and k > 0
    gix, gx, gu, gq = sim.species(0)
    assert len(gq) == len(q)
    assert not np.any(gu) and np.all(gq == q[0])
    got = sorted(zip((gix[:, 0] + k).tolist(), gix[:, 1].tolist(), gx[:, 0].tolist(),
                     gx[:, 1].tolist()))
    want = sorted(zip((ix[:, 0] + k).tolist(), ix[:, 1].tolist(), x[:, 0].tolist(),
                      x[:, 1].tolist()))
    # the same lattice, translated by k cells in global coordinates
    assert got == want
    e, b, j = sim.fields()
    assert not np.any(e) and not np.any(b)
    sim.close()


def test_window_injects_profile(osg):
    nx, dx, dt = [32, 16], [0.05, 0.05], 0.035
    sim = osg.Simulation(nx, dx, dt, order=2, precision=32, engine=osg.ENGINE_TILED, tile=[8, 8])
    empty = np.zeros((0, 2), np.int32), np.zeros((0, 2), np.float32), \
        np.zeros((0, 3), np.float32), np.zeros(0, np.float32)
    sim.add_species(-1.0, *empty)
    L = nx[0] * dx[0]
    px, pf = [L + 0.1, L + 0.6, 1e6], [0.0, 2.0, 2.0]      # ramp over 10 cells, then flat
    sim.set_window(0, [2, 1], px, pf)
    for _ in range(40):
        sim.step(1)
    k = sim.window_moves()
    ix, x, u, q = sim.species(0)
    assert len(q) > 0
    xg = (ix[:, 0].astype(np.float64) + k - 0.5 + x[:, 0].astype(np.float64)) * dx[0]
    den = np.interp(xg, px, pf, left=0.0, right=2.0).astype(np.float32)
    assert np.all(den > 0)
    assert np.allclose(q, -den * np.float32(0.5), rtol=2e-6, atol=0)
    # every injected column holds ny x ppc particles (where the profile is positive)
    cols = np.unique(ix[:, 0] + k)
    assert len(q) == len(cols) * nx[1] * 2
    sim.close()


def test_laser_rides_with_the_window(osg):
    nx, dx, dt, order = [320, 48], [0.2, 0.6], 0.18, 2
    sim = osg.Simulation(nx, dx, dt, order=order, precision=32, engine=osg.ENGINE_TILED,
                         tile=[16, 8])
    gl, gu = osg.GUARD[order]
    shape = tuple(reversed([n + gl + gu for n in nx])) + (3,)
    e, b = np.zeros(shape, np.float32), np.zeros(shape, np.float32)
    osg.zpulse_launch(order, nx, dx, [0.0, 0.0], e, b, omega0=1.0, a0=0.1, pol=0.0,
                      lon_x0=40.0, lon_duration=6.0, lon_range=30.0, per_w0=6.0,
                      per_focus=50.0, per_center=(nx[1] * dx[1] / 2, 0.0))
    sim.set_fields(e, b)
    empty = np.zeros((0, 2), np.int32), np.zeros((0, 2), np.float32), \
        np.zeros((0, 3), np.float32), np.zeros(0, np.float32)
    sim.add_species(-1.0, *empty)
    sim.set_window(0, [1, 1], [0.0, 1.0], [0.0, 0.0])      # vacuum: nothing injected

    def env_peak(f):
        prof = (f[gl:gl + nx[1], gl:gl + nx[0], 1].astype(np.float64) ** 2).sum(axis=0)
        c = np.convolve(prof, np.ones(15) / 15, mode="same")
        return int(np.argmax(c))

    def energy(fe, fb):
        return float((fe.astype(np.float64) ** 2).sum() + (fb.astype(np.float64) ** 2).sum())

    p0, w0 = env_peak(e), energy(e, b)
    sim.step(150)
    e1, b1, _ = sim.fields()
    assert sim.window_moves() > 120
    assert abs(env_peak(e1) - p0) <= 3
    assert abs(energy(e1, b1) / w0 - 1.0) < 0.02
    sim.close()
