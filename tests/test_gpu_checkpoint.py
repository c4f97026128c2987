"""GPU tests of checkpoint / restart of the device-resident simulation (osg_sim_checkpoint,
osg_sim_restore; the role of the reference's write_restart / read_restart,
source/os-main.f03:299-343):

* a restored simulation holds exactly the checkpointed state (every particle, E and B);
* continuing it gives the run that was never interrupted: FP64 plain engine to 1e-12 (the
  current's atomic sums are the only difference), FP32 tiled engine with current smoothing to
  1e-5, and the moving window keeps its count of moves and its injection (a cold plasma stays
  exactly on the lattice);
* a truncated file or a file that is not a checkpoint is refused with an error.
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


def _state(sim):
    e, b, _ = sim.fields()
    sp = []
    for k in range(sim.nspecies):
        ix, x, u, q = sim.species(k)
        o = np.argsort(q, kind="stable")
        sp.append((ix[o], x[o], u[o], q[o]))
    return e, b, sp


def _build(osg, oracle, prec, engine, smooth):
    dim, order, nx = 2, 2, [32, 24]
    p, g, dx, dt, species, e, b = _setup(oracle, prec, dim, order, nx, [2, 2], 7)
    sim = osg.Simulation(nx, dx, dt, order=order, precision=prec, engine=engine,
                         tile=[8, 8] if engine == osg.ENGINE_TILED else None,
                         smooth_type=osg.SMOOTH_BINOMIAL if smooth else osg.SMOOTH_NONE,
                         smooth_order=1 if smooth else 0)
    ge, gb = (np.zeros(sim.grid_shape, sim.dtype) for _ in range(2))
    gl = sim.gcl[0]
    # the oracle's fields, placed into the (possibly wider) guard frame of the simulation
    og = g.gcl[0]
    ge[gl - og:gl - og + e.shape[0], gl - og:gl - og + e.shape[1]] = e
    gb[gl - og:gl - og + b.shape[0], gl - og:gl - og + b.shape[1]] = b
    sim.set_fields(ge, gb)
    for s in species:
        sim.add_species(s["rqm"], s["ix"], s["x"], s["u"], s["q"])
    return sim


@pytest.mark.parametrize("prec,engine,smooth,tol", [(64, "plain", False, 1e-12),
                                                    (32, "tiled", True, 1e-5)])
def test_restart_continues_the_run(osg, oracle, tmp_path, prec, engine, smooth, tol):
    eng = osg.ENGINE_PLAIN if engine == "plain" else osg.ENGINE_TILED
    sim = _build(osg, oracle, prec, eng, smooth)
    sim.step(4)
    path = tmp_path / "state.ckpt"
    sim.checkpoint(path)
    saved = _state(sim)
    sim.step(4)
    full = _state(sim)
    kin_full, fld_full = sim.energy()
    sim.close()

    rs = osg.Simulation.restore(path)
    assert rs.nspecies == 2 and rs.dim == 2 and rs.precision == prec
    now = _state(rs)
    for a, c in zip(now[:2], saved[:2]):
        assert np.array_equal(a, c)
    for sa, sc in zip(now[2], saved[2]):
        for a, c in zip(sa, sc):
            assert np.array_equal(a, c)
    rs.step(4)
    cont = _state(rs)
    kin, fld = rs.energy()
    rs.close()
    for a, c in zip(cont[:2], full[:2]):
        assert _nerr(a, c) <= tol
    for sa, sc in zip(cont[2], full[2]):
        assert np.array_equal(sa[3], sc[3])
        assert _nerr(sa[0] + sa[1], sc[0] + sc[1]) <= tol
        assert _nerr(sa[2], sc[2]) <= tol
    assert np.allclose(kin, kin_full, rtol=10 * tol, atol=0)


def test_restart_keeps_the_moving_window(osg, tmp_path):
    nx, dx, dt = [48, 16], [0.05, 0.05], 0.035
    sim = osg.Simulation(nx, dx, dt, order=2, precision=32, engine=osg.ENGINE_TILED, tile=[8, 8])
    r = osg.Rng(2)
    ix, x, u, q = osg.load_lattice(r, 32, nx, [2, 2], dx, -1.0, [0.0] * 3, [0.0] * 3)
    sim.add_species(-1.0, ix, x, u, q)
    sim.set_window(0, [2, 2], [-1e6, 1e6], [1.0, 1.0])
    sim.step(15)
    path = tmp_path / "win.ckpt"
    sim.checkpoint(path)
    sim.step(15)
    k_full = sim.window_moves()
    full = _state(sim)
    sim.close()
    rs = osg.Simulation.restore(path)
    rs.step(15)
    assert rs.window_moves() == k_full and k_full > 0
    cont = _state(rs)
    rs.close()
    key = lambda s: sorted(zip(s[0][:, 0].tolist(), s[0][:, 1].tolist(), s[1][:, 0].tolist(),
                               s[1][:, 1].tolist()))
    assert len(cont[2][0][3]) == len(full[2][0][3])
    assert key(cont[2][0]) == key(full[2][0])
    assert not np.any(cont[0]) and not np.any(cont[1])


def test_restore_refuses_bad_files(osg, tmp_path):
    nx = [16, 16]
    sim = osg.Simulation(nx, [0.1, 0.1], 0.05, order=2, precision=32, engine=osg.ENGINE_TILED,
                         tile=[8, 8])
    r = osg.Rng(3)
    sim.add_species(-1.0, *osg.load_lattice(r, 32, nx, [2, 2], [0.1, 0.1], -1.0, [0.1] * 3,
                                            [0.0] * 3))
    good = tmp_path / "good.ckpt"
    sim.checkpoint(good)
    sim.close()
    data = good.read_bytes()
    (tmp_path / "short.ckpt").write_bytes(data[: len(data) // 2])
    (tmp_path / "other.ckpt").write_bytes(b"not a checkpoint" * 8)
    for name in ("short.ckpt", "other.ckpt", "missing.ckpt"):
        with pytest.raises(osg.OsirisGB300Error):
            osg.Simulation.restore(tmp_path / name)
    osg.Simulation.restore(good).close()
