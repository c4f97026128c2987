"""The tiled engine's precision pattern on the GPU: FP32 particles and current with a two-sum
compensated tile current and a deterministic FP64 re-summation of the tile currents in tile
order, and the exact pusher inside the tiled push.

* exact pusher, tiled FP32 engine: 1 and 10 steps against the oracle (same tolerances as the
  Boris tests: 1e-5 and 5e-5 normwise);
* compensation: 1000 identical particles in one cell deposit exactly 1000 times the current of
  one of them (the correctly rounded FP32 value; a plain FP32 running sum is off by several
  ulps);
* reproducibility: two runs from the same load agree to 1e-6 (normwise) after 5 steps.  The
  tile flush is deterministic; inside a tile the FP32 sums of a warp's lanes depend on which
  particles share a warp iteration, which follows the order particles arrive in their tile.
"""
import numpy as np
import pytest

from test_gpu_step import _compare, _setup

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def osg():
    import __graft_entry__ as g
    g.build_native()
    import osiris_gb300
    if osiris_gb300.lib().osg_device_count() < 1:
        pytest.fail("no CUDA device visible")
    return osiris_gb300


@pytest.mark.parametrize("steps,tol", [(1, 1e-5), (10, 5e-5)])
@pytest.mark.parametrize("dim,order,nx,tile", [(2, 2, [32, 24], [8, 8]), (2, 3, [16, 16], [8, 4]),
                                               (3, 2, [16, 8, 8], [4, 4, 4])])
def test_tiled_exact_pusher_matches_oracle(osg, oracle, dim, order, nx, tile, steps, tol):
    _compare(osg, oracle, 32, osg.ENGINE_TILED, dim, order, nx, [2] * dim, steps, tol,
             tile=tile, pusher="exact")


def _identical(osg, n, order=2):
    nx, dx, dt = [16, 16], [0.05, 0.05], 0.035
    sim = osg.Simulation(nx, dx, dt, order=order, precision=32, engine=osg.ENGINE_TILED,
                         tile=[8, 8])
    ix = np.tile(np.array([[6, 5]], np.int32), (n, 1))
    x = np.tile(np.array([[0.125, -0.3125]], np.float32), (n, 1))
    u = np.tile(np.array([[0.3, 0.1, 0.05]], np.float32), (n, 1))
    q = np.full(n, -1.0 / 1024, np.float32)
    sim.add_species(-1.0, ix, x, u, q)
    sim.step(1)
    _, _, j = sim.fields()
    sim.close()
    return j


def test_compensated_tile_current_is_correctly_rounded(osg):
    j1 = _identical(osg, 1).astype(np.float64)
    j1000 = _identical(osg, 1000)
    nz = j1 != 0
    assert nz.sum() >= 20
    want = (1000.0 * j1).astype(np.float32)
    assert np.array_equal(j1000[nz], want[nz])
    assert not np.any(j1000[~nz])


def test_tiled_step_is_reproducible(osg, oracle):
    p, g, dx, dt, species, e, b = _setup(oracle, 32, 2, 2, [64, 48], [4, 4], seed=12, uth=0.3)
    out = []
    for _ in range(2):
        sim = osg.Simulation([64, 48], dx, dt, order=2, precision=32, engine=osg.ENGINE_TILED,
                             tile=[8, 8])
        sim.set_fields(e, b)
        for s in species:
            sim.add_species(s["rqm"], s["ix"], s["x"], s["u"], s["q"])
        sim.step(5)
        out.append(sim.fields())
        sim.close()
    for a, c in zip(out[0], out[1]):
        a, c = a.astype(np.float64), c.astype(np.float64)
        assert np.abs(a - c).max() <= 1e-6 * np.abs(c).max()
