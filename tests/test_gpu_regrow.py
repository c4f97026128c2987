"""GPU test of the tiled engine's slab growth under strong density bunching.

A cold 2D plasma converging on the box centre at 0.1 c piles up in the central tiles; with the
slabs sized tightly at the start (capacity 1.0: 1.25 x the initial fullest tile + 64 slots),
osg_sim_step must re-bin into larger slabs before any tile overflows (it checks the occupancy
every 8 steps and grows the slabs by 1.5x at least).  Every particle is kept and the final
occupancy stays below 1.
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


def test_converging_flow_regrows_slabs(osg):
    nx, dx, dt = [64, 64], [0.05, 0.05], 0.035
    ix, x, u, q = osg.load_lattice(osg.Rng(7), 32, nx, [2, 2], dx, -1.0, [0.0] * 3,
                                   [0.0] * 3)
    pos = (ix.astype(np.float64) - 0.5 + x) * np.asarray(dx)
    r = pos - 0.5 * np.asarray(nx) * np.asarray(dx)
    n = np.maximum(np.linalg.norm(r, axis=1, keepdims=True), 1e-9)
    u = np.zeros((len(q), 3), np.float32)
    u[:, :2] = (-0.1 * r / n).astype(np.float32)
    sim = osg.Simulation(nx, dx, dt, order=2, precision=32, engine=osg.ENGINE_TILED,
                         capacity=1.0)
    sim.add_species(-1.0, ix, x, u, q)
    sim.step(120)
    assert sim.num_particles(0) == len(q)
    assert sim.tile_occupancy() < 1.0
    jx, _, _, jq = sim.species(0)
    assert np.array_equal(np.sort(jq), np.sort(q))
    assert (jx >= 1).all() and (jx <= 64).all()
    sim.close()
