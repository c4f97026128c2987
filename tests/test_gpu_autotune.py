"""GPU tests of the single-box autotuner (osg_sim_autotune).

* tiled engine, 2D and 3D: the tuner picks one of its candidate tile shapes and CTA sizes, and
  a run started after tuning evolves as a fresh run built with the chosen tile shape: fields
  within 1e-5 normwise after 6 steps (the tile shape changes only the order of FP32 sums),
  the same particle count, kinetic energies within 1e-5.  That also shows the tuner put the
  state back after its trial steps;
* plain engine (FP64): the tuner returns a cell-sort interval (0 = never) and the tuned run
  matches a fresh run with that interval to 1e-12;
* the tuner refuses to run after the first step.
"""
import numpy as np
import pytest

from test_gpu_configs import _nerr

pytestmark = pytest.mark.gpu

DT = {2: 0.035, 3: 0.025}   # below the Courant limit of dx = 0.05 (2D 0.0354, 3D 0.0289)


@pytest.fixture(scope="module")
def osg():
    import __graft_entry__ as g
    g.build_native()
    import osiris_gb300
    if osiris_gb300.lib().osg_device_count() < 1:
        pytest.fail("no CUDA device visible")
    return osiris_gb300


def _species(osg, nx, ppc, prec, seed=5):
    r = osg.Rng(seed)
    return [osg.load_lattice(r, prec, nx, ppc, [0.05] * len(nx), -1.0, [0.05] * 3,
                             [s * 0.1, 0.0, 0.0], 1e-2, 1.0) for s in (1.0, -1.0)]


def _sim(osg, nx, order, prec, engine, sp, **kw):
    sim = osg.Simulation(nx, [0.05] * len(nx), DT[len(nx)], order=order, precision=prec,
                         engine=engine, **kw)
    for s in sp:
        sim.add_species(-1.0, *s)
    return sim


@pytest.mark.parametrize("nx,order,ppc,cands", [
    ([64, 64], 2, [4, 4], ([8, 8], [16, 8], [8, 4], [16, 16])),
    ([24, 24, 24], 3, [2, 2, 2], ([8, 8, 4], [8, 4, 4], [4, 4, 4], [8, 8, 8])),
])
def test_tiled_autotune_matches_fresh_run(osg, nx, order, ppc, cands):
    sp = _species(osg, nx, ppc, 32)
    a = _sim(osg, nx, order, 32, osg.ENGINE_TILED, sp)
    choice = a.autotune(steps=3)
    assert choice["tile"] in [list(c) for c in cands], choice
    assert choice["threads"] in (128, 256)
    a.step(6)
    b = _sim(osg, nx, order, 32, osg.ENGINE_TILED, sp, tile=choice["tile"])
    b.step(6)
    for fa, fb in zip(a.fields(), b.fields()):
        assert _nerr(fa, fb) <= 1e-5, _nerr(fa, fb)
    for k in range(2):
        assert a.num_particles(k) == b.num_particles(k) == len(sp[k][3])
    ka, _ = a.energy()
    kb, _ = b.energy()
    assert np.allclose(ka, kb, rtol=1e-5)
    a.close()
    b.close()


def test_plain_autotune_sort_interval(osg):
    nx = [48, 48]
    sp = _species(osg, nx, [4, 4], 64)
    a = _sim(osg, nx, 2, 64, osg.ENGINE_PLAIN, sp)
    choice = a.autotune(steps=8)
    n_sort = choice["n_sort"]
    assert n_sort >= 0 and choice["threads"] == 0
    a.step(6)
    b = _sim(osg, nx, 2, 64, osg.ENGINE_PLAIN, sp, n_sort=n_sort)
    b.step(6)
    for fa, fb in zip(a.fields(), b.fields()):
        assert _nerr(fa, fb) <= 1e-12, _nerr(fa, fb)
    ka, _ = a.energy()
    kb, _ = b.energy()
    assert np.allclose(ka, kb, rtol=1e-12)
    a.close()
    b.close()


def test_autotune_only_before_first_step(osg):
    nx = [32, 32]
    sim = _sim(osg, nx, 2, 32, osg.ENGINE_TILED, _species(osg, nx, [2, 2], 32))
    sim.step(1)
    with pytest.raises(Exception):
        sim.autotune(steps=3)
    sim.close()
