"""GPU tests of the thermal-bath particle boundary in the tiled engine (tiled_reemit).

The tiled engine keys its bath draws by tile slot instead of particle index, so its random
stream is not the plain engine's.  Two kinds of check:

* a nearly cold bath with no fluid momentum (uth_bnd 1e-6) makes every re-emission all but
  deterministic (the edge cell, offset -1/2 or just below 1/2, momenta of order 1e-6): the
  tiled FP32 engine then matches the plain FP32 engine, which is pinned to the oracle, after 10
  steps -- fields, and every particle (matched by its distinct charge) within 1e-4 normwise.
  This covers the edge cell and offset, the momenta, the current of the way in (-q back along
  the new momentum) and the migration of re-emitted particles between tiles, in 2D and 3D, on
  walled and open (Lindman) axes.  (A fluid momentum would make the offset depend on the
  uniform draw, u_d / gamma dt/dx_d v, so the two streams would place particles differently.);
* a hot bath (uth_bnd 0.3, with and without a fluid momentum): no particle is lost, every cell
  index stays in the box, and the kinetic energy after 60 steps matches the plain engine's
  within 5%;
* the bath needs the Boris pusher in the tiled engine.
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


def _run(osg, engine, dim, nx, dx, dt, species, e, b, walls, oax, mask, uth, ufl, steps,
         order=2):
    sim = osg.Simulation(nx, dx, dt, order=order, precision=32, engine=engine, walls=walls,
                         open_fields=0 if oax is None else 1 << oax, thermal=mask,
                         uth_bnd=uth, ufl_bnd=ufl, seed=77, capacity=4.0)
    sim.set_fields(e, b)
    for s in species:
        sim.add_species(s["rqm"], s["ix"], s["x"], s["u"], s["q"])
    sim.step(steps)
    out = (sim.fields(), [sim.species(k) for k in range(len(species))], sim.energy()[0])
    sim.close()
    return out


CASES = [  # dim, walls, open axis, thermal mask, ufl
    (2, 1, None, 1, (0.0, 0.0, 0.0)),
    (2, 3, None, 3, (0.0, 0.0, 0.0)),
    (2, 0, 1, 2, (0.0, 0.0, 0.0)),
    (3, 5, None, 5, (0.0, 0.0, 0.0)),
    (3, 2, None, 2, (0.0, 0.0, 0.0)),
]


@pytest.mark.parametrize("dim,walls,oax,mask,ufl", CASES)
def test_cold_bath_tiled_matches_plain(osg, oracle, dim, walls, oax, mask, ufl):
    nx = [24, 16] if dim == 2 else [8, 8, 8]
    p, g, dx, dt, species, e, b = _setup(oracle, 32, dim, 2, nx, [2] * dim, 23, uth=0.6,
                                         ufl=0.1)
    uth = (1e-6, 1e-6, 1e-6)
    ref = _run(osg, osg.ENGINE_PLAIN, dim, nx, dx, dt, species, e, b, walls, oax, mask, uth,
               ufl, 10)
    got = _run(osg, osg.ENGINE_TILED, dim, nx, dx, dt, species, e, b, walls, oax, mask, uth,
               ufl, 10)
    errs = {}
    for name, a, c in zip("EBJ", got[0], ref[0]):
        errs[name] = _nerr(g.interior(a), g.interior(c))
    for k in range(2):
        ix, x, u, q = got[1][k]
        rix, rx, ru, rq = ref[1][k]
        assert len(q) == len(rq)
        assert ix.min() >= 1 and np.all(ix.max(axis=0) <= np.array(nx))
        o, ro = np.argsort(q), np.argsort(rq)
        assert np.array_equal(q[o], rq[ro])
        errs[f"x{k}"] = _nerr((ix + x)[o], (rix + rx)[ro])
        errs[f"u{k}"] = _nerr(u[o], ru[ro])
    bad = {k: v for k, v in errs.items() if not v <= 1e-4}
    assert not bad, (bad, errs)


@pytest.mark.parametrize("dim,ufl", [(2, (0.0, 0.0, 0.0)), (3, (0.0, 0.0, 0.0)),
                                     (2, (0.05, 0.1, -0.1))])
def test_hot_bath_tiled_statistics(osg, oracle, dim, ufl):
    nx = [32, 16] if dim == 2 else [16, 8, 8]
    p, g, dx, dt, species, e, b = _setup(oracle, 32, dim, 2, nx, [3] * dim, 31, uth=0.05,
                                         ufl=0.3)
    e[...] = 0
    b[...] = 0
    uth = (0.3, 0.3, 0.3)
    kin = {}
    for name, eng in (("plain", osg.ENGINE_PLAIN), ("tiled", osg.ENGINE_TILED)):
        fields, sp, k = _run(osg, eng, dim, nx, dx, dt, species, e, b, 1, None, 1, uth, ufl,
                             60)
        for s, s0 in zip(sp, species):
            ix, x, u, q = s
            assert len(q) == len(s0["q"])
            assert ix.min() >= 1 and np.all(ix.max(axis=0) <= np.array(nx))
            if any(ufl):
                # the fluid boost can turn the normal momentum outwards: the reference's
                # placement xpos + u_d / gamma dt/dx_d v then lies a little past the edge
                # offset (both engines, as the oracle)
                assert (np.abs(x) < 1.0).all()
            else:
                assert (x >= -0.5).all() and (x < 0.5).all()
        kin[name] = float(np.sum(k))
    assert abs(kin["tiled"] - kin["plain"]) <= 0.05 * abs(kin["plain"]), kin


def test_tiled_bath_needs_boris(osg):
    with pytest.raises(osg.OsirisGB300Error):
        osg.Simulation([16, 16], [0.1, 0.1], 0.03, order=2, precision=32,
                       engine=osg.ENGINE_TILED, walls=1, thermal=1, uth_bnd=(0.1, 0.1, 0.1),
                       pusher=osg.PUSHER_VAY)
