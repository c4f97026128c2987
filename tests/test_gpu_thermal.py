"""GPU parity of the thermal-bath particle boundary (osg_config.thermal, plain engine) against
the oracle's step: particles crossing a walled or open edge are re-emitted at the edge cell with
momenta from the bath (one Philox4x32-10 draw per re-emission, keyed by seed, species, particle,
step, axis and side) and the current of their way in.  2D and 3D, FP64 1e-12 and FP32 5e-5
after 10 steps, conducting walls and Lindman open edges, with and without a fluid momentum."""
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


CASES = [  # dim, prec, walls, open axis, thermal mask, ufl, thermal type
    (2, 64, 1, None, 1, (0.0, 0.0, 0.0), 0),
    (2, 64, 3, None, 3, (0.05, 0.1, -0.1), 0),
    (2, 32, 2, None, 2, (0.0, 0.0, 0.0), 0),
    (2, 64, 0, 0, 1, (0.0, 0.0, 0.0), 0),
    (2, 32, 0, 1, 2, (0.05, 0.1, -0.1), 0),
    (3, 64, 5, None, 5, (0.0, 0.0, 0.0), 0),
    (2, 64, 3, None, 3, (0.0, 0.0, 0.0), 1),
    (2, 32, 1, None, 1, (0.0, 0.0, 0.0), 2),
    (3, 64, 2, None, 2, (0.0, 0.0, 0.0), 2),
]


@pytest.mark.parametrize("dim,prec,walls,oax,mask,ufl,ttype", CASES)
def test_thermal_bath_matches_oracle(osg, oracle, dim, prec, walls, oax, mask, ufl, ttype):
    nx = [20, 16] if dim == 2 else [10, 9, 8]
    p, g, dx, dt, species, e, b = _setup(oracle, prec, dim, 2, nx, [2] * dim, 21, uth=0.6,
                                         ufl=0.1)
    uth = (0.3, 0.2, 0.25)
    sim = osg.Simulation(nx, dx, dt, order=2, precision=prec, engine=osg.ENGINE_PLAIN,
                         walls=walls, open_fields=0 if oax is None else 1 << oax, thermal=mask,
                         uth_bnd=uth, ufl_bnd=ufl, seed=77, thermal_type=ttype)
    sim.set_fields(e, b)
    for s in species:
        sim.add_species(s["rqm"], s["ix"], s["x"], s["u"], s["q"])
    steps = 10
    sim.step(steps)
    eg, bg, jg = sim.fields()
    ora = [{k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in s.items()}
           for s in species]
    eo, bo, jo = e.copy(), b.copy(), g.zeros(p)
    st = None if oax is None else oracle.lindman_state(g, p, oax)
    for k in range(steps):
        oracle.step(g, p, eo, bo, jo, ora, dt, walls=walls,
                    open_fields=None if oax is None else (oax, st),
                    thermal=dict(mask=mask, uth=uth, ufl=ufl, seed=77, step=k, type=ttype))
    tol = 1e-12 if prec == 64 else 5e-5
    errs = {"E": _nerr(eg, eo), "B": _nerr(bg, bo), "J": _nerr(jg, jo)}
    for k, s in enumerate(ora):
        ix, x, u, q = sim.species(k)
        errs[f"x{k}"] = _nerr(ix + x, s["ix"] + s["x"])
        errs[f"u{k}"] = _nerr(u, s["u"])
        assert np.array_equal(q, s["q"])              # nobody is absorbed
        assert ix.min() >= 1 and np.all(ix.max(axis=0) <= np.array(nx))
    sim.close()
    bad = {k: v for k, v in errs.items() if not v <= tol}
    assert not bad, (bad, errs)


def test_thermal_needs_a_bounded_axis(osg):
    with pytest.raises(osg.OsirisGB300Error):
        osg.Simulation([16, 16], [0.1, 0.1], 0.03, order=2, precision=64,
                       engine=osg.ENGINE_PLAIN, thermal=1, uth_bnd=(0.1, 0.1, 0.1))
