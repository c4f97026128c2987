"""GPU tests of the batched engine (osg_batch_*: many independent periodic boxes in one
persistent push launch and one CUDA graph per step).

* every box of a batch evolves as the same box run alone in the single-box tiled engine
  (osg_sim): fields, current and particles after 6 steps agree to 1e-5 normwise (only the
  order of the per-tile current sums differs), and the particle count is kept;
* the first box is also checked against the CPU oracle's time step (the single-box tolerance
  of the FP32 engines, 5e-5 after 6 steps);
* the autotuner picks one of its candidates and the tuned batch gives the same fields.
"""
import numpy as np
import pytest

from test_gpu_configs import match_particles
from test_gpu_step import _nerr

pytestmark = pytest.mark.gpu

DT = 0.035
BOXES = [([32, 32], 4, 0.1), ([64, 32], 16, 0.05), ([16, 48], 2, 0.2), ([32, 32], 16, 0.02)]


@pytest.fixture(scope="module")
def osg():
    import __graft_entry__ as g
    g.build_native()
    import osiris_gb300
    if osiris_gb300.lib().osg_device_count() < 1:
        pytest.fail("no CUDA device visible")
    return osiris_gb300


def _load(osg, i, nx, ppc, uth):
    r = osg.Rng(40 + i)
    side = int(round(np.sqrt(ppc)))
    out = []
    for s in (1.0, -1.0):
        out.append(osg.load_lattice(r, 32, nx, [side, ppc // side], [0.05, 0.05], -1.0,
                                    [uth] * 3, [s * 0.1, 0.0, 0.0], 1e-2, 1.0))
    return out


def _batch(osg, tile, threads, steps):
    bt = osg.Batch(2, 2, DT, tile=tile, threads=threads)
    for i, (nx, ppc, uth) in enumerate(BOXES):
        k = bt.add_box(nx, [0.05, 0.05])
        for sp in _load(osg, i, nx, ppc, uth):
            bt.add_species(k, -1.0, *sp)
    tuned = bt.tuning()
    bt.step(steps)
    res = [(bt.fields(k), [bt.species(k, s) for s in range(2)], bt.energy(k))
           for k in range(len(BOXES))]
    lps = bt.launches_per_step()
    bt.close()
    return res, tuned, lps


def _single(osg, i, tile, steps):
    nx, ppc, uth = BOXES[i]
    sim = osg.Simulation(nx, [0.05, 0.05], DT, order=2, precision=32, engine=osg.ENGINE_TILED,
                         tile=tile)
    for sp in _load(osg, i, nx, ppc, uth):
        sim.add_species(-1.0, *sp)
    sim.step(steps)
    out = (sim.fields(), [sim.species(s) for s in range(2)], sim.energy())
    sim.close()
    return out


def test_batch_boxes_match_single_box_engine(osg):
    res, tuned, lps = _batch(osg, [8, 8], 256, 6)
    assert tuned == ([8, 8], 256)
    assert lps <= 16          # a fixed launch count, whatever the number of boxes
    for i in range(len(BOXES)):
        (eb, bb, jb), spb, (kb, fb) = res[i]
        (es, bs, js), sps, (ks, fs) = _single(osg, i, [8, 8], 6)
        for a, c in ((eb, es), (bb, bs), (jb, js)):
            assert _nerr(a, c) <= 1e-5, (i, _nerr(a, c))
        for s in range(2):
            assert len(spb[s][3]) == len(sps[s][3])
            # the engines order particles differently: pair them by nearest neighbour
            m, _ = match_particles(BOXES[i][0], sps[s][:3], spb[s][:3])
            ib, xb, ub = (a[m] for a in spb[s][:3])
            i_s, xs, us = sps[s][:3]
            assert _nerr(ub, us) <= 1e-5, (i, s, _nerr(ub, us))
            assert _nerr(ib + xb, i_s + xs) <= 1e-5
        assert np.allclose(kb, ks, rtol=1e-5)
        assert np.allclose(fb, fs, rtol=1e-4, atol=1e-12)


def test_batch_box_matches_oracle(osg, oracle):
    res, _, _ = _batch(osg, [8, 8], 128, 6)
    nx, ppc, uth = BOXES[0]
    g = oracle.Grid(nx, 2, [0.05, 0.05])
    ora = [dict(ix=s[0].copy(), x=s[1].copy(), u=s[2].copy(), q=s[3].copy(), rqm=-1.0)
           for s in _load(osg, 0, nx, ppc, uth)]
    e, b, j = g.zeros("f32"), g.zeros("f32"), g.zeros("f32")
    for _ in range(6):
        oracle.step(g, "f32", e, b, j, ora, DT)
    (eb, bb, jb), _, _ = res[0]
    for a, c in ((eb, e), (bb, b)):
        assert _nerr(g.interior(a), g.interior(c)) <= 5e-5


def test_batch_autotuner_picks_a_candidate(osg):
    res_t, tuned, _ = _batch(osg, None, 0, 4)
    tile, threads = tuned
    assert tile in ([8, 8], [16, 8], [16, 16])
    assert threads in (128, 256)
    res_f, _, _ = _batch(osg, tile, threads, 4)
    for k in range(len(BOXES)):
        for a, c in zip(res_t[k][0], res_f[k][0]):
            assert _nerr(a, c) <= 1e-5
