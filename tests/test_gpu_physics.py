"""Physics of the two-stream configuration on a reduced box (the 512x512 configuration's plasma
parameters on 128x16 cells, 900 steps), from the same seeded OSIRIS load: the mixed-precision
tiled engine and the plain FP64 engine on the GPU, against each other and against the CPU
oracle (the reference's CPU path restated, run in FP64), must show the same linear growth rate
of the E1 field energy and the same total-energy history.

* growth rate: log-linear fit of E1 energy over the linear phase (the samples before the
  first peak that lie between 1e-3x and 10^-0.5x the peak energy); the FP32 tiled rate agrees
  with the FP64 ones within 3%, the FP64 plain engine's with the oracle's within 1e-4;
* energy: total (kinetic + field) energy relative to its initial value; the FP32 history
  differs from the FP64 ones by less than 1e-3 of the initial total at every sample, the FP64
  plain engine's from the oracle's by less than 1e-5.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NX = [128, 16]
PPC = [8, 8]
DX = [0.05, 0.05]
DT = 0.035
STEPS, EVERY = 900, 10


@pytest.fixture(scope="module")
def osg():
    import __graft_entry__ as g
    g.build_native()
    import osiris_gb300
    if osiris_gb300.lib().osg_device_count() < 1:
        pytest.fail("no CUDA device visible")
    return osiris_gb300


def _history(osg, prec, engine):
    r = osg.Rng(2)
    sim = osg.Simulation(NX, DX, DT, order=2, precision=prec, engine=engine,
                         n_sort=25 if engine == osg.ENGINE_PLAIN else 0)
    for s in (1.0, -1.0):
        sim.add_species(-1.0, *osg.load_lattice(r, prec, NX, PPC, DX, -1.0, [0.01] * 3,
                                                [s * 0.2, 0.0, 0.0], 1e-3, 1.0))
    e1, tot = [], []
    for _ in range(STEPS // EVERY):
        sim.step(EVERY)
        kin, fld = sim.energy()
        e1.append(fld[0])
        tot.append(kin.sum() + fld.sum())
    sim.close()
    return np.array(e1), np.array(tot)


def _oracle_history(oracle):
    """The same run on the CPU oracle in FP64: E1 field energy and total energy every EVERY
    steps (kinetic = the time-centred push energy times rqm and the cell volume)."""
    r = oracle.mt_new(2)
    sp = []
    for s in (1.0, -1.0):
        ix, x, u, q = oracle.load(r, "f64", 2, NX, PPC, DX, -1.0, [0.01] * 3,
                                  [s * 0.2, 0.0, 0.0], 1e-3, 1.0)
        sp.append(dict(ix=ix, x=x, u=u, q=q, rqm=-1.0))
    g = oracle.Grid(NX, 2, DX)
    e, b, j = g.zeros("f64"), g.zeros("f64"), g.zeros("f64")
    dv = float(np.prod(DX))
    nthr = oracle.max_threads()
    e1, tot = [], []
    for i in range(STEPS):
        ene = oracle.step(g, "f64", e, b, j, sp, DT, nthreads=nthr)
        if (i + 1) % EVERY == 0:
            fe, fb = oracle.field_energy(g, "f64", e), oracle.field_energy(g, "f64", b)
            e1.append(fe[0])
            tot.append(float((ene * -1.0 * dv).sum() + fe.sum() + fb.sum()))
    return np.array(e1), np.array(tot)


@pytest.fixture(scope="module")
def runs(osg, oracle):
    return {"fp32": _history(osg, 32, osg.ENGINE_TILED),
            "fp64": _history(osg, 64, osg.ENGINE_PLAIN),
            "oracle": _oracle_history(oracle)}


def _growth(e1):
    le = np.log(np.maximum(e1, 1e-300))
    peak = int(np.argmax(le[: len(le) * 3 // 4]))
    lo, hi = le[peak] + np.log(1e-3), le[peak] - 0.5 * np.log(10.0)
    sel = np.where((le > lo) & (le < hi))[0]
    sel = sel[sel < peak]
    assert len(sel) >= 5, "no linear phase found"
    t = (sel + 1) * EVERY * DT
    return np.polyfit(t, le[sel], 1)[0], sel


def test_two_stream_growth_rate_matches_fp64(runs):
    g32, s32 = _growth(runs["fp32"][0])
    g64, s64 = _growth(runs["fp64"][0])
    print(f"growth rate (field energy) FP32 tiled {g32:.5f}  FP64 plain {g64:.5f}  "
          f"windows {s32[0]}-{s32[-1]} / {s64[0]}-{s64[-1]}")
    assert g64 > 0.1
    assert abs(g32 / g64 - 1.0) < 0.03


def test_two_stream_energy_history_matches_fp64(runs):
    t32, t64 = runs["fp32"][1], runs["fp64"][1]
    d32, d64 = t32 / t32[0] - 1.0, t64 / t64[0] - 1.0
    print(f"total energy drift: FP32 tiled max {np.abs(d32).max():.3e}  "
          f"FP64 plain max {np.abs(d64).max():.3e}  max difference {np.abs(d32 - d64).max():.3e}")
    assert np.abs(d32 - d64).max() < 1e-3


def test_two_stream_growth_rate_matches_oracle(runs):
    go, so = _growth(runs["oracle"][0])
    g32, _ = _growth(runs["fp32"][0])
    g64, _ = _growth(runs["fp64"][0])
    print(f"growth rate: oracle FP64 {go:.6f} (window {so[0]}-{so[-1]})  FP32 tiled {g32:.6f}  "
          f"FP64 plain {g64:.6f}")
    assert go > 0.1
    assert abs(g32 / go - 1.0) < 0.03
    assert abs(g64 / go - 1.0) < 1e-4


def test_two_stream_energy_history_matches_oracle(runs):
    to = runs["oracle"][1]
    do = to / to[0] - 1.0
    diffs = {}
    for key in ("fp32", "fp64"):
        t = runs[key][1]
        diffs[key] = np.abs((t / t[0] - 1.0) - do).max()
    print(f"total energy drift: oracle FP64 max {np.abs(do).max():.3e}; difference to it: "
          f"FP32 tiled {diffs['fp32']:.3e}, FP64 plain {diffs['fp64']:.3e}")
    assert diffs["fp32"] < 1e-3
    assert diffs["fp64"] < 1e-5
