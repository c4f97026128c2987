"""Physics of the mixed-precision tiled engine against the FP64 plain engine on the GPU, from
the same seeded OSIRIS load: a reduced two-stream run (the 512x512 configuration's plasma
parameters on 128x16 cells) must show the same linear growth rate of the E1 field energy and
the same total-energy history.

* growth rate: log-linear fit of E1 energy over the linear phase (the samples before the
  first peak that lie between 1e-3x and 10^-0.5x the peak energy); rates agree within 3%;
* energy: total (kinetic + field) energy relative to its initial value; the two histories
  differ by less than 1e-3 of the initial total at every sample.
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


@pytest.fixture(scope="module")
def runs(osg):
    return {"fp32": _history(osg, 32, osg.ENGINE_TILED),
            "fp64": _history(osg, 64, osg.ENGINE_PLAIN)}


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
