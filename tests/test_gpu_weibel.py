"""Physics of the 3D Weibel filamentation configuration (two counter-streaming electron species
at +-0.5 c along z, uth 0.05 c, 8 particles per cell each, cubic splines, dx 0.1, dt 0.05, fixed
neutralising ions) on a reduced 24^3 box: the mixed-precision tiled engine against the FP64
plain engine from the same seeded load.

* every 10 steps the FP64 diagnostics are taken: field and kinetic energy, and the charge
  check max |div E - rho|, which must stay at its t = 0 value (2e-4 of max rho in FP32 over
  400 steps, 1e-10 in FP64);
* the transverse magnetic energy (B1^2 + B2^2) grows at the same rate in both engines (log-
  linear fit over its growth phase, within 10%);
* the total energy histories differ by less than 5e-3 of the initial total;
* against the CPU oracle (the reference's CPU path restated, run in FP64 on the same load):
  the FP32 tiled growth rate within 10% and its energy history within 5e-3, the FP64 plain
  engine's growth rate within 1e-3 and its energy history within 1e-5.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NX = [24, 24, 24]
PPC = [2, 2, 2]
DX = [0.1, 0.1, 0.1]
DT = 0.05
STEPS, EVERY = 400, 10


@pytest.fixture(scope="module")
def osg():
    import __graft_entry__ as g
    g.build_native()
    import osiris_gb300
    if osiris_gb300.lib().osg_device_count() < 1:
        pytest.fail("no CUDA device visible")
    return osiris_gb300


def _history(osg, prec, engine):
    r = osg.Rng(3)
    sim = osg.Simulation(NX, DX, DT, order=3, precision=prec, engine=engine,
                         tile=[8, 8, 8] if engine == osg.ENGINE_TILED else None)
    rho_max = 0.0
    for s in (1.0, -1.0):
        ix, x, u, q = osg.load_lattice(r, prec, NX, PPC, DX, -1.0, [0.05] * 3, [0.0, 0.0, s * 0.5])
        sim.add_species(-1.0, ix, x, u, q)
    g0, _ = sim.gauss_residual()
    bt, tot, gauss = [], [], []
    for _ in range(STEPS // EVERY):
        sim.step(EVERY)
        kin, fld = sim.energy()
        bt.append(fld[3] + fld[4])
        tot.append(kin.sum() + fld.sum())
        gauss.append(sim.gauss_residual()[0])
    sim.close()
    return np.array(bt), np.array(tot), g0, np.array(gauss)


def _oracle_history(oracle):
    """The same run on the CPU oracle in FP64: transverse B energy and total energy every
    EVERY steps."""
    r = oracle.mt_new(3)
    sp = []
    for s in (1.0, -1.0):
        ix, x, u, q = oracle.load(r, "f64", 3, NX, PPC, DX, -1.0, [0.05] * 3, [0.0, 0.0, s * 0.5])
        sp.append(dict(ix=ix, x=x, u=u, q=q, rqm=-1.0))
    g = oracle.Grid(NX, 3, DX)
    e, b, j = g.zeros("f64"), g.zeros("f64"), g.zeros("f64")
    dv = float(np.prod(DX))
    nthr = oracle.max_threads()
    bt, tot = [], []
    for i in range(STEPS):
        ene = oracle.step(g, "f64", e, b, j, sp, DT, nthreads=nthr)
        if (i + 1) % EVERY == 0:
            fe, fb = oracle.field_energy(g, "f64", e), oracle.field_energy(g, "f64", b)
            bt.append(fb[0] + fb[1])
            tot.append(float((ene * -1.0 * dv).sum() + fe.sum() + fb.sum()))
    return np.array(bt), np.array(tot)


@pytest.fixture(scope="module")
def runs(osg, oracle):
    return {"fp32": _history(osg, 32, osg.ENGINE_TILED),
            "fp64": _history(osg, 64, osg.ENGINE_PLAIN),
            "oracle": _oracle_history(oracle)}


def _growth(b):
    lb = np.log(np.maximum(b, 1e-300))
    peak = int(np.argmax(lb))
    lo, hi = lb[0] + np.log(30.0), lb[peak] - np.log(30.0)
    sel = np.where((lb > lo) & (lb < hi))[0]
    sel = sel[sel < peak]
    assert len(sel) >= 4, ("no growth phase found", lb)
    t = (sel + 1) * EVERY * DT
    return np.polyfit(t, lb[sel], 1)[0] / 2.0, sel


def test_weibel_charge_conservation(runs):
    for key, tol in (("fp32", 2e-4), ("fp64", 1e-10)):
        _, _, g0, gauss = runs[key]
        print(f"{key}: div E - rho max {g0:.6e} -> {gauss.min():.6e} .. {gauss.max():.6e}")
        assert np.abs(gauss - g0).max() <= tol * g0


def test_weibel_growth_rate_matches_fp64(runs):
    g32, s32 = _growth(runs["fp32"][0])
    g64, s64 = _growth(runs["fp64"][0])
    print(f"Weibel growth rate (B field) FP32 tiled {g32:.4f}  FP64 plain {g64:.4f}  "
          f"windows {s32[0]}-{s32[-1]} / {s64[0]}-{s64[-1]}")
    assert g64 > 0.1
    assert abs(g32 / g64 - 1.0) < 0.10


def test_weibel_energy_history_matches_fp64(runs):
    t32, t64 = runs["fp32"][1], runs["fp64"][1]
    d32, d64 = t32 / t32[0] - 1.0, t64 / t64[0] - 1.0
    print(f"total energy drift: FP32 tiled max {np.abs(d32).max():.3e}  "
          f"FP64 plain max {np.abs(d64).max():.3e}  max difference {np.abs(d32 - d64).max():.3e}")
    assert np.abs(d32 - d64).max() < 5e-3


def test_weibel_growth_rate_and_energy_match_oracle(runs):
    go, so = _growth(runs["oracle"][0])
    g32, _ = _growth(runs["fp32"][0])
    g64, _ = _growth(runs["fp64"][0])
    to = runs["oracle"][1]
    do = to / to[0] - 1.0
    d32 = np.abs(runs["fp32"][1] / runs["fp32"][1][0] - 1.0 - do).max()
    d64 = np.abs(runs["fp64"][1] / runs["fp64"][1][0] - 1.0 - do).max()
    print(f"Weibel growth rate: oracle FP64 {go:.5f} (window {so[0]}-{so[-1]})  FP32 tiled "
          f"{g32:.5f}  FP64 plain {g64:.5f}; energy history difference FP32 {d32:.3e}  "
          f"FP64 {d64:.3e}")
    assert go > 0.1
    assert abs(g32 / go - 1.0) < 0.10
    assert abs(g64 / go - 1.0) < 1e-3
    assert d32 < 5e-3
    assert d64 < 1e-5
