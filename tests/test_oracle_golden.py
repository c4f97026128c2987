"""The CPU oracle against the golden vectors produced by the reference's own compiled
push/deposit kernels (tests/golden/make_golden.py).

Bit-exact for particle positions, cell indices, momenta, currents and the time-centred energy
in both precisions, all dimensions and interpolation orders -- except the single-precision 3D
cubic/quartic current, where the reference kernel is defective (it offsets z planes by a y
stride, source/simd/os-spec-current-avx2.c:1096,1118); there the current is compared with the
double-precision reference run on the same inputs, at the FP32 tolerance 1e-5 (normwise).
The 2D cylindrical kernels (vadvance_deposit_2d_cyl_sK) have their own eight fixtures,
push_2dcyl_s<order>_<prec>.npz, also bit-exact.
"""
import glob
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = sorted(p for p in glob.glob(os.path.join(GOLD, "push_*.npz")) if "2dcyl" not in p)
CYL = sorted(glob.glob(os.path.join(GOLD, "push_2dcyl_*.npz")))


def _run(po, f, prec):
    dim = f["ix_in"].shape[1]
    order = int(f["order"])
    g = po.Grid(list(f["nx"]), order, list(f["dx"]))
    ix, x, u, q = (np.array(f[k]) for k in ("ix_in", "x_in", "u_in", "q_in"))
    j = g.zeros(prec)
    e, b = np.array(f["e"]), np.array(f["b"])
    ene = po.push(prec, dim, order, ix, x, u, q, 1, len(q), float(f["rqm"]), e, b, j, g.size,
                  g.gcl, g.dx, float(f["dt"]))
    return ix, x, u, j, ene


def test_fixture_set_complete():
    assert len(CASES) == 24
    assert len(CYL) == 8


@pytest.mark.parametrize("path", CASES, ids=[os.path.basename(p)[5:-4] for p in CASES])
def test_oracle_matches_reference(oracle, path):
    f = np.load(path)
    prec = "f32" if path.endswith("_f32.npz") else "f64"
    ix, x, u, j, ene = _run(oracle, f, prec)
    assert np.array_equal(ix, f["ix_out"])
    assert np.array_equal(x, f["x_out"])
    assert np.array_equal(u, f["u_out"])
    assert ene == float(f["ene"])
    if "j_ref64" in f.files:
        ref = f["j_ref64"]
        err = np.abs(j.astype(np.float64) - ref).max() / np.abs(ref).max()
        assert err < 1e-5, err
        # the defective single-precision reference current is far from both
        bad = np.abs(f["j_out"].astype(np.float64) - ref).max() / np.abs(ref).max()
        assert bad > 1e-2
    else:
        assert np.array_equal(j, f["j_out"])


@pytest.mark.parametrize("path", CYL, ids=[os.path.basename(p)[5:-4] for p in CYL])
def test_oracle_cyl_matches_reference(oracle, path):
    f = np.load(path)
    prec = "f32" if path.endswith("_f32.npz") else "f64"
    order = int(f["order"])
    g = oracle.Grid(list(f["nx"]), order, list(f["dx"]))
    ix, x, u, q = (np.array(f[k]) for k in ("ix_in", "x_in", "u_in", "q_in"))
    j = g.zeros(prec)
    ene = oracle.push_cyl(prec, order, ix, x, u, q, 1, len(q), float(f["rqm"]), int(f["ilb2"]),
                          np.array(f["e"]), np.array(f["b"]), j, g.size, g.gcl, g.dx,
                          float(f["dt"]))
    assert np.array_equal(ix, f["ix_out"])
    assert np.array_equal(x, f["x_out"])
    assert np.array_equal(u, f["u_out"])
    assert np.array_equal(j, f["j_out"])
    assert ene == float(f["ene"])
    # the radial step really differs from the Cartesian one on these inputs
    ixc, xc, uc, qc = (np.array(f[k]) for k in ("ix_in", "x_in", "u_in", "q_in"))
    oracle.push(prec, 2, order, ixc, xc, uc, qc, 1, len(qc), float(f["rqm"]), np.array(f["e"]),
                np.array(f["b"]), g.zeros(prec), g.size, g.gcl, g.dx, float(f["dt"]))
    assert not np.array_equal(uc, u)
