"""GPU parity of the drop-in push/deposit entry point (osg_vadvance_deposit_*, the C ABI that
replaces FNAME(vadvance_deposit_{1d,2d,3d}_sN), and osg_vadvance_deposit_cyl_* for
FNAME(vadvance_deposit_2d_cyl_sN)) against the reference's own kernel outputs (golden
fixtures) and against the CPU oracle.

Tolerances: particle positions, cell indices and momenta bit-identical (same roundings as the
reference); current normwise max|a-b|/max|b| <= 1e-12 (FP64) and <= 1e-5 (FP32), the
difference coming only from the order of the atomic current sums; energy sum relative
<= 1e-12 (FP64) / 1e-6 (FP32, the reference sums in float per 464/160-particle chunk).
"""
import glob
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = sorted(p for p in glob.glob(os.path.join(GOLD, "push_*.npz")) if "2dcyl" not in p)
CYL = sorted(glob.glob(os.path.join(GOLD, "push_2dcyl_*.npz")))
TOL_J = {"f32": 1e-5, "f64": 1e-12}
TOL_E = {"f32": 1e-6, "f64": 1e-12}


@pytest.fixture(scope="module")
def osg():
    import __graft_entry__ as g
    g.build_native()
    import osiris_gb300
    if osiris_gb300.lib().osg_device_count() < 1:
        pytest.fail("no CUDA device visible")
    return osiris_gb300


def _nerr(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.mark.parametrize("path", CASES, ids=[os.path.basename(p)[5:-4] for p in CASES])
def test_gpu_push_matches_reference_fixture(osg, path):
    f = np.load(path)
    prec = "f32" if path.endswith("_f32.npz") else "f64"
    dim = f["ix_in"].shape[1]
    order = int(f["order"])
    gl, gu = osg.GUARD[order]
    size = [n + gl + gu for n in f["nx"]]
    ix, x, u, q = (np.array(f[k]) for k in ("ix_in", "x_in", "u_in", "q_in"))
    j = np.zeros_like(f["e"])
    ene = osg.vadvance_deposit(dim, order, ix, x, u, q, 1, len(q), float(f["rqm"]), f["e"],
                               f["b"], size, [gl] * dim, j, size, [gl] * dim, list(f["dx"]),
                               float(f["dt"]))
    assert np.array_equal(ix, f["ix_out"])
    assert np.array_equal(x, f["x_out"])
    assert np.array_equal(u, f["u_out"])
    jref = f["j_ref64"] if "j_ref64" in f.files else f["j_out"]
    assert _nerr(j, jref) <= TOL_J[prec]
    assert abs(ene - float(f["ene"])) <= TOL_E[prec] * abs(float(f["ene"]))


@pytest.mark.parametrize("path", CYL, ids=[os.path.basename(p)[5:-4] for p in CYL])
def test_gpu_cyl_push_matches_reference_fixture(osg, path):
    f = np.load(path)
    prec = "f32" if path.endswith("_f32.npz") else "f64"
    order = int(f["order"])
    gl, gu = osg.GUARD[order]
    size = [n + gl + gu for n in f["nx"]]
    ix, x, u, q = (np.array(f[k]) for k in ("ix_in", "x_in", "u_in", "q_in"))
    j = np.zeros_like(f["e"])
    ene = osg.vadvance_deposit_cyl(order, ix, x, u, q, 1, len(q), float(f["rqm"]),
                                   int(f["ilb2"]), f["e"], f["b"], size, [gl] * 2, j, size,
                                   [gl] * 2, list(f["dx"]), float(f["dt"]))
    assert np.array_equal(ix, f["ix_out"])
    assert np.array_equal(x, f["x_out"])
    assert np.array_equal(u, f["u_out"])
    assert _nerr(j, f["j_out"]) <= TOL_J[prec]
    assert abs(ene - float(f["ene"])) <= TOL_E[prec] * abs(float(f["ene"]))


@pytest.mark.parametrize("prec", ["f32", "f64"])
@pytest.mark.parametrize("order", [1, 2, 3, 4])
def test_gpu_cyl_push_matches_oracle_subrange(osg, oracle, prec, order):
    """A warm plasma off the axis (ilb2 = 4), pushing the sub-range [i0, i1] only, against the
    oracle's cylindrical push on the same arrays."""
    nx, dx = [12, 10], [0.1, 0.12]
    g = oracle.Grid(nx, order, dx)
    rng = np.random.default_rng(40 + order)
    dt_ = np.float32 if prec == "f32" else np.float64
    r = oracle.mt_new(12)
    ix, x, u, q = oracle.load(r, prec, 2, nx, [2, 2], dx, -1.0, [0.6] * 3, [0.1, 0.0, 0.3])
    e = (rng.standard_normal(g.shape) * 0.3).astype(dt_)
    b = (rng.standard_normal(g.shape) * 0.3).astype(dt_)
    n = len(q)
    i0, i1 = 5, n - 3
    a = [v.copy() for v in (ix, x, u, q)]
    j_g = g.zeros(prec)
    ene_g = osg.vadvance_deposit_cyl(order, *a, i0, i1, -1.0, 4, e, b, g.size, g.gcl, j_g,
                                     g.size, g.gcl, dx, 0.04)
    o = [v.copy() for v in (ix, x, u, q)]
    j_o = g.zeros(prec)
    ene_o = oracle.push_cyl(prec, order, *o, i0, i1, -1.0, 4, e, b, j_o, g.size, g.gcl, dx,
                            0.04)
    for k in range(3):
        assert np.array_equal(a[k], o[k]), k
    assert _nerr(j_g, j_o) <= TOL_J[prec]
    assert abs(ene_g - ene_o) <= TOL_E[prec] * abs(ene_o)


@pytest.mark.parametrize("prec", ["f32", "f64"])
@pytest.mark.parametrize("dim,order", [(2, 1), (2, 2), (2, 3), (2, 4), (3, 1), (3, 2), (3, 3),
                                       (1, 2)])
def test_gpu_push_matches_oracle_subrange(osg, oracle, prec, dim, order):
    """A thermal plasma, pushing the sub-range [i0, i1] only (offset handling), against the
    oracle on the same arrays; particles outside the range stay untouched."""
    nx = [12, 10, 8][:dim]
    dx = [0.1, 0.12, 0.15][:dim]
    g = oracle.Grid(nx, order, dx)
    rng = np.random.default_rng(dim * 10 + order)
    dt_ = np.float32 if prec == "f32" else np.float64
    r = oracle.mt_new(11)
    ix, x, u, q = oracle.load(r, prec, dim, nx, [2] * dim, dx, -1.0, [0.6] * 3, [0.2, 0.0, 0.0])
    e = (rng.standard_normal(g.shape) * 0.3).astype(dt_)
    b = (rng.standard_normal(g.shape) * 0.3).astype(dt_)
    n = len(q)
    i0, i1 = 7, n - 5
    a = [v.copy() for v in (ix, x, u, q)]
    j_g = g.zeros(prec)
    ene_g = osg.vadvance_deposit(dim, order, *a, i0, i1, -1.0, e, b, g.size, g.gcl, j_g,
                                 g.size, g.gcl, dx, 0.04)
    o = [v.copy() for v in (ix, x, u, q)]
    j_o = g.zeros(prec)
    ene_o = oracle.push(prec, dim, order, *o, i0, i1, -1.0, e, b, j_o, g.size, g.gcl, dx, 0.04)
    for k in range(3):
        assert np.array_equal(a[k], o[k])
    assert _nerr(j_g, j_o) <= TOL_J[prec]
    assert abs(ene_g - ene_o) <= TOL_E[prec] * abs(ene_o)


@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_gpu_push_chunked_large_range_matches_oracle(osg, oracle, prec):
    """More than 4 Mi particles in one call: the entry point pushes the range in chunks on two
    streams (copies overlapping the push).  Particles stay bit-identical to the oracle and the
    current within the summation-order tolerance; a sub-range offset is included."""
    nx = [128, 64]
    dx = [0.1, 0.1]
    g = oracle.Grid(nx, 2, dx)
    rng = np.random.default_rng(3)
    dt_ = np.float32 if prec == "f32" else np.float64
    r = oracle.mt_new(3)
    ix, x, u, q = oracle.load(r, prec, 2, nx, [24, 24], dx, -1.0, [0.3] * 3, [0.1, 0.0, 0.0])
    e = (rng.standard_normal(g.shape) * 0.2).astype(dt_)
    b = (rng.standard_normal(g.shape) * 0.2).astype(dt_)
    n = len(q)
    assert n > 4 * 2**20
    i0, i1 = 3, n - 2
    a = [v.copy() for v in (ix, x, u, q)]
    j_g = g.zeros(prec)
    ene_g = osg.vadvance_deposit(2, 2, *a, i0, i1, -1.0, e, b, g.size, g.gcl, j_g, g.size,
                                 g.gcl, dx, 0.04)
    o = [v.copy() for v in (ix, x, u, q)]
    j_o = g.zeros(prec)
    ene_o = oracle.push(prec, 2, 2, *o, i0, i1, -1.0, e, b, j_o, g.size, g.gcl, dx, 0.04)
    for k in range(3):
        assert np.array_equal(a[k], o[k])
    assert _nerr(j_g, j_o) <= TOL_J[prec]
    assert abs(ene_g - ene_o) <= 10 * TOL_E[prec] * abs(ene_o)


def test_gpu_push_rejects_out_of_range_cells(osg, oracle):
    """A cell index that would reach outside the arrays is caught by the kernel's own bounds
    check: the call returns OSG_ERR_RANGE and that particle is left as it was."""
    g = oracle.Grid([8, 8], 2, [0.1, 0.1])
    ix = np.array([[3, 3], [40, 3]], np.int32)
    x = np.zeros((2, 2))
    u = np.zeros((2, 3))
    q = np.ones(2)
    e, b, j = g.zeros("f64"), g.zeros("f64"), g.zeros("f64")
    with pytest.raises(osg.OsirisGB300Error) as err:
        osg.vadvance_deposit(2, 2, ix, x, u, q, 1, 2, -1.0, e, b, g.size, g.gcl, j, g.size,
                             g.gcl, [0.1, 0.1], 0.05)
    assert err.value.code == -4
    assert ix[1, 0] == 40


@pytest.mark.parametrize("prec", ["f32", "f64"])
@pytest.mark.parametrize("dim", [2, 3])
def test_gpu_yee_and_periodic_match_oracle(osg, oracle, prec, dim):
    g = oracle.Grid([10, 9, 8][:dim], 2, [0.1, 0.11, 0.12][:dim])
    rng = np.random.default_rng(dim)
    dt_ = np.float32 if prec == "f32" else np.float64
    e = rng.standard_normal(g.shape).astype(dt_)
    b = rng.standard_normal(g.shape).astype(dt_)
    j = rng.standard_normal(g.shape).astype(dt_)
    for add in (0, 1):
        f1, f2 = e.copy(), e.copy()
        osg.periodic(dim, g.nx, g.gcl, g.gcu, f1, add)
        oracle.periodic(g, prec, f2, add)
        assert np.array_equal(f1, f2)
    e1, b1, e2, b2 = e.copy(), b.copy(), e.copy(), b.copy()
    osg.yee_advance(dim, g.nx, g.gcl, g.gcu, e1, b1, j, g.dx, 0.04)
    oracle.yee_advance(g, prec, e2, b2, j, 0.04)
    assert np.array_equal(e1, e2) and np.array_equal(b1, b2)
