"""The reference-named drop-in symbols, called exactly as the Fortran bridge calls them
(source/spec/os-spec-vpush.f03:70-95, 144-169, 217-246, 294-319): every argument a pointer,
the precision chosen by the shim library (libosiris_gb300_single.so: REAL = float,
libosiris_gb300_double.so: REAL = double).  On every golden fixture of the reference's own
kernels (1d, 2d, 2d_cyl and 3d, orders 1-4, both precisions) the outputs must equal the
fixture's: positions, cell indices and momenta bit for bit, the current within 1e-5 (FP32) /
1e-12 (FP64) normwise (atomic summation order), the energy within 1e-6 / 1e-12, and
osg_fortran_status() must report OSG_OK.  A bad call must not exit the process: it leaves the
offending particle untouched and reports its error through osg_fortran_status().
"""
import ctypes as C
import glob
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = sorted(glob.glob(os.path.join(GOLD, "push_*.npz")))
TOL_J = {"f32": 1e-5, "f64": 1e-12}
TOL_E = {"f32": 1e-6, "f64": 1e-12}


@pytest.fixture(scope="module")
def shims():
    import __graft_entry__ as g
    g.build_native()
    import osiris_gb300
    if osiris_gb300.lib().osg_device_count() < 1:
        pytest.fail("no CUDA device visible")
    out = {}
    for prec, name in (("f32", "single"), ("f64", "double")):
        lb = C.CDLL(os.path.join(osiris_gb300.HERE, f"libosiris_gb300_{name}.so"))
        lb.osg_fortran_status.restype = C.c_int
        out[prec] = lb
    return out


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def _nerr(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def _call(lb, prec, name, ix, x, u, q, i0, i1, rqm, ilb2, e, b, size, off, j, dx, dt):
    real = C.c_float if prec == "f32" else C.c_double
    ene = np.zeros(1)
    ci0, ci1, crqm, cdt = C.c_int(i0), C.c_int(i1), real(rqm), C.c_double(dt)
    es, eo = np.asarray(size, np.int32), np.asarray(off, np.int32)
    js, jo = es.copy(), eo.copy()
    dxa = np.asarray(list(dx) + [0.0] * (3 - len(dx)), np.float64)
    args = [_p(ix), _p(x), _p(u), _p(q), C.byref(ci0), C.byref(ci1), C.byref(crqm)]
    if ilb2 is not None:
        cl = C.c_int(ilb2)
        args.append(C.byref(cl))
    args += [_p(e), _p(b), _p(es), _p(eo), _p(j), _p(js), _p(jo), _p(dxa), C.byref(cdt),
             _p(ene)]
    getattr(lb, name)(*args)
    return float(ene[0]), lb.osg_fortran_status()


@pytest.mark.parametrize("path", CASES, ids=[os.path.basename(p)[5:-4] for p in CASES])
def test_reference_named_symbol_matches_fixture(shims, path):
    f = np.load(path)
    prec = "f32" if path.endswith("_f32.npz") else "f64"
    cyl = "2dcyl" in path
    dim = f["ix_in"].shape[1]
    order = int(f["order"])
    gl, gu = {1: (1, 2), 2: (2, 3), 3: (3, 4), 4: (4, 5)}[order]
    size = [int(n) + gl + gu for n in f["nx"]]
    ix, x, u, q = (np.array(f[k]) for k in ("ix_in", "x_in", "u_in", "q_in"))
    e, b = np.array(f["e"]), np.array(f["b"])
    j = np.zeros_like(e)
    name = f"vadvance_deposit_{'2d_cyl' if cyl else f'{dim}d'}_s{order}_"
    ene, status = _call(shims[prec], prec, name, ix, x, u, q, 1, len(q), float(f["rqm"]),
                        int(f["ilb2"]) if cyl else None, e, b, size, [gl] * dim, j,
                        list(f["dx"]), float(f["dt"]))
    assert status == 0
    assert np.array_equal(ix, f["ix_out"])
    assert np.array_equal(x, f["x_out"])
    assert np.array_equal(u, f["u_out"])
    jref = f["j_ref64"] if "j_ref64" in f.files else f["j_out"]
    assert _nerr(j, jref) <= TOL_J[prec]
    assert abs(ene - float(f["ene"])) <= TOL_E[prec] * abs(float(f["ene"]))


@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_bad_call_reports_status_without_exiting(shims, prec):
    """A particle whose stencil would reach outside the field arrays: the reference kernel
    reads out of bounds; the shim returns, leaves that particle as it was and reports
    OSG_ERR_RANGE (-4) through osg_fortran_status()."""
    real = np.float32 if prec == "f32" else np.float64
    size = [11, 11]
    ix = np.array([[1, 1], [40, 3]], np.int32)
    x = np.zeros((2, 2), real)
    u = np.full((2, 3), 0.1, real)
    q = np.full(2, -1.0, real)
    g = np.zeros((11, 11, 3), real)
    ix0, u0 = ix.copy(), u.copy()
    _, status = _call(shims[prec], prec, "vadvance_deposit_2d_s2_", ix, x, u, q, 1, 2, -1.0,
                      None, g, g, size, [2, 2], g.copy(), [0.1, 0.1], 0.05)
    assert status == -4
    assert np.array_equal(ix[1], ix0[1]) and np.array_equal(u[1], u0[1])
