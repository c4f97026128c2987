"""The native library loads without a GPU and exports every entry point the public headers
declare (no compute calls are made here)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INC = os.path.join(ROOT, "include")


def _declared(header, pattern):
    txt = open(os.path.join(INC, header)).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(pattern, txt)))


@pytest.fixture(scope="module")
def built():
    import __graft_entry__ as g
    g.build_native()
    return True


def test_main_library_exports(built):
    import osiris_gb300 as osg
    names = _declared("osiris_gb300.h", r"\b(osg_[a-z0-9_]+)\s*\(")
    assert len(names) >= 25
    lb = ctypes.CDLL(osg.LIB_PATH)
    missing = [n for n in names if not hasattr(lb, n)]
    assert not missing, missing


@pytest.mark.parametrize("prec", ["single", "double"])
def test_fortran_shim_exports(built, prec):
    import osiris_gb300 as osg
    names = _declared("osiris_gb300_fortran.h",
                      r"OSG_FORTRAN_PUSH(?:_CYL)?_DECL\((vadvance_deposit_\w+)\)")
    # every symbol the reference's Fortran bridge calls (source/spec/os-spec-vpush.f03:70-95,
    # 144-169, 217-246, 294-319): 1d, 2d, 2d_cyl and 3d, orders 1-4
    bridge = [f"vadvance_deposit_{g}_s{o}_" for g in ("1d", "2d", "2d_cyl", "3d")
              for o in (1, 2, 3, 4)]
    assert sorted(bridge) == names
    names += ["osg_fortran_status"]
    assert len(names) == 17
    lb = ctypes.CDLL(os.path.join(osg.HERE, f"libosiris_gb300_{prec}.so"))
    missing = [n for n in names if not hasattr(lb, n)]
    assert not missing, missing


def test_error_text_roundtrip_without_gpu(built):
    import osiris_gb300 as osg
    import numpy as np
    # argument validation happens before any CUDA call
    with pytest.raises(osg.OsirisGB300Error) as e:
        osg.vadvance_deposit(5, 2, np.zeros((1, 2), np.int32), np.zeros((1, 2), np.float32),
                             np.zeros((1, 3), np.float32), np.zeros(1, np.float32), 1, 1, -1.0,
                             np.zeros(4, np.float32), np.zeros(4, np.float32), [1, 1], [0, 0],
                             np.zeros(4, np.float32), [1, 1], [0, 0], [0.1, 0.1], 0.05)
    assert e.value.code == -1 and "dim" in str(e.value)
