"""The ctypes mirrors of the C-ABI structs (osiris_gb300.Config, BatchConfig, Zpulse) have the
size and field offsets of the structs include/osiris_gb300.h declares: a small C program
compiled against the header prints them (no GPU, no library load)."""
import ctypes as C
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

STRUCTS = {
    "osg_config": ("Config", ["dim", "order", "precision", "engine", "nx", "dx", "dt", "tile",
                              "n_sort", "capacity", "pusher", "iter_tol", "smooth_type",
                              "smooth_order", "walls", "open_fields", "thermal", "seed",
                              "uth_bnd", "ufl_bnd", "thermal_type", "pmc", "emf_smooth_type",
                              "emf_smooth_order", "pml", "pml_cells",
                              "pml_diffuse"]),
    "osg_batch_config": ("BatchConfig", ["dim", "order", "dt", "tile", "threads", "capacity"]),
    "osg_zpulse": ("Zpulse", ["omega0", "a0", "pol", "lon_x0", "lon_duration", "lon_range",
                              "per_w0", "per_focus", "per_center"]),
}


@pytest.fixture(scope="module")
def c_layout(tmp_path_factory):
    cc = shutil.which("cc") or shutil.which("gcc")
    if not cc:
        pytest.skip("no C compiler")
    d = tmp_path_factory.mktemp("abi")
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "osiris_gb300.h"',
             "int main(void) {"]
    for cname, (_, fields) in STRUCTS.items():
        lines.append(f'printf("{cname} size %zu\\n", sizeof({cname}));')
        for f in fields:
            lines.append(f'printf("{cname} {f} %zu\\n", offsetof({cname}, {f}));')
    lines += ["return 0;", "}"]
    src = d / "abi.c"
    src.write_text("\n".join(lines) + "\n")
    exe = d / "abi"
    subprocess.run([cc, "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)],
                   check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    got = {}
    for line in out.splitlines():
        s, f, v = line.split()
        got[(s, f)] = int(v)
    return got


@pytest.mark.parametrize("cname", sorted(STRUCTS))
def test_ctypes_mirror_matches_header(c_layout, cname):
    import osiris_gb300
    pyname, fields = STRUCTS[cname]
    cls = getattr(osiris_gb300, pyname)
    assert [f for f, _ in cls._fields_] == fields
    assert C.sizeof(cls) == c_layout[(cname, "size")]
    for f in fields:
        assert getattr(cls, f).offset == c_layout[(cname, f)], f
