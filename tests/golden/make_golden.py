"""Generate the golden push/deposit fixtures from the reference's own compiled kernels.

Run from the repository root on an x86_64 machine that has the OSIRIS sources:

    python tests/golden/make_golden.py <osiris checkout>     # or OSIRIS_REF=<checkout>

It builds ``oracle/_ref/libref_{f32,f64}.so`` from ``source/simd/os-spec-push-c.c`` and
``source/simd/os-spec-current-c.c`` of the reference (``make -C oracle ref``), runs every
``vadvance_deposit_{1d,2d,3d}_s{1..4}_`` entry point of both precisions on a seeded input,
and stores inputs and outputs as ``push_<dim>d_s<order>_<prec>.npz``.

The single-precision 3D cubic and quartic reference kernels deposit z planes at a y offset
(source/simd/os-spec-current-avx2.c:1096 and :1118 use ``k3*Dy`` where the other orders use
``k3*Dz``), so for those two fixtures the current is also computed with the double-precision
reference on the same inputs (``j_ref64``), and the parity test uses that.

The 2D cylindrical entry points ``vadvance_deposit_2d_cyl_s{1..4}_`` (x1 = z, x2 = r, with the
node's lower global cell ``ilb2`` along x2) give ``push_2dcyl_s<order>_<prec>.npz`` on the same
kind of input, with the particles kept off the axis (``ilb2`` = 3) and large azimuthal
momenta, so the angular-momentum correction is exercised (``--cyl`` regenerates only these).

A second set, ``mt_kat.npz``, holds the first draws of the OSIRIS-seeded Mersenne Twister for
two seeds, computed with the C++ standard library's ``std::mt19937`` (an independent
implementation): OSIRIS seeds word 0 with ``seed ^ 0x80000000`` and returns the tempered last
initialisation word first (source/random/os-random-mt.f03:84-149), after which the stream is
the standard MT19937 stream of that seed.
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle import pyoracle as po  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))

NX = {1: [9], 2: [7, 6], 3: [6, 5, 5]}
DX = {1: [0.2], 2: [0.2, 0.25], 3: [0.2, 0.25, 0.3]}
DT = 0.08
NP = 203  # not a multiple of the vector width: exercises the padded tail


def make_case(prec, dim, order, seed):
    rng = np.random.default_rng(seed)
    g = po.Grid(NX[dim], order, DX[dim])
    dt_ = po.dtype_of(prec)
    e = (rng.standard_normal(g.shape) * 0.8).astype(dt_)
    b = (rng.standard_normal(g.shape) * 0.8).astype(dt_)
    npad = ((NP + 15) // 16) * 16
    ix = np.ones((npad, dim), np.int32)
    x = np.zeros((npad, dim), dt_)
    u = np.zeros((npad, 3), dt_)
    q = np.zeros(npad, dt_)
    for d in range(dim):
        ix[:NP, d] = rng.integers(1, NX[dim][d] + 1, NP)
    xx = rng.uniform(-0.5, 0.5, (NP, dim))
    edge = rng.random((NP, dim)) < 0.4          # many cell-face crossings, all split cases
    xx[edge] = np.sign(xx[edge]) * rng.uniform(0.42, 0.4999, edge.sum())
    x[:NP] = xx.astype(dt_)
    u[:NP] = (rng.standard_normal((NP, 3)) * 2.0).astype(dt_)
    q[:NP] = rng.uniform(-1.0, 1.0, NP).astype(dt_)
    rqm = -1.0 if seed % 2 else 1836.0
    return g, e, b, ix, x, u, q, rqm


CYL_ILB2 = 3


def run_ref_cyl(prec, order, g, e, b, ix, x, u, q, rqm):
    a = [po.aligned_copy(v) for v in (ix, x, u, q)]
    j = po.aligned(g.shape, po.dtype_of(prec))
    ee, bb = po.aligned_copy(e), po.aligned_copy(b)
    ene = po.push_cyl(prec, order, a[0], a[1], a[2], a[3], 1, NP, rqm, CYL_ILB2, ee, bb, j,
                      g.size, g.gcl, g.dx, DT, impl="ref")
    return a, j, ene


def cyl_fixtures():
    seed = 300
    for prec in ("f64", "f32"):
        for order in (1, 2, 3, 4):
            seed += 1
            g, e, b, ix, x, u, q, rqm = make_case(prec, 2, order, seed)
            u[:NP, 2] *= 3.0            # strong azimuthal motion: the p_theta correction
            a, j, ene = run_ref_cyl(prec, order, g, e, b, ix, x, u, q, rqm)
            np.savez_compressed(
                os.path.join(OUT, f"push_2dcyl_s{order}_{prec}.npz"),
                nx=np.array(g.nx), dx=np.array(g.dx), dt=np.array(DT), np_=np.array(NP),
                rqm=np.array(rqm), order=np.array(order), ilb2=np.array(CYL_ILB2),
                e=e, b=b, ix_in=ix[:NP], x_in=x[:NP], u_in=u[:NP], q_in=q[:NP],
                ix_out=np.asarray(a[0])[:NP], x_out=np.asarray(a[1])[:NP],
                u_out=np.asarray(a[2])[:NP], j_out=np.asarray(j), ene=np.array(ene))
            print(f"push_2dcyl_s{order}_{prec}.npz  ene={ene!r}")


def run_ref(prec, dim, order, g, e, b, ix, x, u, q, rqm):
    a = [po.aligned_copy(v) for v in (ix, x, u, q)]
    j = po.aligned(g.shape, po.dtype_of(prec))
    ee, bb = po.aligned_copy(e), po.aligned_copy(b)
    ene = po.push(prec, dim, order, a[0], a[1], a[2], a[3], 1, NP, rqm, ee, bb, j, g.size,
                  g.gcl, g.dx, DT, impl="ref")
    return a, j, ene


def mt_kat():
    src = r"""
#include <random>
#include <cstdio>
#include <cstdint>
int main(){
  unsigned seeds[2] = {5489u, 20261203u};
  for (int s = 0; s < 2; s++) {
    std::mt19937 g(seeds[s]);
    for (int i = 0; i < 1000; i++) printf("%u\n", (unsigned)g());
  }
}
"""
    with tempfile.TemporaryDirectory() as td:
        cpp = os.path.join(td, "kat.cpp")
        exe = os.path.join(td, "kat")
        open(cpp, "w").write(src)
        subprocess.run(["g++", "-O1", "-o", exe, cpp], check=True)
        out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    v = np.array([int(t) for t in out.split()], dtype=np.uint64).reshape(2, 1000)
    # OSIRIS seed s such that s ^ 0x80000000 == standard seed
    osiris_seed = np.array([(s ^ 0x80000000) - (1 << 32) if (s ^ 0x80000000) >= (1 << 31)
                            else (s ^ 0x80000000) for s in (5489, 20261203)], dtype=np.int64)
    np.savez_compressed(os.path.join(OUT, "mt_kat.npz"), std_seed=np.array([5489, 20261203]),
                        osiris_seed=osiris_seed, stream=v.astype(np.uint32))


def main():
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    if args:
        po.REFERENCE_SRC = args[0]
    if not po.REFERENCE_SRC:
        raise SystemExit("give the OSIRIS source checkout as the argument or in OSIRIS_REF")
    po.build(with_ref=True)
    if po.ref_lib("f64") is None or po.ref_lib("f32") is None:
        raise SystemExit("reference kernels could not be built (needs x86_64 + AVX2 + sources)")
    if "--cyl" in sys.argv:
        cyl_fixtures()
        return
    seed = 100
    for prec in ("f64", "f32"):
        for dim in (1, 2, 3):
            for order in (1, 2, 3, 4):
                seed += 1
                g, e, b, ix, x, u, q, rqm = make_case(prec, dim, order, seed)
                a, j, ene = run_ref(prec, dim, order, g, e, b, ix, x, u, q, rqm)
                extra = {}
                if prec == "f32" and dim == 3 and order >= 3:
                    up = [v.astype(np.float64) if v.dtype != np.int32 else v
                          for v in (e, b, ix, x, u, q)]
                    _, j64, _ = run_ref("f64", dim, order, g, up[0], up[1], up[2], up[3],
                                        up[4], up[5], rqm)
                    extra["j_ref64"] = np.asarray(j64)
                np.savez_compressed(
                    os.path.join(OUT, f"push_{dim}d_s{order}_{prec}.npz"),
                    nx=np.array(g.nx), dx=np.array(g.dx), dt=np.array(DT), np_=np.array(NP),
                    rqm=np.array(rqm), order=np.array(order),
                    e=e, b=b, ix_in=ix[:NP], x_in=x[:NP], u_in=u[:NP], q_in=q[:NP],
                    ix_out=np.asarray(a[0])[:NP], x_out=np.asarray(a[1])[:NP],
                    u_out=np.asarray(a[2])[:NP], j_out=np.asarray(j), ene=np.array(ene),
                    **extra)
                print(f"push_{dim}d_s{order}_{prec}.npz  ene={ene!r}")
    cyl_fixtures()
    mt_kat()
    print("mt_kat.npz")


if __name__ == "__main__":
    main()
