"""ctypes front end of the CPU parity oracle -- TEST INFRASTRUCTURE ONLY.

Loads ``oracle/liboracle.so`` (the plain-C restatement, pic_oracle.c) and, where it was built,
``oracle/_ref/libref_{f32,f64}.so`` (the reference's own AVX2 kernels compiled from source;
x86_64 only).  Arrays follow the reference memory layout:

* particles: ``ix`` int32 (N, dim), ``x`` (N, dim), ``u`` (N, 3), ``q`` (N,) -- the C-order
  view of the Fortran arrays ``ix(dim, N)``, ``x(dim, N)``, ``p(3, N)``, ``q(N)``;
* grids: (size_z, size_y, size_x, 3) -- the C-order view of ``f(3, size_x, size_y, size_z)``
  with ``size = nx + gcl + gcu`` guard cells (source/vdf/os-vdf-define.f03:35-116).
"""
from __future__ import annotations

import ctypes as C
import os
import platform
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")
# an OSIRIS source checkout, for building oracle/_ref (no default: set OSIRIS_REF)
REFERENCE_SRC = os.environ.get("OSIRIS_REF", "")

# guard cells required by each interpolation order (source/particles/os-particles.f03:321-360)
GUARD = {1: (1, 2), 2: (2, 3), 3: (3, 4), 4: (4, 5)}
PUSHERS = {"boris": 0, "exact": 1, "vay": 2, "hc": 3, "fullrot": 4, "euler": 5,
           "cond_vay": 6}

_lib = None
_ref = {}


def build(with_ref: bool = True) -> None:
    """Compile the oracle (and, on x86_64 with the reference sources present, oracle/_ref)."""
    subprocess.run(["make", "-s", "-C", HERE, "liboracle.so", "liboracle_fast.so"], check=True)
    if (with_ref and platform.machine() in ("x86_64", "AMD64") and REFERENCE_SRC
            and os.path.isdir(REFERENCE_SRC)):
        subprocess.run(["make", "-s", "-C", HERE, "ref", "OSIRIS_REF=" + REFERENCE_SRC],
                       check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build(with_ref=False)
        _lib = C.CDLL(LIB_PATH)
        _declare(_lib)
    return _lib


_fast = None


def fast_lib():
    """The same oracle compiled with -O3 -ffast-math: the timed CPU baseline only."""
    global _fast, _lib
    if _fast is None:
        path = os.path.join(HERE, "liboracle_fast.so")
        if not os.path.exists(path):
            build(with_ref=False)
        _fast = C.CDLL(path)
        _declare(_fast)
    return _fast


def ref_lib(prec: str):
    """The reference's compiled AVX2 kernels, or None where they could not be built."""
    if prec not in _ref:
        path = os.path.join(REF_DIR, f"libref_{prec}.so")
        _ref[prec] = C.CDLL(path) if os.path.exists(path) else None
    return _ref[prec]


P = C.c_void_p
I = C.c_int
D = C.c_double


def _declare(L):
    L.ora_push_f32.argtypes = [I, I, P, P, P, P, I, I, C.c_float, P, P, P, P, P, P, P, P, D, P]
    L.ora_push_f64.argtypes = [I, I, P, P, P, P, I, I, D, P, P, P, P, P, P, P, P, D, P]
    for s_ in ("f32", "f64"):
        getattr(L, f"ora_smooth_{s_}").argtypes = [I, P, P, P, P, P, P]
        getattr(L, f"ora_set_smooth_{s_}").argtypes = [P, P]
        getattr(L, f"ora_set_emf_smooth_{s_}").argtypes = [P, P]
        getattr(L, f"ora_walls_{s_}").argtypes = [I, P, P, P, P, I, I, I]
        getattr(L, f"ora_set_walls_{s_}").argtypes = [I]
        getattr(L, f"ora_set_pmc_{s_}").argtypes = [I]
        getattr(L, f"ora_set_open_{s_}").argtypes = [I, P]
        getattr(L, f"ora_set_window_{s_}").argtypes = [I]
        getattr(L, f"ora_lindman_phase_{s_}").argtypes = [I, P, P, P, I, I, P, P, P, P, D]
        getattr(L, f"ora_pml_state_size_{s_}").argtypes = [I, P, P, P, I, I]
        getattr(L, f"ora_pml_state_size_{s_}").restype = C.c_long
        getattr(L, f"ora_pml_init_{s_}").argtypes = [I, P, P, P, I, I, P, D, P]
        getattr(L, f"ora_pml_phase_{s_}").argtypes = [I, P, P, P, I, I, I, P, P, P, P, D]
        getattr(L, f"ora_set_pml_{s_}").argtypes = [I, I, P]
        getattr(L, f"ora_pml_shift_x_{s_}").argtypes = [I, P, P, P, I, I, P]
    L.ora_set_thermal.argtypes = [I, P, P, C.c_uint32, C.c_uint64, I]
    L.ora_push_cyl_f32.argtypes = [I, P, P, P, P, I, I, C.c_float, I, P, P, P, P, P, P, P, P, D,
                                   P]
    L.ora_push_cyl_f64.argtypes = [I, P, P, P, P, I, I, D, I, P, P, P, P, P, P, P, P, D, P]
    L.ora_push_pusher_f32.argtypes = [I, I, I, P, P, P, P, I, I, C.c_float, P, P, P, P, P, P, P,
                                      P, D, D, P]
    L.ora_push_pusher_f64.argtypes = [I, I, I, P, P, P, P, I, I, D, P, P, P, P, P, P, P, P, D, D,
                                      P]
    L.ora_dudt_exact_f32.argtypes = [I, P, P, P, P, C.c_float, D, D, P]
    L.ora_dudt_exact_f64.argtypes = [I, P, P, P, P, D, D, D, P]
    L.ora_dudt_pusher_f32.argtypes = [I, I, P, P, P, P, C.c_float, D, D, P]
    L.ora_dudt_pusher_f64.argtypes = [I, I, P, P, P, P, D, D, D, P]
    for s in ("f32", "f64"):
        getattr(L, f"ora_yee_advance_{s}").argtypes = [I, P, P, P, P, P, P, P, D]
        getattr(L, f"ora_periodic_{s}").argtypes = [I, P, P, P, P, I]
        getattr(L, f"ora_field_energy_{s}").argtypes = [I, P, P, P, P, P, P]
        getattr(L, f"ora_deposit_rho_{s}").argtypes = [I, I, P, P, P, P, I, P, P, P]
        getattr(L, f"ora_div_{s}").argtypes = [I, P, P, P, P, P, P]
        getattr(L, f"ora_load_{s}").argtypes = [P, I, P, P, P, D, P, P, D, D, P, P, P, P]
        getattr(L, f"ora_step_{s}").argtypes = [I, I, P, P, P, P, D, P, P, P, I, P, P, P, P, P,
                                                P, P, I]
        getattr(L, f"ora_step_pusher_{s}").argtypes = [I, I, I, P, P, P, P, D, P, P, P, I, P, P,
                                                       P, P, P, P, P, I, D]
    L.ora_wrap.argtypes = [I, P, I, P]
    L.ora_sort_index.argtypes = [I, P, I, P, P]
    L.ora_mt_seed.argtypes = [P, I]
    L.ora_mt_int32.argtypes = [P]
    L.ora_mt_int32.restype = C.c_int32
    L.ora_gaussian.argtypes = [P]
    L.ora_gaussian.restype = D
    L.ora_load_f32.restype = I
    L.ora_load_f64.restype = I
    L.ora_max_threads.restype = I


def _p(a):
    return a.ctypes.data_as(P) if a is not None else None


def _i32(v):
    return np.ascontiguousarray(np.asarray(v, dtype=np.int32))


def _f64(v):
    return np.ascontiguousarray(np.asarray(v, dtype=np.float64))


def dtype_of(prec: str):
    return np.float32 if prec == "f32" else np.float64


# ------------------------------------------------------------------------------ grids

class Grid:
    """Periodic box with the guard cells the interpolation order needs."""

    def __init__(self, nx, order, dx, guard=None):
        self.dim = len(nx)
        self.nx = list(nx)
        self.order = order
        gl, gu = guard if guard else GUARD[order]
        self.gcl = [gl] * self.dim
        self.gcu = [gu] * self.dim
        self.size = [n + gl + gu for n in self.nx]
        self.dx = list(dx)

    @property
    def shape(self):
        return tuple(reversed(self.size)) + (3,)

    def zeros(self, prec):
        return np.zeros(self.shape, dtype=dtype_of(prec))

    def interior(self, f):
        """View of the interior points 1..nx of a grid array."""
        sl = tuple(slice(gl, gl + n) for gl, n in zip(reversed(self.gcl), reversed(self.nx)))
        return f[sl]

    def args(self):
        return _i32(self.nx), _i32(self.gcl), _i32(self.gcu)


# ------------------------------------------------------------------------------ push

def push(prec, dim, order, ix, x, u, q, i0, i1, rqm, e, b, j, emf_size, emf_off, dx, dt,
         impl="oracle", pusher="boris", iter_tol=1e-3):
    """One vadvance_deposit call; arrays are updated in place; returns the energy sum.
    pusher "exact", "vay" or "hc" replaces the Boris momentum update by dudt_exact / dudt_vay /
    dudt_cary with the double dt (the Fortran advance_deposit path)."""
    ene = np.zeros(1, dtype=np.float64)
    es, eo = _i32(emf_size), _i32(emf_off)
    dxa = _f64(list(dx) + [0.0] * (3 - len(dx)))
    if pusher != "boris":
        if impl != "oracle":
            raise ValueError("the reference kernels have the Boris pusher only")
        f = getattr(lib(), f"ora_push_pusher_{prec}")
        rc = f(PUSHERS[pusher], dim, order, _p(ix), _p(x), _p(u), _p(q), int(i0), int(i1), rqm,
               _p(e), _p(b), _p(es), _p(eo), _p(j), _p(es), _p(eo), _p(dxa), float(dt),
               float(iter_tol), _p(ene))
        if rc != 0:
            raise ValueError("bad dim/order")
    elif impl == "oracle":
        f = getattr(lib(), f"ora_push_{prec}")
        rc = f(dim, order, _p(ix), _p(x), _p(u), _p(q), int(i0), int(i1), rqm, _p(e), _p(b),
               _p(es), _p(eo), _p(j), _p(es), _p(eo), _p(dxa), float(dt), _p(ene))
        if rc != 0:
            raise ValueError("bad dim/order")
    else:
        L = ref_lib(prec)
        if L is None:
            raise RuntimeError("reference kernels not built (oracle/_ref)")
        name = {1: "1d", 2: "2d", 3: "3d"}[dim]
        f = getattr(L, f"vadvance_deposit_{name}_s{order}_")
        ctype = C.c_float if prec == "f32" else C.c_double
        a0, a1, rq, dtv = C.c_int(int(i0)), C.c_int(int(i1)), ctype(rqm), C.c_double(dt)
        f(_p(ix), _p(x), _p(u), _p(q), C.byref(a0), C.byref(a1), C.byref(rq), _p(e), _p(b),
          _p(es), _p(eo), _p(j), _p(es), _p(eo), _p(dxa), C.byref(dtv), _p(ene))
    return float(ene[0])


def push_cyl(prec, order, ix, x, u, q, i0, i1, rqm, ilb2, e, b, j, emf_size, emf_off, dx, dt,
             impl="oracle"):
    """One 2D cylindrical vadvance_deposit_2d_cyl_sK call (x1 = z, x2 = r; ilb2 = the lower
    global cell of the node along x2); arrays updated in place; returns the energy sum."""
    ene = np.zeros(1, dtype=np.float64)
    es, eo = _i32(emf_size), _i32(emf_off)
    dxa = _f64(list(dx) + [0.0] * (3 - len(dx)))
    if impl == "oracle":
        f = getattr(lib(), f"ora_push_cyl_{prec}")
        rc = f(int(order), _p(ix), _p(x), _p(u), _p(q), int(i0), int(i1), rqm, int(ilb2),
               _p(e), _p(b), _p(es), _p(eo), _p(j), _p(es), _p(eo), _p(dxa), float(dt), _p(ene))
        if rc != 0:
            raise ValueError("bad order")
    else:
        L = ref_lib(prec)
        if L is None:
            raise RuntimeError("reference kernels not built (oracle/_ref)")
        f = getattr(L, f"vadvance_deposit_2d_cyl_s{order}_")
        ctype = C.c_float if prec == "f32" else C.c_double
        a0, a1, rq, dtv = C.c_int(int(i0)), C.c_int(int(i1)), ctype(rqm), C.c_double(dt)
        lb = C.c_int(int(ilb2))
        f(_p(ix), _p(x), _p(u), _p(q), C.byref(a0), C.byref(a1), C.byref(rq), C.byref(lb),
          _p(e), _p(b), _p(es), _p(eo), _p(j), _p(es), _p(eo), _p(dxa), C.byref(dtv), _p(ene))
    return float(ene[0])


def dudt(pusher, prec, e, b, u, q, rqm, dt, iter_tol=1e-3):
    """Momentum update ("exact", "vay", "hc", "fullrot", "euler") of n particles in given fields e (n,3), b (n,3);
    u updated in place; returns the energy sum the reference pusher reports."""
    ene = np.zeros(1, dtype=np.float64)
    f = getattr(lib(), f"ora_dudt_pusher_{prec}")
    f(PUSHERS[pusher], len(q), _p(e), _p(b), _p(u), _p(q), rqm, float(dt), float(iter_tol),
      _p(ene))
    return float(ene[0])


def dudt_exact(prec, e, b, u, q, rqm, dt, iter_tol=1e-3):
    """Exact momentum update of n particles in given fields e (n,3), b (n,3); u updated in
    place; returns sum q (gamma - 1) of the new momenta."""
    ene = np.zeros(1, dtype=np.float64)
    f = getattr(lib(), f"ora_dudt_exact_{prec}")
    f(len(q), _p(e), _p(b), _p(u), _p(q), rqm, float(dt), float(iter_tol), _p(ene))
    return float(ene[0])


# ------------------------------------------------------------------------------ grid phases

def yee_advance(g: Grid, prec, e, b, j, dt):
    nx, gl, gu = g.args()
    getattr(lib(), f"ora_yee_advance_{prec}")(g.dim, _p(nx), _p(gl), _p(gu), _p(e), _p(b),
                                               _p(j), _p(_f64(g.dx + [0.0] * 3)), float(dt))


def periodic(g: Grid, prec, f, add):
    nx, gl, gu = g.args()
    getattr(lib(), f"ora_periodic_{prec}")(g.dim, _p(nx), _p(gl), _p(gu), _p(f), int(add))


def field_energy(g: Grid, prec, f):
    nx, gl, gu = g.args()
    out = np.zeros(3)
    getattr(lib(), f"ora_field_energy_{prec}")(g.dim, _p(nx), _p(gl), _p(gu), _p(f),
                                                _p(_f64(g.dx + [0.0] * 3)), _p(out))
    return out


def deposit_rho(g: Grid, prec, ix, x, q):
    nx, gl, gu = g.args()
    rho = np.zeros(g.shape, dtype=np.float64)
    getattr(lib(), f"ora_deposit_rho_{prec}")(g.dim, g.order, _p(nx), _p(gl), _p(gu), _p(rho),
                                               len(q), _p(ix), _p(x), _p(q))
    return rho


def div(g: Grid, prec, f):
    nx, gl, gu = g.args()
    out = np.zeros(tuple(reversed(g.nx)), dtype=np.float64)
    getattr(lib(), f"ora_div_{prec}")(g.dim, _p(nx), _p(gl), _p(gu), _p(f),
                                       _p(_f64(g.dx + [0.0] * 3)), _p(out))
    return out


def wrap(g: Grid, ix):
    lib().ora_wrap(g.dim, _p(_i32(g.nx)), ix.shape[0], _p(ix))


def sort_index(g: Grid, ix):
    idx = np.zeros(ix.shape[0], dtype=np.int32)
    lib().ora_sort_index(g.dim, _p(_i32(g.nx)), ix.shape[0], _p(ix), _p(idx))
    return idx


# ------------------------------------------------------------------------------ RNG / load

class MT(C.Structure):
    _fields_ = [("mt", C.c_uint32 * 624), ("mti", C.c_int), ("have_gauss", C.c_int),
                ("gauss", C.c_double)]


def mt_new(seed: int) -> MT:
    r = MT()
    lib().ora_mt_seed(C.byref(r), int(seed))
    return r


def mt_int32(r: MT) -> int:
    return lib().ora_mt_int32(C.byref(r))


def gaussian(r: MT) -> float:
    return lib().ora_gaussian(C.byref(r))


def load(rng: MT, prec, dim, nx, ppc, dx, rqm, uth, ufl, amp=0.0, kmode=1.0):
    """Lattice load of one species (returns ix, x, u, q)."""
    n = int(np.prod(nx)) * int(np.prod(ppc))
    dt_ = dtype_of(prec)
    ix = np.zeros((n, dim), np.int32)
    x = np.zeros((n, dim), dt_)
    u = np.zeros((n, 3), dt_)
    q = np.zeros(n, dt_)
    got = getattr(lib(), f"ora_load_{prec}")(C.byref(rng), dim, _p(_i32(nx)), _p(_i32(ppc)),
                                              _p(_f64(list(dx) + [0.0] * 3)), float(rqm),
                                              _p(_f64(uth)), _p(_f64(ufl)), float(amp),
                                              float(kmode), _p(ix), _p(x), _p(u), _p(q))
    assert got == n
    return ix, x, u, q


# ------------------------------------------------------------------------------ full step

def walls(g: "Grid", prec, f, kind, mask):
    """Conducting-wall images on the axes in `mask` (bit d), in place: kind 0 E, 1 B (guard
    points set from their images), 2 J (guard values added into the box); 3 E, 4 B of a perfect
    magnetic conductor."""
    nx, gl, gu = g.args()
    getattr(lib(), f"ora_walls_{prec}")(g.dim, _p(nx), _p(gl), _p(gu), _p(f), int(kind),
                                        int(mask), g.order)


def lindman_state(g: "Grid", prec, axis):
    """Zeroed state of Lindman open boundaries at both edges of `axis` (15 reals per interior
    point of the other axes), kept by the caller between steps."""
    n = 1
    for a in range(g.dim):
        if a != axis:
            n *= g.nx[a]
    return np.zeros(15 * n, dtype=dtype_of(prec))


def lindman_phase(g: "Grid", prec, axis, what, e, b, state, dt):
    """One phase of the Lindman boundaries on `axis`, in place (what 0 after the E step, 1
    after a B half step, 2 the restore of the boundary planes)."""
    nx, gl, gu = g.args()
    getattr(lib(), f"ora_lindman_phase_{prec}")(g.dim, _p(nx), _p(gl), _p(gu), int(axis),
                                                 int(what), _p(e), _p(b), _p(state),
                                                 _p(_f64(g.dx + [0.0] * 3)), float(dt))


def pml_state(g: "Grid", prec, mask, nb, dt):
    """State of PML walls of nb cells at both edges of the axes in `mask` (2D): zeroed walls
    and the attenuation tables, kept by the caller between steps."""
    nx, gl, gu = g.args()
    L = lib()
    n = getattr(L, f"ora_pml_state_size_{prec}")(g.dim, _p(nx), _p(gl), _p(gu), int(mask),
                                                 int(nb))
    st = np.zeros(n, dtype=dtype_of(prec))
    getattr(L, f"ora_pml_init_{prec}")(g.dim, _p(nx), _p(gl), _p(gu), int(mask), int(nb),
                                       _p(_f64(g.dx + [0.0] * 3)), float(dt), _p(st))
    return st


def pml_phase(g: "Grid", prec, mask, nb, what, e, b, state, dt):
    """One PML phase for the axes in `mask`, in place (what 0 the walls' guard update, 1 E
    walls with the B interfaces, 2 B walls with the E interfaces)."""
    nx, gl, gu = g.args()
    getattr(lib(), f"ora_pml_phase_{prec}")(g.dim, _p(nx), _p(gl), _p(gu), int(mask), int(nb),
                                             int(what), _p(e), _p(b), _p(state),
                                             _p(_f64(g.dx + [0.0] * 3)), float(dt))


def step(g: Grid, prec, e, b, j, species, dt, nthreads=1, fast=False, pusher="boris",
         iter_tol=1e-3, smooth=None, walls=0, open_fields=None, thermal=None, pmc=0,
         window=False, smooth_emf=None, pml=None):
    """One full time step; species = list of dicts with ix, x, u, q, rqm.  walls (bit d):
    axis d bounded by conducting walls instead of periodic.  open_fields = (axis, state from
    lindman_state): Lindman open boundaries at both edges of that axis, particles absorbed
    there (left in the arrays with charge and momentum 0).  pml = (mask, nb, state from
    pml_state): PML walls of nb cells at both edges of the axes in mask (bit 3: x1 is a moving
    window's axis), particles absorbed there the same way.  thermal = dict(mask, uth, ufl, seed,
    step, type: 0 thermal, 1 random dir, 2 waterbag): particles crossing the edges of the axes in mask (walled or open) are re-emitted from
    a thermal bath; step keys the random stream.  pmc (bit d, d walled): perfect magnetic
    instead of electric conductor walls.  window=True: x1 is the axis of a moving window (no
    guard update along it, particles absorbed below cell 1 -- removed from the species arrays
    after the step -- and reflected above nx); the window's moves are Window.start_step.
    smooth = (type, order) filters the folded current; smooth_emf = (type, order) gives the
    particles smoothed copies of E and B (the reference's e_part / b_part, smooth_type
    "stand"), E and B themselves unchanged.
    Returns the per-species energy sums (Boris: time-centred u^2/(gamma+1); exact pusher:
    gamma - 1 of the new momentum; both times q).  fast=True runs the -O3 -ffast-math build
    (timing only)."""
    nx, gl, gu = g.args()
    ns = len(species)
    np_ = _i32([len(s["q"]) for s in species])
    PA = P * ns
    ixs = PA(*[_p(s["ix"]) for s in species])
    xs = PA(*[_p(s["x"]) for s in species])
    us = PA(*[_p(s["u"]) for s in species])
    qs = PA(*[_p(s["q"]) for s in species])
    rqm = np.asarray([s["rqm"] for s in species], dtype=dtype_of(prec))
    ene = np.zeros(ns)
    L = fast_lib() if fast else lib()
    if smooth is not None:
        ordv, coef = _smooth_tables(g.dim, prec, [smooth[0]] * g.dim, [smooth[1]] * g.dim)
        getattr(L, f"ora_set_smooth_{prec}")(_p(ordv), _p(coef))
    if smooth_emf is not None:
        eord, ecoef = _smooth_tables(g.dim, prec, [smooth_emf[0]] * g.dim,
                                     [smooth_emf[1]] * g.dim)
        getattr(L, f"ora_set_emf_smooth_{prec}")(_p(eord), _p(ecoef))
    args = (g.dim, g.order, _p(nx), _p(gl), _p(gu), _p(_f64(g.dx + [0.0] * 3)), float(dt), _p(e),
            _p(b), _p(j), ns, _p(np_), ixs, xs, us, qs, _p(rqm), _p(ene), int(nthreads))
    getattr(L, f"ora_set_walls_{prec}")(int(walls))
    getattr(L, f"ora_set_pmc_{prec}")(int(pmc))
    getattr(L, f"ora_set_window_{prec}")(1 if window else 0)
    if open_fields is not None:
        getattr(L, f"ora_set_open_{prec}")(int(open_fields[0]), _p(open_fields[1]))
    if pml is not None:
        getattr(L, f"ora_set_pml_{prec}")(int(pml[0]), int(pml[1]), _p(pml[2]))
    if thermal is not None:
        L.ora_set_thermal(int(thermal["mask"]), _p(_f64(thermal["uth"])),
                          _p(_f64(thermal.get("ufl", [0.0] * 3))), int(thermal.get("seed", 0)),
                          int(thermal["step"]), int(thermal.get("type", 0)))
    try:
        if pusher != "boris":
            getattr(L, f"ora_step_pusher_{prec}")(PUSHERS[pusher], *args, float(iter_tol))
        else:
            getattr(L, f"ora_step_{prec}")(*args)
    finally:
        getattr(L, f"ora_set_walls_{prec}")(0)
        getattr(L, f"ora_set_pmc_{prec}")(0)
        getattr(L, f"ora_set_window_{prec}")(0)
        getattr(L, f"ora_set_open_{prec}")(-1, None)
        getattr(L, f"ora_set_pml_{prec}")(0, 0, None)
        L.ora_set_thermal(0, None, None, 0, 0, 0)
    if smooth is not None:
        getattr(L, f"ora_set_smooth_{prec}")(None, None)
    if smooth_emf is not None:
        getattr(L, f"ora_set_emf_smooth_{prec}")(None, None)
    if window:
        for sp in species:
            keep = sp["ix"][:, 0] > ORA_GONE // 2
            if not keep.all():
                for k in ("ix", "x", "u", "q"):
                    sp[k] = np.ascontiguousarray(sp[k][keep])
    return ene


ORA_GONE = -(1 << 28)


class Window:
    """Moving window along x1 at c (the oracle's restatement):

    * move_boundary_space_global (source/os-space.f90:508-566): every step starts by adding dt
      to the window motion; once it reaches dx1 the window moves one cell;
    * a move shifts E and B one cell down along x1, guard cells included, the last x1 plane
      becoming zero (move_window_vdf, source/vdf/os-vdf.f03:56-205), lowers every particle's
      x1 cell index by one (move_window_species, source/spec/os-species.f03:171-229) and fills
      the new last plane of cells with plasma of the injected species (inject_std,
      source/spec/psource/os-psource-std.f03:759-1120): ppc[d] particles per cell on the
      OSIRIS lattice, at rest, charge sign(rqm) den / prod(ppc) with den the piecewise-linear
      profile (prof_x, prof_f; 0 outside) at the particle's global x1 position.
    Call start_step before every step(..., window=True)."""

    def __init__(self, g: Grid, prec, species_index, ppc, prof_x, prof_f):
        self.g, self.prec = g, prec
        self.k = species_index
        self.ppc = list(ppc) + [1] * (3 - len(ppc))
        self.prof_x, self.prof_f = list(prof_x), list(prof_f)
        self.xmoved = 0.0
        self.moves = 0

    def _den(self, x):
        px, pf = self.prof_x, self.prof_f
        if x < px[0] or x > px[-1]:
            return 0.0
        for i in range(1, len(px)):
            if x <= px[i]:
                w = (x - px[i - 1]) / (px[i] - px[i - 1])
                return pf[i - 1] + w * (pf[i] - pf[i - 1])
        return pf[-1]

    def start_step(self, e, b, species, dt, pml=None):
        """Advance the window motion; on a move shift the fields and particles and inject.
        pml = (mask, nb, state): PML walls of other axes shift with the fields.  Returns True
        when the window moved."""
        self.xmoved += dt
        if self.xmoved < self.g.dx[0]:
            return False
        self.xmoved -= self.g.dx[0]
        self.moves += 1
        for f in (e, b):
            f[..., :-1, :] = f[..., 1:, :].copy()
            f[..., -1, :] = 0
        if pml is not None:
            nx, gl, gu = self.g.args()
            getattr(lib(), f"ora_pml_shift_x_{self.prec}")(self.g.dim, _p(nx), _p(gl), _p(gu),
                                                            int(pml[0]), int(pml[1]),
                                                            _p(pml[2]))
        for sp in species:
            sp["ix"][:, 0] -= 1
        self._inject(species[self.k])
        return True

    def _inject(self, sp):
        g, dim = self.g, self.g.dim
        dt_ = dtype_of(self.prec)
        ppc = self.ppc
        per = int(np.prod(ppc[:dim]))
        unit = np.float32(1.0) / np.float32(per) if dt_ == np.float32 else 1.0 / per
        unit = (-1.0 if sp["rqm"] < 0 else 1.0) * float(unit)
        ny = g.nx[1] if dim > 1 else 1
        nz = g.nx[2] if dim > 2 else 1
        ix, x, q = [], [], []
        for ck in range(nz):
            for cj in range(ny):
                for sa in range(ppc[0]):
                    for sb in range(ppc[1] if dim > 1 else 1):
                        for sc in range(ppc[2] if dim > 2 else 1):
                            # lattice offset (2 (s + 1) - 1 - ppc) * (0.5 / ppc), in the
                            # particles' precision
                            off = [dt_(2 * (s + 1) - 1 - p) * (dt_(0.5) / dt_(p))
                                   for s, p in zip((sa, sb, sc), ppc)]
                            xg = (self.moves + g.nx[0] - 0.5 + float(off[0])) * g.dx[0]
                            den = self._den(xg)
                            if dt_ == np.float32:
                                den = float(np.float32(den))
                            if not den > 0.0:
                                continue
                            ix.append([g.nx[0], 1 + cj, 1 + ck][:dim])
                            x.append(off[:dim])
                            q.append(den * unit)
        if not q:
            return
        sp["ix"] = np.ascontiguousarray(np.vstack([sp["ix"], np.array(ix, np.int32)]))
        sp["x"] = np.ascontiguousarray(np.vstack([sp["x"], np.array(x, dt_)]))
        sp["u"] = np.ascontiguousarray(np.vstack([sp["u"], np.zeros((len(q), 3), dt_)]))
        sp["q"] = np.ascontiguousarray(np.concatenate([sp["q"], np.array(q, dt_)]))


def max_threads() -> int:
    return lib().ora_max_threads()


def aligned(shape, dtype, align=64):
    """Zeroed array whose data pointer is `align`-byte aligned (the reference kernels use
    aligned 256-bit loads)."""
    dtype = np.dtype(dtype)
    n = int(np.prod(shape)) * dtype.itemsize
    buf = np.zeros(n + align, dtype=np.uint8)
    off = (-buf.ctypes.data) % align
    return buf[off:off + n].view(dtype).reshape(shape)


def aligned_copy(a, align=64):
    out = aligned(a.shape, a.dtype, align)
    out[...] = a
    return out


# ------------------------------------------------------------------------ laser launch

def zpulse(dim, order, nx, dx, xmin, prec, omega0, a0, pol, lon_x0, lon_duration, lon_range,
           per_w0, per_focus, per_center):
    """Numpy restatement of the zpulse launch at t = 0 (forward, gaussian longitudinal,
    Hermite-Gaussian TEM00 transverse; source/zpulse/os-zpulse-std.f03: launch_zpulse_2d
    :1072-1212, launch_zpulse_3d :1218-1390, lon_envelope :2480-2561, per_envelope_2d/3d
    :2599-3049).  Returns (e, b) on a zeroed grid with guard cells."""
    gl, gu = GUARD[order]
    size = [n + gl + gu for n in nx]
    dt_ = dtype_of(prec)
    half = order in (2, 4)
    idx = [np.arange(sz) - gl + 1 for sz in size]      # Fortran cell index incl. guards
    base = [xmin[d] + (dx[d] / 2 if half else 0.0) for d in range(dim)]
    amp = omega0 * a0
    k = omega0

    def lon(z):
        s_ = (z - lon_x0) / lon_duration
        return np.where(np.abs(z - lon_x0) > lon_range / 2, 0.0, np.exp(-2 * (s_ * s_)))

    def per(x1, x2, x3):
        ox = x2 - per_center[0]
        rho2 = ox * ox if dim == 2 else ox * ox + (x3 - per_center[1]) ** 2
        z = x1 - per_focus
        z0 = k * per_w0 ** 2 / 2
        nz = z != 0
        rwl2 = np.where(nz, z0 ** 2 / (z0 ** 2 + z ** 2), 1.0)
        curv = np.where(nz, 0.5 * rho2 * z / (z ** 2 + z0 ** 2), 0.0)
        gouy = np.where(nz, np.arctan2(z, z0), 0.0)
        a = np.sqrt(rwl2) if dim == 3 else np.sqrt(np.sqrt(rwl2))
        return a * np.exp(-rho2 * rwl2 / per_w0 ** 2) * np.cos(k * (x1 - lon_x0) + k * curv - gouy)

    z = base[0] + (idx[0] - 1) * dx[0]
    r1 = base[1] + (idx[1] - 1) * dx[1]
    z2, r12 = z + dx[0] / 2, r1 + dx[1] / 2
    cp, sp = np.cos(pol), np.sin(pol)
    shape = tuple(reversed(size)) + (3,)
    e = np.zeros(shape, dt_)
    b = np.zeros(shape, dt_)
    if dim == 2:
        Z, R = np.meshgrid(z, r1, indexing="xy")
        Z2, R2 = np.meshgrid(z2, r12, indexing="xy")
        le, le2 = amp * lon(Z), amp * lon(Z2)
        b[..., 1] = (-le2 * per(Z2, R, 0) * sp).astype(dt_)
        b[..., 2] = (le2 * per(Z2, R2, 0) * cp).astype(dt_)
        e[..., 1] = (le * per(Z, R2, 0) * cp).astype(dt_)
        e[..., 2] = (le * per(Z, R, 0) * sp).astype(dt_)
    else:
        r2 = base[2] + (idx[2] - 1) * dx[2]
        r22 = r2 + dx[2] / 2

        def grid(a1, a2, a3):
            A3, A2, A1 = np.meshgrid(a3, a2, a1, indexing="ij")
            return A1, A2, A3

        X1, X2, X3 = grid(z2, r1, r22)
        b[..., 1] = b[..., 1] - (amp * lon(X1) * per(X1, X2, X3) * sp).astype(dt_)
        X1, X2, X3 = grid(z2, r12, r2)
        b[..., 2] = b[..., 2] + (amp * lon(X1) * per(X1, X2, X3) * cp).astype(dt_)
        X1, X2, X3 = grid(z, r12, r2)
        e[..., 1] = e[..., 1] + (amp * lon(X1) * per(X1, X2, X3) * cp).astype(dt_)
        X1, X2, X3 = grid(z, r1, r22)
        e[..., 2] = e[..., 2] + (amp * lon(X1) * per(X1, X2, X3) * sp).astype(dt_)
    return e, b


# ------------------------------------------------------------------------ smoothing

SMOOTH = dict(none=0, binomial=2, compensated=3, fivepass=4, tri6=5, tri8=6)


def _combine_kernel3(k3, n):
    """combine_kernel3 (source/vdf/os-vdf-smooth.f90:151-183): n 3-point kernels -> 2n+1."""
    out = [0.0] * (2 * n + 1)
    out[n] = 1.0
    for k in range(n):
        f1 = 0.0
        for j in range(n - k, n + k + 2):
            out[j - 1] = k3[k][2] * out[j] + out[j - 1]
            f2 = k3[k][0] * out[j]
            out[j] = k3[k][1] * out[j] + f1
            f1 = f2
    return out


def smooth_coefficients(stype, order, prec="f64"):
    """setup_smooth restated (source/vdf/os-vdf-smooth.f90:373-467): the normalised kernel of
    one axis.  prec "f32" follows the single-precision build (coefficients held in float,
    normalised with a double total); returns (n, list of 2n+1 floats)."""
    if stype == 0:
        return 0, [1.0]
    if stype == 2:
        n = order
        k3 = [(1.0, 2.0, 1.0)] * n
    elif stype == 3:
        n = max(2, order)
        comp = float(np.float32(np.float32(4.0) + np.float32(2.0) * np.float32(n - 1)) /
                     np.float32(n - 1))
        k3 = [(1.0, 2.0, 1.0)] * (n - 1) + [(-1.0, comp, -1.0)]
    elif stype == 4:
        n = 5
        k3 = [(1.0, 2.0, 1.0)] * 4 + [(-5.0, 15.0, -5.0)]
    elif stype == 5:
        n, c = 3, [0.015625, -0.09375, 0.234375, 0.6875, 0.234375, -0.09375, 0.015625]
    elif stype == 6:
        n, c = 4, [-0.00390625, 0.03125, -0.109375, 0.21875, 0.7265625, 0.21875, -0.109375,
                   0.03125, -0.00390625]
    else:
        raise ValueError("unknown smoothing type")
    if stype in (2, 3, 4):
        c = _combine_kernel3(k3, n)
    if prec == "f32":
        c = [float(np.float32(v)) for v in c]
    total = 0.0
    for v in c:
        total = total + v
    c = [v / total for v in c]
    if prec == "f32":
        c = [float(np.float32(v)) for v in c]
    return n, c


def _smooth_tables(dim, prec, types, orders):
    ordv = np.zeros(3, np.int32)
    coef = np.zeros(3 * 31, dtype_of(prec))
    for d in range(dim):
        n, c = smooth_coefficients(types[d], orders[d], prec)
        ordv[d] = n
        coef[31 * d: 31 * d + len(c)] = c
    return ordv, coef


def smooth(g: Grid, prec, f, types, orders):
    """filter_2d/3d in place (source/vdf/os-vdf-smooth.f90:639-1000)."""
    nx, gl, gu = g.args()
    ordv, coef = _smooth_tables(g.dim, prec, types, orders)
    getattr(lib(), f"ora_smooth_{prec}")(g.dim, _p(nx), _p(gl), _p(gu), _p(f), _p(ordv), _p(coef))
