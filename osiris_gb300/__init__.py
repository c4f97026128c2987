"""osiris_gb300 -- GB300 (sm_103a) implementation of the OSIRIS particle-in-cell time step.

Python front end of the C ABI in ``include/osiris_gb300.h`` (ctypes over the in-tree
``libosiris_gb300.so``).  Two layers, mirroring the reference:

* drop-in calls with the reference's arguments on host arrays in the reference layout:
  :func:`vadvance_deposit` (FNAME(vadvance_deposit_{1d,2d,3d}_sN), source/simd/
  os-spec-push-avx2{,d}.c), :func:`yee_advance` (advance_yee, source/emf/solver/
  os-emf-solver-yee.f03:542-568), :func:`periodic` (update_periodic_vdf, source/vdf/
  os-vdf-comm.f90:142-326);
* :class:`Simulation`, a device-resident time stepper (phase order of iter_sim,
  source/os-simulation.f03:498-666) with the plain (reference layout, FP64 or FP32) and the
  tiled (FP32) particle engines.

Array conventions (C-order views of the Fortran arrays): particles ``ix`` int32 (N, dim),
``x`` (N, dim), ``u`` (N, 3), ``q`` (N,); grids (size_z, size_y, size_x, 3) with
``size = nx + gcl + gcu``.  Errors raise :class:`OsirisGB300Error`; there is no CPU fallback:
if the library is missing or no GPU is present the calls fail.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libosiris_gb300.so")

OSG_OK = 0
ENGINE_PLAIN = 0
ENGINE_TILED = 1
PUSHER_BORIS = 0
PUSHER_EXACT = 1
PUSHER_VAY = 2
PUSHER_HC = 3
PUSHER_FULLROT = 4
PUSHER_EULER = 5
PUSHER_COND_VAY = 6
SMOOTH_NONE, SMOOTH_BINOMIAL, SMOOTH_COMPENSATED = 0, 2, 3
SMOOTH_5PASS, SMOOTH_TRI6, SMOOTH_TRI8 = 4, 5, 6
RNG_BYTES = 2512

# guard cells per interpolation order (source/particles/os-particles.f03:321-360)
GUARD = {1: (1, 2), 2: (2, 3), 3: (3, 4), 4: (4, 5)}


class OsirisGB300Error(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"osiris_gb300 error {code}: {msg}")
        self.code = code


_lib = None


def lib():
    """The loaded native library (built by ``__graft_entry__.build()`` / osiris_gb300.build)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise OsirisGB300Error(-2, f"native library not built: {LIB_PATH}")
        _lib = C.CDLL(LIB_PATH)
        _declare(_lib)
        _declare_batch(_lib)
    return _lib


P, I, L, D, F = C.c_void_p, C.c_int, C.c_long, C.c_double, C.c_float


class Config(C.Structure):
    _fields_ = [("dim", I), ("order", I), ("precision", I), ("engine", I), ("nx", I * 3),
                ("dx", D * 3), ("dt", D), ("tile", I * 3), ("n_sort", I), ("capacity", D),
                ("pusher", I), ("iter_tol", D), ("smooth_type", I), ("smooth_order", I),
                ("walls", I),
                ("open_fields", I),
                ("thermal", I), ("seed", C.c_uint), ("uth_bnd", D * 3), ("ufl_bnd", D * 3),
                ("thermal_type", I), ("pmc", I), ("emf_smooth_type", I),
                ("emf_smooth_order", I), ("pml", I), ("pml_cells", I),
                ("pml_diffuse", I)]


def _declare(lb):
    lb.osg_last_error.restype = C.c_char_p
    lb.osg_version.restype = I
    lb.osg_device_count.restype = I
    lb.osg_device_memory.argtypes = [P, P]
    lb.osg_host_alloc.argtypes = [C.c_size_t]
    lb.osg_host_alloc.restype = P
    lb.osg_host_free.argtypes = [P]
    lb.osg_vadvance_deposit_f32.argtypes = [I, I, P, P, P, P, I, I, F, P, P, P, P, P, P, P, P, D, P]
    lb.osg_vadvance_deposit_f64.argtypes = [I, I, P, P, P, P, I, I, D, P, P, P, P, P, P, P, P, D, P]
    lb.osg_advance_deposit_exact_f32.argtypes = [I, I, P, P, P, P, I, I, F, P, P, P, P, P, P, P,
                                                 P, D, D, P]
    lb.osg_advance_deposit_exact_f64.argtypes = [I, I, P, P, P, P, I, I, D, P, P, P, P, P, P, P,
                                                 P, D, D, P]
    lb.osg_advance_deposit_f32.argtypes = [I, I, P, P, P, P, I, I, F, P, P, P, P, P, P, P, P, D,
                                           I, D, P]
    lb.osg_advance_deposit_f64.argtypes = [I, I, P, P, P, P, I, I, D, P, P, P, P, P, P, P, P, D,
                                           I, D, P]
    lb.osg_vadvance_deposit_cyl_f32.argtypes = [I, P, P, P, P, I, I, F, I, P, P, P, P, P, P, P,
                                                P, D, P]
    lb.osg_vadvance_deposit_cyl_f64.argtypes = [I, P, P, P, P, I, I, D, I, P, P, P, P, P, P, P,
                                                P, D, P]
    lb.osg_vadvance_deposit_noalloc_f32.argtypes = [I, I, P, P, P, P, I, I, F, P, P, P, P, P, P,
                                                    P, P, D, P]
    for s in ("f32", "f64"):
        getattr(lb, f"osg_yee_advance_{s}").argtypes = [I, P, P, P, P, P, P, P, D]
        getattr(lb, f"osg_periodic_{s}").argtypes = [I, P, P, P, P, I]
        getattr(lb, f"osg_walls_{s}").argtypes = [I, P, P, P, P, I, I, I]
        getattr(lb, f"osg_lindman_{s}").argtypes = [I, P, P, P, I, I, P, P, P, P, D]
        getattr(lb, f"osg_pml_init_{s}").argtypes = [I, P, P, P, I, I, P, D, P]
        getattr(lb, f"osg_pml_{s}").argtypes = [I, P, P, P, I, I, I, P, P, P, P, D]
    lb.osg_particle_wrap.argtypes = [I, P, L, P]
    lb.osg_rng_seed.argtypes = [P, I]
    lb.osg_load_lattice.argtypes = [P, I, I, P, P, P, D, P, P, D, D, P, P, P, P]
    lb.osg_load_lattice.restype = L
    lb.osg_sim_create.argtypes = [C.POINTER(Config), C.POINTER(P)]
    lb.osg_sim_destroy.argtypes = [P]
    lb.osg_sim_add_species.argtypes = [P, D, L, P, P, P, P]
    lb.osg_sim_set_fields.argtypes = [P, P, P]
    lb.osg_sim_get_fields.argtypes = [P, P, P, P]
    lb.osg_sim_num_particles.argtypes = [P, I, C.POINTER(L)]
    lb.osg_sim_get_species.argtypes = [P, I, P, P, P, P]
    lb.osg_sim_step.argtypes = [P, I]
    lb.osg_sim_step_async.argtypes = [P, I]
    lb.osg_sim_sync.argtypes = [P]
    lb.osg_sim_stream.argtypes = [P]
    lb.osg_sim_stream.restype = P
    lb.osg_sim_energy.argtypes = [P, P, P]
    lb.osg_sim_gauss_residual.argtypes = [P, C.POINTER(D), C.POINTER(D)]
    lb.osg_sim_profile.argtypes = [P, I, P]
    lb.osg_sim_autotune.argtypes = [P, I, P, C.POINTER(I), C.POINTER(I)]
    lb.osg_sim_launches_per_step.argtypes = [P]
    lb.osg_sim_time_steps.argtypes = [P, I, C.POINTER(F)]
    lb.osg_sim_tile_occupancy.argtypes = [P, C.POINTER(D)]
    lb.osg_set_device.argtypes = [I]


class BatchConfig(C.Structure):
    _fields_ = [("dim", I), ("order", I), ("dt", D), ("tile", I * 3), ("threads", I),
                ("capacity", D)]


class Zpulse(C.Structure):
    _fields_ = [("omega0", D), ("a0", D), ("pol", D), ("lon_x0", D), ("lon_duration", D),
                ("lon_range", D), ("per_w0", D), ("per_focus", D), ("per_center", D * 2)]


def _declare_batch(lb):
    lb.osg_zpulse_launch.argtypes = [I, I, I, P, P, P, P, P, P, P, P]
    lb.osg_sim_set_window.argtypes = [P, I, P, I, P, P]
    lb.osg_sim_window_moves.argtypes = [P, P]
    lb.osg_sim_guard_cells.argtypes = [P, P, P]
    lb.osg_sim_checkpoint.argtypes = [P, C.c_char_p]
    lb.osg_sim_restore.argtypes = [C.c_char_p, C.POINTER(P)]
    lb.osg_sim_get_config.argtypes = [P, C.POINTER(Config), C.POINTER(I), P]
    lb.osg_smooth_f32.argtypes = [I, P, P, P, P, P, P]
    lb.osg_smooth_f64.argtypes = [I, P, P, P, P, P, P]
    lb.osg_smooth_coefficients.argtypes = [I, I, P, P]
    lb.osg_batch_create.argtypes = [P, P]
    lb.osg_batch_destroy.argtypes = [P]
    lb.osg_batch_add_box.argtypes = [P, P, P]
    lb.osg_batch_add_species.argtypes = [P, I, D, L, P, P, P, P]
    lb.osg_batch_tuning.argtypes = [P, P, P]
    lb.osg_batch_step.argtypes = [P, I]
    lb.osg_batch_time_steps.argtypes = [P, I, P]
    lb.osg_batch_stream.argtypes = [P]
    lb.osg_batch_stream.restype = P
    lb.osg_batch_num_boxes.argtypes = [P]
    lb.osg_batch_launches_per_step.argtypes = [P]
    lb.osg_batch_energy.argtypes = [P, I, P, P]
    lb.osg_batch_get_fields.argtypes = [P, I, P, P, P]
    lb.osg_batch_num_particles.argtypes = [P, I, I, P]
    lb.osg_batch_get_species.argtypes = [P, I, I, P, P, P, P]


def _check(rc):
    if rc < 0:
        raise OsirisGB300Error(rc, lib().osg_last_error().decode(errors="replace"))
    return rc


def _p(a):
    return None if a is None else a.ctypes.data_as(P)


def _i32(v):
    return np.ascontiguousarray(np.asarray(v, dtype=np.int32))


def _f64(v):
    return np.ascontiguousarray(np.asarray(v, dtype=np.float64))


def _prec(a):
    if a.dtype == np.float32:
        return "f32"
    if a.dtype == np.float64:
        return "f64"
    raise TypeError("real arrays must be float32 or float64")


def _need(a, dtype, name):
    if not (isinstance(a, np.ndarray) and a.dtype == dtype and a.flags.c_contiguous
            and a.flags.writeable):
        raise TypeError(f"{name} must be a writable C-contiguous {np.dtype(dtype)} array")


# ------------------------------------------------------------------------ drop-in calls

def vadvance_deposit(dim, order, ix, x, u, q, i0, i1, rqm, efield, bfield, emf_size,
                     emf_offset, j, j_size, j_offset, dx, dt, pusher=PUSHER_BORIS,
                     iter_tol=1e-3):
    """Push particles i0..i1 (1-based, inclusive) and add their current into ``j``.

    Same arguments and in-place semantics as FNAME(vadvance_deposit_<dim>d_s<order>);
    returns the time-centred energy sum the reference adds into ``*ene``.  With
    ``pusher=PUSHER_EXACT`` the momentum update is the exact pusher (push_type = "exact",
    osg_advance_deposit_exact_*) and the energy is sum q (gamma - 1) of the new momenta;
    ``PUSHER_VAY`` / ``PUSHER_HC`` / ``PUSHER_FULLROT`` / ``PUSHER_EULER`` /
    ``PUSHER_COND_VAY`` select the Vay, Higuera-Cary, full-rotation, Euler-rotation and
    conditional Vay updates (push_type "vay", "cary", "fullrot", "euler", "cond_vay";
    osg_advance_deposit_*) with the energy those reference pushers report."""
    prec = _prec(x)
    dt_ = np.float32 if prec == "f32" else np.float64
    _need(ix, np.int32, "ix")
    for a, n in ((x, "x"), (u, "u"), (q, "q"), (j, "j")):
        _need(a, dt_, n)
    for a, n in ((efield, "efield"), (bfield, "bfield")):
        if a.dtype != dt_ or not a.flags.c_contiguous:
            raise TypeError(f"{n} must be C-contiguous {np.dtype(dt_)}")
    ene = np.zeros(1)
    args = (dim, order, _p(ix), _p(x), _p(u), _p(q), int(i0), int(i1), rqm, _p(efield),
            _p(bfield), _p(_i32(emf_size)), _p(_i32(emf_offset)), _p(j), _p(_i32(j_size)),
            _p(_i32(j_offset)), _p(_f64(list(dx) + [0.0] * (3 - len(dx)))), float(dt))
    if pusher == PUSHER_EXACT:
        _check(getattr(lib(), f"osg_advance_deposit_exact_{prec}")(*args, float(iter_tol),
                                                                    _p(ene)))
    elif pusher != PUSHER_BORIS:
        _check(getattr(lib(), f"osg_advance_deposit_{prec}")(*args, int(pusher),
                                                              float(iter_tol), _p(ene)))
    else:
        _check(getattr(lib(), f"osg_vadvance_deposit_{prec}")(*args, _p(ene)))
    return float(ene[0])


def vadvance_deposit_cyl(order, ix, x, u, q, i0, i1, rqm, ilb2, efield, bfield, emf_size,
                         emf_offset, j, j_size, j_offset, dx, dt):
    """2D cylindrical push (x1 = z, x2 = r) of particles i0..i1 with the current added into
    ``j``: FNAME(vadvance_deposit_2d_cyl_s<order>) (osg_vadvance_deposit_cyl_*); ilb2 is the
    lower global cell along x2.  Returns the time-centred energy sum."""
    prec = _prec(x)
    dt_ = np.float32 if prec == "f32" else np.float64
    _need(ix, np.int32, "ix")
    for a, n in ((x, "x"), (u, "u"), (q, "q"), (j, "j")):
        _need(a, dt_, n)
    for a, n in ((efield, "efield"), (bfield, "bfield")):
        if a.dtype != dt_ or not a.flags.c_contiguous:
            raise TypeError(f"{n} must be C-contiguous {np.dtype(dt_)}")
    ene = np.zeros(1)
    _check(getattr(lib(), f"osg_vadvance_deposit_cyl_{prec}")(
        int(order), _p(ix), _p(x), _p(u), _p(q), int(i0), int(i1), rqm, int(ilb2), _p(efield),
        _p(bfield), _p(_i32(emf_size)), _p(_i32(emf_offset)), _p(j), _p(_i32(j_size)),
        _p(_i32(j_offset)), _p(_f64(list(dx) + [0.0] * (3 - len(dx)))), float(dt), _p(ene)))
    return float(ene[0])


NOALLOC_SCRATCH_BYTES = 16 << 20


def vadvance_deposit_noalloc(dim, order, ix, x, u, q, i0, i1, rqm, efield, bfield, emf_size,
                             emf_offset, j, j_size, j_offset, dx, dt):
    """vadvance_deposit (float32 only) without any device allocation: the staging lives in a
    fixed NOALLOC_SCRATCH_BYTES array of the library; larger calls raise (split i0..i1)."""
    _need(ix, np.int32, "ix")
    for a, n in ((x, "x"), (u, "u"), (q, "q"), (j, "j")):
        _need(a, np.float32, n)
    for a, n in ((efield, "efield"), (bfield, "bfield")):
        if a.dtype != np.float32 or not a.flags.c_contiguous:
            raise TypeError(f"{n} must be C-contiguous float32")
    ene = np.zeros(1)
    _check(lib().osg_vadvance_deposit_noalloc_f32(
        dim, order, _p(ix), _p(x), _p(u), _p(q), int(i0), int(i1), rqm, _p(efield), _p(bfield),
        _p(_i32(emf_size)), _p(_i32(emf_offset)), _p(j), _p(_i32(j_size)), _p(_i32(j_offset)),
        _p(_f64(list(dx) + [0.0] * (3 - len(dx)))), float(dt), _p(ene)))
    return float(ene[0])


def yee_advance(dim, nx, gcl, gcu, e, b, j, dx, dt):
    """B half step, E full step, B half step on guard-celled host grids (in place)."""
    prec = _prec(e)
    _check(getattr(lib(), f"osg_yee_advance_{prec}")(
        dim, _p(_i32(nx)), _p(_i32(gcl)), _p(_i32(gcu)), _p(e), _p(b), _p(j),
        _p(_f64(list(dx) + [0.0] * 3)), float(dt)))


def lindman(dim, nx, gcl, gcu, axis, what, e, b, state, dx, dt):
    """One phase of the Lindman open boundaries on host arrays (osg_lindman_*): what 0 after
    the E step, 1 after a B half step (dt the full step), 2 the restore of the boundary planes;
    `state` (15 reals per interior point of the other axes) is kept by the caller."""
    s = _prec(e)
    dt_ = e.dtype
    for a, n in ((e, "e"), (b, "b"), (state, "state")):
        _need(a, dt_, n)
    npts = 3 * int(np.prod([int(nx[d]) + int(gcl[d]) + int(gcu[d]) for d in range(dim)]))
    if e.size != npts or b.size != npts:
        raise ValueError(f"e and b must hold {npts} reals (3 x the guard-celled grid)")
    if not 0 <= int(axis) < dim:
        raise ValueError(f"axis {axis} outside 0..{dim - 1}")
    nperp = int(np.prod([nx[d] for d in range(dim) if d != int(axis)])) if dim > 1 else 1
    if state.size < 15 * nperp:
        raise ValueError(f"state holds {state.size} reals, needs {15 * nperp}")
    _check(getattr(lib(), f"osg_lindman_{s}")(dim, _p(_i32(nx)), _p(_i32(gcl)), _p(_i32(gcu)),
                                              int(axis), int(what), _p(e), _p(b), _p(state),
                                              _p(_f64(list(dx) + [0.0] * 3)), float(dt)))


def pml_state(dim, nx, gcl, gcu, mask, nb, dx, dt, dtype):
    """State of PML walls of nb cells at both edges of the axes in `mask` on a host grid
    (osg_pml_init_*): zeroed split-field walls and the attenuation tables."""
    lb = lib()
    lb.osg_pml_state_size.argtypes = [I, P, P, P, I, I]
    lb.osg_pml_state_size.restype = C.c_long
    n = lb.osg_pml_state_size(dim, _p(_i32(nx)), _p(_i32(gcl)), _p(_i32(gcu)), int(mask), int(nb))
    if n < 0:
        raise OsirisGB300Error(-1, lb.osg_last_error().decode(errors="replace"))
    st = np.zeros(n, dtype=dtype)
    s = "f32" if st.dtype == np.float32 else "f64"
    _check(getattr(lb, f"osg_pml_init_{s}")(dim, _p(_i32(nx)), _p(_i32(gcl)), _p(_i32(gcu)),
                                            int(mask), int(nb), _p(_f64(list(dx) + [0.0] * 3)),
                                            float(dt), _p(st)))
    return st


def pml(dim, nx, gcl, gcu, mask, nb, what, e, b, state, dx, dt):
    """One phase of the PML walls on host arrays (osg_pml_*): what 0 the walls' guard update,
    1 after the first B half step (B interfaces, E walls), 2 after the E step (E interfaces,
    B walls); `state` from pml_state is kept by the caller."""
    s = _prec(state)
    dt_ = state.dtype
    for a, n in ((e, "e"), (b, "b")):
        _need(a, dt_, n)
    npts = 3 * int(np.prod([int(nx[d]) + int(gcl[d]) + int(gcu[d]) for d in range(dim)]))
    if e.size != npts or b.size != npts:
        raise ValueError(f"e and b must hold {npts} reals (3 x the guard-celled grid)")
    _need(state, dt_, "state")
    lb = lib()
    lb.osg_pml_state_size.argtypes = [I, P, P, P, I, I]
    lb.osg_pml_state_size.restype = C.c_long
    need = lb.osg_pml_state_size(dim, _p(_i32(nx)), _p(_i32(gcl)), _p(_i32(gcu)), int(mask) & 7,
                                 int(nb))
    if need < 0:
        raise OsirisGB300Error(-1, lb.osg_last_error().decode(errors="replace"))
    if state.size < need:
        raise ValueError(f"state holds {state.size} reals, needs {need}")
    _check(getattr(lb, f"osg_pml_{s}")(dim, _p(_i32(nx)), _p(_i32(gcl)), _p(_i32(gcu)),
                                          int(mask), int(nb), int(what), _p(e), _p(b), _p(state),
                                          _p(_f64(list(dx) + [0.0] * 3)), float(dt)))


def walls(dim, nx, gcl, gcu, f, kind, mask, order):
    """Conducting-wall images on a host grid (osg_walls_*): kind 0 E, 1 B, 2 J (perfect electric
    conductor; the current's images serve both conductors), 3 E, 4 B (perfect magnetic
    conductor); mask bit d walls axis d."""
    s = _prec(f)
    _check(getattr(lib(), f"osg_walls_{s}")(dim, _p(_i32(nx)), _p(_i32(gcl)), _p(_i32(gcu)),
                                            _p(f), int(kind), int(mask), int(order)))


def periodic(dim, nx, gcl, gcu, f, add):
    """Single-node periodic guard update (add=1: fold, add=0: replace), in place."""
    prec = _prec(f)
    _check(getattr(lib(), f"osg_periodic_{prec}")(dim, _p(_i32(nx)), _p(_i32(gcl)),
                                                   _p(_i32(gcu)), _p(f), int(add)))


def particle_wrap(nx, ix):
    """Periodic particle boundary on host cell indices (in place)."""
    _need(ix, np.int32, "ix")
    _check(lib().osg_particle_wrap(len(nx), _p(_i32(nx)), ix.shape[0], _p(ix)))


def pinned_empty(shape, dtype):
    """numpy array on page-locked host memory (freed when the array is collected)."""
    dtype = np.dtype(dtype)
    n = int(np.prod(shape)) * dtype.itemsize
    ptr = lib().osg_host_alloc(max(n, 1))
    if not ptr:
        raise OsirisGB300Error(-6, lib().osg_last_error().decode(errors="replace"))
    buf = (C.c_char * max(n, 1)).from_address(ptr)
    arr = np.frombuffer(buf, dtype=np.uint8, count=n).view(dtype).reshape(shape)
    _Pinned.keep[id(arr)] = ptr
    return arr


class _Pinned:
    keep = {}


def pinned_free(arr):
    ptr = _Pinned.keep.pop(id(arr), None)
    if ptr:
        lib().osg_host_free(ptr)


# ------------------------------------------------------------------------ seeded load

class Rng:
    """OSIRIS-seeded Mersenne Twister state shared by successive species loads."""

    def __init__(self, seed):
        self.buf = np.zeros(RNG_BYTES, dtype=np.uint8)
        _check(lib().osg_rng_seed(_p(self.buf), int(seed)))


def load_lattice(rng, precision, nx, ppc, dx, rqm, uth, ufl, amp=0.0, kmode=1.0):
    """Regular-lattice species over the periodic box; returns (ix, x, u, q)."""
    dim = len(nx)
    n = int(np.prod(nx)) * int(np.prod(ppc))
    dt_ = np.float32 if precision == 32 else np.float64
    ix = np.zeros((n, dim), np.int32)
    x = np.zeros((n, dim), dt_)
    u = np.zeros((n, 3), dt_)
    q = np.zeros(n, dt_)
    got = lib().osg_load_lattice(_p(rng.buf), precision, dim, _p(_i32(nx)), _p(_i32(ppc)),
                                 _p(_f64(list(dx) + [0.0] * 3)), float(rqm), _p(_f64(uth)),
                                 _p(_f64(ufl)), float(amp), float(kmode), _p(ix), _p(x), _p(u),
                                 _p(q))
    _check(got)
    assert got == n
    return ix, x, u, q


def zpulse_launch(order, nx, dx, xmin, e, b, omega0=1.0, a0=1.0, pol=0.0, lon_x0=0.0,
                  lon_duration=1.0, lon_range=1.0, per_w0=1.0, per_focus=0.0,
                  per_center=(0.0, 0.0)):
    """Add a Gaussian laser pulse (t = 0, forward) to host E/B arrays (osg_zpulse_launch)."""
    dim = len(nx)
    prec = 32 if e.dtype == np.float32 else 64
    gl, gu = GUARD[order]
    zp = Zpulse(omega0, a0, pol, lon_x0, lon_duration, lon_range, per_w0, per_focus,
                (D * 2)(*per_center))
    for a, n in ((e, "e"), (b, "b")):
        if a.dtype != e.dtype or not a.flags.c_contiguous:
            raise TypeError(f"{n} must be C-contiguous like e")
    _check(lib().osg_zpulse_launch(prec, dim, order, _p(_i32(nx)), _p(_i32([gl] * dim)),
                                   _p(_i32([gu] * dim)), _p(_f64(dx)), _p(_f64(xmin)),
                                   C.byref(zp), _p(e), _p(b)))


def smooth(dim, nx, gcl, gcu, f, types, orders):
    """Current smoothing of a host grid in place (osg_smooth_*): per axis the type
    (SMOOTH_*) and order; FP64 coefficients and sums."""
    prec = _prec(f)
    if not f.flags.c_contiguous:
        raise TypeError("f must be C-contiguous")
    _check(getattr(lib(), f"osg_smooth_{prec}")(dim, _p(_i32(nx)), _p(_i32(gcl)), _p(_i32(gcu)),
                                                _p(f), _p(_i32(types)), _p(_i32(orders))))


def smooth_coefficients(stype, order):
    """The normalised FP64 filter coefficients of one axis (osg_smooth_coefficients)."""
    c = np.zeros(31)
    n = C.c_int()
    _check(lib().osg_smooth_coefficients(int(stype), int(order), _p(c), C.byref(n)))
    return n.value, c[: 2 * n.value + 1].copy()


# ------------------------------------------------------------------------ simulation

class Simulation:
    """Device-resident periodic PIC simulation (fields + species stay on the GPU)."""

    def __init__(self, nx, dx, dt, order=2, precision=32, engine=ENGINE_TILED, tile=None,
                 n_sort=0, capacity=0.0, pusher=PUSHER_BORIS, iter_tol=0.0,
                 smooth_type=SMOOTH_NONE, smooth_order=0, walls=0, open_fields=0, thermal=0,
                 uth_bnd=(0.0, 0.0, 0.0), ufl_bnd=(0.0, 0.0, 0.0), seed=0, pmc=0,
                 thermal_type=0, emf_smooth_type=SMOOTH_NONE, emf_smooth_order=0, pml=0,
                 pml_cells=0, pml_diffuse=0):
        self.dim = len(nx)
        self.nx = list(nx)
        self.order = order
        self.precision = precision
        self.dtype = np.float32 if precision == 32 else np.float64
        gl, gu = GUARD[order]
        self.gcl, self.gcu = [gl] * self.dim, [gu] * self.dim
        self.size = [n + gl + gu for n in self.nx]
        cfg = Config()
        cfg.dim, cfg.order, cfg.precision, cfg.engine = self.dim, order, precision, engine
        for d in range(self.dim):
            cfg.nx[d] = nx[d]
            cfg.dx[d] = dx[d]
            cfg.tile[d] = (tile[d] if tile else 0)
        cfg.dt = dt
        cfg.n_sort = n_sort
        cfg.capacity = capacity
        cfg.pusher = pusher
        cfg.iter_tol = iter_tol
        cfg.smooth_type = smooth_type
        cfg.smooth_order = smooth_order
        cfg.walls = walls
        cfg.open_fields = open_fields
        cfg.thermal = thermal
        cfg.pmc = pmc
        cfg.thermal_type = thermal_type
        cfg.emf_smooth_type = emf_smooth_type
        cfg.emf_smooth_order = emf_smooth_order
        cfg.pml = pml
        cfg.pml_cells = pml_cells
        cfg.pml_diffuse = pml_diffuse
        cfg.seed = seed
        for c in range(3):
            cfg.uth_bnd[c] = uth_bnd[c]
            cfg.ufl_bnd[c] = ufl_bnd[c]
        self.cfg = cfg
        self.dx = list(dx)
        self.dt = dt
        self.h = P()
        _check(lib().osg_sim_create(C.byref(cfg), C.byref(self.h)))
        self._guards()
        self.nspecies = 0
        self.rqm = []

    def _guards(self):
        # guard cells as created (wider than the interpolation needs when smoothing)
        gcl, gcu = np.zeros(3, np.int32), np.zeros(3, np.int32)
        _check(lib().osg_sim_guard_cells(self.h, _p(gcl), _p(gcu)))
        self.gcl, self.gcu = [int(v) for v in gcl[: self.dim]], [int(v) for v in gcu[: self.dim]]
        self.size = [n + a + b for n, a, b in zip(self.nx, self.gcl, self.gcu)]

    def checkpoint(self, path):
        """Write the device-resident state to `path` (osg_sim_checkpoint)."""
        _check(lib().osg_sim_checkpoint(self.h, os.fsencode(str(path))))

    @classmethod
    def restore(cls, path):
        """A simulation that continues the run checkpointed in `path` (osg_sim_restore)."""
        self = cls.__new__(cls)
        self.h = P()
        _check(lib().osg_sim_restore(os.fsencode(str(path)), C.byref(self.h)))
        cfg, ns, rqm = Config(), I(), np.zeros(16)
        _check(lib().osg_sim_get_config(self.h, C.byref(cfg), C.byref(ns), _p(rqm)))
        self.cfg = cfg
        self.dim, self.order, self.precision = cfg.dim, cfg.order, cfg.precision
        self.dtype = np.float32 if cfg.precision == 32 else np.float64
        self.nx = [int(cfg.nx[d]) for d in range(self.dim)]
        self.dx = [float(cfg.dx[d]) for d in range(self.dim)]
        self.dt = float(cfg.dt)
        self._guards()
        self.nspecies = int(ns.value)
        self.rqm = [float(v) for v in rqm[: self.nspecies]]
        return self

    def close(self):
        if self.h:
            lib().osg_sim_destroy(self.h)
            self.h = P()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def grid_shape(self):
        return tuple(reversed(self.size)) + (3,)

    def add_species(self, rqm, ix, x, u, q):
        ix, x, u, q = (np.ascontiguousarray(ix, np.int32), np.ascontiguousarray(x, self.dtype),
                       np.ascontiguousarray(u, self.dtype), np.ascontiguousarray(q, self.dtype))
        k = _check(lib().osg_sim_add_species(self.h, float(rqm), len(q), _p(ix), _p(x), _p(u),
                                             _p(q)))
        self.nspecies += 1
        self.rqm.append(rqm)
        return k

    def set_fields(self, e=None, b=None):
        e = None if e is None else np.ascontiguousarray(e, self.dtype)
        b = None if b is None else np.ascontiguousarray(b, self.dtype)
        _check(lib().osg_sim_set_fields(self.h, _p(e), _p(b)))

    def fields(self):
        e, b, j = (np.zeros(self.grid_shape, self.dtype) for _ in range(3))
        _check(lib().osg_sim_get_fields(self.h, _p(e), _p(b), _p(j)))
        return e, b, j

    def num_particles(self, k):
        n = L()
        _check(lib().osg_sim_num_particles(self.h, k, C.byref(n)))
        return n.value

    def species(self, k):
        n = self.num_particles(k)
        ix = np.zeros((n, self.dim), np.int32)
        x = np.zeros((n, self.dim), self.dtype)
        u = np.zeros((n, 3), self.dtype)
        q = np.zeros(n, self.dtype)
        _check(lib().osg_sim_get_species(self.h, k, _p(ix), _p(x), _p(u), _p(q)))
        return ix, x, u, q

    def step(self, n=1):
        _check(lib().osg_sim_step(self.h, int(n)))

    def step_async(self, n=1):
        _check(lib().osg_sim_step_async(self.h, int(n)))

    def sync(self):
        _check(lib().osg_sim_sync(self.h))

    @property
    def stream(self):
        return lib().osg_sim_stream(self.h)

    def energy(self):
        kin = np.zeros(16)
        fld = np.zeros(6)
        _check(lib().osg_sim_energy(self.h, _p(kin), _p(fld)))
        return kin[: self.nspecies], fld

    def gauss_residual(self):
        m, l2 = D(), D()
        _check(lib().osg_sim_gauss_residual(self.h, C.byref(m), C.byref(l2)))
        return m.value, l2.value

    def set_window(self, species, ppc, prof_x, prof_f):
        """Moving window along x1 at c; `species` receives cold particles (ppc per axis) in
        the new cells with the piecewise-linear density profile (prof_x, prof_f)."""
        _check(lib().osg_sim_set_window(self.h, species, _p(_i32(ppc)), len(prof_x),
                                        _p(_f64(prof_x)), _p(_f64(prof_f))))

    def window_moves(self):
        n = C.c_long()
        _check(lib().osg_sim_window_moves(self.h, C.byref(n)))
        return n.value

    def autotune(self, steps=4):
        """Autotuner (osg_sim_autotune): TILED, the fastest tile shape and push CTA size over
        `steps` timed steps per candidate (the engine is re-binned for it); PLAIN, the cell-sort
        interval from the measured sort cost and slow-down of unsorted steps.  Call after the
        species are added, before the first step.  Returns {"tile", "threads", "n_sort"}."""
        tile = np.zeros(3, np.int32)
        th, ns = C.c_int(), C.c_int()
        _check(lib().osg_sim_autotune(self.h, int(steps), _p(tile), C.byref(th), C.byref(ns)))
        return {"tile": [int(v) for v in tile[:self.dim]], "threads": th.value,
                "n_sort": ns.value}

    def profile(self, n):
        ms = np.zeros(5, np.float32)
        _check(lib().osg_sim_profile(self.h, int(n), _p(ms)))
        return {"push": float(ms[0]), "fold": float(ms[1]), "yee": float(ms[2]),
                "replace": float(ms[3]), "sort": float(ms[4])}

    def launches_per_step(self):
        return lib().osg_sim_launches_per_step(self.h)

    def tile_occupancy(self):
        m = D()
        _check(lib().osg_sim_tile_occupancy(self.h, C.byref(m)))
        return m.value

    def time_steps(self, n):
        """Run n steps between two CUDA events on the simulation stream; returns device ms."""
        ms = F()
        _check(lib().osg_sim_time_steps(self.h, int(n), C.byref(ms)))
        return float(ms.value)


def device_memory():
    """(free, total) bytes of the current device (cudaMemGetInfo)."""
    f, t = C.c_size_t(0), C.c_size_t(0)
    _check(lib().osg_device_memory(C.byref(f), C.byref(t)))
    return f.value, t.value


def set_device(device):
    _check(lib().osg_set_device(int(device)))


class Batch:
    """Many independent periodic boxes advanced together (osg_batch_*): one persistent push
    launch over the tiles of all boxes, one launch per field phase, one CUDA graph per step.
    ``tile``/``threads`` left at None/0 are chosen by the autotuner on the first step."""

    def __init__(self, dim, order, dt, tile=None, threads=0, capacity=0.0):
        cfg = BatchConfig()
        cfg.dim, cfg.order, cfg.dt, cfg.threads, cfg.capacity = dim, order, dt, threads, capacity
        for d in range(dim):
            cfg.tile[d] = tile[d] if tile else 0
        self.dim, self.order, self.dt = dim, order, dt
        self.h = P()
        _check(lib().osg_batch_create(C.byref(cfg), C.byref(self.h)))
        self.boxes = []

    def close(self):
        if self.h:
            lib().osg_batch_destroy(self.h)
            self.h = P()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_box(self, nx, dx):
        rc = lib().osg_batch_add_box(self.h, _p(_i32(nx)), _p(_f64(dx)))
        _check(min(rc, 0))
        gl, gu = GUARD[self.order]
        self.boxes.append(dict(nx=list(nx), dx=list(dx), size=[n + gl + gu for n in nx],
                               species=0))
        return rc

    def add_species(self, box, rqm, ix, x, u, q):
        _need(ix, np.int32, "ix")
        for a, n in ((x, "x"), (u, "u"), (q, "q")):
            _need(a, np.float32, n)
        rc = lib().osg_batch_add_species(self.h, box, float(rqm), len(q), _p(ix), _p(x), _p(u),
                                         _p(q))
        _check(min(rc, 0))
        self.boxes[box]["species"] += 1
        return rc

    def tuning(self):
        t = np.zeros(3, np.int32)
        th = C.c_int()
        _check(lib().osg_batch_tuning(self.h, _p(t), C.byref(th)))
        return [int(v) for v in t[: self.dim]], th.value

    def step(self, n=1):
        _check(lib().osg_batch_step(self.h, int(n)))

    def time_steps(self, n):
        ms = C.c_float()
        _check(lib().osg_batch_time_steps(self.h, int(n), C.byref(ms)))
        return ms.value

    def launches_per_step(self):
        return lib().osg_batch_launches_per_step(self.h)

    def energy(self, box):
        kin = np.zeros(max(1, self.boxes[box]["species"]))
        fld = np.zeros(6)
        _check(lib().osg_batch_energy(self.h, box, _p(kin), _p(fld)))
        return kin[: self.boxes[box]["species"]], fld

    def fields(self, box):
        shape = tuple(reversed(self.boxes[box]["size"])) + (3,)
        e, b, j = (np.zeros(shape, np.float32) for _ in range(3))
        _check(lib().osg_batch_get_fields(self.h, box, _p(e), _p(b), _p(j)))
        return e, b, j

    def num_particles(self, box, k):
        n = C.c_long()
        _check(lib().osg_batch_num_particles(self.h, box, k, C.byref(n)))
        return n.value

    def species(self, box, k):
        n = self.num_particles(box, k)
        ix = np.zeros((n, self.dim), np.int32)
        x = np.zeros((n, self.dim), np.float32)
        u = np.zeros((n, 3), np.float32)
        q = np.zeros(n, np.float32)
        _check(lib().osg_batch_get_species(self.h, box, k, _p(ix), _p(x), _p(u), _p(q)))
        return ix, x, u, q
