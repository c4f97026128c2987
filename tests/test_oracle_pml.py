"""The oracle's PML walls (Vay's split-field perfectly matched layer, "vpml", at both edges of
one axis of a 2D box), on the CPU:

* the attenuation tables follow the reference's formulas (setup_att_coeff, source/emf/
  boundary/os-emf-vpml.f03:3586-3684) for the default 8 cells, where s1 = -2 and s2 = 0.2 (the
  reference's note on its earlier constants): checked entry by entry against a restatement here,
  and deep in the wall the damped update tends to the plain Yee update at the interface;
* a plane pulse travelling along the PML axis, in either direction, leaves the box with less
  than 1e-4 of its energy, while the same box without PML keeps its energy to 1e-5;
* with PML on both axes (the x1 walls covering the corners) a cylindrical pulse leaves the box
  with less than 1e-5 of its energy; with one PML axis most of it stays (the other is periodic);
* 3D, one PML axis (six split components per wall point): a plane pulse along that axis, either
  direction, leaves less than 1e-8 of its energy; with PML on all three axes (the walls covering
  the edge regions of the higher axes) a divergence-free spherical pulse leaves less than 1e-6,
  and with none it keeps its energy;
* the diffusion correction (2D) moves a tenth of the damped B_z part into the other one every
  step, which the walls damp only along the other axis: a plane pulse along the PML axis then
  leaves about 2% of its energy for a while, below 1e-3 after 400 steps, the same for either
  axis (without it: 1e-21);
* a window move shifts every wall of an axis other than x1 one cell down along x1, its last
  plane zero, and leaves the tables alone;
* the state is four split-field walls per PML axis plus the tables.
"""
import numpy as np
import pytest

from oracle import pyoracle as po

NB = 8


def _tables(st, nb, axis):
    return st[len(st) - 24 * nb:].reshape(2, 4, 3, nb)[axis]


@pytest.mark.parametrize("axis", [0, 1])
def test_attenuation_tables(axis):
    nx = [24, 20]
    dx = [0.1, 0.2]
    dt = 0.04
    g = po.Grid(nx, 2, dx)
    st = po.pml_state(g, "f64", 1 << axis, NB, dt)
    t = _tables(st, NB, axis)
    dtdx = dt / dx[axis]
    dif = (1 - dtdx) / (1 + dtdx)
    att = lambda x: np.exp(-2.0 * (0.2 * x) ** 4)
    for j in range(NB):
        n = NB - 1 - j          # lower tables are stored from the outside in
        b1e = dtdx * (1 + dif * (1 - att(j)))
        b1b = dtdx * (1 + dif * (1 - att(j + 0.5)))
        assert t[0, :, n] == pytest.approx([1 - b1e + att(j) * dtdx, att(j - 0.5) * b1e, dtdx],
                                           rel=1e-14)
        assert t[2, :, n] == pytest.approx([1 - b1b + att(j + 0.5) * dtdx, att(j) * b1b, dtdx],
                                           rel=1e-14)
        b1e = dtdx * (1 + dif * (1 - att(j + 0.5)))
        b1b = dtdx * (1 + dif * (1 - att(j + 1.0)))
        assert t[1, :, j] == pytest.approx([1 - b1e + att(j + 0.5) * dtdx, dtdx, att(j) * b1e],
                                           rel=1e-14)
        assert t[3, :, j] == pytest.approx([1 - b1b + att(j + 1.0) * dtdx, dtdx,
                                            att(j + 0.5) * b1b], rel=1e-14)
    # next to the interface the damped update is nearly the plain one (1, dtdx, dtdx)
    assert t[1, :, 0] == pytest.approx([1.0, dtdx, dtdx], rel=1e-3)
    # the walls start at zero
    assert not st[:len(st) - 24 * NB].any()


def _energy(g, e, b):
    return float(np.sum(g.interior(e) ** 2) + np.sum(g.interior(b) ** 2))


@pytest.mark.parametrize("axis", [0, 1])
@pytest.mark.parametrize("sign", [1, -1])
def test_plane_pulse_is_absorbed(axis, sign):
    nx = [96, 16] if axis == 0 else [16, 96]
    g = po.Grid(nx, 2, [0.1, 0.1])
    dt = 0.05
    n = g.size[axis]
    pos = (np.arange(n) - n / 2) * 0.1
    prof, prof_h = np.exp(-(pos / 0.6) ** 2), np.exp(-((pos + 0.05) / 0.6) ** 2)
    res = {}
    for pml in (True, False):
        e, b, j = g.zeros("f64"), g.zeros("f64"), g.zeros("f64")
        if axis == 0:
            e[..., 1] = prof[None, :]
            b[..., 2] = sign * prof_h[None, :]
        else:
            e[..., 0] = prof[:, None]
            b[..., 2] = -sign * prof_h[:, None]
        w0 = _energy(g, e, b)
        st = po.pml_state(g, "f64", 1 << axis, NB, dt)
        for _ in range(200):
            po.step(g, "f64", e, b, j, [], dt, pml=(1 << axis, NB, st) if pml else None)
        res[pml] = _energy(g, e, b) / w0
    assert res[True] < 1e-4, res
    assert abs(res[False] - 1.0) < 1e-5, res


def test_state_size():
    g = po.Grid([24, 20], 2, [0.1, 0.1])
    gl, gu = po.GUARD[2]
    for axis in (0, 1):
        nt = g.nx[1 - axis]
        nte = nt + max(gl, 1) + max(gu, 2)
        st = po.pml_state(g, "f32", 1 << axis, NB, 0.04)
        assert st.dtype == np.float32 and len(st) == 4 * nte * NB * 4 + 24 * NB


def test_corners_absorb_a_cylindrical_pulse():
    nx = [48, 40]
    g = po.Grid(nx, 2, [0.1, 0.1])
    left = {}
    for mask in (1, 3):
        e, b, j = g.zeros("f64"), g.zeros("f64"), g.zeros("f64")
        st = po.pml_state(g, "f64", mask, NB, 0.05)
        yy, xx = np.meshgrid(np.arange(g.size[1]), np.arange(g.size[0]), indexing="ij")
        e[..., 2] = np.exp(-((xx - g.size[0] / 2) ** 2 + (yy - g.size[1] / 2) ** 2) / 8.0)
        w0 = _energy(g, e, b)
        for _ in range(400):
            po.step(g, "f64", e, b, j, [], 0.05, pml=(mask, NB, st))
        assert np.isfinite(e).all() and np.isfinite(b).all()
        left[mask] = _energy(g, e, b) / w0
    assert left[3] < 1e-5 and left[1] > 1e-2, left


@pytest.mark.parametrize("axis", [0, 1, 2])
@pytest.mark.parametrize("sign", [1, -1])
def test_3d_plane_pulse_is_absorbed(axis, sign):
    nx = [8, 8, 8]
    nx[axis] = 64
    g = po.Grid(nx, 2, [0.1, 0.1, 0.1])
    e, b, j = g.zeros("f64"), g.zeros("f64"), g.zeros("f64")
    n = g.size[axis]
    pos = (np.arange(n) - n / 2) * 0.1
    shp = [1, 1, 1]
    shp[2 - axis] = n
    # E along the next axis, B along the one after: E x B points along +axis
    e[..., (axis + 1) % 3] = np.exp(-(pos / 0.5) ** 2).reshape(shp)
    b[..., (axis + 2) % 3] = sign * np.exp(-((pos + 0.05) / 0.5) ** 2).reshape(shp)
    w0 = _energy(g, e, b)
    st = po.pml_state(g, "f64", 1 << axis, NB, 0.04)
    for _ in range(200):
        po.step(g, "f64", e, b, j, [], 0.04, pml=(1 << axis, NB, st))
    assert _energy(g, e, b) / w0 < 1e-8


def test_3d_edges_absorb_a_spherical_pulse():
    nx = [24, 20, 16]
    g = po.Grid(nx, 2, [0.1, 0.1, 0.1])
    z, y, x = np.meshgrid(np.arange(g.size[2]), np.arange(g.size[1]), np.arange(g.size[0]),
                          indexing="ij")
    az = np.exp(-((x - g.size[0] / 2) ** 2 + (y - g.size[1] / 2) ** 2 +
                  (z - g.size[2] / 2) ** 2) / 6.0)
    left = {}
    for mask in (7, 0):
        e, b, j = g.zeros("f64"), g.zeros("f64"), g.zeros("f64")
        # B = curl (0, 0, A_z) by the grid's differences: no divergence, so it all radiates
        b[:, :-1, :, 0] = (az[:, 1:, :] - az[:, :-1, :]) / 0.1
        b[:, :, :-1, 1] = -(az[:, :, 1:] - az[:, :, :-1]) / 0.1
        w0 = _energy(g, e, b)
        st = po.pml_state(g, "f64", mask, NB, 0.04)
        for _ in range(240):
            po.step(g, "f64", e, b, j, [], 0.04, pml=(mask, NB, st) if mask else None)
        assert np.isfinite(e).all() and np.isfinite(b).all()
        left[mask] = _energy(g, e, b) / w0
    assert left[7] < 1e-6 and abs(left[0] - 1.0) < 0.05, left


@pytest.mark.parametrize("axis", [0, 1])
def test_diffusion_correction_keeps_the_absorption(axis):
    nx = [96, 16] if axis == 0 else [16, 96]
    g = po.Grid(nx, 2, [0.1, 0.1])
    n = g.size[axis]
    pos = (np.arange(n) - n / 2) * 0.1
    e, b, j = g.zeros("f64"), g.zeros("f64"), g.zeros("f64")
    if axis == 0:
        e[..., 1] = np.exp(-(pos / 0.6) ** 2)[None, :]
        b[..., 2] = np.exp(-((pos + 0.05) / 0.6) ** 2)[None, :]
    else:
        e[..., 0] = np.exp(-(pos / 0.6) ** 2)[:, None]
        b[..., 2] = -np.exp(-((pos + 0.05) / 0.6) ** 2)[:, None]
    w0 = _energy(g, e, b)
    mask = 1 << axis
    st = po.pml_state(g, "f64", mask, NB, 0.05)
    left = []
    for it in range(400):
        po.step(g, "f64", e, b, j, [], 0.05, pml=(mask | (mask << 4), NB, st))
        if it in (199, 399):
            left.append(_energy(g, e, b) / w0)
    assert np.isfinite(e).all() and np.isfinite(b).all()
    assert 1e-3 < left[0] < 0.05 and left[1] < 1e-3, left


@pytest.mark.parametrize("dim,mask", [(2, 2), (3, 2), (3, 4), (3, 6)])
def test_window_shift_moves_the_walls_along_x1(dim, mask):
    """ora_pml_shift_x (a window move): every wall of an axis other than x1 shifts one x1 cell
    down, its last x1 plane becoming zero (move_window_wall)."""
    nx = [12, 10] if dim == 2 else [12, 10, 9]
    g = po.Grid(nx, 2, [0.1] * dim)
    st = po.pml_state(g, "f64", mask, NB, 0.03)
    ntab = 12 * dim * NB
    rng = np.random.default_rng(2)
    st[:len(st) - ntab] = rng.standard_normal(len(st) - ntab)
    before = st.copy()
    nx_, gl, gu = g.args()
    po.lib().ora_pml_shift_x_f64(dim, po._p(nx_), po._p(gl), po._p(gu), mask, NB, po._p(st))
    # the walls' x1 extent: nx + max(gcl, 2) + max(gcu, 2) points; a wall is lines of one x1
    # point (4 nb reals in 2D, 6 nb in 3D) repeated along x1, per point of the remaining axis
    n1 = nx[0] + max(g.gcl[0], 2) + max(g.gcu[0], 2)
    line = (4 if dim == 2 else 6) * NB
    walls = st[:len(st) - ntab]
    assert np.array_equal(st[len(st) - ntab:], before[len(st) - ntab:])
    w = walls.reshape(-1, n1, line)
    b = before[:len(st) - ntab].reshape(-1, n1, line)
    assert np.array_equal(w[:, :-1], b[:, 1:])
    assert not w[:, -1].any()
