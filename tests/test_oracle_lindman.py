"""Oracle tests of Lindman open boundaries (p_bc_lindman, source/emf/boundary/os-emf-lindman.f90)
and of the absorbing particle boundary that goes with them (p_bc_absorbing,
source/spec/os-spec-boundary.f03:501-511).

* the first step from a zero state follows the update rule: E_t(0) = -k E_t(1) and
  E_t(nx+2) = -k E_t(nx+1) for the tangential components, k = (1 - dt/dx)/(1 + dt/dx)
  (update_lindman_2d_e :454-535, disp_corr :237-238), E_n(0) stays 0, and the state holds the
  planes it copied (E at 0, 1, nx+1, nx+2; B at 0 equal to the grid's Yee value there);
* a plane pulse leaves the box through either edge of any axis, in 2D and 3D, FP32 and FP64,
  with less than 1e-4 of its energy left behind (a periodic box keeps all of it);
* particles leaving through an open edge are absorbed after their deposit: charge and
  momentum 0, at offset 0 of the edge cell; the others keep their charge.
"""
import numpy as np
import pytest

from test_gpu_step import _setup


def _state_planes(g, st, axis):
    """state as [slot, other-axes point (lower axis fastest), component]"""
    return st.reshape(5, -1, 3)


def _plane(g, f, axis, i):
    """the plane at reference index i along `axis`, interior of the other axes, as
    [point (lower other axis fastest), component]"""
    sl = []
    for a in reversed(range(g.dim)):
        if a == axis:
            sl.append(i - 1 + g.gcl[a])
        else:
            sl.append(slice(g.gcl[a], g.gcl[a] + g.nx[a]))
    return f[tuple(sl)].reshape(-1, 3)


@pytest.mark.parametrize("dim,axis", [(2, 0), (2, 1), (3, 0), (3, 2)])
def test_first_step_follows_the_update_rule(oracle, dim, axis):
    nx = [10, 8] if dim == 2 else [8, 7, 6]
    dx = [0.1, 0.12, 0.09][:dim]
    dt = 0.5 / np.sqrt(sum(1 / d ** 2 for d in dx))
    g = oracle.Grid(nx, 2, dx)
    rng = np.random.default_rng(3 + axis)
    e = rng.standard_normal(g.shape)
    b = rng.standard_normal(g.shape)
    j = g.zeros("f64")
    st = oracle.lindman_state(g, "f64", axis)
    oracle.step(g, "f64", e, b, j, [], dt, open_fields=(axis, st))
    k = (1 - dt / dx[axis]) / (1 + dt / dx[axis])
    n = nx[axis]
    tang = [c for c in range(3) if c != axis]
    e0, e1 = _plane(g, e, axis, 0), _plane(g, e, axis, 1)
    f1, f2 = _plane(g, e, axis, n + 1), _plane(g, e, axis, n + 2)
    assert np.array_equal(e0[:, tang], -k * e1[:, tang])
    assert np.array_equal(f2[:, tang], -k * f1[:, tang])
    assert not np.any(e0[:, axis])
    S = _state_planes(g, st, axis)
    for slot, plane in ((0, e0), (1, e1), (3, f1), (4, f2)):
        assert np.array_equal(S[slot][:, tang], plane[:, tang])
        assert not np.any(S[slot][:, axis])
    # the lower B buffer took the same increments as the grid's B(0), which the step's guard
    # update had set to the (zero) buffer
    np.testing.assert_allclose(S[2], _plane(g, b, axis, 0), rtol=0, atol=1e-13)


def _pulse(oracle, prec, dim, axis, forward, open_):
    nx = [96, 8] if dim == 2 else [64, 6, 6]
    nx[0], nx[axis] = nx[axis], nx[0]
    dx = [0.2] * dim
    dt = 0.9 / np.sqrt(sum(1 / d ** 2 for d in dx))
    g = oracle.Grid(nx, 2, dx)
    e, b, j = g.zeros(prec), g.zeros(prec), g.zeros(prec)
    t, s = (axis + 1) % 3, (axis + 2) % 3
    L = nx[axis] * dx[axis]
    coord = np.indices(g.shape[:-1])[dim - 1 - axis] - g.gcl[axis]
    prof = lambda x: np.exp(-((x - 0.5 * L) / (0.08 * L)) ** 2)
    # E_t at integer points, B_s half a cell up: a pulse moving along +axis (or -axis)
    e[..., t] = prof(coord * dx[axis])
    b[..., s] = (1.0 if forward else -1.0) * prof((coord + 0.5) * dx[axis])
    st = oracle.lindman_state(g, prec, axis) if open_ else None

    def energy():
        return float((g.interior(e).astype(np.float64) ** 2).sum() +
                     (g.interior(b).astype(np.float64) ** 2).sum())

    w0 = energy()
    for _ in range(int(L / dt)):
        oracle.step(g, prec, e, b, j, [], dt, open_fields=(axis, st) if open_ else None)
    return energy() / w0


@pytest.mark.parametrize("prec", ["f32", "f64"])
@pytest.mark.parametrize("dim,axis", [(2, 0), (2, 1), (3, 1), (3, 2)])
@pytest.mark.parametrize("forward", [True, False])
def test_pulse_leaves_the_box(oracle, prec, dim, axis, forward):
    assert _pulse(oracle, prec, dim, axis, forward, True) < 1e-4


def test_periodic_box_keeps_the_pulse(oracle):
    assert abs(_pulse(oracle, "f64", 2, 0, True, False) - 1.0) < 1e-2


@pytest.mark.parametrize("prec", [32, 64])
@pytest.mark.parametrize("axis", [0, 1])
def test_particles_absorbed_at_open_edges(oracle, prec, axis):
    """A particle absorbed in a step is left at offset 0 of the edge cell with charge and
    momentum 0; later steps still move it (its charge-to-mass ratio is the species') but it
    deposits nothing."""
    nx = [12, 10]
    p, g, dx, dt, species, e, b = _setup(oracle, prec, 2, 2, nx, [2, 2], 7, uth=0.6, ufl=0.1)
    st = oracle.lindman_state(g, p, axis)
    q_init = [s["q"].copy() for s in species]
    j = g.zeros(p)
    gone = 0
    for _ in range(6):
        before = [s["q"].copy() for s in species]
        oracle.step(g, p, e, b, j, species, dt, open_fields=(axis, st))
        for s, q0 in zip(species, before):
            new = (q0 != 0) & (s["q"] == 0)
            gone += int(new.sum())
            assert not np.any(s["u"][new]) and not np.any(s["x"][new, axis])
            assert np.all(np.isin(s["ix"][new, axis], [1, nx[axis]]))
            assert s["ix"].min() >= 1 and np.all(s["ix"].max(axis=0) <= np.array(nx))
    for s, q0 in zip(species, q_init):
        live = s["q"] != 0
        assert np.array_equal(s["q"][live], q0[live])
    assert gone > 0
