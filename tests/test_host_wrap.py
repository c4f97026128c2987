"""The host-array periodic particle boundary (osg_particle_wrap, the replacement of the periodic
branch of phys_boundary_species, source/spec/os-spec-boundary.f03:1280-1290) gives the same
cell indices as the oracle's restatement, on the single-threaded path (small arrays) and on the
multi-threaded one (more than 2^20 particles)."""
import numpy as np
import pytest


@pytest.fixture(scope="module")
def osg():
    import __graft_entry__ as g
    g.build_native()
    import osiris_gb300
    return osiris_gb300


@pytest.mark.parametrize("np_", [0, 1, 1000, 3_000_001])
@pytest.mark.parametrize("dim", [1, 2, 3])
def test_particle_wrap_matches_oracle(osg, oracle, dim, np_):
    nx = [17, 9, 5][:dim]
    rng = np.random.default_rng(dim * 7 + np_ % 13)
    # cells one step after a push: inside [0, nx + 1] (a particle moves at most one cell)
    ix = np.stack([rng.integers(0, n + 2, size=np_) for n in nx], axis=1).astype(np.int32)
    ix = np.ascontiguousarray(ix)
    ref = ix.copy()
    g = oracle.Grid(nx, 2, [0.1] * dim)
    oracle.wrap(g, ref)
    got = ix.copy()
    osg.particle_wrap(nx, got)
    assert np.array_equal(got, ref)
    if np_:
        assert got.min() >= 1 and (got <= np.array(nx)).all()
