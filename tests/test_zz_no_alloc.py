"""The allocation-free push entry point (osg_vadvance_deposit_noalloc_f32) against the regular
one (osg_vadvance_deposit_f32), through the C ABI.

It exists for hosts that cannot let a library call cudaMalloc (the GPU is handed to their own
pool allocator, or device memory is budgeted once before stepping): its device staging is one
fixed array inside the library.  Two calls in a row must each reproduce the regular entry point
(bit-identical particles, current within the FP32 tolerance 1e-5 normwise, energy within 1e-6)
-- the second call checks that nothing left in the shared array by the first leaks through --
and the second call must leave the device's free memory unchanged (nothing allocated).  A call
just under the documented size limit (8*dim + 16 bytes per particle plus three grid copies)
must succeed; one too large for the array must be rejected with a clear error before any GPU
work.  This file is collected last so that a stop-at-first-failure run has run everything else
first.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def osg():
    import __graft_entry__ as g
    g.build_native()
    import osiris_gb300
    if osiris_gb300.lib().osg_device_count() < 1:
        pytest.fail("no CUDA device visible")
    return osiris_gb300


def _case(osg, seed, dim, order, nx, ppc):
    r = osg.Rng(seed)
    ix, x, u, q = osg.load_lattice(r, 32, nx, [ppc] * dim, [0.1] * dim, -1.0, [0.5] * 3,
                                   [0.3, -0.1, 0.2])
    gl, gu = osg.GUARD[order]
    size = [n + gl + gu for n in nx]
    shape = tuple(reversed(size)) + (3,)
    rng = np.random.default_rng(seed)
    e = (rng.standard_normal(shape) * 0.3).astype(np.float32)
    b = (rng.standard_normal(shape) * 0.3).astype(np.float32)
    j0 = (rng.standard_normal(shape) * 0.01).astype(np.float32)   # the call ADDS into j
    return (ix, x, u, q), e, b, j0, size, [gl] * dim


def _nerr(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


@pytest.mark.parametrize("dim,order,nx,ppc", [(2, 2, [40, 32], 3), (3, 3, [12, 10, 8], 2)])
def test_noalloc_matches_regular_entry_point_twice(osg, dim, order, nx, ppc):
    for call, seed in enumerate((11, 12)):
        parts, e, b, j0, size, off = _case(osg, seed + dim, dim, order, nx, ppc)
        n = len(parts[3])
        i0, i1 = 3, n - 2
        a = [v.copy() for v in parts]
        ja = j0.copy()
        free0 = osg.device_memory()[0]
        ene_a = osg.vadvance_deposit_noalloc(dim, order, *a, i0, i1, -1.0, e, b, size, off, ja,
                                             size, off, [0.1] * dim, 0.04)
        if call == 1:
            # the first call set up the array's address (and loaded the kernels); the second
            # may not take any device memory
            assert osg.device_memory()[0] == free0, "the no-allocation entry point allocated"
        r = [v.copy() for v in parts]
        jr = j0.copy()
        ene_r = osg.vadvance_deposit(dim, order, *r, i0, i1, -1.0, e, b, size, off, jr, size,
                                     off, [0.1] * dim, 0.04)
        for k in range(3):
            assert np.array_equal(a[k], r[k]), (call, k)
        assert _nerr(ja, jr) <= 1e-5, call
        assert abs(ene_a - ene_r) <= 1e-6 * abs(ene_r), call


def _limit_particles(osg, size, dim):
    """Largest particle count one call can carry with this grid (8*dim + 16 bytes per particle,
    three 256-byte-aligned grid copies, 256 bytes of counters, 256-byte alignment of the four
    particle arrays)."""
    a256 = lambda n: (n + 255) // 256 * 256
    grid = a256(4 * 3 * int(np.prod(size)))
    room = osg.NOALLOC_SCRATCH_BYTES - 256 - 3 * grid - 4 * 255
    return room // (8 * dim + 16)


def test_noalloc_accepts_a_call_just_under_its_limit(osg):
    size = [13, 13]
    n = _limit_particles(osg, size, 2)
    rng = np.random.default_rng(5)
    ix = rng.integers(1, 9, (n, 2)).astype(np.int32)
    x = (rng.random((n, 2)) - 0.5).astype(np.float32)
    u = (rng.standard_normal((n, 3)) * 0.1).astype(np.float32)
    q = np.full(n, -1e-3, np.float32)
    g = (rng.standard_normal((13, 13, 3)) * 0.1).astype(np.float32)
    a = [v.copy() for v in (ix, x, u, q)]
    ja = np.zeros_like(g)
    osg.vadvance_deposit_noalloc(2, 2, *a, 1, n, -1.0, g, g, size, [2, 2], ja, size, [2, 2],
                                 [0.1, 0.1], 0.04)
    r = [v.copy() for v in (ix, x, u, q)]
    jr = np.zeros_like(g)
    osg.vadvance_deposit(2, 2, *r, 1, n, -1.0, g, g, size, [2, 2], jr, size, [2, 2],
                         [0.1, 0.1], 0.04)
    for k in range(3):
        assert np.array_equal(a[k], r[k]), k
    assert _nerr(ja, jr) <= 1e-5


def test_noalloc_rejects_calls_larger_than_its_array(osg):
    size = [13, 13]
    n = _limit_particles(osg, size, 2) + 64        # 32 bytes per 2D particle: past the limit
    ix = np.ones((n, 2), np.int32) * 4
    x = np.zeros((n, 2), np.float32)
    u = np.zeros((n, 3), np.float32)
    q = np.zeros(n, np.float32)
    g = np.zeros((13, 13, 3), np.float32)
    with pytest.raises(osg.OsirisGB300Error) as err:
        osg.vadvance_deposit_noalloc(2, 2, ix, x, u, q, 1, n, -1.0, g, g, size, [2, 2],
                                     g.copy(), size, [2, 2], [0.1, 0.1], 0.04)
    assert err.value.code == -1 and "bytes of device scratch" in str(err.value)
    assert (ix == 4).all()
