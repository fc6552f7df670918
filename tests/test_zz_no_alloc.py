"""csmc_energy_diff_static: the allocation-free variant of csmc_energy_diff.

It exists for callers that cannot let the library allocate device memory on
every call (a host process whose pool allocator already holds the GPU's
memory, or a proposal loop that cannot absorb a synchronising cudaFree).  It
stages through a fixed static device array of CSMC_ENERGY_DIFF_STATIC_MAX
proposals.  Checked here through the C ABI against csmc_energy_diff, on two
calls in a row, with the tolerance the parity tests use.  Collected last so
that a stop at the first failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

STATIC_MAX = 65536
TOL = {"fp64": 1e-12, "fp32": 1e-6}


def _ptr(a, t):
    return a.ctypes.data_as(C.POINTER(t))


def _energy_diff(ctx, name, slot, sites, new_rows):
    n = len(sites)
    out = np.zeros(n)
    code = getattr(ctx.lib, name)(ctx.handle, slot, n, _ptr(sites, C.c_int64), _ptr(new_rows, C.c_double),
                                  _ptr(out, C.c_double))
    return code, out


class _Ctx:
    def __init__(self, m, precision, lat, seed):
        self.lib = m.lib()
        self.mc = m.MonteCarlo([0.5, 1.0], lat, {}, precision=precision, seed=seed)
        self.handle = self.mc.ctx.handle


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_static_energy_diff_matches_allocating_entry(m, precision):
    E = m.examples
    lat = m.Lattice((3, 3, 3), E.pyrochlore_ckq(), 1.0, rng=np.random.default_rng(1))
    ctx = _Ctx(m, precision, lat, seed=2)
    rng = np.random.default_rng(3)
    for slot in (0, 1):
        spins = rng.normal(size=(3, lat.size))
        spins = np.asfortranarray(spins / np.linalg.norm(spins, axis=0))
        ctx.mc.set_spins(spins, slot)
    scale = 2 * (np.abs(lat.tables()["bilinear_matrices"]).sum(axis=(1, 2, 3))
                 + np.abs(lat.tables()["cubic_tensors"]).sum(axis=(1, 2, 3, 4))
                 + np.abs(lat.tables()["quartic_tensors"]).sum(axis=(1, 2, 3, 4, 5)) + 1.0)
    for call, n in enumerate((5000, 777)):  # two calls in a row, different sizes
        slot = call % 2
        sites = rng.integers(0, lat.size, n).astype(np.int64)
        new = rng.normal(size=(n, 3))
        new = np.ascontiguousarray(new / np.linalg.norm(new, axis=1, keepdims=True))
        c0, ref = _energy_diff(ctx, "csmc_energy_diff", slot, sites, new)
        c1, got = _energy_diff(ctx, "csmc_energy_diff_static", slot, sites, new)
        assert c0 == 0 and c1 == 0, ctx.lib.csmc_last_error()
        assert np.all(np.abs(got - ref) <= TOL[precision] * scale[sites])


def test_static_energy_diff_limits(m):
    lat = m.Lattice((8, 8), m.examples.square_heisenberg(), 1.0, rng=np.random.default_rng(4))
    ctx = _Ctx(m, "fp64", lat, seed=5)
    rng = np.random.default_rng(6)
    n = STATIC_MAX  # the largest accepted size
    sites = rng.integers(0, lat.size, n).astype(np.int64)
    new = np.ascontiguousarray(np.tile([0.0, 0.0, 1.0], (n, 1)))
    c0, ref = _energy_diff(ctx, "csmc_energy_diff", 0, sites, new)
    c1, got = _energy_diff(ctx, "csmc_energy_diff_static", 0, sites, new)
    assert c0 == 0 and c1 == 0
    assert np.all(np.abs(got - ref) <= 1e-12 * 10)
    code, _ = _energy_diff(ctx, "csmc_energy_diff_static", 0, np.zeros(n + 1, np.int64),
                           np.zeros((n + 1, 3)))
    assert code == 1 and b"CSMC_ENERGY_DIFF_STATIC_MAX" in ctx.lib.csmc_last_error()


def _allocs(lib):
    n = C.c_int64()
    assert lib.csmc_debug_device_allocs(C.byref(n)) == 0
    return n.value


def test_static_energy_diff_allocates_nothing(m):
    """Repeated calls make no device allocation (the library's own count of
    cudaMalloc calls stays put), while the allocating entry point's calls are
    counted; n = 0 is a no-op and a slot out of range is an error."""
    lat = m.Lattice((6, 6), m.examples.triangular_afm(h=0.3), 1.0, rng=np.random.default_rng(7))
    ctx = _Ctx(m, "fp32", lat, seed=8)
    rng = np.random.default_rng(9)
    sites = rng.integers(0, lat.size, 300).astype(np.int64)
    new = np.ascontiguousarray(np.tile([0.6, 0.0, 0.8], (300, 1)))
    c, first = _energy_diff(ctx, "csmc_energy_diff_static", 1, sites, new)
    assert c == 0
    before = _allocs(ctx.lib)
    for _ in range(4):
        c, again = _energy_diff(ctx, "csmc_energy_diff_static", 1, sites, new)
        assert c == 0 and np.array_equal(again, first)
    c, _ = _energy_diff(ctx, "csmc_energy_diff_static", 0, sites[:0], new[:0])
    assert c == 0
    assert _allocs(ctx.lib) == before
    c, ref = _energy_diff(ctx, "csmc_energy_diff", 1, sites, new)
    assert c == 0 and _allocs(ctx.lib) == before + 3  # sites, new spins and results staged
    assert np.all(np.abs(first - ref) <= TOL["fp32"] * 2 * (6 + 0.3 + 1))
    c, _ = _energy_diff(ctx, "csmc_energy_diff_static", 2, sites, new)  # two slots: 0 and 1
    assert c == 1 and b"slot" in ctx.lib.csmc_last_error()
