"""Spins across the host boundary: csmc_set_spins_all / csmc_get_spins_all
(the reference layout, 3 x N Float64 per replica in slot order) with pageable
host arrays (staged through one bulk copy) and with pinned host memory (read
or written in place by the conversion kernel; two doubles per thread when
every replica's block starts on a 16-byte boundary, one otherwise).

Gates: every path gives the same device state bit for bit -- the Float64
input rounded to the context's precision -- and the same values back.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _pinned(n):
    torch = pytest.importorskip("torch")
    return torch.empty(n, dtype=torch.float64).pin_memory().numpy()


def _p(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
@pytest.mark.parametrize("name,shape", [("sc", (4, 4, 4)), ("square", (5, 5))])  # N = 64 (even), 25 (odd)
def test_spins_round_trip_pinned_and_pageable(m, name, shape, precision):
    E = m.examples
    uc = {"sc": E.sc_heisenberg, "square": E.square_heisenberg}[name]()
    lat = m.Lattice(shape, uc, 1.0)
    R = 3
    ctx = m.monte_carlo.Context([lat], [R], precision=precision, seed=11)
    n = 3 * lat.size * R
    rng = np.random.default_rng(7)
    v = rng.normal(size=(R, lat.size, 3))
    v /= np.linalg.norm(v, axis=2, keepdims=True)
    src = np.ascontiguousarray(v.reshape(-1))
    want = src.astype(np.float32).astype(np.float64) if precision == "fp32" else src

    # pageable in, pageable out
    ctx.call("csmc_set_spins_all", _p(src))
    out = np.zeros(n)
    ctx.call("csmc_get_spins_all", _p(out))
    assert np.array_equal(out, want)

    # pinned out (in place), aligned and (one double in) unaligned
    pin = _pinned(n + 2)
    for off in (0, 1):
        view = pin[off:off + n]
        view[:] = 0.0
        ctx.call("csmc_get_spins_all", _p(view))
        assert np.array_equal(view, want), off

    # pinned in (in place), aligned and unaligned; read back pageable
    for off in (0, 1):
        ctx.call("csmc_random_spins", C.c_uint64(3 + off))
        view = pin[off:off + n]
        view[:] = src
        ctx.call("csmc_set_spins_all", _p(view))
        out[:] = 0.0
        ctx.call("csmc_get_spins_all", _p(out))
        assert np.array_equal(out, want), off
