"""csmc_autotune: the launch-configuration autotuner of the resident kernel.

It times every cluster size that fits and two block sizes on the context's
own replicas, then restores the replicas and counters exactly, so a chain that
was tuned before running equals one that was not (same tolerances as the
cluster-size equality test: the configurations run the same arithmetic per
site).
"""
import numpy as np
import pytest

from test_gpu_parity import obs_tol, rand_spins, setup

pytestmark = pytest.mark.gpu


def _pt(m, mc, lat, tune):
    mc.ctx.set_temperatures(np.array([0.2, 0.4, 0.8, 1.6]))
    for r in range(4):
        mc.set_spins(rand_spins(lat.size, 40 + r), r)
    mc.path = "resident"
    p = mc.parameters
    p.t_thermalization, p.t_measurement, p.report_interval, p.checkpoint_rate = 5, 35, 40, 10
    p.probe_rate, p.swap_rate, p.overrelaxation_rate = 5, 5, 5
    entries = m.autotune(mc, n_windows=2, alg=m.MetropolisAdaptive()) if tune else []
    out = m.parallel_tempering(mc, alg=m.MetropolisAdaptive(), verbose=False)
    return entries, (np.stack([mc.spins(r) for r in range(4)]), out["energy"], out["magnetization"],
                     mc.accepted.copy(), mc.exchanged.copy(), np.atleast_1d(mc.sigma))


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("name", ["sc", "honeycomb"])
def test_autotune_leaves_the_chain_unchanged(m, orc, name, precision):
    lat, _, mc0 = setup(m, orc, name, precision, R=4, seed=9)
    _, ref = _pt(m, mc0, lat, tune=False)
    lat, _, mc1 = setup(m, orc, name, precision, R=4, seed=9)
    entries, got = _pt(m, mc1, lat, tune=True)
    assert len(entries) >= 1 and sum(e["chosen"] for e in entries) == 1
    assert all(e["ms_per_window"] > 0 and e["block"] % 32 == 0 for e in entries)
    assert {e["cluster"] for e in entries} <= {1, 2, 4}
    assert np.abs(ref[0] - got[0]).max() <= 1e-12 * (1 if precision == "fp64" else 1e6)
    assert np.abs(ref[1] - got[1]).max() <= obs_tol(precision) * lat.size
    assert np.abs(ref[2] - got[2]).max() <= obs_tol(precision) * lat.size
    assert np.array_equal(ref[3], got[3]) and np.array_equal(ref[4], got[4])
    assert np.allclose(ref[5], got[5], rtol=1e-12)


def test_autotune_on_the_global_path_is_a_no_op(m, orc):
    """A run that takes the global path has no resident configuration to tune."""
    lat, _, mc = setup(m, orc, "pyrochlore", "fp32", R=2, seed=3)
    mc.path = "global"
    before = mc.spins(1).copy()
    assert m.autotune(mc, n_windows=1) == []
    assert np.array_equal(mc.spins(1), before)


def _set_persistent(mc, on):
    import ctypes as C
    mc.ctx.call("csmc_set_persistent", 1 if on else 0)
    got = C.c_int32()
    mc.ctx.call("csmc_persistent", C.byref(got))
    return got.value


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("name", ["sc", "honeycomb", "triangular_open", "pyrochlore"])
def test_persistent_windows_equal_one_launch_per_window(m, orc, name, precision):
    """Exchange windows in one cooperative launch (one grid barrier per
    window, each replica deciding its own pair's exchange) give the same
    chain, records and counters as one launch per window with a separate
    exchange launch."""
    res = []
    for on in (False, True):
        lat, _, mc = setup(m, orc, name, precision, R=4, seed=9)
        assert _set_persistent(mc, on) in ((0,) if not on else (0, 1))
        res.append(_pt(m, mc, lat, tune=False)[1])
    ref, got = res
    assert np.abs(ref[0] - got[0]).max() <= 1e-12 * (1 if precision == "fp64" else 1e6)
    assert np.abs(ref[1] - got[1]).max() <= obs_tol(precision) * lat.size
    assert np.abs(ref[2] - got[2]).max() <= obs_tol(precision) * lat.size
    assert np.array_equal(ref[3], got[3]) and np.array_equal(ref[4], got[4])
    assert np.allclose(ref[5], got[5], rtol=1e-12)


def test_autotune_automatic_path_also_times_the_global_sweeps(m, orc):
    """With the automatic path the global colour sweeps are one more
    candidate; whichever is kept, the chain runs on and its energies match
    the oracle's total energy of the final spins."""
    lat, ol, mc = setup(m, orc, "pyrochlore", "fp32", R=2, seed=3)
    mc.path = "auto"
    mc.ctx.set_temperatures(np.array([0.3, 0.9]))
    entries = m.autotune(mc, n_windows=2)
    assert any(e["path"] == "global" for e in entries) and any(e["path"] == "resident" for e in entries)
    assert sum(e["chosen"] for e in entries) == 1
    p = mc.parameters
    p.t_thermalization, p.t_measurement, p.report_interval, p.checkpoint_rate = 0, 20, 20, 10
    p.probe_rate, p.swap_rate, p.overrelaxation_rate = 5, 5, 5
    m.parallel_tempering(mc, verbose=False)
    for r in range(2):
        s = mc.spins(r)
        assert abs(m.total_energy(mc, r) - ol.total_energy(np.asfortranarray(s))) <= 1e-4 * lat.size


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_persistent_exchange_of_several_lattices(m, precision):
    """Two lattices of different sizes with three replicas each in one
    context, parallel tempering in one cooperative launch: each replica takes
    its own pair's exchange within its lattice's slots (monte_carlo.jl:308-349),
    and the chains, probe records and accepted and exchange counters equal
    those of one launch per window with the stand-alone exchange kernel; both
    lattices exchange."""
    import ctypes as C
    from importlib import import_module
    L = import_module(m.__name__ + "._lib")
    E = m.examples
    lats = [m.Lattice((6, 6), E.triangular_afm(h=0.2), 1.0, rng=np.random.default_rng(6)),
            m.Lattice((8, 8), E.triangular_afm(h=0.5), 1.0, rng=np.random.default_rng(8))]
    T = np.array([0.50, 0.52, 0.54, 0.60, 0.62, 0.64])  # close rungs: exchanges are frequent
    n_slots, cap = 6, 16
    res = []
    for on in (0, 1):
        ctx = m.monte_carlo.Context(lats, [3, 3], precision=precision, seed=5)
        ctx.set_temperatures(T)
        for k in range(n_slots):
            ctx.set_spins(k, lats[k // 3].spins)
        ctx.call("csmc_set_persistent", on)
        rec_E, rec_M = np.zeros((cap, n_slots)), np.zeros((cap, n_slots))
        acc, exch = np.zeros(n_slots), np.zeros(n_slots)
        rp = L.RunParams()
        rp.sweep_start, rp.n_sweeps, rp.t_thermalization = 1, 60, 0
        rp.overrelaxation_rate, rp.swap_rate, rp.probe_rate = 2, 4, 4
        rp.kind, rp.path = L.METROPOLIS, L.PATH_RESIDENT
        rp.probe_energy = rec_E.ctypes.data_as(C.POINTER(C.c_double))
        rp.probe_magnetization = rec_M.ctypes.data_as(C.POINTER(C.c_double))
        rp.probe_capacity = cap
        rp.accepted = acc.ctypes.data_as(C.POINTER(C.c_double))
        rp.exchanged = exch.ctypes.data_as(C.POINTER(C.c_double))
        ctx.call("csmc_run", C.byref(rp))
        res.append(([ctx.get_spins(k) for k in range(n_slots)], rec_E, rec_M, acc, exch, rp.n_probes_out))
    ref, got = res
    for k in range(n_slots):
        assert np.abs(ref[0][k] - got[0][k]).max() <= 1e-12 * (1 if precision == "fp64" else 1e6), k
    assert ref[5] == got[5] == 15  # probes at iterations 4, 8, ..., 60
    assert np.abs(ref[1] - got[1]).max() <= obs_tol(precision) * 64
    assert np.abs(ref[2] - got[2]).max() <= obs_tol(precision) * 64
    assert np.array_equal(ref[3], got[3]) and np.array_equal(ref[4], got[4])
    assert got[4][:3].sum() > 0 and got[4][3:].sum() > 0  # both lattices exchanged
