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
    """Exchange windows in one cooperative launch (grid barriers, exchange by
    block 0) give the same chain, records and counters as one launch per
    window with a separate exchange launch."""
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
