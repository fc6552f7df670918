"""Failure detection without a GPU fault: every device wait in the kernels
is bounded, and a wait that gives up becomes CSMC_ERR_TIMEOUT on the host
while the context stays usable.  csmc_selftest_timeout runs a kernel whose
wait can never complete (an mbarrier phase expecting bytes no copy delivers;
a grid barrier expecting one more CTA than the launch has)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CSMC_ERR_TIMEOUT = 4


@pytest.mark.parametrize("which", [0, 1])
def test_bounded_wait_times_out_into_an_error_and_the_context_survives(m, orc, which):
    lat = m.Lattice((8, 8), m.examples.square_heisenberg(), 1.0, rng=np.random.default_rng(5))
    mc = m.MonteCarlo([0.5, 1.0], lat, {"overrelaxation_rate": 5}, precision="fp32", seed=3)
    lib = m.lib()
    code = lib.csmc_selftest_timeout(mc.ctx.handle, which)
    assert code == CSMC_ERR_TIMEOUT, lib.csmc_last_error()
    assert b"bounded device wait" in lib.csmc_last_error()
    # the flag was cleared: the same context keeps working
    ol = orc.OracleLattice(m.examples.square_heisenberg(), (8, 8), 1.0)
    m.overrelaxation(mc)
    acc = np.atleast_1d(m.Metropolis()(mc, 0.5))
    assert np.all((acc >= 0) & (acc <= lat.size))
    s = mc.spins(0)
    assert abs(m.total_energy(mc) - ol.total_energy(np.asfortranarray(s))) <= 1e-4 * lat.size


def test_selftest_rejects_unknown_waits(m):
    lat = m.Lattice((4, 4), m.examples.square_heisenberg(), 1.0)
    mc = m.MonteCarlo(0.5, lat, {}, precision="fp64", seed=1)
    assert m.lib().csmc_selftest_timeout(mc.ctx.handle, 7) == 1


def test_device_allocation_failure_is_an_error_code(m):
    """A context whose replicas cannot fit (131072 replicas of 262144 sites:
    550 GB of spins on a 288 GB device) fails with CSMC_ERR_OOM, frees what it
    had allocated, and the device stays usable."""
    big = m.Lattice((64, 64, 64), m.examples.sc_heisenberg(), 1.0, initialCondition="none")
    with pytest.raises(m.CSMCError) as e:
        m.monte_carlo.Context([big], [131072], precision="fp32", seed=1)
    assert e.value.code == 2  # CSMC_ERR_OOM
    lat = m.Lattice((8, 8), m.examples.square_heisenberg(), 1.0)
    mc = m.MonteCarlo(0.5, lat, {"overrelaxation_rate": 5}, precision="fp32", seed=2)
    assert 0 <= m.Metropolis()(mc, 0.5) <= lat.size
