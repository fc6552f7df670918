"""Constrained Metropolis (metropolis_constraint!, metropolis_constraint_adaptive!,
metropolis.jl:36-58,155-179) on the GPU against the oracle's restatement.

The constraint is the closed form c = g.V + q|V|^2 + p|V| + c0 of
V = sum_i w_i s_i.  The FP64 replay evaluates c over the whole lattice at
every proposal, as the reference calls its constraint function, with the
reference's arithmetic: every decision equal to the oracle's, spins and
lambda to rounding (sin/cos may differ from libm in the last bit).  The
production sweep keeps V as a running sum (c then differs from the
oracle's by rounding only): decisions equal, spins within 1e-12, lambda
within 1e-9 relative."""
import ctypes as C

import numpy as np
import pytest

from test_gpu_parity import model, rand_spins

pytestmark = pytest.mark.gpu

KINDS = {"MetropolisConstraint": 0, "MetropolisConstraintAdaptive": 1}  # oracle: cone flag


def _constraint(m, orc, lat, weight):
    """A staggered-weight constraint using every term of the closed form."""
    w = np.where(np.arange(lat.size) % 3 == 0, -1.0, 1.0) * 0.5
    args = dict(g=(0.3, -0.2, 0.7), q=0.01, p=-0.05, c0=0.4)
    return m.Constraint(site_weights=w, **args), orc.constraint(w, weight=weight, **args)


def _setup(m, orc, name, precision, weight=0.3, seed=77, T=0.6, R=1):
    uc, shape, bc = model(m, name)
    lat = m.Lattice(shape, uc, 1.0, bc=bc)
    ol = orc.OracleLattice(uc, shape, 1.0, bc=bc)
    kd, ko = _constraint(m, orc, lat, weight)
    mc = m.MonteCarlo([T] * R if R > 1 else T, lat, {"overrelaxation_rate": 5}, precision=precision, seed=seed,
                      constraint=kd, weight=weight, sigma0=2.0)
    return lat, ol, mc, kd, ko


@pytest.mark.parametrize("kind", list(KINDS))
@pytest.mark.parametrize("name", ["square", "honeycomb", "pyrochlore", "asym_open", "selfloop"])
def test_constraint_replay_exact(m, orc, name, kind):
    """Replay of given proposals: every decision and sigma identical, lambda to rounding."""
    lat, ol, mc, kd, ko = _setup(m, orc, name, "fp64")
    s = rand_spins(lat.size, 21)
    mc.set_spins(s)
    rng = np.random.default_rng(22)
    n = 2 * lat.size
    sites = rng.integers(0, lat.size, n)
    up, uz, ua = rng.random(n), rng.random(n), rng.random(n)
    mc.ctx.call("csmc_set_sigma", np.array([0.5]).ctypes.data_as(C.POINTER(C.c_double)))
    mc.lambda_ = 0.25
    acc, sigma = m.replay(mc, sites, up, uz, ua, alg=getattr(m, kind)(), T=0.6)
    acc_o, sigma_o, lam_o = ol.constraint_replay(s, 0.6, KINDS[kind], 0.5, 2.0, ko, 0.25, sites, up, uz, ua)
    assert 0 < acc.sum() and (acc.sum() < n or lat.size < 8)
    assert np.array_equal(acc, acc_o)
    assert np.abs(mc.spins(0) - s).max() <= 1e-13
    # sin/cos of the proposals may differ from the oracle's libm in the last
    # bit, so the spins (and through c, lambda) agree to rounding
    assert mc.lambda_ == pytest.approx(lam_o, rel=1e-12, abs=1e-14)
    assert sigma == pytest.approx(sigma_o, rel=1e-15)
    assert abs(kd(s) - ol.constraint_value(s, ko)) <= 1e-12 * lat.size


@pytest.mark.parametrize("kind", list(KINDS))
@pytest.mark.parametrize("name", ["square", "honeycomb", "pyrochlore", "asym_open"])
def test_constraint_sweep_fp64_matches_oracle(m, orc, name, kind):
    """Three FP64 sweeps of N random-site proposals each == the oracle fed the
    same Philox draws (counters (q, sweep, chain, 5) and (q, sweep, chain, 6))."""
    seed = 31
    lat, ol, mc, kd, ko = _setup(m, orc, name, "fp64", seed=seed)
    s = rand_spins(lat.size, 23)
    mc.set_spins(s)
    mc.ctx.call("csmc_set_sigma", np.array([0.7]).ctypes.data_as(C.POINTER(C.c_double)))
    alg = getattr(m, kind)()
    sigma, lam = 0.7, 0.0
    for sweep in range(3):
        acc = alg(mc, 0.6)
        acc_o, sigma, lam = ol.constraint_sweep(s, 0.6, KINDS[kind], sigma, 2.0, ko, lam, seed, 0, sweep)
        assert acc == acc_o
        assert np.abs(mc.spins(0) - s).max() <= 1e-12
        assert mc.lambda_ == pytest.approx(lam, rel=1e-9, abs=1e-12)
        assert mc.sigma == pytest.approx(sigma, rel=1e-12)


def test_constraint_sweep_fp32_flips(m, orc):
    """FP32 sweep against the FP64 oracle on the same draws: decisions may
    differ only where the exponent sits within single-precision rounding."""
    seed = 41
    lat, ol, mc, kd, ko = _setup(m, orc, "honeycomb", "fp32", seed=seed)
    s = np.asfortranarray(rand_spins(lat.size, 24).astype(np.float32).astype(np.float64))
    mc.set_spins(s)
    acc = m.MetropolisConstraint()(mc, 0.6)
    acc_o, _, lam_o = ol.constraint_sweep(s, 0.6, 0, 60.0, 2.0, ko, 0.0, seed, 0, 0)
    flips = abs(acc - acc_o)
    print(f"fp32 accepted {acc}, oracle {acc_o}, lambda {mc.lambda_} vs {lam_o}")
    assert flips <= max(2, 0.02 * lat.size)


def test_zero_weight_without_constraint_is_plain_random_site_metropolis(m, orc):
    """weight 0 and c = 0: lambda stays 0 and the sweep is metropolis! with N
    random-site proposals (metropolis.jl:65-82)."""
    seed = 5
    uc, shape, bc = model(m, "sc")
    lat = m.Lattice(shape, uc, 1.0, bc=bc)
    ol = orc.OracleLattice(uc, shape, 1.0, bc=bc)
    mc = m.MonteCarlo(0.5, lat, {"overrelaxation_rate": 5}, precision="fp64", seed=seed)
    s = rand_spins(lat.size, 25)
    mc.set_spins(s)
    acc = m.MetropolisConstraint()(mc, 0.5)
    acc_o, _, lam_o = ol.constraint_sweep(s, 0.5, 0, 60.0, 60.0, orc.constraint(), 0.0, seed, 0, 0)
    assert acc == acc_o and lam_o == 0.0 and mc.lambda_ == 0.0
    assert np.abs(mc.spins(0) - s).max() <= 1e-12


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_parallel_tempering_with_constraint(m, orc, precision):
    """parallel_tempering! with alg=MetropolisConstraintAdaptive() runs on the
    global path; lambda is per slot (it stays with the temperature when
    replicas exchange), the probe energies are those of the slots' chains."""
    lat, ol, mc, kd, ko = _setup(m, orc, "square", precision, weight=0.05, R=4)
    mc.temperatures[:] = [0.3, 0.5, 0.8, 1.3]
    mc.ctx.set_temperatures(mc.temperatures)
    p = mc.parameters
    p.t_thermalization, p.t_measurement, p.report_interval, p.checkpoint_rate = 10, 20, 10, 10
    p.probe_rate, p.swap_rate = 5, 5
    out = m.parallel_tempering(mc, alg=m.MetropolisConstraintAdaptive(), verbose=False)
    lam = mc.lambda_
    assert np.all(np.isfinite(lam)) and np.any(lam != 0.0)
    assert mc.accepted.sum() > 0
    E = np.array([ol.total_energy(mc.spins(r)) for r in range(4)])
    assert np.allclose(out["energy"][-1], E, rtol=1e-4 if precision == "fp32" else 1e-10, atol=1e-4)


def test_constraint_rejects_resident_path_and_callables(m):
    uc, shape, bc = model(m, "square")
    lat = m.Lattice(shape, uc, 1.0, bc=bc)
    with pytest.raises(TypeError):
        m.MonteCarlo(0.5, lat, {}, constraint=lambda lattice: 0.0, weight=1.0)
    mc = m.MonteCarlo([0.5, 0.7], lat, {"overrelaxation_rate": 5, "swap_rate": 5, "probe_rate": 5,
                                        "t_thermalization": 5, "t_measurement": 5, "report_interval": 5,
                                        "checkpoint_rate": 5}, path="resident")
    with pytest.raises(m.CSMCError):
        m.parallel_tempering(mc, alg=m.MetropolisConstraint(), verbose=False)
