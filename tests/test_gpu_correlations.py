"""Equal-time spin correlations (compute_equal_time_correlations,
spin_correlations.jl:6-43) on the GPU against the oracle's restatement, for
every slot of a parallel-tempering context, in both precisions.

Tolerances: FP64 1e-10 and FP32 2e-5 relative to N, the largest possible
|S_a(k)|^2 / N (all spins aligned), since the sums run over N sites in a
different order (device order) than the oracle's."""
import numpy as np
import pytest

from test_gpu_parity import rand_spins

pytestmark = pytest.mark.gpu

TOL = {"fp64": 1e-10, "fp32": 2e-5}


def _wavevectors(lat, n, seed):
    rng = np.random.default_rng(seed)
    D = lat.site_positions.shape[0]
    ks = rng.uniform(-np.pi, np.pi, size=(D, n))
    ks[:, 0] = 0.0  # k = 0: |M|^2 / N
    return ks


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("name,shape,R", [("square", (8, 8), 3), ("honeycomb", (6, 5), 2), ("sc", (6, 6, 6), 17),
                                          ("pyrochlore", (2, 2, 3), 1), ("sc", (4, 4, 4), 40)])
def test_structure_factor_matches_oracle(m, orc, name, shape, R, precision):
    E = m.examples
    uc = {"square": E.square_heisenberg, "honeycomb": lambda: E.honeycomb_kitaev(K=-1, J=0.1, G=0.05),
          "sc": E.sc_heisenberg, "pyrochlore": E.pyrochlore_ckq}[name]()
    lat = m.Lattice(shape, uc, 1.0)
    mc = m.MonteCarlo([0.5 + 0.1 * r for r in range(R)] if R > 1 else 0.5, lat, {}, precision=precision, seed=5)
    spins = [rand_spins(lat.size, 70 + r) for r in range(R)]
    for r, s in enumerate(spins):
        mc.set_spins(s, r)
    ks = _wavevectors(lat, 77, 3)  # n_k not a multiple of the 64-wavevector tile
    got = m.structure_factors(mc, ks)
    assert got.shape == (R, 9, 77)
    for r in range(R):
        ref = orc.structure_factor(mc.spins(r), lat.site_positions, ks)
        assert np.abs(got[r] - ref).max() <= TOL[precision] * lat.size, (r, np.abs(got[r] - ref).max())
    # k = 0 is |sum_i s_i|^2 / N
    for r in range(R):
        assert got[r][0, 0] + got[r][4, 0] + got[r][8, 0] == pytest.approx(
            m.get_magnetization(mc, r) ** 2 / lat.size, rel=1e-4 if precision == "fp32" else 1e-10)


def test_structure_factor_follows_the_slots_after_exchanges(m, orc):
    """The record is by slot: after a PT run with exchanges, slot r's
    correlations are those of the configuration now in slot r."""
    lat = m.Lattice((6, 6), m.examples.triangular_afm(h=0.5), 1.0)
    mc = m.MonteCarlo([0.2, 0.3, 0.5, 0.8], lat, {"overrelaxation_rate": 5}, precision="fp64", seed=2)
    p = mc.parameters
    p.t_thermalization, p.t_measurement, p.report_interval, p.checkpoint_rate = 0, 50, 50, 10
    p.probe_rate, p.swap_rate = 5, 5
    m.parallel_tempering(mc, verbose=False)
    assert mc.exchanged.sum() > 0
    ks = _wavevectors(lat, 9, 4)
    got = m.structure_factors(mc, ks)
    for r in range(4):
        ref = orc.structure_factor(mc.spins(r), lat.site_positions, ks)
        assert np.abs(got[r] - ref).max() <= 1e-10 * lat.size


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_parallel_tempering_measures_correlations_at_every_probe(m, orc, precision):
    """MonteCarlo(corr=true, ks) (monte_carlo.jl:371-375): one 9 x N_k sample
    per probe and slot, taken after the exchange; at k = 0 the trace of a
    sample is |M|^2 / N of the same probe."""
    lat = m.Lattice((8, 8), m.examples.triangular_afm(h=0.3), 1.0)
    ks = _wavevectors(lat, 5, 6)
    mc = m.MonteCarlo([0.2, 0.4, 0.9], lat, {"overrelaxation_rate": 5}, precision=precision, seed=8, corr=True, ks=ks)
    p = mc.parameters
    p.t_thermalization, p.t_measurement, p.report_interval, p.checkpoint_rate = 10, 40, 25, 10
    p.probe_rate, p.swap_rate = 5, 10
    out = m.parallel_tempering(mc, verbose=False)
    n_probes = out["magnetization"].shape[0]
    assert n_probes == 8
    for r in range(3):
        samples = np.array(mc.observables[r].correlations)
        assert samples.shape == (n_probes, 9, 5)
        trace0 = samples[:, 0, 0] + samples[:, 4, 0] + samples[:, 8, 0]
        rel = 1e-4 if precision == "fp32" else 1e-10
        assert np.allclose(trace0, out["magnetization"][:, r] ** 2 / lat.size, rtol=rel, atol=rel)


def test_parallel_tempering_saves_initial_configurations(m, orc):
    """saveIC (monte_carlo.jl:353-364): at every checkpoint of the measurement
    phase the listed ranks' configurations are kept; each equals the
    configuration the probe of the same iteration measured."""
    uc = m.examples.triangular_afm(h=0.3)
    lat = m.Lattice((6, 6), uc, 1.0)
    ol = orc.OracleLattice(uc, (6, 6), 1.0)
    mc = m.MonteCarlo([0.2, 0.4, 0.9], lat, {"overrelaxation_rate": 5}, precision="fp64", seed=4)
    p = mc.parameters
    p.t_thermalization, p.t_measurement, p.report_interval, p.checkpoint_rate = 10, 30, 15, 10
    p.probe_rate, p.swap_rate = 5, 5
    out = m.parallel_tempering(mc, saveIC=(0, 2), verbose=False)
    ics = mc.initial_configurations
    assert sorted(ics) == [0, 2]
    for r in (0, 2):
        assert sorted(ics[r]) == [0, 1, 2]  # iterations 10, 20, 30
        for ts in range(3):
            k = 2 * ts  # probes at 10, 15, 20, ...
            s = ics[r][ts]
            assert ol.total_energy(s) == pytest.approx(out["energy"][k, r], rel=1e-12, abs=1e-12)
            assert ol.magnetization(s) == pytest.approx(out["magnetization"][k, r], rel=1e-12, abs=1e-12)


@pytest.mark.parametrize("name,shape,R,n_k,aligned", [("sc", (4, 4, 4), 17, 77, False), ("sc", (6, 6, 6), 70, 130, False),
                                                       ("square", (8, 8), 3, 200, False), ("sc", (6, 6, 6), 5, 40, True),
                                                       ("pyrochlore", (2, 2, 3), 1, 129, False),
                                                       ("sc", (4, 4, 4), 1, 19456, False)])
def test_tensor_core_structure_factor(m, orc, name, shape, R, n_k, aligned):
    """Single precision on the tensor cores (tcgen05, each operand split into
    two TF32 halves) against the oracle and against the CUDA-core kernel, with
    the FP32 tolerance 2e-5 x N: wavevector counts that are not multiples of
    the 128-wavevector tile, more than 64 replicas (two replica tiles), and all
    spins aligned (|S(0)|^2 / N = N, the largest sums).  The sites of a tile
    are split over several CTAs when there are fewer tiles than SMs (4 splits
    of 1 chunk at 64 sites; 8 asked for 14 chunks, 7 run), and not at 152
    tiles (19456 wavevectors)."""
    E = m.examples
    uc = {"square": E.square_heisenberg, "sc": E.sc_heisenberg, "pyrochlore": E.pyrochlore_ckq}[name]()
    lat = m.Lattice(shape, uc, 1.0)
    mc = m.MonteCarlo([0.5 + 0.01 * r for r in range(R)] if R > 1 else 0.5, lat, {}, precision="fp32", seed=5)
    for r in range(R):
        s = rand_spins(lat.size, 300 + r)
        if aligned:
            s = np.asfortranarray(np.tile(s[:, :1], (1, lat.size)))
        mc.set_spins(s, r)
    ks = _wavevectors(lat, n_k, 8)
    tc = m.structure_factors(mc, ks)
    mc.ctx.call("csmc_set_tensor_cores", 0)
    cc = m.structure_factors(mc, ks)
    mc.ctx.call("csmc_set_tensor_cores", 1)
    tol = TOL["fp32"] * lat.size
    assert np.abs(tc - cc).max() <= tol, np.abs(tc - cc).max()
    for r in range(R):
        ref = orc.structure_factor(mc.spins(r), lat.site_positions, ks)
        assert np.abs(tc[r] - ref).max() <= tol, (r, np.abs(tc[r] - ref).max())
    if aligned:
        assert tc[0][0, 0] + tc[0][4, 0] + tc[0][8, 0] == pytest.approx(lat.size, rel=1e-5)
