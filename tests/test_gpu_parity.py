"""GPU kernels (through the C ABI) against the CPU oracle.

Tolerances (the parity gates of the path):
  local field / dE, FP64: |gpu - oracle| <= 1e-12 * sum|terms|
  local field / dE, FP32: |gpu - oracle| <= 1e-6  * sum|terms|
  colour-order overrelaxation / deterministic / Metropolis sweeps, FP64: 1e-12
  replay: every accept/reject decision identical
"""
import json
import math
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = {"fp64": 1e-12, "fp32": 1e-6}


def model(m, name):
    E = m.examples
    if name == "square":
        return E.square_heisenberg(), (8, 8), "periodic"
    if name == "honeycomb":
        return E.honeycomb_kitaev(K=-1, J=0.1, G=0.05, Gp=-0.02, h=0.1), (6, 6), "periodic"
    if name == "sc":
        return E.sc_heisenberg(J=1.0, D=0.2), (4, 4, 4), "periodic"
    if name == "sc24":  # the benchmark lattice
        return E.sc_heisenberg(J=1.0, D=0.2), (24, 24, 24), "periodic"
    if name == "triangular_open":
        return E.triangular_afm(h=0.7), (6, 6), "open"
    if name == "pyrochlore":
        return E.pyrochlore_ckq(), (2, 2, 2), "periodic"
    if name == "pyrochlore_dense":  # tensors without an isotropic form: the dense contractions
        uc = E.pyrochlore_ckq(cubic=False, quartic=False)
        rng = np.random.default_rng(3)
        C, Q = 0.02 * rng.normal(size=(3, 3, 3)), 0.05 * rng.normal(size=(3, 3, 3, 3))
        for face in [(1, 2, 3), (2, 3, 4)]:
            m.addCubic(uc, *face, C, (0, 0, 0), (0, 0, 0))
        m.addQuartic(uc, 1, 2, 3, 4, Q, (0, 0, 0), (0, 0, 0), (0, 0, 0))
        m.addQuartic(uc, 1, 3, 2, 4, 0.05 * np.einsum("ab,cd->abcd", np.eye(3), np.eye(3)), (0, 0, 0), (0, 0, 0),
                     (0, 0, 0))  # isotropic beside dense in one lattice
        return uc, (2, 2, 2), "periodic"
    if name == "asym_open":
        uc = m.Honeycomb()
        a = np.arange(9.0).reshape(3, 3) / 9 - 0.4
        m.addBilinear(uc, 1, 2, a, (0, -1))
        m.addBilinear(uc, 2, 1, a.T, (1, 0))
        m.addOnSite(uc, 1, np.diag([0.1, 0.2, 0.3]))
        m.addOnSite(uc, 2, np.diag([0.3, 0.2, 0.1]))
        m.addZeemanCoupling(uc, 1, [0.1, 0.0, 0.0])
        m.addZeemanCoupling(uc, 2, [0.0, 0.2, 0.0])
        return uc, (3, 4), "open"
    if name == "selfloop":
        uc = E.square_heisenberg(J=-0.5)
        return uc, (1, 2), "periodic"
    raise KeyError(name)


MODELS = ["square", "honeycomb", "sc", "triangular_open", "pyrochlore", "pyrochlore_dense", "asym_open", "selfloop"]


def setup(m, orc, name, precision, R=1, seed=20261203, T=1.0):
    uc, shape, bc = model(m, name)
    lat = m.Lattice(shape, uc, 1.0, bc=bc)
    ol = orc.OracleLattice(uc, shape, 1.0, bc=bc)
    mc = m.MonteCarlo([T] * R if R > 1 else T, lat, {"overrelaxation_rate": 5}, precision=precision, seed=seed)
    return lat, ol, mc


def obs_tol(precision):
    """Per-site tolerance of energies and |M| between launch configurations:
    single precision adds each thread's sites in FP32 before the FP64 sum, and
    the split of sites over threads differs between configurations."""
    return 1e-9 if precision == "fp64" else 1e-6


def term_scale(lat):
    """Per-site sum of |coefficients| (|s| = 1): bounds sum|terms| of the local field."""
    t = lat.tables()
    s = 2 * np.abs(t["onsite"]).sum(axis=(1, 2)) + np.abs(t["field"]).sum(axis=1)
    s += np.abs(t["bilinear_matrices"]).sum(axis=(1, 2, 3))
    s += np.abs(t["cubic_tensors"]).sum(axis=(1, 2, 3, 4))
    s += np.abs(t["quartic_tensors"]).sum(axis=(1, 2, 3, 4, 5))
    return np.maximum(s, 1e-300)


def rand_spins(n, seed):
    rng = np.random.default_rng(seed)
    v = rng.normal(size=(3, n))
    v /= np.linalg.norm(v, axis=0)
    return np.asfortranarray(v)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("name", MODELS)
def test_local_field(m, orc, name, precision):
    lat, ol, mc = setup(m, orc, name, precision)
    s = rand_spins(lat.size, 1)
    if precision == "fp32":
        s = np.asfortranarray(s.astype(np.float32).astype(np.float64))
    mc.set_spins(s)
    H = m.local_fields(mc)
    Ho = ol.local_fields(s)
    err = np.abs(H - Ho).max(axis=0) / term_scale(lat)
    assert err.max() <= TOL[precision], err.max()


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("name", MODELS)
def test_energy_diff(m, orc, name, precision):
    import ctypes as C
    lat, ol, mc = setup(m, orc, name, precision)
    s = rand_spins(lat.size, 2)
    if precision == "fp32":
        s = np.asfortranarray(s.astype(np.float32).astype(np.float64))
    mc.set_spins(s)
    rng = np.random.default_rng(3)
    n = 64
    sites = rng.integers(0, lat.size, n).astype(np.int64)
    new = rand_spins(n, 4)
    if precision == "fp32":
        new = np.asfortranarray(new.astype(np.float32).astype(np.float64))
    new_c = np.ascontiguousarray(new.T)
    dE = np.zeros(n)
    mc.ctx.call("csmc_energy_diff", 0, n, sites.ctypes.data_as(C.POINTER(C.c_int64)),
                new_c.ctypes.data_as(C.POINTER(C.c_double)), dE.ctypes.data_as(C.POINTER(C.c_double)))
    ref = np.array([ol.energy_diff(s, sites[q], new[:, q]) for q in range(n)])
    scale = 2 * term_scale(lat)[sites]
    assert (np.abs(dE - ref) / scale).max() <= TOL[precision]


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("name", MODELS)
def test_total_energy_and_magnetization(m, orc, name, precision):
    lat, ol, mc = setup(m, orc, name, precision, R=2)
    s0, s1 = rand_spins(lat.size, 5), rand_spins(lat.size, 6)
    if precision == "fp32":
        s0, s1 = (np.asfortranarray(x.astype(np.float32).astype(np.float64)) for x in (s0, s1))
    mc.set_spins(s0, 0)
    mc.set_spins(s1, 1)
    E = mc.ctx.per_slot("csmc_total_energy")
    M = mc.ctx.per_slot("csmc_magnetization")
    scale = term_scale(lat).sum()
    for k, s in enumerate((s0, s1)):
        assert abs(E[k] - ol.total_energy(s)) <= TOL[precision] * scale
        assert abs(M[k] - ol.magnetization(s)) <= TOL[precision] * lat.size
        assert np.array_equal(mc.spins(k), s) or precision == "fp32"


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("name", MODELS)
def test_overrelax_and_deterministic_in_colour_order(m, orc, name, precision):
    """OR / deterministic colour sweeps == the oracle's single-site routines in the same order."""
    lat, ol, mc = setup(m, orc, name, precision)
    _, order, _ = lat.colouring()
    s = rand_spins(lat.size, 7)
    if precision == "fp32":
        s = np.asfortranarray(s.astype(np.float32).astype(np.float64))
    mc.set_spins(s)
    tol = 1e-12 if precision == "fp64" else 2e-5
    m.overrelaxation(mc)
    ol.overrelax_order(s, order)
    assert np.abs(mc.spins(0) - s).max() <= tol
    mc.ctx.call("csmc_deterministic_sweeps", 1)
    ol.deterministic_order(s, order)
    assert np.abs(mc.spins(0) - s).max() <= tol
    # a second overrelaxation after alignment changes nothing the oracle does not
    m.overrelaxation(mc)
    ol.overrelax_order(s, order)
    assert np.abs(mc.spins(0) - s).max() <= tol


@pytest.mark.parametrize("kind", ["Metropolis", "MetropolisAdaptive", "MetropolisFixedCone"])
@pytest.mark.parametrize("name", ["honeycomb", "sc", "pyrochlore", "pyrochlore_dense", "asym_open"])
def test_metropolis_colour_sweep_fp64(m, orc, name, kind):
    """One FP64 colour sweep == the oracle fed the same Philox stream (53-bit uniforms)."""
    seed = 99
    lat, ol, mc = setup(m, orc, name, "fp64", seed=seed, T=0.7)
    _, order, _ = lat.colouring()
    s = rand_spins(lat.size, 8)
    mc.set_spins(s)
    import ctypes as C
    sig = np.array([0.8])
    mc.ctx.call("csmc_set_sigma", sig.ctypes.data_as(C.POINTER(C.c_double)))
    alg = getattr(m, kind)()
    okind = {"Metropolis": orc.UNIFORM, "MetropolisAdaptive": orc.ADAPTIVE, "MetropolisFixedCone": orc.FIXED_CONE}[kind]
    sigma = 0.8
    for sweep in range(3):
        acc = alg(mc, 0.7)
        acc_o, sigma = ol.colour_sweep(s, 0.7, okind, sigma, order, seed, 0, sweep, 53)
        assert acc == acc_o
        assert np.abs(mc.spins(0) - s).max() <= 1e-12
        assert abs(mc.sigma - sigma) <= 1e-12


@pytest.mark.parametrize("name", ["honeycomb", "sc", "pyrochlore"])
def test_metropolis_colour_sweep_fp32_flips(m, orc, name):
    """FP32 sweep against the oracle on the same 24-bit stream: decisions may differ
    only where dE or the acceptance threshold sits within single-precision
    rounding; the count of such flips is reported, not gated."""
    seed = 5
    lat, ol, mc = setup(m, orc, name, "fp32", seed=seed, T=0.7)
    _, order, _ = lat.colouring()
    s = np.asfortranarray(rand_spins(lat.size, 9).astype(np.float32).astype(np.float64))
    mc.set_spins(s)
    acc = m.Metropolis()(mc, 0.7)
    acc_o, _ = ol.colour_sweep(s, 0.7, orc.UNIFORM, 60.0, order, seed, 0, 0, 24)
    flips = abs(acc - acc_o)
    print(f"{name}: fp32 accepted {acc}, oracle {acc_o}, flips {flips}")
    assert flips <= max(2, 0.01 * lat.size)


@pytest.mark.parametrize("kind", ["Metropolis", "MetropolisAdaptive", "MetropolisFixedCone"])
@pytest.mark.parametrize("name", ["honeycomb", "sc", "pyrochlore", "asym_open", "selfloop"])
def test_replay_exact(m, orc, name, kind):
    """Replay of the reference's proposals: every decision identical."""
    lat, ol, mc = setup(m, orc, name, "fp64", T=0.4)
    s = rand_spins(lat.size, 10)
    mc.set_spins(s)
    rng = np.random.default_rng(11)
    n = 3 * lat.size
    sites = rng.integers(0, lat.size, n)
    up, uz, ua = rng.random(n), rng.random(n), rng.random(n)
    okind = {"Metropolis": orc.UNIFORM, "MetropolisAdaptive": orc.ADAPTIVE, "MetropolisFixedCone": orc.FIXED_CONE}[kind]
    import ctypes as C
    mc.ctx.call("csmc_set_sigma", np.array([0.5]).ctypes.data_as(C.POINTER(C.c_double)))
    acc, sigma = m.replay(mc, sites, up, uz, ua, alg=getattr(m, kind)(), T=0.4)
    acc_o, sigma_o = ol.replay(s, 0.4, okind, 0.5, sites, up, uz, ua)
    assert np.array_equal(acc, acc_o)
    assert np.abs(mc.spins(0) - s).max() <= 1e-13
    assert sigma == pytest.approx(sigma_o, rel=1e-15)


def _run_once(m, mc, start, n, or_rate, path, block=0):
    import ctypes as C
    from importlib import import_module
    L = import_module(m.__name__ + "._lib")
    rp = L.RunParams()
    rp.sweep_start, rp.n_sweeps, rp.overrelaxation_rate = start, n, or_rate
    rp.path = {"resident": L.PATH_RESIDENT, "global": L.PATH_GLOBAL, "per_replica": L.PATH_PER_REPLICA}[path]
    rp.resident_block = block
    acc = np.zeros(mc.n_replicas)
    rp.accepted = acc.ctypes.data_as(C.POINTER(C.c_double))
    mc.ctx.call("csmc_run", C.byref(rp))
    return acc


SINGLE_SWEEP_CASES = [(n, p) for n in ["square", "honeycomb", "sc", "triangular_open", "pyrochlore", "pyrochlore_dense",
                                        "asym_open"]
                      for p in ["resident", "resident1024", "global"]] + [("sc24", "global")]


@pytest.mark.parametrize("name,path", SINGLE_SWEEP_CASES)
def test_run_paths_single_sweeps_match_oracle(m, orc, name, path):
    """One iteration of csmc_run on each execution path (the resident kernel
    picks its specialised form for every model here but the pyrochlore) ==
    the oracle: an overrelaxation-only iteration in colour order, and a
    Metropolis-only iteration on the same Philox stream (FP64)."""
    seed = 21
    lat, ol, mc = setup(m, orc, name, "fp64", seed=seed, T=0.6)
    _, order, _ = lat.colouring()
    s = rand_spins(lat.size, 30)
    mc.set_spins(s)
    block = 1024 if path == "resident1024" else 0
    path = "resident" if path.startswith("resident") else path
    _run_once(m, mc, 1, 1, 1000, path, block)  # iteration 1: overrelaxation only
    ol.overrelax_order(s, order)
    assert np.abs(mc.spins(0) - s).max() <= 1e-12
    acc = _run_once(m, mc, 0, 1, 0, path, block)  # iteration 0, no overrelaxation: one Metropolis sweep
    acc_o, _ = ol.colour_sweep(s, 0.6, orc.UNIFORM, 60.0, order, seed, 0, 0, 53)
    assert acc[0] == acc_o
    assert np.abs(mc.spins(0) - s).max() <= 1e-12


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("name", ["square", "sc", "pyrochlore", "triangular_open"])
def test_run_paths_agree(m, orc, name, precision):
    """Resident, per-colour and per-replica execution of a short window with
    overrelaxation, Metropolis, energies and probes.  The paths associate the
    same sums differently (the resident kernel folds 2O+P), so they agree to
    rounding and the agreement is checked over few sweeps (the dynamics
    amplify rounding differences)."""
    res = []
    for path in ("resident", "global", "per_replica"):
        lat, ol, mc = setup(m, orc, name, precision, R=3, seed=3)
        mc.ctx.set_temperatures(np.array([0.3, 0.6, 1.2]))
        for r in range(3):
            mc.set_spins(rand_spins(lat.size, 20 + r), r)
        _run_once(m, mc, 1, 3, 2, path)  # iterations 1..3: 3 OR sweeps, 1 Metropolis sweep
        res.append(np.stack([mc.spins(r) for r in range(3)]))
    tol = 1e-11 if precision == "fp64" else 1e-4
    for other in res[1:]:
        diff = np.abs(res[0] - other).max(axis=1)  # per replica and site
        # FP32: a proposal whose dE sits within rounding of the threshold may flip
        assert np.mean(diff > tol) <= (0.0 if precision == "fp64" else 0.01), diff.max()


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("name", ["square", "sc", "pyrochlore", "triangular_open"])
def test_generic_paths_give_the_same_chain(m, orc, name, precision):
    """The per-colour and per-replica launches run identical arithmetic: the
    same chain over a whole window, probes and counters included."""
    res = []
    for path in ("global", "per_replica"):
        lat, ol, mc = setup(m, orc, name, precision, R=3, seed=3)
        mc.path = path
        mc.ctx.set_temperatures(np.array([0.3, 0.6, 1.2]))
        for r in range(3):
            mc.set_spins(rand_spins(lat.size, 20 + r), r)
        mc.parameters.t_thermalization = 10
        mc.parameters.t_measurement = 30
        mc.parameters.report_interval = 40
        mc.parameters.checkpoint_rate = 10
        mc.parameters.probe_rate = 5
        mc.parameters.swap_rate = 0
        mc.parameters.overrelaxation_rate = 4
        out = m.parallel_tempering(mc, verbose=False)
        res.append((np.stack([mc.spins(r) for r in range(3)]), out["energy"], out["magnetization"], mc.accepted.copy()))
    tol = 1e-12 if precision == "fp64" else 1e-5
    for other in res[1:]:
        assert np.abs(res[0][0] - other[0]).max() <= tol
        assert np.array_equal(res[0][3], other[3])
        assert np.abs(res[0][1] - other[1]).max() <= tol * 100
        assert np.abs(res[0][2] - other[2]).max() <= tol * 100


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_honeycomb_anneal_kat(m, orc, precision):
    """test/mctests.jl:1-50 on the GPU: anneal to 1e-7 + deterministic updates, E/N rounds to -0.6444."""
    c = json.loads((Path(__file__).parent / "golden" / "reference_kats.json").read_text())["cases"][3]
    md = c["model"]
    uc = m.examples.honeycomb_kitaev(K=md["K"], J=md["J"], G=md["G"], Gp=md["Gp"], h=md["h"])
    lat = m.Lattice(tuple(md["shape"]), uc, md["S"], rng=np.random.default_rng(1))
    mc = m.MonteCarlo(md["T"], lat, dict(md["params"]), precision=precision, seed=17)
    m.simulated_annealing(mc, lambda x: md["T0"] * 0.9 ** x, md["T0"], verbose=False)
    m.deterministic_updates(mc)
    E = m.energy_density(mc)
    assert round(E, 4) == c["expect"]["energy_density_4dp"], E


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("path", ["resident", "size_groups", "global"])
def test_batch_of_lattices_matches_single(m, orc, precision, path):
    """Independent chains of different sizes in one context (the uneven batch
    of independent chains) == each chain run alone: with the same chain id
    (csmc_set_chain_ids), seed and initial spins, a chain draws the same
    numbers wherever it runs, so its spins and accepted counts agree bit for
    bit.  The batch runs every lattice in one launch (one work list), or as
    size groups (one launch shape per band of sizes, side by side); alone,
    each context picks its own launch shape."""
    import ctypes as C
    from importlib import import_module
    L = import_module(m.__name__ + "._lib")
    E = m.examples
    specs = [(12, 0.2, 0.5), (18, 0.6, 1.5), (6, 1.0, 2.5), (24, 0.35, 0.0)]
    ids = np.array([7, 1000, 3, 42], np.uint32)
    lats = [m.Lattice((Ls, Ls), E.triangular_afm(h=h), 1.0, rng=np.random.default_rng(Ls)) for Ls, _, h in specs]
    Ts = np.array([t for _, t, _ in specs])

    def run(ctx, T, ids_):
        ctx.set_temperatures(T)
        ctx.call("csmc_set_chain_ids", ids_.ctypes.data_as(C.POINTER(C.c_uint32)))
        rp = L.RunParams()
        rp.sweep_start, rp.n_sweeps, rp.overrelaxation_rate = 1, 30, 3
        rp.path = L.PATH_GLOBAL if path == "global" else L.PATH_RESIDENT
        acc = np.zeros(ctx.n_slots)
        rp.accepted = acc.ctypes.data_as(C.POINTER(C.c_double))
        ctx.call("csmc_run", C.byref(rp))
        return acc

    batch = m.monte_carlo.Context(lats, [1] * len(lats), precision=precision, seed=4)
    if path == "size_groups":
        batch.call("csmc_set_size_groups", 1)
        n = C.c_int32()
        batch.call("csmc_size_groups", C.byref(n))
        assert n.value >= 2  # padded sizes of about 600 and 400 | 220 and 130
    for k, lat in enumerate(lats):
        batch.set_spins(k, lat.spins)
    acc_b = run(batch, Ts, ids)
    for k, lat in enumerate(lats):
        one = m.monte_carlo.Context([lat], [1], precision=precision, seed=4)
        one.set_spins(0, lat.spins)
        acc_1 = run(one, Ts[k:k + 1], ids[k:k + 1])
        assert acc_1[0] == acc_b[k], (k, acc_1[0], acc_b[k])
        assert np.array_equal(one.get_spins(0), batch.get_spins(k)), k
    assert acc_b.min() > 0


@pytest.mark.parametrize("block", [512, 1024])
def test_resident_fp32_benchmark_lattice(m, orc, block):
    """The benchmark lattice (SC L=24) in single precision on the resident
    kernel: one overrelaxation sweep in colour order and one Metropolis sweep
    on the 24-bit Philox stream against the FP64 oracle.  Metropolis decisions
    whose dE sits within single-precision rounding of the threshold may flip;
    at most 1% of the sites may differ."""
    seed = 21
    lat, ol, mc = setup(m, orc, "sc24", "fp32", seed=seed, T=0.6)
    _, order, _ = lat.colouring()
    s = np.asfortranarray(rand_spins(lat.size, 30).astype(np.float32).astype(np.float64))
    mc.set_spins(s)
    _run_once(m, mc, 1, 1, 1000, "resident", block)
    ol.overrelax_order(s, order)
    assert np.abs(mc.spins(0) - s).max() <= 2e-5
    s = np.asfortranarray(mc.spins(0))
    acc = _run_once(m, mc, 0, 1, 0, "resident", block)
    acc_o, _ = ol.colour_sweep(s, 0.6, orc.UNIFORM, 60.0, order, seed, 0, 0, 24)
    assert abs(acc[0] - acc_o) <= 0.01 * lat.size
    assert np.mean(np.abs(mc.spins(0) - s).max(axis=0) > 1e-4) <= 0.01


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("name", ["sc_afm", "triangular_field"])
def test_pt_statistics_vs_oracle(m, orc, precision, name):
    """Parallel tempering on the GPU (colour sweeps, device exchanges) against
    the oracle's restatement of parallel_tempering! (random-site Metropolis,
    sequential overrelaxation, in-process exchanges): E/N, |M|/N and C_v per
    temperature agree within 3 combined standard errors (binned).

    Models without onsite terms: with an onsite term the reference's
    overrelaxation reflects about a local field that contains 2 O s
    (monte_carlo.jl:135-137) and does not conserve energy, so the chain's
    steady state is not the Boltzmann distribution and depends on the update
    order; there parity is exact per sweep in the same order (the colour-order
    tests above), not statistical across orders."""
    from importlib import import_module
    obs = import_module(m.__name__ + ".observables")
    if name == "sc_afm":
        uc, shape, T = m.examples.sc_heisenberg(J=1.0, D=0.0), (4, 4, 4), [0.4, 0.7, 1.1, 1.8]
    else:
        uc, shape, T = m.examples.triangular_afm(h=0.5), (6, 6), [0.15, 0.3, 0.6, 1.2]
    params = dict(t_thermalization=2000, t_measurement=20000, probe_rate=10, swap_rate=10, overrelaxation_rate=5,
                  report_interval=11000, checkpoint_rate=1000)
    lat = m.Lattice(shape, uc, 1.0, rng=np.random.default_rng(7))
    mc = m.MonteCarlo(T, lat, params, precision=precision, seed=8)
    out = m.parallel_tempering(mc, verbose=False)
    ol = orc.OracleLattice(uc, shape, 1.0)
    spins = [ol.random_spins(9, r) for r in range(len(T))]
    ref = ol.parallel_tempering(spins, T, params["t_thermalization"], params["t_measurement"], 10, 10, 5,
                                n_threads=4, seed=10)
    N = lat.size
    assert out["energy"].shape == ref["energy"].shape
    for r, t in enumerate(T):
        for gpu, cpu, f in ((out["energy"][:, r] / N, ref["energy"][:, r] / N, obs.mean_and_error),
                            (out["magnetization"][:, r] / N, ref["magnetization"][:, r] / N, obs.mean_and_error),
                            (out["energy"][:, r], ref["energy"][:, r], lambda x: obs.specific_heat(x, t, N))):
            a, da = f(gpu)
            b, db = f(cpu)
            assert abs(a - b) <= 3 * math.hypot(da, db), (t, a, da, b, db)
    # exchanges happened and the slot permutation stayed a permutation
    assert mc.exchanged.sum() > 0
    perm = np.zeros(len(T), np.int32)
    import ctypes as C
    mc.ctx.call("csmc_get_permutation", perm.ctypes.data_as(C.POINTER(C.c_int32)))
    assert sorted(perm.tolist()) == list(range(len(T)))


def test_fp32_energy_density_vs_fp64_oracle(m, orc):
    """FP32 spins and fields with FP64 energy accumulation: E/N of the same
    configurations within 1e-4 of the FP64 oracle on the benchmark lattice."""
    uc = m.examples.sc_heisenberg(J=1.0, D=0.2)
    lat = m.Lattice((24, 24, 24), uc, 1.0, initialCondition="none")
    ol = orc.OracleLattice(uc, (24, 24, 24), 1.0)
    mc = m.MonteCarlo([0.1, 2.0], lat, {"overrelaxation_rate": 5}, precision="fp32", seed=1)
    mc.ctx.call("csmc_random_spins", 5)
    _run_once(m, mc, 1, 20, 5, "resident")  # partly ordered at T=0.1
    E = mc.ctx.per_slot("csmc_total_energy")
    for r in range(2):
        s = mc.spins(r)
        assert abs(E[r] / lat.size - ol.total_energy(s) / lat.size) <= 1e-4


def _cluster(mc, ranks=None):
    import ctypes as C
    if ranks is not None:
        mc.ctx.call("csmc_set_cluster_size", ranks)
    out = C.c_int32()
    mc.ctx.call("csmc_cluster_size", C.byref(out))
    return out.value


@pytest.mark.parametrize("ranks", [2, 4])
@pytest.mark.parametrize("name", ["square", "honeycomb", "sc", "sc24", "triangular_open", "asym_open", "selfloop",
                                  "pyrochlore"])
def test_cluster_resident_single_sweeps_match_oracle(m, orc, name, ranks):
    """The resident kernel split over a cluster of 2 or 4 CTAs (partners of
    other ranks read through distributed shared memory) == the oracle, one
    overrelaxation and one Metropolis sweep in colour order, FP64.  The
    pyrochlore with cubic and quartic terms runs the generic kernel."""
    seed = 23
    lat, ol, mc = setup(m, orc, name, "fp64", seed=seed, T=0.6)
    assert _cluster(mc, ranks) == ranks
    _, order, _ = lat.colouring()
    s = rand_spins(lat.size, 31)
    mc.set_spins(s)
    _run_once(m, mc, 1, 1, 1000, "resident")
    ol.overrelax_order(s, order)
    assert np.abs(mc.spins(0) - s).max() <= 1e-12
    acc = _run_once(m, mc, 0, 1, 0, "resident")
    acc_o, _ = ol.colour_sweep(s, 0.6, orc.UNIFORM, 60.0, order, seed, 0, 0, 53)
    assert acc[0] == acc_o
    assert np.abs(mc.spins(0) - s).max() <= 1e-12


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("name", ["sc", "honeycomb", "triangular_open", "pyrochlore"])
def test_cluster_sizes_give_the_same_chain(m, orc, name, precision):
    """One CTA per replica and clusters of 2 and 4 CTAs run the same
    arithmetic per site: a parallel-tempering window with exchanges, probes and
    adaptive sigma gives the same spins, records and counters."""
    res = []
    for ranks in (1, 2, 4):
        lat, ol, mc = setup(m, orc, name, precision, R=4, seed=9)
        assert _cluster(mc, ranks) == ranks
        mc.ctx.set_temperatures(np.array([0.2, 0.4, 0.8, 1.6]))
        for r in range(4):
            mc.set_spins(rand_spins(lat.size, 40 + r), r)
        mc.path = "resident"
        p = mc.parameters
        p.t_thermalization, p.t_measurement, p.report_interval, p.checkpoint_rate = 5, 35, 40, 10
        p.probe_rate, p.swap_rate, p.overrelaxation_rate = 5, 5, 5
        out = m.parallel_tempering(mc, alg=m.MetropolisAdaptive(), verbose=False)
        res.append((np.stack([mc.spins(r) for r in range(4)]), out["energy"], out["magnetization"],
                    mc.accepted.copy(), mc.exchanged.copy(), np.atleast_1d(mc.sigma)))
    for other in res[1:]:
        assert np.abs(res[0][0] - other[0]).max() <= 1e-12 * (1 if precision == "fp64" else 1e6)
        assert np.abs(res[0][1] - other[1]).max() <= obs_tol(precision) * lat.size
        assert np.abs(res[0][2] - other[2]).max() <= obs_tol(precision) * lat.size
        assert np.array_equal(res[0][3], other[3]) and np.array_equal(res[0][4], other[4])
        assert np.allclose(res[0][5], other[5], rtol=1e-12)
