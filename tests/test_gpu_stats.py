"""Chain-level parity through the C ABI: the random streams, the replica
exchange decision by decision, the single-precision chain of the benchmark
configuration against the double-precision chain, the statistics of the
cubic/quartic Hamiltonian against the oracle, and the plug point alg(mc, T)
at a temperature other than mc.T.

Gates:
  Philox4x32-10 on the device: the published known-answer vectors, bit for bit
  exchange: every accept/reject decision of monte_carlo.jl:308-349 given the
    recorded energies and the Philox uniform, identical
  FP32 vs FP64 chain (SC L=24, D=0.2): |<E/N>_32 - <E/N>_64| <= max(1e-4, 3 sigma)
    and the same for <|M|>/N, sigma the combined binned standard error
  cubic/quartic PT statistics: E/N, |M|/N, C_v within 3 combined sigma
  alg(mc, T): the oracle's colour sweep at that T, identical decisions, 1e-12
"""
import ctypes as C
import math
from importlib import import_module

import numpy as np
import pytest

from test_oracle_kats import PHILOX_KATS

pytestmark = pytest.mark.gpu

PURPOSE_SWAP = 3


def _lib(m):
    return import_module(m.__name__ + "._lib")


def test_philox_known_answers_on_device(m):
    """The device generator behind every draw reproduces the published vectors."""
    L = _lib(m)
    ctr = np.array([c for c, _, _ in PHILOX_KATS], np.uint32)
    key = np.array([k for _, k, _ in PHILOX_KATS], np.uint32)
    out = np.zeros((len(PHILOX_KATS), 4), np.uint32)
    L.call("csmc_debug_philox", L.ptr(ctr, C.c_uint32), L.ptr(key, C.c_uint32), len(PHILOX_KATS),
           L.ptr(out, C.c_uint32))
    assert [tuple(int(x) for x in row) for row in out] == [o for _, _, o in PHILOX_KATS]


def _u53(a, b):
    return (((a >> 5) << 26) | (b >> 6)) * (1.0 / 9007199254740992.0)


def _perm(mc):
    p = np.zeros(mc.n_replicas, np.int32)
    mc.ctx.call("csmc_get_permutation", p.ctypes.data_as(C.POINTER(C.c_int32)))
    return p


@pytest.mark.parametrize("precision,path,persistent", [("fp32", "resident", 1), ("fp32", "resident", 0),
                                                        ("fp64", "global", 0)])
def test_exchange_decisions_exact(m, orc, precision, path, persistent):
    """Each exchange decision equals the reference's rule (monte_carlo.jl:308-349):
    at sweep q (a multiple of swap_rate) the pairs (a, a+1) with
    a = (q / swap_rate) % 2 + 2m exchange when the even slot's uniform is below
    min(1, exp((1/T_odd - 1/T_even)(E_odd - E_even))).  The energies are the
    ones the device recorded at q, the uniform is word pair (x, y) of
    Philox(a, q, lattice, SWAP) under the context's seed, recomputed by the
    oracle's Philox.  One csmc_run call per exchange window, the permutation
    read before and after."""
    L = _lib(m)
    R, seed, swap_rate = 8, 0x1234_0000_0042, 2
    T = np.geomspace(0.3, 3.0, R)
    lat = m.Lattice((4, 4, 4), m.examples.sc_heisenberg(J=1.0, D=0.2), 1.0, rng=np.random.default_rng(1))
    mc = m.MonteCarlo(T, lat, {}, precision=precision, seed=seed)
    mc.ctx.call("csmc_random_spins", 3)
    mc.ctx.call("csmc_set_persistent", persistent)
    k0, k1 = seed & 0xFFFFFFFF, seed >> 32
    rec = np.zeros(R)
    n_acc = n_rej = 0
    for w in range(120):
        q = (w + 1) * swap_rate
        before = _perm(mc)  # replica of each slot
        rp = L.RunParams()
        rp.sweep_start, rp.n_sweeps = q - swap_rate + 1, swap_rate
        rp.t_thermalization, rp.overrelaxation_rate, rp.swap_rate, rp.probe_rate = 0, 1, swap_rate, swap_rate
        rp.path = {"resident": L.PATH_RESIDENT, "global": L.PATH_GLOBAL}[path]
        rp.probe_energy, rp.probe_capacity = rec.ctypes.data_as(C.POINTER(C.c_double)), 1
        mc.ctx.call("csmc_run", C.byref(rp))
        assert rp.n_probes_out == 1
        after = _perm(mc)
        E_rep = np.zeros(R)
        E_rep[after] = rec  # the probe records each slot's replica after the exchange
        expect = before.copy()
        for a in range((q // swap_rate) % 2, R - 1, 2):
            ev, od = (a, a + 1) if a % 2 == 0 else (a + 1, a)
            x = math.exp((1 / T[od] - 1 / T[ev]) * (E_rep[before[od]] - E_rep[before[ev]]))
            wx, wy, _, _ = orc.philox((a, q, 0, PURPOSE_SWAP), (k0, k1))
            if _u53(wx, wy) < min(1.0, x):
                expect[a], expect[a + 1] = expect[a + 1], expect[a]
                n_acc += 1
            else:
                n_rej += 1
        assert np.array_equal(after, expect), (w, before, after, expect)
    assert n_acc > 20 and n_rej > 20, (n_acc, n_rej)


@pytest.mark.slow
def test_fp32_chain_vs_fp64_chain_config3(m):
    """The precision pattern on the benchmark configuration (SC L=24, J=+I,
    D Sz^2 with D=0.2, geometric T ladder 0.1..2.0, exchanges every 10 sweeps,
    1 Metropolis + 5 overrelaxation sweeps): batched single-precision chains
    (resident kernel) and double-precision chains, in the same colour order,
    give the same thermal averages.  Every fourth temperature of the 64-slot
    ladder, four independent chains per precision (45000 sweeps each).  Per
    temperature |<E/N>_32 - <E/N>_64| <= max(1e-4, 3 sigma) and the same for
    <|M|>/N, where sigma combines the two precisions' errors of the mean, each
    the larger of the binned standard error and the spread of the four chains;
    the spin-length drift of the FP32 chains is reported and bounded."""
    obs = import_module(m.__name__ + ".observables")
    T = np.geomspace(0.1, 2.0, 64)[::4]
    params = dict(t_thermalization=5000, t_measurement=40000, probe_rate=10, swap_rate=10, overrelaxation_rate=5,
                  report_interval=45000, checkpoint_rate=45000)
    uc = m.examples.sc_heisenberg(J=1.0, D=0.2)
    seeds = (11, 12, 13, 14)
    stats = {}  # precision -> [temperature][quantity] -> (mean over chains, error of that mean)
    drift = {}
    for precision in ("fp32", "fp64"):
        per_chain = []
        for seed in seeds:
            lat = m.Lattice((24, 24, 24), uc, 1.0, initialCondition="none")
            mc = m.MonteCarlo(T, lat, params, precision=precision, seed=seed)
            mc.ctx.call("csmc_random_spins", seed)
            out = m.parallel_tempering(mc, verbose=False)
            d = C.c_double()
            mc.ctx.call("csmc_spin_length_drift", C.byref(d))
            drift[precision] = max(drift.get(precision, 0.0), d.value)
            per_chain.append([[obs.mean_and_error(out[q][:, r] / lat.size) for q in ("energy", "magnetization")]
                              for r in range(len(T))])
        stats[precision] = []
        for r in range(len(T)):
            row = []
            for q in range(2):
                means = np.array([per_chain[k][r][q][0] for k in range(len(seeds))])
                errs = np.array([per_chain[k][r][q][1] for k in range(len(seeds))])
                binned = math.sqrt(float((errs ** 2).sum())) / len(seeds)
                spread = float(means.std(ddof=1)) / math.sqrt(len(seeds))
                row.append((float(means.mean()), max(binned, spread)))
            stats[precision].append(row)
    worst = [0.0, 0.0]
    for r, t in enumerate(T):
        (e32, se32), (m32, sm32) = stats["fp32"][r]
        (e64, se64), (m64, sm64) = stats["fp64"][r]
        se, sm = math.hypot(se32, se64), math.hypot(sm32, sm64)
        print(f"T={t:.4f} E/N fp32 {e32:.7f} fp64 {e64:.7f} d={e32 - e64:+.2e} (sigma {se:.1e}) | "
              f"|M|/N fp32 {m32:.6f} fp64 {m64:.6f} d={m32 - m64:+.2e} (sigma {sm:.1e})")
        assert abs(e32 - e64) <= max(1e-4, 3 * se), (t, e32, e64, se)
        assert abs(m32 - m64) <= max(1e-4, 3 * sm), (t, m32, m64, sm)
        worst = [max(worst[0], abs(e32 - e64)), max(worst[1], abs(m32 - m64))]
    print(f"max |d(E/N)| {worst[0]:.2e}, max |d(|M|/N)| {worst[1]:.2e}, max ||S|-1| fp32 {drift['fp32']:.2e}, "
          f"fp64 {drift['fp64']:.2e}")
    assert drift["fp32"] <= 1e-5  # renormalised every 64 sweeps


def test_pt_statistics_cubic_quartic_vs_oracle(m, orc):
    """The pyrochlore with nearest-neighbour J1, scalar chirality on every
    face and biquadratic terms over the three pairings of each tetrahedron
    (hamiltonian.jl:36-65, 106-128), in parallel tempering on the GPU (colour
    sweeps, device exchanges) against the oracle's parallel_tempering!
    (random-site Metropolis, sequential overrelaxation): E/N, |M|/N and C_v per
    temperature within 3 combined standard errors.  The model has no onsite
    term, so overrelaxation conserves the energy and the stationary
    distribution does not depend on the update order."""
    obs = import_module(m.__name__ + ".observables")
    uc = m.examples.pyrochlore_ckq(J1=1.0, kappa=0.3, q=0.4, h=0.2)
    shape, T = (2, 2, 2), [0.1, 0.25, 0.6, 1.5]
    params = dict(t_thermalization=2000, t_measurement=20000, probe_rate=10, swap_rate=10, overrelaxation_rate=5,
                  report_interval=22000, checkpoint_rate=22000)
    ol = orc.OracleLattice(uc, shape, 1.0)
    spins = [ol.random_spins(9, r) for r in range(len(T))]
    ref = ol.parallel_tempering(spins, T, params["t_thermalization"], params["t_measurement"], 10, 10, 5,
                                n_threads=4, seed=10)
    for precision in ("fp64", "fp32"):
        lat = m.Lattice(shape, uc, 1.0, rng=np.random.default_rng(7))
        mc = m.MonteCarlo(T, lat, params, precision=precision, seed=8)
        out = m.parallel_tempering(mc, verbose=False)
        N = lat.size
        for r, t in enumerate(T):
            for gpu, cpu, f in ((out["energy"][:, r] / N, ref["energy"][:, r] / N, obs.mean_and_error),
                                (out["magnetization"][:, r] / N, ref["magnetization"][:, r] / N, obs.mean_and_error),
                                (out["energy"][:, r], ref["energy"][:, r], lambda x: obs.specific_heat(x, t, N))):
                a, da = f(gpu)
                b, db = f(cpu)
                assert abs(a - b) <= 3 * math.hypot(da, db), (precision, t, a, da, b, db)
        assert mc.exchanged.sum() > 0


def test_alg_at_other_temperature(m, orc):
    """alg(mc, T) with T != mc.T, as simulated_annealing! calls it with the
    schedule's temperature (monte_carlo.jl:172-182), on a context of three
    slots: every slot sweeps at that T (one value, or one per slot), equal to
    the oracle's colour sweep at that T, while mc.T and the slot permutation
    stay as they were."""
    import test_gpu_parity as P
    seed = 41
    lat, ol, mc = P.setup(m, orc, "honeycomb", "fp64", R=3, seed=seed, T=2.0)
    _, order, _ = lat.colouring()
    s = [P.rand_spins(lat.size, 60 + r) for r in range(3)]
    for r in range(3):
        mc.set_spins(s[r], r)
    alg = m.Metropolis()
    T_mc = np.array(mc.temperatures)
    acc = alg(mc, 0.35)  # one temperature for every slot
    for r in range(3):
        acc_o, _ = ol.colour_sweep(s[r], 0.35, orc.UNIFORM, 60.0, order, seed, r, 0, 53)
        assert acc[r] == acc_o
        assert np.abs(mc.spins(r) - s[r]).max() <= 1e-12
    Ts = np.array([0.2, 0.5, 0.9])
    acc = alg(mc, Ts)  # one temperature per slot
    for r in range(3):
        acc_o, _ = ol.colour_sweep(s[r], Ts[r], orc.UNIFORM, 60.0, order, seed, r, 1, 53)
        assert acc[r] == acc_o
        assert np.abs(mc.spins(r) - s[r]).max() <= 1e-12
    assert np.array_equal(np.array(mc.temperatures), T_mc)
    assert np.array_equal(_perm(mc), np.arange(3))
    # the slots' own temperatures are still in force for a sweep without T
    acc = alg(mc)
    for r in range(3):
        acc_o, _ = ol.colour_sweep(s[r], 2.0, orc.UNIFORM, 60.0, order, seed, r, 2, 53)
        assert acc[r] == acc_o
    assert np.abs(mc.lattice.spins - s[0]).max() <= 1e-12  # lattice.spins follows slot 0
