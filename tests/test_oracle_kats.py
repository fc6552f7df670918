"""The CPU oracle against the reference's own known-answer tests
(tests/golden/reference_kats.json, generated from ClassicalSpinMC.jl's
test/latticetests.jl and test/mctests.jl), plus self-consistency checks."""
import json
import math
from pathlib import Path

import numpy as np
import pytest

KATS = {c["name"]: c for c in json.loads((Path(__file__).parent / "golden" / "reference_kats.json").read_text())["cases"]}


def test_zeeman_kat(m, orc):
    c = KATS["zeeman_energy"]
    uc = m.Square()
    m.addZeemanCoupling(uc, 1, [1.0, 0.0, 0.0])
    ol = orc.OracleLattice(uc, (1, 1), 1.0)
    s = orc.spins_array(1)
    s[:, 0] = [1.0, 0.0, 0.0]
    assert ol.total_energy(s) == c["expect"]["total_energy"]
    H = ol.local_field(s, 0)
    assert tuple(H) == tuple(KATS["zeeman_local_field"]["expect"]["local_field_site1"])


def test_bilinear_fm_kat(m, orc):
    c = KATS["bilinear_fm_energy_density"]
    uc = m.examples.square_heisenberg(J=-1.0, h=(0.0, 0.0, 0.0))
    ol = orc.OracleLattice(uc, (2, 2), 1.0)
    s = orc.spins_array(4)
    s[0, :] = 1.0
    assert ol.total_energy(s) / 4 == c["expect"]["energy_density"]


@pytest.mark.parametrize("name", ["honeycomb_kitaev_gamma_anneal", "honeycomb_kitaev_gamma_anneal_adaptive"])
def test_honeycomb_anneal_kat(m, orc, name):
    """test/mctests.jl:1-58: anneal T0=1 -> 1e-7 with x -> 0.9^x, E/N rounds to -0.6444."""
    c = KATS[name]
    md = c["model"]
    uc = m.examples.honeycomb_kitaev(K=md["K"], J=md["J"], G=md["G"], Gp=md["Gp"], h=md["h"])
    ol = orc.OracleLattice(uc, tuple(md["shape"]), md["S"])
    temps = m.annealing_temperatures(lambda x: md["T0"] * 0.9 ** x, md["T0"], md["T"])
    assert len(temps) == 153
    p = md["params"]
    kind = orc.UNIFORM if md["alg"] == "Metropolis" else orc.ADAPTIVE
    spins = ol.random_spins(seed=11)
    ol.simulated_annealing(spins, temps, p["t_thermalization"], p["overrelaxation_rate"], kind=kind, seed=5)
    if md["deterministic"]:
        ol.deterministic_ref(spins, p["t_deterministic"], seed=6)
    E = ol.total_energy(spins) / ol.N
    assert round(E, 4) == c["expect"]["energy_density_4dp"]


def test_literal_and_arithmetic_lookup_agree(m, orc):
    """findfirst over the sorted site list (lattice.jl:196,228,273) == index arithmetic."""
    E = m.examples
    cases = [(E.honeycomb_kitaev(G=0.1), (3, 2), "periodic"), (E.pyrochlore_ckq(), (2, 1, 2), "periodic"),
             (E.pyrochlore_ckq(), (2, 2, 1), "open"), (E.triangular_afm(h=1.0), (3, 4), "open")]
    for uc, shape, bc in cases:
        a = orc.OracleLattice(uc, shape, 1.0, bc=bc, literal=True).tables()
        b = orc.OracleLattice(uc, shape, 1.0, bc=bc, literal=False).tables()
        for k in a:
            assert np.array_equal(a[k], b[k]), (shape, bc, k)


def test_philox_stream_properties(orc):
    """Philox4x32-10: distinct counters give uniform, uncorrelated words."""
    words = np.array([orc.philox((i, 3, 7, 1), (0x1234, 0x5678)) for i in range(4096)], dtype=np.uint64)
    u = words.astype(np.float64) / 2 ** 32
    assert abs(u.mean() - 0.5) < 0.01
    assert abs(u.var() - 1 / 12) < 0.005
    c = np.corrcoef(u[:, 0], u[:, 1])[0, 1]
    assert abs(c) < 0.05
    assert orc.philox((0, 0, 0, 0), (0, 0)) != orc.philox((1, 0, 0, 0), (0, 0))


# Known-answer vectors of Philox4x32-10 published with the algorithm (Salmon,
# Moraes, Dror, Shaw, SC'11; the Random123 distribution's kat_vectors):
# (counter, key) -> output, four 32-bit words each.
PHILOX_KATS = [
    ((0x00000000, 0x00000000, 0x00000000, 0x00000000), (0x00000000, 0x00000000),
     (0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8)),
    ((0xffffffff, 0xffffffff, 0xffffffff, 0xffffffff), (0xffffffff, 0xffffffff),
     (0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd)),
    ((0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344), (0xa4093822, 0x299f31d0),
     (0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1)),
]


def test_philox_known_answers(orc):
    """The oracle's Philox4x32-10 (the stream the GPU replays decision for
    decision in the colour-sweep parity tests) reproduces the published
    known-answer vectors."""
    for ctr, key, out in PHILOX_KATS:
        assert orc.philox(ctr, key) == out


def test_random_spins_on_sphere(m, orc):
    ol = orc.OracleLattice(m.examples.sc_heisenberg(), (3, 3, 3), 1.5)
    s = ol.random_spins(seed=3)
    assert np.allclose(np.linalg.norm(s, axis=0), 1.5, atol=1e-12)
    assert abs(s[2].mean()) < 0.5


def test_replay_matches_direct_energy_difference(m, orc):
    """Replayed proposals reproduce energy(new) - energy(old) decisions (metropolis.jl:65-101)."""
    uc = m.examples.pyrochlore_ckq()
    ol = orc.OracleLattice(uc, (2, 2, 2), 1.0)
    s0 = ol.random_spins(seed=1)
    rng = np.random.default_rng(2)
    n = 200
    sites = rng.integers(0, ol.N, n)
    up, uz, ua = rng.random(n), rng.random(n), rng.random(n)
    s = s0.copy(order="F")
    acc, _ = ol.replay(s, 0.3, orc.UNIFORM, 60.0, sites, up, uz, ua)
    # recompute by hand
    t = s0.copy(order="F")
    for p in range(n):
        phi, z = 2 * math.pi * up[p], 2 * uz[p] - 1
        r = math.sqrt(1 - z * z)
        new = np.array([r * math.cos(phi), r * math.sin(phi), z])
        dE = ol.energy_diff(t, sites[p], new)
        a = dE < 0 or ua[p] < math.exp(-dE / 0.3)
        assert bool(acc[p]) == a
        if a:
            t[:, sites[p]] = new
    assert np.array_equal(s, t)


def test_constraint_replay_matches_the_reference_loop(m, orc):
    """The oracle's metropolis_constraint_adaptive! (metropolis.jl:155-179)
    against the reference's loop written out here: cone proposal, dE,
    c = constraint(lattice) with the new spin in place, new_lambda =
    lambda - weight c, accept dE - new_lambda c < 0 or u < exp(-(...)/T),
    lambda kept on acceptance, sigma rule at the end.  Cubic and quartic
    terms included (pyrochlore)."""
    uc = m.examples.pyrochlore_ckq()
    ol = orc.OracleLattice(uc, (2, 1, 2), 1.0)
    N = ol.N
    w = np.linspace(-1.0, 1.0, N)
    g, q, pn, c0, weight = (0.2, 0.5, -0.3), 0.02, 0.1, -0.7, 0.4
    k = orc.constraint(w, g=g, q=q, p=pn, c0=c0, weight=weight)

    def c_of(t):
        V = [0.0, 0.0, 0.0]
        for i in range(N):
            for a in range(3):
                V[a] = V[a] + w[i] * t[a, i]
        vv = V[0] * V[0] + V[1] * V[1] + V[2] * V[2]
        return g[0] * V[0] + g[1] * V[1] + g[2] * V[2] + q * vv + pn * math.sqrt(vv) + c0

    s0 = ol.random_spins(seed=3)
    rng = np.random.default_rng(4)
    n, T, sigma, sigma0, lam0 = 150, 0.5, 0.6, 9.0, 0.1
    sites = rng.integers(0, N, n)
    up, uz, ua = rng.random(n), rng.random(n), rng.random(n)
    s = s0.copy(order="F")
    acc, sig, lam = ol.constraint_replay(s, T, 1, sigma, sigma0, k, lam0, sites, up, uz, ua)
    t, lt, na = s0.copy(order="F"), lam0, 0
    for p in range(n):
        i = sites[p]
        old = t[:, i].copy()
        phi, z = 2 * math.pi * up[p], 2 * uz[p] - 1
        r = math.sqrt(1 - z * z)
        u = np.array([r * math.cos(phi), r * math.sin(phi), z])
        v = old + sigma * u
        new = v / math.sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2])
        dE = ol.energy_diff(t, i, new)
        t[:, i] = new
        c = c_of(t)
        nl = lt - weight * c
        x = dE - nl * c
        a = x < 0 or ua[p] < math.exp(-x / T)
        assert bool(acc[p]) == a, p
        if a:
            lt, na = nl, na + 1
        else:
            t[:, i] = old
    assert np.abs(s - t).max() <= 1e-14
    assert lam == pytest.approx(lt, rel=1e-12, abs=1e-14)
    rate = na / n
    assert sig == pytest.approx(sigma * 0.5 / (1 - rate) if rate < 0.5 else sigma0, rel=1e-15)
