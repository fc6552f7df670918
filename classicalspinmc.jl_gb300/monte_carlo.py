"""MonteCarlo and the sweep drivers, mirroring metropolis.jl, monte_carlo.jl,
hamiltonian.jl and observables.jl on top of the GPU library.

``MonteCarlo(T, lattice, parameters)`` creates a device context holding the
lattice's flattened tables and one replica per temperature: ``T`` may be a
single temperature (the reference's one MPI rank) or a sequence (the ranks of
a parallel-tempering ladder, batched on the one GPU).  Spins live on the
device; ``mc.lattice.spins`` follows the device after every driver call (read back on access).

The sweep plug point of the reference, ``alg(mc, T)``
(``alg::FunctionWrapper{Float64,Tuple{MonteCarlo,Float64}}``, metropolis.jl:181-199),
is kept: ``Metropolis()``, ``MetropolisAdaptive()`` and
``MetropolisFixedCone()`` return callables that run one device sweep and
return the accepted count.  The constrained variants (metropolis.jl:36-58,
:155-179) take a ``Constraint`` of closed form instead of a host closure.
Output files (``outpath``) follow hdf5.jl's layout (``hdf5.py``).
"""
from __future__ import annotations

import copy
import ctypes as C
import math
import os
import warnings
from dataclasses import dataclass

import numpy as np

from . import _lib, hdf5
from .lattice import Lattice
from .observables import Observables, mean_and_error, specific_heat, susceptibility


@dataclass
class SimulationParameters:
    """SimulationParameters (metropolis.jl:4-13)."""

    t_thermalization: int = 1
    t_deterministic: int = 1
    t_measurement: int = 1
    probe_rate: int = 1
    swap_rate: int = 1
    overrelaxation_rate: int = 10
    report_interval: int = 0
    checkpoint_rate: int = 0


_ALLOWED = ["t_thermalization", "t_deterministic", "t_measurement", "probe_rate", "swap_rate",
            "overrelaxation_rate", "report_interval", "checkpoint_rate"]


def MCParamsBuffer(d: dict) -> SimulationParameters:
    """MCParamsBuffer (monte_carlo.jl:10-27): defaults, and a warning per unknown key."""
    for key in d:
        if key not in _ALLOWED:
            warnings.warn(f"'{key}' not a valid MC parameter; ignoring")
    return SimulationParameters(**{k: int(d[k]) for k in _ALLOWED if k in d})


class _Alg:
    """A Metropolis sweep kind usable as alg(mc, T)."""

    def __init__(self, kind: int, name: str):
        self.kind = kind
        self.name = name

    def __call__(self, mc: "MonteCarlo", T=None):
        return mc._metropolis(self.kind, T)

    def __repr__(self):
        return f"{self.name}()"


def Metropolis() -> _Alg:
    """Metropolis() -> metropolis! (metropolis.jl:65-82, :181-183)."""
    return _Alg(_lib.METROPOLIS, "Metropolis")


def MetropolisAdaptive() -> _Alg:
    """MetropolisAdaptive() -> metropolis_adaptive! (metropolis.jl:113-133, :185-187)."""
    return _Alg(_lib.METROPOLIS_ADAPTIVE, "MetropolisAdaptive")


def MetropolisFixedCone() -> _Alg:
    """MetropolisFixedCone() -> metropolis_fixed_cone! (metropolis.jl:136-153, :189-191)."""
    return _Alg(_lib.METROPOLIS_FIXED_CONE, "MetropolisFixedCone")


def MetropolisConstraint() -> _Alg:
    """MetropolisConstraint() -> metropolis_constraint! (metropolis.jl:36-58, :193-195).

    The reference's body calls ``e_diff``, which the package does not define;
    here the proposal is the uniform one of metropolis! (calculate_energy_diff!
    without a cone, metropolis.jl:94-101)."""
    return _Alg(_lib.METROPOLIS_CONSTRAINT, "MetropolisConstraint")


def MetropolisConstraintAdaptive() -> _Alg:
    """MetropolisConstraintAdaptive() -> metropolis_constraint_adaptive! (metropolis.jl:155-179, :197-199)."""
    return _Alg(_lib.METROPOLIS_CONSTRAINT_ADAPTIVE, "MetropolisConstraintAdaptive")


class Constraint:
    """The ``constraint`` function of MonteCarlo (monte_carlo.jl:57) in the
    closed form the device evaluates: with V = sum_i w_i s_i over the sites
    (``site_weights`` w in site order, default 1 everywhere),

        c(lattice) = g . V + q |V|^2 + p |V| + c0.

    A linear constraint on the magnetisation along an axis, on its square or
    on its norm, on a staggered magnetisation (weights +1/-1), and sums of
    these, have this form.  Calling the object on a lattice or on a 3 x N spin
    array evaluates c on the host."""

    def __init__(self, site_weights=None, g=(0.0, 0.0, 0.0), q: float = 0.0, p: float = 0.0, c0: float = 0.0):
        self.site_weights = None if site_weights is None else np.ascontiguousarray(site_weights, np.float64)
        self.g = tuple(float(x) for x in g)
        if len(self.g) != 3:
            raise ValueError("g has 3 components")
        self.q, self.p, self.c0 = float(q), float(p), float(c0)

    def __call__(self, lattice_or_spins) -> float:
        s = getattr(lattice_or_spins, "spins", lattice_or_spins)
        s = np.asarray(s, dtype=np.float64)
        w = np.ones(s.shape[1]) if self.site_weights is None else self.site_weights
        V = (s * w).sum(axis=1)
        vv = float(V @ V)
        return float(np.dot(self.g, V)) + self.q * vv + self.p * np.sqrt(vv) + self.c0

    def desc(self, n_sites: int, weight: float) -> "_lib.ConstraintDesc":
        d = _lib.ConstraintDesc()
        if self.site_weights is not None:
            if self.site_weights.shape != (n_sites,):
                raise ValueError(f"site_weights must have one entry per site ({n_sites})")
            d.site_weights = _lib.ptr(self.site_weights, C.c_double)
        for a in range(3):
            d.g[a] = self.g[a]
        d.q, d.p, d.c0, d.weight = self.q, self.p, self.c0, float(weight)
        return d


_PRECISION = {"fp64": _lib.FP64, "fp32": _lib.FP32}
_PATHS = {"auto": _lib.PATH_AUTO, "resident": _lib.PATH_RESIDENT, "global": _lib.PATH_GLOBAL,
          "per_replica": _lib.PATH_PER_REPLICA}


class Context:
    """Owner of one libcsmc context (csmc_create / csmc_destroy)."""

    def __init__(self, lattices, replicas, precision="fp64", seed=20261203):
        lattices = list(lattices)
        self.lattices = lattices
        self.replicas = [int(r) for r in replicas]
        self.precision = precision
        self.handle = C.c_void_p()
        descs = (_lib.LatticeDesc * len(lattices))(*[l.desc.desc for l in lattices])
        reps = np.asarray(self.replicas, dtype=np.int32)
        _lib.call("csmc_create_batch", descs, len(lattices), _lib.ptr(reps, C.c_int32), _PRECISION[precision],
                  C.c_uint64(seed), C.byref(self.handle))
        n = C.c_int32()
        _lib.call("csmc_num_slots", self.handle, C.byref(n))
        self.n_slots = n.value

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value:
            try:
                _lib.lib().csmc_destroy(h)
            except Exception:
                pass
            self.handle = C.c_void_p()

    def call(self, name, *args):
        _lib.call(name, self.handle, *args)

    def slot_sizes(self):
        out = []
        for l, r in zip(self.lattices, self.replicas):
            out += [l.size] * r
        return out

    def set_spins(self, slot: int, spins: np.ndarray):
        s = np.asfortranarray(spins, dtype=np.float64)
        self.call("csmc_set_spins", int(slot), _lib.ptr(s, C.c_double))

    def get_spins(self, slot: int) -> np.ndarray:
        n = self.slot_sizes()[slot]
        s = np.zeros((3, n), np.float64, order="F")
        self.call("csmc_get_spins", int(slot), _lib.ptr(s, C.c_double))
        return s

    def set_temperatures(self, T):
        t = np.ascontiguousarray(T, dtype=np.float64)
        self.call("csmc_set_temperatures", _lib.ptr(t, C.c_double))

    def per_slot(self, name) -> np.ndarray:
        out = np.zeros(self.n_slots, np.float64)
        self.call(name, _lib.ptr(out, C.c_double))
        return out


class MonteCarlo:
    """MonteCarlo(T, lattice, parameters; ...) (monte_carlo.jl:56-118).

    Extra keywords of this implementation: ``precision`` ("fp64" or "fp32"),
    ``seed`` (Philox key), ``path`` ("auto", "resident", "global",
    "per_replica").  With ``outpath`` (a directory with its trailing
    separator, as in the reference) the params file and one configuration
    file per replica are created as monte_carlo.jl:95-116 does for its ranks
    (replica r plays rank r): ``mc.outpath`` is the file of the one replica,
    or the list of the replicas' files.
    """

    def __init__(self, T, lattice: Lattice, parameters: dict, *, constraint=None, weight: float = 0.0,
                 outpath: str = "", outprefix: str = "configuration", inparams=None, overwrite: bool = True,
                 sigma0: float = 60, corr: bool = False, ks=None, precision: str = "fp64", seed: int = 20261203,
                 path: str = "auto"):
        if corr and (ks is None or np.asarray(ks).shape[1] == 0):
            raise ValueError("No momentum vectors provided for correlation calculations!")
        if constraint is not None and not isinstance(constraint, Constraint):
            raise TypeError("constraint must be a Constraint: the device evaluates c = g.V + q|V|^2 + p|V| + c0 "
                            "of V = sum_i w_i s_i, not an arbitrary function")
        self.temperatures = np.atleast_1d(np.asarray(T, dtype=np.float64)).copy()
        self.lattice = copy.deepcopy(lattice)  # monte_carlo.jl:74
        self.parameters = MCParamsBuffer(dict(parameters))
        self.sigma0 = float(sigma0)
        self.outpath = outpath
        self.path = path
        R = len(self.temperatures)
        self.ctx = Context([self.lattice], [R], precision=precision, seed=seed)
        self.ctx.set_temperatures(self.temperatures)
        self.ctx.call("csmc_set_sigma", _lib.ptr(np.full(R, self.sigma0), C.c_double))
        self.ctx.call("csmc_set_sigma0", C.c_double(self.sigma0))
        self.constraint, self.weight = constraint, float(weight)  # monte_carlo.jl:77-78
        if constraint is not None:
            self.ctx.call("csmc_set_constraint", 0, C.byref(constraint.desc(self.lattice.size, weight)))
        for r in range(R):
            self.ctx.set_spins(r, self.lattice.spins)
        self.observables = [Observables() for _ in range(R)]
        self.corr = bool(corr)  # monte_carlo.jl:81-82
        self.momentum_vectors = None if ks is None else np.asfortranarray(ks, dtype=np.float64)
        self.accepted = np.zeros(R)
        self.exchanged = np.zeros(R)
        self.initial_configurations = {}  # parallel_tempering(saveIC=...): {rank: {timestep: spins}}
        self.outpaths = []
        if outpath:  # monte_carlo.jl:95-113
            self.outpaths = [f"{outpath}{outprefix}_{r}.h5" for r in range(R)]
            if not os.path.isdir(outpath):
                os.mkdir(outpath)
            paramsfile = f"{outpath}{outprefix}.h5.params"
            if not os.path.isfile(paramsfile) and overwrite:
                hdf5.create_params_file(self, paramsfile)
                if inparams:
                    hdf5.write_attributes(paramsfile, dict(inparams))
            for r, fn in enumerate(self.outpaths):
                if not os.path.isfile(fn) and overwrite:
                    print(f"Creating new file {os.path.basename(fn)} for output on rank {r}")
                    hdf5.initialize_hdf5(self, paramsfile, r)
            self.outpath = self.outpaths[0] if R == 1 else list(self.outpaths)

    # -- state --------------------------------------------------------------
    @property
    def T(self):
        return float(self.temperatures[0]) if len(self.temperatures) == 1 else self.temperatures

    @property
    def n_replicas(self) -> int:
        return len(self.temperatures)

    @property
    def lambda_(self):
        """mc.lambda (metropolis.jl:21) per slot: the running Lagrange
        multiplier of the constrained kinds, 0 at creation."""
        lm = self.ctx.per_slot("csmc_get_lambda")
        return float(lm[0]) if len(lm) == 1 else lm

    @lambda_.setter
    def lambda_(self, value):
        v = np.ascontiguousarray(np.broadcast_to(np.asarray(value, np.float64), (self.n_replicas,)))
        self.ctx.call("csmc_set_lambda", _lib.ptr(v, C.c_double))

    @property
    def sigma(self):
        s = self.ctx.per_slot("csmc_get_sigma")
        return float(s[0]) if len(s) == 1 else s

    def spins(self, slot: int = 0) -> np.ndarray:
        return self.ctx.get_spins(slot)

    def set_spins(self, spins: np.ndarray, slot: int = 0) -> None:
        self.ctx.set_spins(slot, spins)
        if slot == 0:
            self.lattice.spins[:] = spins

    def sync(self) -> None:
        """mc.lattice.spins follows slot 0 on the device: read back when next accessed."""
        ctx = self.ctx
        self.lattice.__dict__["_pull"] = lambda: ctx.get_spins(0)

    # -- plug point ---------------------------------------------------------
    def _metropolis(self, kind: int, T=None):
        """alg(mc, T): one sweep of every slot.  T (a number, or one per slot)
        is the temperature of this sweep, as simulated_annealing! passes the
        schedule's T (monte_carlo.jl:172-182); mc.T stays as it is."""
        acc = np.zeros(self.n_replicas)
        if T is None:
            self.ctx.call("csmc_metropolis_sweep", int(kind), _lib.ptr(acc, C.c_double))
        else:
            Ts = np.ascontiguousarray(np.atleast_1d(np.asarray(T, dtype=np.float64)))
            self.ctx.call("csmc_metropolis_sweep_at", int(kind), _lib.ptr(Ts, C.c_double), len(Ts),
                          _lib.ptr(acc, C.c_double))
        self.sync()
        return float(acc[0]) if self.n_replicas == 1 else acc


def _context_of(x):
    """A MonteCarlo's context, or a cached FP64 context for a bare Lattice with its spins uploaded."""
    if isinstance(x, MonteCarlo):
        return x.ctx, x
    lat = x
    ctx = getattr(lat, "_ctx", None)
    if ctx is None:
        ctx = Context([lat], [1], precision="fp64")
        lat._ctx = ctx
    ctx.set_spins(0, lat.spins)
    return ctx, None


def overrelaxation(x) -> None:
    """overrelaxation! (monte_carlo.jl:126-139): one sweep, colour class by colour class."""
    ctx, mc = _context_of(x)
    ctx.call("csmc_overrelax_sweep")
    if mc is None:
        x.spins[:] = ctx.get_spins(0)
    else:
        mc.sync()


def total_energy(x, slot: int = 0) -> float:
    """total_energy (hamiltonian.jl:70-132)."""
    ctx, _ = _context_of(x)
    return float(ctx.per_slot("csmc_total_energy")[slot])


def energy_density(x, slot: int = 0) -> float:
    """energy_density (hamiltonian.jl:134-136)."""
    ctx, mc = _context_of(x)
    n = (mc.lattice if mc else x).size
    return float(ctx.per_slot("csmc_total_energy")[slot]) / n


def get_magnetization(x, slot: int = 0) -> float:
    """get_magnetization (observables.jl:12-18): |sum_i s_i|."""
    ctx, _ = _context_of(x)
    return float(ctx.per_slot("csmc_magnetization")[slot])


def structure_factors(x, ks) -> np.ndarray:
    """compute_equal_time_correlations (spin_correlations.jl:6-43) of every
    slot at once: ks is dim x N_k (the reference's layout); returns an array
    [slot, 9, N_k] of Re(S_a(k) conj(S_b(k))) / N, row 3a+b."""
    ctx, mc = _context_of(x)
    return context_structure_factors(ctx, mc.lattice if mc is not None else x, ks)


def context_structure_factors(ctx: Context, lat: Lattice, ks) -> np.ndarray:
    """structure_factors of every slot of a context of one lattice."""
    ks = np.asfortranarray(np.atleast_2d(np.asarray(ks, dtype=np.float64)))
    pos = np.asfortranarray(lat.site_positions, dtype=np.float64)
    dim, n_k = ks.shape
    if pos.shape[0] != dim:
        raise ValueError(f"ks has {dim} rows, the lattice is {pos.shape[0]}-dimensional")
    R = ctx.replicas[0]
    out = np.zeros((R, n_k, 9), np.float64)
    ctx.call("csmc_structure_factor", 0, dim, _lib.ptr(pos, C.c_double), n_k, _lib.ptr(ks, C.c_double),
             _lib.ptr(out, C.c_double))
    return np.ascontiguousarray(out.transpose(0, 2, 1))


def compute_equal_time_correlations(x, ks, slot: int = 0) -> np.ndarray:
    """compute_equal_time_correlations (spin_correlations.jl:6-43) of one slot: 9 x N_k."""
    return structure_factors(x, ks)[slot]


def get_local_field(x, point: int, slot: int = 0) -> tuple:
    """get_local_field (hamiltonian.jl:3-67) at 1-based site `point`."""
    ctx, mc = _context_of(x)
    n = (mc.lattice if mc else x).size
    H = np.zeros((3, n), np.float64, order="F")
    ctx.call("csmc_local_field", int(slot), _lib.ptr(H, C.c_double))
    return tuple(float(v) for v in H[:, point - 1])


def local_fields(x, slot: int = 0) -> np.ndarray:
    """get_local_field at every site, as a 3 x N array."""
    ctx, mc = _context_of(x)
    n = (mc.lattice if mc else x).size
    H = np.zeros((3, n), np.float64, order="F")
    ctx.call("csmc_local_field", int(slot), _lib.ptr(H, C.c_double))
    return H


def annealing_temperatures(schedule, T0: float, T_target: float) -> list[float]:
    """The temperatures simulated_annealing! visits: T0, schedule(1), ... while T > target (monte_carlo.jl:159-185)."""
    temps, T, time = [], T0, 1
    while T > T_target:
        temps.append(T)
        T = schedule(time)
        time += 1
    return temps


def simulated_annealing(mc: MonteCarlo, schedule, T0: float = 1.0, alg: _Alg | None = None,
                        verbose: bool = True) -> np.ndarray:
    """simulated_annealing! (monte_carlo.jl:157-190).

    Every replica anneals through the same temperature sequence down to the
    MonteCarlo's target temperature (all replicas must share it).  Returns the
    accepted proposals per temperature and replica.
    """
    alg = Metropolis() if alg is None else alg
    if not isinstance(alg, _Alg):
        raise NotImplementedError("alg must be one of Metropolis(), MetropolisAdaptive(), MetropolisFixedCone(), "
                                  "MetropolisConstraint(), MetropolisConstraintAdaptive()")
    if len(set(mc.temperatures.tolist())) != 1:
        raise ValueError("simulated_annealing needs one target temperature for all replicas")
    temps = annealing_temperatures(schedule, T0, float(mc.temperatures[0]))
    p = mc.parameters
    R = mc.n_replicas
    acc = np.zeros((len(temps), R))
    t = np.asarray(temps, dtype=np.float64)
    # with output files, one call per temperature and the checkpoint after it
    # (monte_carlo.jl:186-188); the random streams are keyed by the sweep
    # counters the context carries, so the chains do not depend on the split
    steps = [(k, k + 1) for k in range(len(temps))] if mc.outpaths else ([(0, len(temps))] if temps else [])
    for a, b in steps:
        mc.ctx.call("csmc_anneal", _lib.ptr(t[a:], C.c_double), b - a, p.t_thermalization,
                    p.overrelaxation_rate, alg.kind, C.c_double(mc.sigma0), _PATHS[mc.path],
                    _lib.ptr(acc[a:], C.c_double))
        if mc.outpaths:
            hdf5.write_MC_checkpoint(mc)
    if verbose:
        total = p.t_thermalization * mc.lattice.size / (p.overrelaxation_rate or 1)
        for T, a in zip(temps, acc[:, 0]):
            print(f"Acceptance rate at T={T}: {round(a / total * 100, 5)} % ")
    mc.sync()
    return acc


def deterministic_updates(mc: MonteCarlo) -> None:
    """deterministic_updates! (monte_carlo.jl:201-213).

    The reference makes t_deterministic-1 single-site updates at random sites;
    here they are ceil((t_deterministic-1)/N) colour sweeps, every site once
    per sweep.
    """
    n = max(mc.parameters.t_deterministic - 1, 0)
    sweeps = -(-n // mc.lattice.size)
    mc.ctx.call("csmc_deterministic_sweeps", int(sweeps))
    mc.sync()


def parallel_tempering(mc: MonteCarlo, saveIC=(), alg: _Alg | None = None, verbose: bool = True,
                       resident_block: int = 0) -> dict:
    """parallel_tempering! (monte_carlo.jl:235-398) with the ranks as replicas on one GPU.

    Like the reference, report_interval and checkpoint_rate must be nonzero
    (``sweep % 0`` throws a DivideError at monte_carlo.jl:355 and :383).
    ``saveIC`` lists ranks (slots) whose configuration is saved at every
    checkpoint of the measurement phase (monte_carlo.jl:353-364): kept in
    ``mc.initial_configurations[rank][timestep]`` (3 x N arrays) and, with
    output files, written to ``IC_<rank>/IC_<timestep>.h5`` beside them.
    With output files every replica's file also gets the spins at those
    checkpoints (write_MC_checkpoint) and the observables at the end
    (write_final_observables, monte_carlo.jl:387-391).
    Returns the per-replica energy and |M| series and the derived observables.
    """
    alg = Metropolis() if alg is None else alg
    if not isinstance(alg, _Alg):
        raise NotImplementedError("alg must be one of Metropolis(), MetropolisAdaptive(), MetropolisFixedCone(), "
                                  "MetropolisConstraint(), MetropolisConstraintAdaptive()")
    p = mc.parameters
    if p.report_interval == 0:
        raise ZeroDivisionError("integer division error: report_interval is 0 (monte_carlo.jl:383)")
    if p.checkpoint_rate == 0 and p.t_measurement > 0:
        raise ZeroDivisionError("integer division error: checkpoint_rate is 0 (monte_carlo.jl:355)")
    R = mc.n_replicas
    if R == 1 and verbose:
        warnings.warn("MPI commSize of 1; no replica exchanges will occur!")
    total = p.t_thermalization + p.t_measurement
    Es, Ms = [], []
    start = 0

    save = sorted({int(r) for r in saveIC})
    if any(r < 0 or r >= R for r in save):
        raise ValueError(f"saveIC ranks must be in 0..{R - 1}")

    def is_corr(it):  # correlations at the probe, after the exchange (monte_carlo.jl:371-375)
        return mc.corr and p.probe_rate > 0 and it >= p.t_thermalization and it % p.probe_rate == 0

    out = bool(mc.outpaths)

    def is_ic(it):  # checkpoints of the measurement phase (monte_carlo.jl:353-364)
        return (out or bool(save)) and it >= p.t_thermalization and it % p.checkpoint_rate == 0

    if out and save:
        for r in save:
            d = os.path.join(os.path.dirname(mc.outpaths[r]), f"IC_{r}")
            if not os.path.isdir(d):
                os.mkdir(d)

    def pieces(a, b):
        """[a, b) split after every iteration whose end state is read on the host."""
        out, q = [], a
        for it in range(a, b):
            if is_corr(it) or is_ic(it):
                out.append((q, it + 1))
                q = it + 1
        if q < b:
            out.append((q, b))
        return out

    while start < total:
        n = min(p.report_interval, total - start)
        acc = np.zeros(R)
        exc = np.zeros(R)
        for a, b in pieces(start, start + n):
            k, E_, M_ = _run_piece(mc, a, b - a, alg, resident_block, acc, exc)
            Es.append(E_[:k])
            Ms.append(M_[:k])
            if is_corr(b - 1):
                ssf = structure_factors(mc, mc.momentum_vectors)
                for r in range(R):
                    mc.observables[r].push_correlations(ssf[r])
            if is_ic(b - 1):
                timestep = (b - 1 - p.t_thermalization) // p.checkpoint_rate
                spins = [mc.spins(r) for r in range(R)] if out else {r: mc.spins(r) for r in save}
                if out:
                    hdf5.write_MC_checkpoint(mc, spins)
                for r in save:
                    mc.initial_configurations.setdefault(r, {})[timestep] = spins[r]
                    if out:
                        hdf5.write_initial_configuration(
                            os.path.join(os.path.dirname(mc.outpaths[r]), f"IC_{r}", f"IC_{timestep}.h5"),
                            mc, r, spins[r])
        mc.accepted += acc
        mc.exchanged += exc
        start += n
        if verbose:
            _print_runtime_statistics(mc, start, acc, exc, n)
    E = np.concatenate(Es) if Es else np.zeros((0, R))
    M = np.concatenate(Ms) if Ms else np.zeros((0, R))
    for r in range(R):
        for e, m in zip(E[:, r], M[:, r]):
            mc.observables[r].push(e, m)
    mc.sync()
    if out:
        hdf5.write_final_observables(mc, verbose)
    return {"energy": E, "magnetization": M, "summary": summarize(mc, E, M)}


def _run_piece(mc, start, n, alg, resident_block, acc, exc):
    """csmc_run over iterations [start, start + n) with the PT schedule; the
    probe records and counters of the piece (counters added to acc, exc)."""
    p = mc.parameters
    R = mc.n_replicas
    cap = n // max(p.probe_rate, 1) + 2
    rec_E = np.zeros((cap, R))
    rec_M = np.zeros((cap, R))
    rp = _lib.RunParams()
    rp.sweep_start = start
    rp.n_sweeps = n
    rp.t_thermalization = p.t_thermalization
    rp.overrelaxation_rate = p.overrelaxation_rate
    rp.swap_rate = p.swap_rate if R > 1 else 0
    rp.probe_rate = p.probe_rate
    rp.kind = alg.kind
    rp.path = _PATHS[mc.path]
    rp.resident_block = resident_block
    rp.probe_energy = _lib.ptr(rec_E, C.c_double)
    rp.probe_magnetization = _lib.ptr(rec_M, C.c_double)
    rp.probe_capacity = cap
    rp.accepted = _lib.ptr(acc, C.c_double)
    rp.exchanged = _lib.ptr(exc, C.c_double)
    mc.ctx.call("csmc_run", C.byref(rp))
    return rp.n_probes_out, rec_E, rec_M


def autotune(mc: MonteCarlo, n_windows: int = 4, alg: _Alg | None = None) -> list[dict]:
    """Time the resident kernel's launch configurations (CTAs per replica,
    threads per CTA) on this MonteCarlo's replicas with its PT schedule, keep
    the fastest for later runs, and return the candidates.  The replicas and
    every counter are restored exactly, so the chain is unaffected.  No
    counterpart in the reference (its knobs are this library's)."""
    alg = Metropolis() if alg is None else alg
    p = mc.parameters
    rp = _lib.RunParams()
    rp.sweep_start = 0
    rp.n_sweeps = 0
    rp.t_thermalization = p.t_thermalization
    rp.overrelaxation_rate = p.overrelaxation_rate
    rp.swap_rate = p.swap_rate if mc.n_replicas > 1 else 0
    rp.probe_rate = p.probe_rate
    rp.kind = alg.kind
    rp.path = _PATHS[mc.path]
    cap = 64  # more than the candidates the library tries
    entries = (_lib.TuneEntry * cap)()
    n = C.c_int32()
    mc.ctx.call("csmc_autotune", C.byref(rp), int(n_windows), entries, cap, C.byref(n))
    paths = {_lib.PATH_RESIDENT: "resident", _lib.PATH_GLOBAL: "global"}
    return [{"path": paths.get(e.path, "resident"), "cluster": e.cluster, "block": e.block,
             "persistent": bool(e.persistent),
             "ms_per_window": e.ms_per_window, "chosen": bool(e.chosen)} for e in entries[:min(n.value, cap)]]


def _print_runtime_statistics(mc, t, acc, exc, n):
    """print_runtime_statistics! (helper.jl:25-78), one line per replica."""
    p = mc.parameters
    total = p.t_thermalization + p.t_measurement
    attempted = n * mc.lattice.size / (p.overrelaxation_rate or 1)
    lines = [f"Sweep {t} / {total} ({100.0 * t / total:.1f}%)",
             f"\t\tthermalized : {'YES' if t >= p.t_thermalization else 'NO'}"]
    sig = np.atleast_1d(mc.sigma)
    for r in range(mc.n_replicas):
        lines.append(f"\t\tsimulation {r} update acceptance rate : {acc[r] / attempted * 100:.2f}%\tsigma : "
                     f"{sig[r]:.2f}")
        if mc.n_replicas > 1 and p.swap_rate > 0:
            att = n / p.swap_rate / (2.0 if r in (0, mc.n_replicas - 1) else 1.0)
            lines.append(f"\t\tsimulation {r} replica exchange acceptance rate : {exc[r] / att * 100:.2f}%")
    print("\n".join(lines) + "\n")


def summarize(mc: MonteCarlo, E: np.ndarray, M: np.ndarray) -> list[dict]:
    """The derived observables of write_final_observables (hdf5.jl:204-239) per
    replica, with absolute errors throughout (the files hold the reference's
    relative errors for the specific heat and the susceptibility)."""
    out = []
    N = mc.lattice.size
    for r in range(mc.n_replicas):
        T = float(mc.temperatures[r])
        e, de = mean_and_error(E[:, r]) if len(E) else (float("nan"), float("nan"))
        m, dm = mean_and_error(M[:, r]) if len(M) else (float("nan"), float("nan"))
        c, dc = specific_heat(E[:, r], T, N) if len(E) else (float("nan"), float("nan"))
        x, dx = susceptibility(M[:, r], T, N) if len(M) else (float("nan"), float("nan"))
        out.append(dict(T=T, energy=e, energy_err=de, magnetization=m, magnetization_err=dm,
                        specific_heat=c, specific_heat_err=dc, susceptibility=x, susceptibility_err=dx))
    return out


def replay(mc: MonteCarlo, sites, u_phi, u_z, u_acc, alg: _Alg | None = None, T=None, slot: int = 0):
    """Replay of one reference Metropolis sweep's proposals (0-based sites and uniforms), FP64."""
    alg = Metropolis() if alg is None else alg
    n = len(sites)
    s = np.ascontiguousarray(sites, dtype=np.int64)
    up, uz, ua = (np.ascontiguousarray(a, dtype=np.float64) for a in (u_phi, u_z, u_acc))
    acc = np.zeros(n, np.uint8)
    sig = C.c_double(float(np.atleast_1d(mc.sigma)[slot]))
    T = float(mc.temperatures[slot]) if T is None else float(T)
    mc.ctx.call("csmc_replay", int(slot), alg.kind, C.c_double(T), C.byref(sig), n, _lib.ptr(s, C.c_int64),
                _lib.ptr(up, C.c_double), _lib.ptr(uz, C.c_double), _lib.ptr(ua, C.c_double),
                _lib.ptr(acc, C.c_uint8))
    return acc, sig.value
