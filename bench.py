#!/usr/bin/env python3
"""Benchmark: site updates/s of the batched parallel-tempering sweep.

Workload (the single-GPU headline configuration): simple-cubic Heisenberg
model, L=24 (13824 sites), J=+I on the 6 nearest neighbours, onsite D*Sz^2
with D=0.2, S=1; 64 replicas on a geometric temperature ladder 0.1..2.0;
overrelaxation_rate=5 (1 Metropolis + 5 overrelaxation sweeps), exchanges
every 10 sweeps, probes every 10 sweeps.  Spins, fields and dE in FP32;
energies, the exchange exponent and observables in FP64.  Synthetic: random
initial spins from the Philox INIT stream.

One step = 100 iterations of the reference's loop (monte_carlo.jl:295-388):
10 exchange windows, each 10 overrelaxation + 2 Metropolis sweeps of all 64
replicas, the energies, one replica exchange and one probe (E, |M|) -- one
csmc_run call, as a caller running report_interval >= 100 makes.
Site updates per step = 64 * 13824 * 120.

`value` is device throughput (CUDA events on the library's stream) with the
replicas resident in HBM; L2 is flushed (256 MB write) between steps.
`e2e` goes through the public C ABI with host buffers every step:
csmc_set_spins_all (FP64 reference layout, all replicas) -> csmc_run ->
csmc_get_spins_all + probe records.

--impl reference times the CPU restatement of the reference's algorithm
(the oracle: random-site Metropolis, sequential overrelaxation, total energy
after every Metropolis sweep, in-process replica exchange) on all host cores,
one replica per thread, on a bounded sample of the same workload.
Multi-GPU (torchrun): independent replica sets per GPU, no collective on the
data path ("scaling": "weak").
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))
import __graft_entry__ as G  # noqa: E402

L_SIDE, R_REPL, OR_RATE, SWAP_RATE, PROBE_RATE = 24, 64, 5, 10, 10
ITER_PER_STEP = 100
SEED = 20261203
BYTES_PER_UPDATE_FP32 = 12 * (2 + 6)  # s_b * (2 + z): own spin read+write, 6 neighbours read
RESIDENT_BLOCK = 0
RUN_PATH = 0  # CSMC_PATH_AUTO; --path selects another execution path


def workload_config(extra=None):
    cfg = {"workload": "sc_heisenberg_onsite_pt", "lattice": "simple cubic L=24 (13824 sites)", "replicas": R_REPL,
           "T_ladder": "geometric 0.1..2.0", "overrelaxation_rate": OR_RATE, "swap_rate": SWAP_RATE,
           "probe_rate": PROBE_RATE, "iterations_per_step": ITER_PER_STEP,
           "site_updates_per_step": R_REPL * L_SIDE ** 3 * (ITER_PER_STEP + ITER_PER_STEP // OR_RATE),
           "l2": "flushed between steps (256 MB write)", "parallelism": "replicas"}
    if extra:
        cfg.update(extra)
    return cfg


def temperatures():
    return np.exp(np.linspace(math.log(0.1), math.log(2.0), R_REPL))


def make_lattice(m):
    return m.Lattice((L_SIDE,) * 3, m.examples.sc_heisenberg(J=1.0, D=0.2), 1.0, initialCondition="none")


class Clocks:
    """nvidia-smi sampling of SM clock and throttle reasons during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.rows, self.proc, self.index = [], None, index

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in self.rows for k in range(4) if len(r) > 3 + k and r[3 + k] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def job_throughput(t_rank_s, updates_per_rank, world, dist, device):
    """Whole-job site updates/s of N independent replica sets (one per rank):
    every rank did `updates_per_rank` in `t_rank_s` seconds; the job took the
    slowest rank's time.  Returns (updates/s, that time)."""
    t = t_rank_s
    if dist:
        import torch
        tt = torch.tensor([t], dtype=torch.float64, device=device)
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        t = float(tt.item())
    return world * updates_per_rank / t, t


def run_params(L, start, n, rec_E=None, rec_M=None, cap=0, path=None):
    path = RUN_PATH if path is None else path
    rp = L.RunParams()
    rp.sweep_start = start
    rp.n_sweeps = n
    rp.t_thermalization = 0
    rp.overrelaxation_rate = OR_RATE
    rp.swap_rate = SWAP_RATE
    rp.probe_rate = PROBE_RATE
    rp.kind = L.METROPOLIS
    rp.path = path
    rp.resident_block = RESIDENT_BLOCK
    if rec_E is not None:
        rp.probe_energy = rec_E.ctypes.data_as(C.POINTER(C.c_double))
        rp.probe_magnetization = rec_M.ctypes.data_as(C.POINTER(C.c_double))
        rp.probe_capacity = cap
    return rp


def stats(ctx):
    ms, n, kms, kn = C.c_double(), C.c_int64(), C.c_double(), C.c_int64()
    ctx.call("csmc_last_run_stats", C.byref(ms), C.byref(n), C.byref(kms), C.byref(kn))
    return ms.value, n.value, kms.value, kn.value


def bench_ours(args, rank, world, dist):
    import torch
    m = G.load()
    from importlib import import_module
    L = import_module(m.__name__ + "._lib")
    dev = rank % max(torch.cuda.device_count(), 1)
    torch.cuda.set_device(dev)
    lat = make_lattice(m)
    ctx = m.monte_carlo.Context([lat], [R_REPL], precision="fp32", seed=SEED + rank)
    ctx.set_temperatures(temperatures())
    ctx.call("csmc_random_spins", C.c_uint64(SEED + 1000 * rank))
    tuned = []
    if args.no_persistent:
        ctx.call("csmc_set_persistent", 0)
    if args.cluster:
        ctx.call("csmc_set_cluster_size", args.cluster)
    elif not args.no_autotune and not args.block:
        # the library's autotuner picks CTAs per replica and threads per CTA on
        # these replicas (state restored exactly afterwards)
        entries = (L.TuneEntry * 64)()
        n = C.c_int32()
        ctx.call("csmc_autotune", C.byref(run_params(L, 1, 0)), 8, entries, 64, C.byref(n))
        tuned = [{"path": "global" if e.path == L.PATH_GLOBAL else "resident", "cluster": e.cluster,
                  "block": e.block, "persistent": bool(e.persistent),
                  "ms_per_window": round(e.ms_per_window, 5), "chosen": bool(e.chosen)} for e in entries[:n.value]]
    ranks = C.c_int32()
    ctx.call("csmc_cluster_size", C.byref(ranks))
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    upd = R_REPL * lat.size * (ITER_PER_STEP + ITER_PER_STEP // OR_RATE)
    it = 1  # steps cover iterations [10k+1, 10k+10]: one exchange window each
    for _ in range(args.warmup):
        ctx.call("csmc_run", C.byref(run_params(L, it, ITER_PER_STEP)))
        it += ITER_PER_STEP

    def barrier():
        if dist:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    dev_ms = kern_ms = 0.0
    launches = kern_launches = 0
    barrier()
    with Clocks(dev) as clk:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            ctx.call("csmc_run", C.byref(run_params(L, it, ITER_PER_STEP)))
            it += ITER_PER_STEP
            a, b, c, d = stats(ctx)
            dev_ms += a
            launches += b
            kern_ms += c
            kern_launches += d
        barrier()
        wall = time.perf_counter() - t0
    value, t_dev = job_throughput(dev_ms / 1e3, upd * args.steps, world, dist, "cuda")
    out = {"value": value, "ms_per_step": 1e3 * t_dev / args.steps, "wall_ms_per_step": 1e3 * wall / args.steps,
           "gpu_launches": launches, "clocks": clk.summary(), "ctas_per_replica": ranks.value, "autotune": tuned}
    # roofline of the dominant kernel, per exchange window (the unit a
    # per-window launch processes; a persistent launch runs 10 windows)
    windows = args.steps * ITER_PER_STEP // SWAP_RATE
    kernel = "k_resident<float>"
    if kern_launches == 0:  # global path: every launch of a step (colour sweeps, energies, exchange)
        kern_ms, kernel = dev_ms, "global colour sweeps (whole step)"
    per_window_s = kern_ms / 1e3 / windows
    bytes_per_window = upd * BYTES_PER_UPDATE_FP32 * args.steps / windows
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    achieved = bytes_per_window / per_window_s / 1e9
    resident = kernel.startswith("k_res")
    traffic = None
    tf = ROOT / "profiles" / "traffic.json"
    if tf.exists() and resident:
        traffic = json.loads(tf.read_text()).get("k_resident_fp32_sc_L24_R64_per_window")
    sm_mhz = clk.summary().get("sm_mhz") or peaks.get("sm_max_mhz", 2070.0)
    if resident:
        # the replicas stay in shared memory: the level that binds is the SMs'
        # shared memory, nominally 128 B per clock per SM at the sampled clock
        peak = 152 * 128 * sm_mhz * 1e6 / 1e9
        out["roofline"] = {"bound": "smem", "achieved": achieved, "peak": peak, "unit": "GB/s",
                           "frac": achieved / peak, "traffic": traffic, "kernel": kernel, "per": "exchange window",
                           "algorithmic_bytes": bytes_per_window, "kernel_ms": per_window_s * 1e3,
                           "peak_source": f"nominal 152 SMs x 128 B/clk x {sm_mhz:.0f} MHz (sampled)",
                           "hbm_equivalent": {"peak": hbm_peak, "frac": achieved / hbm_peak}}
    else:
        out["roofline"] = {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                           "frac": achieved / hbm_peak, "traffic": None, "kernel": kernel, "per": "exchange window",
                           "algorithmic_bytes": bytes_per_window, "kernel_ms": per_window_s * 1e3,
                           "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)" if peaks else "fallback"}

    # end to end through the C ABI with host buffers
    nh = R_REPL * lat.size * 3
    h_in = torch.empty(nh, dtype=torch.float64).pin_memory().numpy()
    h_out = torch.empty(nh, dtype=torch.float64).pin_memory().numpy()
    ctx.call("csmc_get_spins_all", h_in.ctypes.data_as(C.POINTER(C.c_double)))
    cap = ITER_PER_STEP // PROBE_RATE + 2
    rec_E = np.zeros((cap, R_REPL))
    rec_M = np.zeros((cap, R_REPL))
    e2e_steps = max(3, min(args.steps, args.e2e_steps))
    rp = run_params(L, it, ITER_PER_STEP, rec_E, rec_M, cap)  # one parameter block, advanced per step
    p_in, p_out = h_in.ctypes.data_as(C.POINTER(C.c_double)), h_out.ctypes.data_as(C.POINTER(C.c_double))
    for k in range(e2e_steps + 2):
        if k == 2:
            barrier()
            t0 = time.perf_counter()
        ctx.call("csmc_set_spins_all", p_in)
        rp.sweep_start = it
        ctx.call("csmc_run", C.byref(rp))
        it += ITER_PER_STEP
        ctx.call("csmc_get_spins_all", p_out)
        p_in, p_out = p_out, p_in
    barrier()
    t_e2e = time.perf_counter() - t0
    out["e2e"] = {"value": world * upd * e2e_steps / t_e2e, "unit": "site updates/s",
                  "h2d_bytes_per_step": nh * 8, "d2h_bytes_per_step": nh * 8 + 2 * cap * R_REPL * 8,
                  "ms_per_step": 1e3 * t_e2e / e2e_steps,
                  "api": "csmc_set_spins_all + csmc_run + csmc_get_spins_all"}

    # the plain FP64 one-replica-per-launch path on the same workload (the metric compares against it)
    if rank == 0 and args.plain_steps > 0:
        ctx64 = m.monte_carlo.Context([lat], [R_REPL], precision="fp64", seed=SEED)
        ctx64.set_temperatures(temperatures())
        ctx64.call("csmc_random_spins", C.c_uint64(SEED))
        ctx64.call("csmc_run", C.byref(run_params(L, 1, ITER_PER_STEP, path=L.PATH_PER_REPLICA)))
        t = 0.0
        for k in range(args.plain_steps):
            ctx64.call("csmc_run", C.byref(run_params(L, 1 + ITER_PER_STEP * (k + 1), ITER_PER_STEP,
                                                      path=L.PATH_PER_REPLICA)))
            t += stats(ctx64)[0] / 1e3
        out["plain_fp64_per_replica"] = {"value": upd * args.plain_steps / t, "unit": "site updates/s",
                                         "ms_per_step": 1e3 * t / args.plain_steps,
                                         "batched_fp32_speedup": value / world / (upd * args.plain_steps / t)}
    return out


def _tuned_summary(tuned):
    """The autotuner's candidates go to stderr; the JSON line keeps their count and the one chosen."""
    if tuned:
        print("autotune candidates: " + json.dumps(tuned), file=sys.stderr)
    chosen = [t for t in tuned if t["chosen"]]
    return {"candidates": len(tuned), "chosen": chosen[0] if chosen else None}


def oracle_sample(target_s: float, threads: int):
    """The oracle's parallel tempering on the same workload; returns updates/s and the sample."""
    m = G.load()
    orc = G.load_oracle()
    uc = m.examples.sc_heisenberg(J=1.0, D=0.2)
    ol = orc.OracleLattice(uc, (L_SIDE,) * 3, 1.0)
    spins = [ol.random_spins(SEED, r) for r in range(R_REPL)]
    T = temperatures()

    def run(n_iter):
        t0 = time.perf_counter()
        ol.parallel_tempering(spins, T, 0, n_iter, PROBE_RATE, SWAP_RATE, OR_RATE, n_threads=threads, seed=SEED)
        return time.perf_counter() - t0

    t1 = run(ITER_PER_STEP)
    n = max(ITER_PER_STEP, int(round(target_s / max(t1, 1e-6) * ITER_PER_STEP / 10.0)) * 10)
    t = run(n)
    upd = R_REPL * ol.N * (n + n // OR_RATE)
    return upd / t, {"iterations": n, "seconds": t,
                     "sample": f"{n} iterations (= {n // ITER_PER_STEP} steps) of the 64-replica L=24 workload"}


# ------------------------------------------------------------------ other configurations
# The remaining configurations of the path, each measured the same way
# (device time of csmc_run / csmc_anneal through the C ABI, L2 flushed between
# steps) beside the oracle on the host cores.  The driver's default line is the
# 64-replica simple-cubic workload above; these are selected with --workload.

def _triangular_batch(m, n=256, seed=4):
    """256 independent triangular antiferromagnets: (L, T, h) per chain from a seeded generator."""
    rng = np.random.default_rng(seed)
    Ls = rng.choice([12, 18, 24, 36, 48, 72], size=n)
    Ts = np.exp(rng.uniform(math.log(0.05), math.log(1.0), size=n))
    hs = rng.uniform(0.0, 3.0, size=n)
    lats = [m.Lattice((int(L), int(L)), m.examples.triangular_afm(h=float(h)), 1.0, initialCondition="none")
            for L, h in zip(Ls, hs)]
    return lats, Ts, hs


def other_workload(name, m):
    """(lattices, replicas per lattice, temperatures per slot, precision, run kwargs, description)."""
    E = m.examples
    if name == "square_fp64":
        lat = m.Lattice((32, 32), E.square_heisenberg(), 1.0, initialCondition="none")
        return ([lat], [1], np.array([0.5]), "fp64", dict(or_rate=10, swap_rate=0, probe_rate=10, iters=100),
                "square Heisenberg L=32 (1024 sites), h=(0,0,0.1), T=0.5, FP64, 100 iterations per step")
    if name == "honeycomb_fp32":
        lat = m.Lattice((48, 48), E.honeycomb_kitaev(K=-1.0, J=0.1, G=0.05), 1.0, initialCondition="none")
        return ([lat], [1], np.array([1.0]), "fp32", dict(or_rate=10, swap_rate=0, probe_rate=0, iters=1000),
                "honeycomb K-J-Gamma L=48 (4608 sites), one annealing temperature of 1000 iterations per step, FP32")
    if name == "triangular_batch_fp32":
        lats, Ts, _ = _triangular_batch(m)
        return (lats, [1] * len(lats), Ts, "fp32", dict(or_rate=5, swap_rate=0, probe_rate=10, iters=10),
                f"256 triangular AFM chains, L in {{12..72}} ({sum(l.size for l in lats)} sites), FP32")
    if name in ("pyrochlore_fp32", "pyrochlore_large_fp32"):
        shape = (16, 16, 16) if name == "pyrochlore_fp32" else (32, 32, 16)
        lat = m.Lattice(shape, E.pyrochlore_ckq(), 1.0, initialCondition="none")
        Ts = np.exp(np.linspace(math.log(0.05), math.log(1.5), 32))
        return ([lat], [32], Ts, "fp32", dict(or_rate=5, swap_rate=10, probe_rate=10, iters=10),
                f"pyrochlore J1 + cubic + quartic, shape {shape} ({lat.size} sites), 32 PT replicas, FP32")
    if name == "sc_constraint_fp32":  # MetropolisConstraintAdaptive: sequential proposals per replica
        lat = m.Lattice((24, 24, 24), E.sc_heisenberg(J=1.0, D=0.2), 1.0, initialCondition="none")
        Ts = np.exp(np.linspace(math.log(0.1), math.log(2.0), 64))
        return ([lat], [64], Ts, "fp32", dict(or_rate=5, swap_rate=10, probe_rate=10, iters=10, kind=4),
                "simple cubic L=24 (13824 sites), 64 PT replicas, MetropolisConstraintAdaptive with "
                "c = M_z / N - 0.1 (weight 0.01), FP32, global path")
    if name == "sc_large_fp32":  # replicas beyond shared memory and beyond L2: the global sweeps from HBM
        lat = m.Lattice((64, 64, 64), E.sc_heisenberg(J=1.0, D=0.2), 1.0, initialCondition="none")
        Ts = np.exp(np.linspace(math.log(0.1), math.log(2.0), 64))
        return ([lat], [64], Ts, "fp32", dict(or_rate=5, swap_rate=10, probe_rate=10, iters=10),
                "simple cubic L=64 (262144 sites), 64 PT replicas (268 MB of spins), FP32, global colour sweeps")
    raise SystemExit(f"unknown workload {name}")


def bench_other(args):
    import torch
    m = G.load()
    from importlib import import_module
    L = import_module(m.__name__ + "._lib")
    torch.cuda.set_device(0)
    lats, reps, Ts, prec, kw, desc = other_workload(args.workload, m)
    ctx = m.monte_carlo.Context(lats, reps, precision=prec, seed=SEED)
    ctx.set_temperatures(Ts)
    ctx.call("csmc_random_spins", C.c_uint64(SEED))
    if args.no_persistent:
        ctx.call("csmc_set_persistent", 0)
    kind = kw.get("kind", L.METROPOLIS)
    if kind >= L.METROPOLIS_CONSTRAINT:
        k = L.ConstraintDesc()
        k.g[2] = 1.0 / lats[0].size
        k.c0, k.weight = -0.1, 0.01
        ctx.call("csmc_set_constraint", 0, C.byref(k))
    sites = sum(l.size * r for l, r in zip(lats, reps))
    iters = kw["iters"]
    anneal = args.workload == "honeycomb_fp32"
    if anneal:
        upd = sites * ((iters - 1) + (iters - 1) // kw["or_rate"])
    else:
        upd = sites * (iters + iters // kw["or_rate"])
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    it = [1]
    tuned = []
    if not args.no_autotune:  # resident configuration or global sweeps, timed on these replicas
        rp = L.RunParams()
        rp.sweep_start, rp.n_sweeps, rp.t_thermalization = 1, 0, 0
        rp.overrelaxation_rate, rp.swap_rate, rp.probe_rate = kw["or_rate"], kw["swap_rate"], kw["probe_rate"]
        rp.kind, rp.path = kind, RUN_PATH
        entries = (L.TuneEntry * 64)()
        n = C.c_int32()
        ctx.call("csmc_autotune", C.byref(rp), 4, entries, 64, C.byref(n))
        tuned = [{"path": "global" if e.path == L.PATH_GLOBAL else "resident", "cluster": e.cluster,
                  "block": e.block, "persistent": bool(e.persistent), "ms_per_window": round(e.ms_per_window, 5),
                  "chosen": bool(e.chosen)} for e in entries[:n.value]]

    def step():
        if anneal:
            temps = np.array([1.0])
            ctx.call("csmc_anneal", temps.ctypes.data_as(C.POINTER(C.c_double)), 1, C.c_int64(iters),
                     kw["or_rate"], L.METROPOLIS, C.c_double(60.0), RUN_PATH, None)
        else:
            rp = L.RunParams()
            rp.sweep_start, rp.n_sweeps, rp.t_thermalization = it[0], iters, 0
            rp.overrelaxation_rate, rp.swap_rate, rp.probe_rate = kw["or_rate"], kw["swap_rate"], kw["probe_rate"]
            rp.kind, rp.path = kind, RUN_PATH
            ctx.call("csmc_run", C.byref(rp))
            it[0] += iters
        return stats(ctx)

    for _ in range(args.warmup):
        step()
    t_dev = 0.0
    launches = 0
    torch.cuda.synchronize()
    with Clocks(0) as clk:
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            ms, n, _, _ = step()
            t_dev += ms / 1e3
            launches += n
    value = upd * args.steps / t_dev
    cl = C.c_int32()
    ctx.call("csmc_cluster_size", C.byref(cl))
    # algorithmic bytes s_b (2 + z) per update against the measured HBM copy
    # bandwidth; with the working set inside L2 the figure is the rate a
    # streaming kernel would need, not DRAM traffic
    z = max(l.info.width_bilinear for l in lats)
    s_b = 12 if prec == "fp32" else 24
    ws = sum(l.info.padded_sites * r for l, r in zip(lats, reps)) * (16 if prec == "fp32" else 24)
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    peak = peaks.get("hbm_gbs", 6800.0)
    ach = upd * args.steps * s_b * (2 + z) / t_dev / 1e9
    roof = {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak, "traffic": None,
            "kernel": "whole step (every launch)", "bytes_per_update": s_b * (2 + z),
            "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)" if peaks else "fallback",
            "working_set_bytes": ws, "working_set_in_l2": ws < 126 * 2**20}
    line = {"metric": "site updates/s (Metropolis+OR)", "value": value, "unit": "site updates/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t_dev / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if prec == "fp64" else "f32", "data": "synthetic",
            "config": {"workload": args.workload, "description": desc, "site_updates_per_step": upd,
                       "ctas_per_replica": cl.value, "l2": "flushed between steps (256 MB write)",
                       "autotune": _tuned_summary(tuned)},
            "roofline": roof, "clocks": clk.summary(), "gpu_launches": launches}
    print(json.dumps(line))


def bench_structure_factor(args):
    """compute_equal_time_correlations of all 64 replicas of the simple-cubic
    L=24 workload at every allowed wavevector 2 pi n / L (13824 k-points),
    FP32: site-phase products (k-points x sites x replicas) per second of
    device time.  `--cuda-cores` times the CUDA-core kernel instead of the
    tensor-core one (csmc_set_tensor_cores)."""
    import torch
    m = G.load()
    torch.cuda.set_device(0)
    lat = make_lattice(m)
    mc = m.MonteCarlo(list(temperatures()), lat, {}, precision="fp32", seed=SEED)
    mc.ctx.call("csmc_random_spins", C.c_uint64(SEED))
    if args.cuda_cores:
        mc.ctx.call("csmc_set_tensor_cores", 0)
    n = np.stack(np.unravel_index(np.arange(L_SIDE ** 3), (L_SIDE,) * 3), axis=0)
    ks = np.asfortranarray(2 * np.pi * n / L_SIDE, dtype=np.float64)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    for _ in range(args.warmup):
        m.structure_factors(mc, ks)
    t = 0.0
    with Clocks(0) as clk:
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            m.structure_factors(mc, ks)
            t += stats(mc.ctx)[0] / 1e3
    n_k, N = ks.shape[1], lat.size
    products = n_k * N * R_REPL
    line = {"metric": "structure factor: k-point x site x replica products per second", "value": products * args.steps / t,
            "unit": "products/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * t / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic",
            "config": {"workload": "structure_factor", "lattice": "simple cubic L=24 (13824 sites)",
                       "replicas": R_REPL, "k_points": int(n_k),
                       "kernel": "CUDA cores (6 FP32 FMA per product)" if args.cuda_cores else
                                 "tensor cores (tcgen05 TF32, operands split hi+lo, 3 products)",
                       "l2": "flushed between steps (256 MB write)"},
            "clocks": clk.summary(), "gpu_launches": args.steps * (1 if args.cuda_cores else 2)}
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    if args.cuda_cores:
        flop = 12.0 * products  # 6 FMA per product
        peak = 152 * 128 * 2 * (clk.summary().get("sm_mhz") or 2070.0) * 1e6 / 1e12  # FP32 FMA, sampled clock
        line["roofline"] = {"bound": "fp32", "achieved": flop * args.steps / t / 1e12, "peak": peak,
                            "unit": "TFLOP/s", "frac": flop * args.steps / t / 1e12 / peak, "traffic": None,
                            "peak_source": "nominal 152 SMs x 128 FP32 FMA/clk at the sampled clock"}
    else:
        # the MMAs' work: cos and sin, three split products, 2 FLOP per MAC, over
        # the padded sites (multiple of 16) and 192 spin columns per 64 replicas
        n_pad = -(-N // 16) * 16
        flop = 3 * 2 * 2.0 * n_k * n_pad * 3 * (-(-R_REPL // 64) * 64)
        peak = peaks.get("bf16_tflops", 1900.0) / 2  # TF32 runs at half the bf16 rate
        line["roofline"] = {"bound": "tensor", "achieved": flop * args.steps / t / 1e12, "peak": peak,
                            "unit": "TFLOP/s", "frac": flop * args.steps / t / 1e12 / peak, "traffic": None,
                            "peak_source": "TF32 = half of MEASURED_PEAKS.json bf16_tflops (measured cuBLAS bf16)",
                            "note": "time includes the spin-packing launch; 108 tiles of 128 wavevectors x "
                                    "64 replicas, sites split 7 ways (756 CTAs on 152 SMs), the last CTA of a "
                                    "tile adding its partial sums"}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--e2e-steps", type=int, default=50)
    ap.add_argument("--plain-steps", type=int, default=3)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--block", type=int, default=0, help="threads per CTA of the resident kernel (0: library default)")
    ap.add_argument("--cluster", type=int, default=0, help="CTAs per replica (0: autotuned; 1, 2 or 4)")
    ap.add_argument("--no-autotune", action="store_true", help="skip csmc_autotune (library heuristics)")
    ap.add_argument("--path", default="auto", choices=["auto", "resident", "global"],
                    help="execution path of csmc_run (auto: the autotuner's choice)")
    ap.add_argument("--cuda-cores", action="store_true",
                    help="structure_factor workload: the CUDA-core kernel instead of the tensor cores")
    ap.add_argument("--no-persistent", action="store_true",
                    help="one launch per exchange window (csmc_set_persistent 0), e.g. under a profiler")
    ap.add_argument("--workload", default="sc_pt",
                    choices=["sc_pt", "square_fp64", "honeycomb_fp32", "triangular_batch_fp32", "pyrochlore_fp32",
                             "pyrochlore_large_fp32", "sc_large_fp32", "sc_constraint_fp32", "structure_factor"],
                    help="sc_pt (default): the 64-replica simple-cubic line; the others measure the remaining "
                         "configurations (device throughput only)")
    args = ap.parse_args()
    global RESIDENT_BLOCK, RUN_PATH
    RESIDENT_BLOCK = args.block
    RUN_PATH = {"auto": 0, "resident": 1, "global": 2}[args.path]
    if args.workload == "structure_factor":
        bench_structure_factor(args)
        return
    if args.workload != "sc_pt":
        bench_other(args)
        return
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", str(args.gpus)))
    threads = os.cpu_count() or 1
    metric = "site updates/s (Metropolis+OR), batched FP32 vs plain FP64 GPU, |dE/N|<=1e-4"
    unit = "site updates/s"

    if args.impl == "reference":
        if rank != 0:
            return
        v, sample = oracle_sample(args.cpu_seconds, threads)
        line = {"metric": metric, "value": v, "unit": unit, "impl": "reference", "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": workload_config({"parallelism": "threads (one replica per thread)"}),
                "cpu_baseline": {"value": v, "unit": unit, "cores": threads, "kind": "port",
                                 "sample": sample["sample"]},
                "e2e": {"value": v, "unit": unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    dist = world > 1
    if dist:
        import torch
        torch.distributed.init_process_group("nccl")
    res = bench_ours(args, rank, world, dist)
    if rank != 0:
        return
    cpu = None
    if world == 1:
        v, sample = oracle_sample(args.cpu_seconds, threads)
        cpu = {"value": v, "unit": unit, "cores": threads, "kind": "port", "sample": sample["sample"]}
    line = {"metric": metric, "value": res["value"], "unit": unit, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": res["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": workload_config({"precision": "FP32 spins/fields/dE, FP64 energies+exchange+observables",
                                       "wall_ms_per_step": res["wall_ms_per_step"],
                                       "ctas_per_replica": res["ctas_per_replica"],
                                       "autotune": _tuned_summary(res["autotune"])}),
            "roofline": res["roofline"], "cpu_baseline": cpu, "e2e": res["e2e"], "clocks": res["clocks"],
            "gpu_launches": res["gpu_launches"]}
    if "plain_fp64_per_replica" in res:
        line["plain_fp64_per_replica"] = res["plain_fp64_per_replica"]
    print(json.dumps(line))


if __name__ == "__main__":
    main()
