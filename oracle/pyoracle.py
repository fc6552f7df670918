"""ctypes wrapper of the CPU oracle (oracle/csmc_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, never by the product package.  Builds the
oracle with ``make -C oracle`` on first use.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "libcsmc_oracle.so"

i32p = C.POINTER(C.c_int32)
i64p = C.POINTER(C.c_int64)
f64p = C.POINTER(C.c_double)
u8p = C.POINTER(C.c_uint8)
UNIFORM, ADAPTIVE, FIXED_CONE = 0, 1, 2


class Desc(C.Structure):
    _fields_ = [
        ("dim", C.c_int32), ("n_basis", C.c_int32), ("shape", C.c_int32 * 3), ("periodic", C.c_int32),
        ("spin_length", C.c_double),
        ("n_field", C.c_int32), ("field_basis", i32p), ("field_vec", f64p),
        ("n_onsite", C.c_int32), ("onsite_basis", i32p), ("onsite_mat", f64p),
        ("n_bilinear", C.c_int32), ("bilinear_basis", i32p), ("bilinear_mat", f64p), ("bilinear_offset", i32p),
        ("n_cubic", C.c_int32), ("cubic_basis", i32p), ("cubic_tensor", f64p), ("cubic_offset", i32p),
        ("n_quartic", C.c_int32), ("quartic_basis", i32p), ("quartic_tensor", f64p), ("quartic_offset", i32p),
    ]


class PTParams(C.Structure):
    _fields_ = [("t_thermalization", C.c_int64), ("t_measurement", C.c_int64), ("probe_rate", C.c_int32),
                ("swap_rate", C.c_int32), ("overrelaxation_rate", C.c_int32), ("kind", C.c_int32),
                ("sigma0", C.c_double), ("n_threads", C.c_int32), ("seed", C.c_uint64)]


class Constraint(C.Structure):
    """orc_constraint: c = g.V + q |V|^2 + p |V| + c0 with V = sum_i w_i s_i."""
    _fields_ = [("w", f64p), ("g", C.c_double * 3), ("q", C.c_double), ("p", C.c_double), ("c0", C.c_double),
                ("weight", C.c_double)]


def constraint(weights=None, g=(0.0, 0.0, 0.0), q=0.0, p=0.0, c0=0.0, weight=0.0):
    """An orc_constraint (the weights array is kept alive on the structure)."""
    k = Constraint()
    if weights is not None:
        w = np.ascontiguousarray(weights, np.float64)
        k._keep = w
        k.w = w.ctypes.data_as(f64p)
    for a in range(3):
        k.g[a] = float(g[a])
    k.q, k.p, k.c0, k.weight = float(q), float(p), float(c0), float(weight)
    return k


class Rng(C.Structure):
    _fields_ = [("s", C.c_uint64 * 4)]


_L = None


def build() -> Path:
    r = subprocess.run(["make", "-s", "-C", str(HERE)], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    return LIB


def lib() -> C.CDLL:
    global _L
    if _L is None:
        if not LIB.exists() or LIB.stat().st_mtime < (HERE / "csmc_oracle.c").stat().st_mtime:
            build()
        L = C.CDLL(str(LIB))
        sig = {
            "orc_lattice_new": (C.c_void_p, [C.POINTER(Desc), C.c_int, C.c_char_p, C.c_int]),
            "orc_lattice_free": (None, [C.c_void_p]),
            "orc_n_sites": (C.c_int64, [C.c_void_p]),
            "orc_term_counts": (None, [C.c_void_p, i32p]),
            "orc_export_tables": (None, [C.c_void_p, i64p, f64p, i64p, f64p, i64p, f64p, f64p, f64p]),
            "orc_local_field": (None, [C.c_void_p, f64p, C.c_int64, f64p]),
            "orc_site_energy": (C.c_double, [C.c_void_p, f64p, C.c_int64]),
            "orc_total_energy": (C.c_double, [C.c_void_p, f64p]),
            "orc_magnetization": (C.c_double, [C.c_void_p, f64p]),
            "orc_structure_factor": (None, [f64p, C.c_int64, f64p, C.c_int, f64p, C.c_int64, f64p]),
            "orc_random_spin_orientation": (None, [C.c_double, C.c_double, C.c_double, f64p]),
            "orc_gaussian_move": (None, [C.c_double, f64p, C.c_double, C.c_double, C.c_double, f64p]),
            "orc_energy_diff": (C.c_double, [C.c_void_p, f64p, C.c_int64, f64p]),
            "orc_metropolis_replay": (C.c_int64, [C.c_void_p, f64p, C.c_double, C.c_int, f64p, C.c_int64, i64p,
                                                  f64p, f64p, f64p, u8p]),
            "orc_constraint_value": (C.c_double, [C.c_void_p, f64p, C.POINTER(Constraint)]),
            "orc_metropolis_constraint_replay": (C.c_int64, [C.c_void_p, f64p, C.c_double, C.c_int, f64p, C.c_double,
                                                             C.POINTER(Constraint), f64p, C.c_int64, i64p, f64p,
                                                             f64p, f64p, u8p]),
            "orc_metropolis_constraint_sweep": (C.c_int64, [C.c_void_p, f64p, C.c_double, C.c_int, f64p, C.c_double,
                                                            C.POINTER(Constraint), f64p, C.c_uint64, C.c_uint32,
                                                            C.c_uint32]),
            "orc_overrelax_order": (None, [C.c_void_p, f64p, i64p, C.c_int64]),
            "orc_deterministic_order": (None, [C.c_void_p, f64p, i64p, C.c_int64]),
            "orc_overrelax_sweep": (None, [C.c_void_p, f64p]),
            "orc_philox4x32_10": (None, [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]),
            "orc_metropolis_colour_sweep": (C.c_int64, [C.c_void_p, f64p, C.c_double, C.c_int, f64p, i64p,
                                                        C.c_int64, C.c_uint64, C.c_uint32, C.c_uint32, C.c_int]),
            "orc_random_spins": (None, [C.c_void_p, f64p, C.c_uint64, C.c_uint32]),
            "orc_rng_seed": (None, [C.POINTER(Rng), C.c_uint64]),
            "orc_rng_uniform": (C.c_double, [C.POINTER(Rng)]),
            "orc_metropolis_sweep_ref": (C.c_double, [C.c_void_p, f64p, C.c_double, C.c_int, f64p,
                                                      C.POINTER(Rng)]),
            "orc_deterministic_ref": (None, [C.c_void_p, f64p, C.c_int64, C.POINTER(Rng)]),
            "orc_simulated_annealing": (C.c_double, [C.c_void_p, f64p, f64p, C.c_int32, C.c_int64, C.c_int32,
                                                     C.c_int, C.c_double, C.POINTER(Rng)]),
            "orc_parallel_tempering": (C.c_int64, [C.c_void_p, C.POINTER(f64p), f64p, C.c_int32,
                                                   C.POINTER(PTParams), f64p, f64p, f64p, f64p, C.c_int64]),
        }
        for k, (res, args) in sig.items():
            f = getattr(L, k)
            f.restype = res
            f.argtypes = args
        _L = L
    return _L


def _p(a, t=C.c_double):
    return None if a is None else a.ctypes.data_as(C.POINTER(t))


def spins_array(n: int) -> np.ndarray:
    return np.zeros((3, n), np.float64, order="F")


class OracleLattice:
    """The reference's Lattice (lattice.jl:65-291) built by the oracle from a unit cell."""

    def __init__(self, uc, shape, S: float, bc: str = "periodic", literal: bool = False):
        D = len(uc.lattice_vectors)
        self.keep = []
        d = Desc()
        d.dim = D
        d.n_basis = len(uc.basis)
        for k in range(3):
            d.shape[k] = int(shape[k]) if k < D else 1
        d.periodic = 1 if bc == "periodic" else 0
        d.spin_length = float(S)

        def arr(rows, width, dt):
            a = np.ascontiguousarray(np.asarray(rows, dtype=dt).reshape(-1, width) if rows else
                                     np.zeros((0, width), dt))
            self.keep.append(a)
            return a.ctypes.data_as(C.POINTER(C.c_int32 if dt == np.int32 else C.c_double))

        d.n_field = len(uc.field)
        d.field_basis = arr([b for b, _ in uc.field], 1, np.int32)
        d.field_vec = arr([np.asarray(h).reshape(3) for _, h in uc.field], 3, np.float64)
        d.n_onsite = len(uc.onsite)
        d.onsite_basis = arr([b for b, _ in uc.onsite], 1, np.int32)
        d.onsite_mat = arr([np.asarray(m).reshape(9) for _, m in uc.onsite], 9, np.float64)
        d.n_bilinear = len(uc.bilinear)
        d.bilinear_basis = arr([t[:2] for t in uc.bilinear], 2, np.int32)
        d.bilinear_mat = arr([np.asarray(t[2]).reshape(9) for t in uc.bilinear], 9, np.float64)
        d.bilinear_offset = arr([t[3] for t in uc.bilinear], D, np.int32)
        d.n_cubic = len(uc.cubic)
        d.cubic_basis = arr([t[:3] for t in uc.cubic], 3, np.int32)
        d.cubic_tensor = arr([np.asarray(t[3]).reshape(27) for t in uc.cubic], 27, np.float64)
        d.cubic_offset = arr([tuple(t[4]) + tuple(t[5]) for t in uc.cubic], 2 * D, np.int32)
        d.n_quartic = len(uc.quartic)
        d.quartic_basis = arr([t[:4] for t in uc.quartic], 4, np.int32)
        d.quartic_tensor = arr([np.asarray(t[4]).reshape(81) for t in uc.quartic], 81, np.float64)
        d.quartic_offset = arr([tuple(t[5]) + tuple(t[6]) + tuple(t[7]) for t in uc.quartic], 3 * D, np.int32)
        err = C.create_string_buffer(512)
        self.h = lib().orc_lattice_new(C.byref(d), 1 if literal else 0, err, 512)
        if not self.h:
            raise ValueError(err.value.decode())
        self.N = lib().orc_n_sites(self.h)
        cnt = (C.c_int32 * 3)()
        lib().orc_term_counts(self.h, cnt)
        self.N2, self.N3, self.N4 = cnt[0], cnt[1], cnt[2]
        self.S = float(S)

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_lattice_free(self.h)
            self.h = None

    def tables(self) -> dict:
        N, n2, n3, n4 = self.N, self.N2, self.N3, self.N4
        t = dict(bilinear_sites=np.zeros((N, n2), np.int64), bilinear_matrices=np.zeros((N, n2, 3, 3)),
                 cubic_sites=np.zeros((N, n3, 2), np.int64), cubic_tensors=np.zeros((N, n3, 3, 3, 3)),
                 quartic_sites=np.zeros((N, n4, 3), np.int64), quartic_tensors=np.zeros((N, n4, 3, 3, 3, 3)),
                 field=np.zeros((N, 3)), onsite=np.zeros((N, 3, 3)))
        lib().orc_export_tables(self.h, _p(t["bilinear_sites"], C.c_int64), _p(t["bilinear_matrices"]),
                                _p(t["cubic_sites"], C.c_int64), _p(t["cubic_tensors"]),
                                _p(t["quartic_sites"], C.c_int64), _p(t["quartic_tensors"]), _p(t["field"]),
                                _p(t["onsite"]))
        return t

    # -- Hamiltonian --------------------------------------------------------
    def local_field(self, spins, i: int) -> np.ndarray:
        H = np.zeros(3)
        lib().orc_local_field(self.h, _p(spins), int(i), _p(H))
        return H

    def local_fields(self, spins) -> np.ndarray:
        H = spins_array(self.N)
        for i in range(self.N):
            H[:, i] = self.local_field(spins, i)
        return H

    def site_energy(self, spins, i: int) -> float:
        return lib().orc_site_energy(self.h, _p(spins), int(i))

    def total_energy(self, spins) -> float:
        return lib().orc_total_energy(self.h, _p(spins))

    def magnetization(self, spins) -> float:
        return lib().orc_magnetization(self.h, _p(spins))

    def energy_diff(self, spins, i: int, new) -> float:
        """dE of moving site i to `new`, spins left unchanged."""
        s = np.asfortranarray(spins.copy())
        n = np.ascontiguousarray(new, dtype=np.float64)
        return lib().orc_energy_diff(self.h, _p(s), int(i), _p(n))

    # -- updates ------------------------------------------------------------
    def replay(self, spins, T, kind, sigma, sites, u_phi, u_z, u_acc):
        n = len(sites)
        s = np.ascontiguousarray(sites, np.int64)
        a = [np.ascontiguousarray(x, np.float64) for x in (u_phi, u_z, u_acc)]
        acc = np.zeros(n, np.uint8)
        sg = C.c_double(sigma)
        lib().orc_metropolis_replay(self.h, _p(spins), T, kind, C.byref(sg), n, _p(s, C.c_int64), _p(a[0]),
                                    _p(a[1]), _p(a[2]), _p(acc, C.c_uint8))
        return acc, sg.value

    def constraint_value(self, spins, k) -> float:
        return lib().orc_constraint_value(self.h, _p(spins), C.byref(k))

    def constraint_replay(self, spins, T, cone, sigma, sigma0, k, lam, sites, u_phi, u_z, u_acc):
        """metropolis_constraint(_adaptive)! fed with the given proposals;
        returns (accepted flags, sigma, lambda)."""
        n = len(sites)
        s = np.ascontiguousarray(sites, np.int64)
        a = [np.ascontiguousarray(x, np.float64) for x in (u_phi, u_z, u_acc)]
        acc = np.zeros(n, np.uint8)
        sg, lm = C.c_double(sigma), C.c_double(lam)
        lib().orc_metropolis_constraint_replay(self.h, _p(spins), T, int(cone), C.byref(sg), sigma0, C.byref(k),
                                               C.byref(lm), n, _p(s, C.c_int64), _p(a[0]), _p(a[1]), _p(a[2]),
                                               _p(acc, C.c_uint8))
        return acc, sg.value, lm.value

    def constraint_sweep(self, spins, T, cone, sigma, sigma0, k, lam, seed, chain, sweep):
        """One constrained sweep with the GPU kernel's Philox draws;
        returns (accepted count, sigma, lambda)."""
        sg, lm = C.c_double(sigma), C.c_double(lam)
        acc = lib().orc_metropolis_constraint_sweep(self.h, _p(spins), T, int(cone), C.byref(sg), sigma0,
                                                    C.byref(k), C.byref(lm), C.c_uint64(seed), chain, sweep)
        return acc, sg.value, lm.value

    def overrelax_order(self, spins, order):
        o = np.ascontiguousarray(order, np.int64)
        lib().orc_overrelax_order(self.h, _p(spins), _p(o, C.c_int64), len(o))

    def deterministic_order(self, spins, order):
        o = np.ascontiguousarray(order, np.int64)
        lib().orc_deterministic_order(self.h, _p(spins), _p(o, C.c_int64), len(o))

    def overrelax_sweep(self, spins):
        lib().orc_overrelax_sweep(self.h, _p(spins))

    def colour_sweep(self, spins, T, kind, sigma, order, seed, chain, sweep, bits):
        o = np.ascontiguousarray(order, np.int64)
        sg = C.c_double(sigma)
        acc = lib().orc_metropolis_colour_sweep(self.h, _p(spins), T, kind, C.byref(sg), _p(o, C.c_int64), len(o),
                                                C.c_uint64(seed), chain, sweep, bits)
        return acc, sg.value

    def random_spins(self, seed: int, chain: int = 0) -> np.ndarray:
        s = spins_array(self.N)
        lib().orc_random_spins(self.h, _p(s), C.c_uint64(seed), chain)
        return s

    def simulated_annealing(self, spins, temps, t_therm, or_rate, kind=UNIFORM, sigma0=60.0, seed=1):
        r = Rng()
        lib().orc_rng_seed(C.byref(r), C.c_uint64(seed))
        t = np.ascontiguousarray(temps, np.float64)
        return lib().orc_simulated_annealing(self.h, _p(spins), _p(t), len(t), int(t_therm), int(or_rate), kind,
                                             sigma0, C.byref(r))

    def deterministic_ref(self, spins, t_det, seed=2):
        r = Rng()
        lib().orc_rng_seed(C.byref(r), C.c_uint64(seed))
        lib().orc_deterministic_ref(self.h, _p(spins), int(t_det), C.byref(r))

    def metropolis_sweep_ref(self, spins, T, kind=UNIFORM, sigma=60.0, rng=None):
        sg = C.c_double(sigma)
        return lib().orc_metropolis_sweep_ref(self.h, _p(spins), T, kind, C.byref(sg), C.byref(rng)), sg.value

    def parallel_tempering(self, spins_list, T, t_therm, t_meas, probe_rate, swap_rate, or_rate, kind=UNIFORM,
                           sigma0=60.0, n_threads=1, seed=7):
        R = len(spins_list)
        arrs = (f64p * R)(*[_p(s) for s in spins_list])
        p = PTParams(int(t_therm), int(t_meas), int(probe_rate), int(swap_rate), int(or_rate), kind, sigma0,
                     int(n_threads), seed)
        cap = (t_therm + t_meas) // max(probe_rate, 1) + 2
        E = np.zeros((cap, R))
        M = np.zeros((cap, R))
        acc = np.zeros(R)
        exc = np.zeros(R)
        Tt = np.ascontiguousarray(T, np.float64)
        n = lib().orc_parallel_tempering(self.h, arrs, _p(Tt), R, C.byref(p), _p(acc), _p(exc), _p(E), _p(M), cap)
        # the oracle swaps the arrays in place of MPI.Sendrecv!: report final configurations by slot
        finals = [np.ctypeslib.as_array(C.cast(arrs[r], C.POINTER(C.c_double)), shape=(self.N * 3,)).copy()
                  for r in range(R)]
        return dict(energy=E[:n], magnetization=M[:n], accepted=acc, exchanged=exc,
                    spins=[f.reshape(3, self.N, order="F") for f in finals])


def structure_factor(spins, pos, ks) -> np.ndarray:
    """compute_equal_time_correlations (spin_correlations.jl:6-43): spins 3 x N,
    pos dim x N, ks dim x n_k (column-major) -> Suv 9 x n_k."""
    spins = np.asfortranarray(spins, np.float64)
    pos = np.asfortranarray(pos, np.float64)
    ks = np.asfortranarray(ks, np.float64)
    n_k = ks.shape[1]
    out = np.zeros((9, n_k), np.float64, order="F")
    lib().orc_structure_factor(_p(spins), spins.shape[1], _p(pos), pos.shape[0], _p(ks), n_k, _p(out))
    return out


def philox(ctr, key) -> tuple:
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    lib().orc_philox4x32_10(c, k, o)
    return tuple(o)
