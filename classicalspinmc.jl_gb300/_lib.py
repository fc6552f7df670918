"""ctypes binding of libcsmc.so (include/csmc.h).

The library is loaded from ``classicalspinmc.jl_gb300/lib/libcsmc.so``, built
in-tree by ``build.py``.  There is no fallback: if the library is missing or
a call fails, an exception is raised.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "lib" / "libcsmc.so"

CSMC_OK = 0
ERRORS = {1: "CSMC_ERR_INVALID", 2: "CSMC_ERR_OOM", 3: "CSMC_ERR_CUDA", 4: "CSMC_ERR_TIMEOUT",
          5: "CSMC_ERR_COLOURING", 6: "CSMC_ERR_UNSUPPORTED"}
FP64, FP32 = 0, 1
METROPOLIS, METROPOLIS_ADAPTIVE, METROPOLIS_FIXED_CONE = 0, 1, 2
METROPOLIS_CONSTRAINT, METROPOLIS_CONSTRAINT_ADAPTIVE = 3, 4
PATH_AUTO, PATH_RESIDENT, PATH_GLOBAL, PATH_PER_REPLICA = 0, 1, 2, 3

i32p = C.POINTER(C.c_int32)
i64p = C.POINTER(C.c_int64)
f64p = C.POINTER(C.c_double)
u8p = C.POINTER(C.c_uint8)
u32p = C.POINTER(C.c_uint32)


class CSMCError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class LatticeDesc(C.Structure):
    _fields_ = [
        ("dim", C.c_int32), ("n_basis", C.c_int32), ("shape", C.c_int32 * 3), ("periodic", C.c_int32),
        ("spin_length", C.c_double),
        ("n_field", C.c_int32), ("field_basis", i32p), ("field_vec", f64p),
        ("n_onsite", C.c_int32), ("onsite_basis", i32p), ("onsite_mat", f64p),
        ("n_bilinear", C.c_int32), ("bilinear_basis", i32p), ("bilinear_mat", f64p), ("bilinear_offset", i32p),
        ("n_cubic", C.c_int32), ("cubic_basis", i32p), ("cubic_tensor", f64p), ("cubic_offset", i32p),
        ("n_quartic", C.c_int32), ("quartic_basis", i32p), ("quartic_tensor", f64p), ("quartic_offset", i32p),
    ]


class LatticeInfo(C.Structure):
    _fields_ = [
        ("n_sites", C.c_int64), ("n_colours", C.c_int32), ("n_bilinear", C.c_int32), ("n_cubic", C.c_int32),
        ("n_quartic", C.c_int32), ("width_bilinear", C.c_int32), ("width_cubic", C.c_int32),
        ("width_quartic", C.c_int32), ("n_matrices", C.c_int32), ("n_cubic_tensors", C.c_int32),
        ("n_quartic_tensors", C.c_int32), ("padded_sites", C.c_int64), ("n_isotropic_cubic", C.c_int32),
        ("n_isotropic_quartic", C.c_int32),
    ]


class ConstraintDesc(C.Structure):
    """csmc_constraint: c = g.V + q |V|^2 + p |V| + c0, V = sum_i w_i s_i."""
    _fields_ = [("site_weights", f64p), ("g", C.c_double * 3), ("q", C.c_double), ("p", C.c_double),
                ("c0", C.c_double), ("weight", C.c_double)]


class RunParams(C.Structure):
    _fields_ = [
        ("sweep_start", C.c_int64), ("n_sweeps", C.c_int64), ("t_thermalization", C.c_int64),
        ("overrelaxation_rate", C.c_int32), ("swap_rate", C.c_int32), ("probe_rate", C.c_int32),
        ("kind", C.c_int32), ("path", C.c_int32), ("resident_block", C.c_int32),
        ("probe_energy", f64p), ("probe_magnetization", f64p), ("probe_capacity", C.c_int64),
        ("accepted", f64p), ("exchanged", f64p), ("n_probes_out", C.c_int64),
    ]


class TuneEntry(C.Structure):
    _fields_ = [("path", C.c_int32), ("cluster", C.c_int32), ("block", C.c_int32), ("persistent", C.c_int32),
                ("ms_per_window", C.c_double), ("chosen", C.c_int32)]


# name -> (restype, argtypes); every entry point declared in include/csmc.h
_vp = C.c_void_p
SIGNATURES = {
    "csmc_last_error": (C.c_char_p, []),
    "csmc_version": (C.c_char_p, []),
    "csmc_lattice_plan": (C.c_int, [C.POINTER(LatticeDesc), C.POINTER(LatticeInfo)]),
    "csmc_lattice_tables": (C.c_int, [C.POINTER(LatticeDesc), i64p, f64p, i64p, f64p, i64p, f64p, f64p, f64p]),
    "csmc_lattice_colouring": (C.c_int, [C.POINTER(LatticeDesc), i32p, i64p, i64p]),
    "csmc_create": (C.c_int, [C.POINTER(LatticeDesc), C.c_int32, C.c_int32, C.c_uint64, C.POINTER(_vp)]),
    "csmc_create_batch": (C.c_int, [C.POINTER(LatticeDesc), C.c_int32, i32p, C.c_int32, C.c_uint64,
                                    C.POINTER(_vp)]),
    "csmc_destroy": (C.c_int, [_vp]),
    "csmc_num_slots": (C.c_int, [_vp, i32p]),
    "csmc_lattice_info_of": (C.c_int, [_vp, C.c_int32, C.POINTER(LatticeInfo)]),
    "csmc_set_spins": (C.c_int, [_vp, C.c_int32, f64p]),
    "csmc_get_spins": (C.c_int, [_vp, C.c_int32, f64p]),
    "csmc_set_spins_all": (C.c_int, [_vp, f64p]),
    "csmc_get_spins_all": (C.c_int, [_vp, f64p]),
    "csmc_random_spins": (C.c_int, [_vp, C.c_uint64]),
    "csmc_set_chain_ids": (C.c_int, [_vp, u32p]),
    "csmc_set_temperatures": (C.c_int, [_vp, f64p]),
    "csmc_set_sigma": (C.c_int, [_vp, f64p]),
    "csmc_get_sigma": (C.c_int, [_vp, f64p]),
    "csmc_get_permutation": (C.c_int, [_vp, i32p]),
    "csmc_set_sigma0": (C.c_int, [_vp, C.c_double]),
    "csmc_set_constraint": (C.c_int, [_vp, C.c_int32, C.c_void_p]),
    "csmc_set_lambda": (C.c_int, [_vp, f64p]),
    "csmc_get_lambda": (C.c_int, [_vp, f64p]),
    "csmc_local_field": (C.c_int, [_vp, C.c_int32, f64p]),
    "csmc_energy_diff": (C.c_int, [_vp, C.c_int32, C.c_int64, i64p, f64p, f64p]),
    "csmc_energy_diff_static": (C.c_int, [_vp, C.c_int32, C.c_int64, i64p, f64p, f64p]),
    "csmc_total_energy": (C.c_int, [_vp, f64p]),
    "csmc_magnetization": (C.c_int, [_vp, f64p]),
    "csmc_metropolis_sweep": (C.c_int, [_vp, C.c_int32, f64p]),
    "csmc_metropolis_sweep_at": (C.c_int, [_vp, C.c_int32, f64p, C.c_int32, f64p]),
    "csmc_overrelax_sweep": (C.c_int, [_vp]),
    "csmc_deterministic_sweeps": (C.c_int, [_vp, C.c_int64]),
    "csmc_replay": (C.c_int, [_vp, C.c_int32, C.c_int32, C.c_double, f64p, C.c_int64, i64p, f64p, f64p, f64p,
                              u8p]),
    "csmc_run": (C.c_int, [_vp, C.POINTER(RunParams)]),
    "csmc_anneal": (C.c_int, [_vp, f64p, C.c_int32, C.c_int64, C.c_int32, C.c_int32, C.c_double, C.c_int32,
                              f64p]),
    "csmc_set_cluster_size": (C.c_int, [_vp, C.c_int32]),
    "csmc_cluster_size": (C.c_int, [_vp, i32p]),
    "csmc_set_size_groups": (C.c_int, [_vp, C.c_int32]),
    "csmc_size_groups": (C.c_int, [_vp, i32p]),
    "csmc_autotune": (C.c_int, [_vp, C.POINTER(RunParams), C.c_int32, C.POINTER(TuneEntry), C.c_int32, i32p]),
    "csmc_structure_factor": (C.c_int, [_vp, C.c_int32, C.c_int32, f64p, C.c_int64, f64p, f64p]),
    "csmc_set_tensor_cores": (C.c_int, [_vp, C.c_int32]),
    "csmc_selftest_timeout": (C.c_int, [_vp, C.c_int32]),
    "csmc_set_persistent": (C.c_int, [_vp, C.c_int32]),
    "csmc_persistent": (C.c_int, [_vp, i32p]),
    "csmc_set_renormalize": (C.c_int, [_vp, C.c_int32]),
    "csmc_spin_length_drift": (C.c_int, [_vp, f64p]),
    "csmc_debug_philox": (C.c_int, [u32p, u32p, C.c_int64, u32p]),
    "csmc_debug_device_allocs": (C.c_int, [i64p]),
    "csmc_last_run_stats": (C.c_int, [_vp, f64p, i64p, f64p, i64p]),
}

_LIB = None


def lib() -> C.CDLL:
    """Load libcsmc.so once; raise if it has not been built."""
    global _LIB
    if _LIB is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH} is missing: build it with classicalspinmc.jl_gb300/build.py")
        L = C.CDLL(str(LIB_PATH))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = L
    return _LIB


def check(code: int) -> None:
    if code != CSMC_OK:
        raise CSMCError(code, lib().csmc_last_error().decode())


def call(name: str, *args) -> None:
    check(getattr(lib(), name)(*args))


def ptr(a: np.ndarray, ctype):
    """Pointer to a contiguous numpy buffer (None for None)."""
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"] or a.flags["F_CONTIGUOUS"]
    return a.ctypes.data_as(C.POINTER(ctype))
