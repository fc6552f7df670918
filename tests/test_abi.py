"""The C ABI: libcsmc.so loads and exports every entry point include/csmc.h
declares; the ctypes signatures cover them; without a GPU, contexts fail with
CSMC_ERR_CUDA instead of crashing."""
import ctypes as C
import re
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent.parent


def declared_symbols():
    text = (ROOT / "include" / "csmc.h").read_text()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(csmc_\w+)\s*\(", text, re.M)))


def test_header_symbols_exported(m):
    lib = m.lib()
    syms = declared_symbols()
    assert len(syms) >= 30
    for s in syms:
        assert hasattr(lib, s), s


def test_ctypes_signatures_cover_header(m):
    from importlib import import_module
    L = import_module(m.__name__ + "._lib")
    assert sorted(L.SIGNATURES) == declared_symbols()


def test_struct_sizes_match_header(m):
    from importlib import import_module
    L = import_module(m.__name__ + "._lib")
    # 64-bit layouts of csmc_lattice_info / csmc_run_params
    assert C.sizeof(L.LatticeInfo) == 8 + 10 * 4 + 8 + 2 * 4
    assert C.sizeof(L.RunParams) == 3 * 8 + 6 * 4 + 2 * 8 + 8 + 2 * 8 + 8


def test_errors_are_codes_not_crashes(m):
    lib = m.lib()
    from importlib import import_module
    L = import_module(m.__name__ + "._lib")
    d = m.Lattice((4, 4), m.examples.square_heisenberg(), 1.0).desc
    h = C.c_void_p()
    code = lib.csmc_create(d.ref(), 7, 1, 0, C.byref(h))  # bad precision
    assert code == 1 and b"precision" in lib.csmc_last_error()
    code = lib.csmc_create(d.ref(), 0, 0, 0, C.byref(h))  # no replicas
    assert code == 1
    assert lib.csmc_create(None, 0, 1, 0, C.byref(h)) == 1
    assert lib.csmc_total_energy(None, None) == 1
    assert lib.csmc_destroy(None) == 0
    code = lib.csmc_create(d.ref(), 0, 1, 0, C.byref(h))
    if code == 0:  # a GPU is present
        assert lib.csmc_destroy(h) == 0
    else:
        assert code == 3 and len(lib.csmc_last_error()) > 0


def test_host_api_reaches_the_device(m):
    """MonteCarlo's host path (deepcopy, description, validation) runs to the CUDA
    context; without a GPU it stops there with CSMC_ERR_CUDA."""
    lat = m.Lattice((4, 4), m.examples.square_heisenberg(), 1.0)
    try:
        mc = m.MonteCarlo([0.5, 1.0], lat, {"overrelaxation_rate": 5}, precision="fp32")
    except m.CSMCError as e:
        assert e.code == 3
    else:
        assert mc.n_replicas == 2
