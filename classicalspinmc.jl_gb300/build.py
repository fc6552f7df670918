"""Build libcsmc.so in-tree for sm_103a.

Every CUDA translation unit is compiled by nvcc with
``-gencode arch=compute_103a,code=sm_103a -lineinfo`` in parallel, the host
flattener (plan.cpp) by g++, and the objects are linked into
``classicalspinmc.jl_gb300/lib/libcsmc.so`` (static CUDA runtime).  exact.cu,
the sequential FP64 replay kernel, is compiled with ``-fmad=false`` so that
its arithmetic matches the reference's unfused evaluation.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
OUT = PKG / "lib"
OBJ = PKG / "_build"
LIB = OUT / "libcsmc.so"

GENCODE = "-gencode=arch=compute_103a,code=sm_103a"
NVCC_FLAGS = [GENCODE, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-Wall"]


def _nvcc() -> str:
    for cand in (os.environ.get("CUDACXX"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _cuda_include(nvcc: str) -> str:
    return str(Path(nvcc).resolve().parent.parent / "include")


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose: bool = False, force: bool = False, ptxas_info: bool = False) -> Path:
    nvcc = _nvcc()
    OBJ.mkdir(exist_ok=True)
    OUT.mkdir(exist_ok=True)
    headers = sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.hpp")) + [PKG.parent / "include" / "csmc.h"]
    jobs = []
    for src in sorted(CSRC.glob("*.cu")):
        obj = OBJ / (src.stem + ".o")
        flags = list(NVCC_FLAGS)
        if src.name == "exact.cu":
            flags.append("-fmad=false")
        if ptxas_info:
            flags += ["-Xptxas", "-v"]
        jobs.append((obj, [nvcc, *flags, "-c", str(src), "-o", str(obj)], [src, *headers]))
    for src in sorted(CSRC.glob("*.cpp")):
        obj = OBJ / (src.stem + ".o")
        jobs.append((obj, ["g++", *CXX_FLAGS, "-I", _cuda_include(nvcc), "-c", str(src), "-o", str(obj)],
                     [src, *headers]))
    todo = [(o, c) for o, c, d in jobs if force or ptxas_info or _stale(o, d)]
    with cf.ThreadPoolExecutor(max_workers=min(8, max(1, len(todo)))) as ex:
        futs = {ex.submit(_run, c): o for o, c in todo}
        for f in cf.as_completed(futs):
            f.result()
            if verbose:
                print("compiled", futs[f].name, file=sys.stderr)
    objs = [o for o, _, _ in jobs]
    if force or todo or _stale(LIB, objs):
        _run([nvcc, GENCODE, "-shared", "-o", str(LIB), *map(str, objs), "-lpthread"])
    return LIB


if __name__ == "__main__":
    build(verbose=True, force="--force" in sys.argv, ptxas_info="--ptxas" in sys.argv)
    print(LIB)
