"""Structure factors of stored configurations, mirroring spin_correlations.jl:45-145.

``runEqualTimeStructureFactor(path, lat, ks)`` computes the equal-time
correlations of every ``IC_<i>.h5`` configuration in ``path`` (the files
parallel_tempering writes for ``saveIC``) and stores them in the file's
``spin_correlations`` group; ``compute_equal_time_structure_factor(path,
dest)`` averages the stored correlations into ``dest``.

The reference runs one configuration at a time per MPI rank.  Here the
configurations of a rank are loaded as the replicas of one device context,
``batch`` at a time, and one ``csmc_structure_factor`` launch computes all of
them.  ``rank`` and ``world`` split the files over processes as the
reference splits them over MPI ranks (the first N_IC % world ranks take one
more).  The reference calls ``read_spin_configuration!(file, lat)`` with its
arguments swapped (hdf5.jl:266 takes the lattice first), which Julia rejects;
here the configuration is read as that function intends.
"""
from __future__ import annotations

import os

import numpy as np

from . import hdf5
from .monte_carlo import Context, context_structure_factors


def rank_share(n_ic: int, rank: int = 0, world: int = 1) -> tuple[int, int]:
    """(first configuration, count) of ``rank`` (spin_correlations.jl:63-79)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside a world of {world}")
    per, rem = divmod(n_ic, world)
    counts = [per + (1 if r < rem else 0) for r in range(world)]
    return sum(counts[:rank]), counts[rank]


def runEqualTimeStructureFactor(path: str, lat, ks, override: bool = False, *, rank: int = 0, world: int = 1,
                                batch: int = 64, precision: str = "fp64", verbose: bool = True) -> list[int]:
    """runEqualTimeStructureFactor! (spin_correlations.jl:48-108); returns the
    indices of the configurations computed (skipped ones, which already hold
    ``spin_correlations`` and are not overridden, are left out)."""
    ks = np.asfortranarray(np.atleast_2d(np.asarray(ks, dtype=np.float64)))
    n_ic = len(os.listdir(path))
    first, count = rank_share(n_ic, rank, world)
    todo = []
    for ic in range(first, first + count):
        fn = f"{path}IC_{ic}.h5"
        with hdf5.h5open(fn, "r") as f:
            exists = "spin_correlations" in f
        if exists and not override:
            if verbose:
                print(f"Skipping IC_{ic}")
            continue
        todo.append(ic)
    for b in range(0, len(todo), max(1, batch)):
        group = todo[b:b + max(1, batch)]
        ctx = Context([lat], [len(group)], precision=precision)
        for slot, ic in enumerate(group):
            with hdf5.h5open(f"{path}IC_{ic}.h5", "r") as f:
                s = np.asfortranarray(np.asarray(f["spins"].read(), dtype=np.float64).T)
            if s.shape != (3, lat.size):
                raise ValueError(f"IC_{ic}.h5 holds {s.shape[1]} spins, the lattice has {lat.size} sites")
            ctx.set_spins(slot, s)
        if verbose:
            print(f"Computing SSF {b + 1}-{b + len(group)}/{len(todo)} on rank {rank}")
        S = context_structure_factors(ctx, lat, ks)
        for slot, ic in enumerate(group):
            if verbose:
                print(f"Writing IC {ic} to file on rank {rank}")
            with hdf5.h5open(f"{path}IC_{ic}.h5", "r+") as f:
                g = f["spin_correlations"] if "spin_correlations" in f else f.create_group("spin_correlations")
                hdf5.overwrite_keys(g, {"SSF": hdf5._jl(S[slot]), "SSF_momentum": hdf5._jl(ks)}, verbose)
        del ctx
    return todo


def compute_equal_time_structure_factor(path: str, dest: str, verbose: bool = True) -> np.ndarray:
    """compute_equal_time_structure_factor (spin_correlations.jl:114-145): the
    mean of the stored correlations of every file in ``path`` (in name order),
    written with the wavevectors of the first into ``dest`` (which must
    exist); returns the mean as a 9 x N_k array."""
    files = sorted(os.listdir(path))
    if verbose:
        print(f"Initializing LogBinner in {path}")
    with hdf5.h5open(path + files[0], "r") as f0:
        shape = f0["spin_correlations/SSF"].shape
        ks = f0["spin_correlations/SSF_momentum"].read()
    total = np.zeros(shape)
    if verbose:
        print(f"Collecting correlations from {len(files)} files")
    for fn in files:
        with hdf5.h5open(path + fn, "r") as f:
            total += f["spin_correlations/SSF"].read()
    mean = total / len(files)
    if verbose:
        print(f"Writing to {dest}")
    with hdf5.h5open(dest, "r+") as d:
        g = d["spin_correlations"] if "spin_correlations" in d else d.create_group("spin_correlations")
        hdf5.overwrite_keys(g, {"SSF": mean, "SSF_momentum": ks}, verbose)
    if verbose:
        print("Done")
    return np.ascontiguousarray(mean.T)
