"""Observables, mirroring observables.jl.

The reference pushes (E, E^2) and (|M|, |M|^2) into BinningAnalysis.jl 0.6.1
ErrorPropagators (observables.jl:20-25) and derives the specific heat and
susceptibility with standard errors from the gradient of the estimator at the
binning level it deems reliable (observables.jl:30-63).  That package is not
available here; its published method is restated below: logarithmic binning
(bin size 2^l), the deepest level that still holds at least 32 bins, and the
standard error of g(mean) as sqrt(var(grad g . x_bin) / n_bins).  Error bars
are unpinned against the reference (it has no test for them).
"""
from __future__ import annotations

import numpy as np


class Observables:
    """Observables (observables.jl:5-10): per-probe energy and |M| samples."""

    def __init__(self):
        self.energy: list[float] = []
        self.magnetization: list[float] = []
        self.correlations: list[np.ndarray] = []

    def push(self, E: float, M: float) -> None:
        """update_observables! (observables.jl:20-25)."""
        self.energy.append(float(E))
        self.magnetization.append(float(M))

    def push_correlations(self, Suv: np.ndarray) -> None:
        """update_correlations! (observables.jl:27-30): one 9 x N_k sample."""
        self.correlations.append(np.array(Suv, dtype=np.float64))

    def mean_correlations(self) -> np.ndarray | None:
        """The mean of the correlation samples (the LogBinner's mean)."""
        return np.mean(self.correlations, axis=0) if self.correlations else None


def _reliable_bins(x: np.ndarray, min_bins: int = 32) -> np.ndarray:
    """Bin means (rows) at the deepest 2^l level with >= min_bins full bins."""
    n = x.shape[0]
    size = 1
    while n // (size * 2) >= min_bins:
        size *= 2
    nb = n // size
    return x[: nb * size].reshape(nb, size, -1).mean(axis=1)


def _propagate(samples: np.ndarray, g, grad) -> tuple[float, float]:
    x = np.stack([samples, samples ** 2], axis=1)
    mean = x.mean(axis=0)
    value = g(mean)
    if len(samples) < 2:
        return float(value), float("nan")
    bins = _reliable_bins(x)
    proj = bins @ np.asarray(grad(mean))
    err = np.sqrt(abs(np.var(proj, ddof=1) / len(proj))) if len(proj) > 1 else float("nan")
    return float(value), float(err)


def specific_heat(E: np.ndarray, T: float, N: int) -> tuple[float, float]:
    """specific_heat (observables.jl:36-49): (<E^2> - <E>^2) / (T^2 N) and its error."""
    c = lambda e: 1 / T ** 2 * (e[1] - e[0] * e[0]) / N
    dc = lambda e: [-2.0 / T ** 2 * e[0] / N, 1 / T ** 2 / N]
    return _propagate(np.asarray(E, dtype=np.float64), c, dc)


def susceptibility(M: np.ndarray, T: float, N: int) -> tuple[float, float]:
    """susceptibility (observables.jl:51-63): (<M^2> - <M>^2) / (T N) and its error."""
    x = lambda m: 1 / T * (m[1] - m[0] * m[0]) / N
    dx = lambda m: [-2 / T * m[0] / N, 1 / T / N]
    return _propagate(np.asarray(M, dtype=np.float64), x, dx)


def mean_and_error(samples: np.ndarray) -> tuple[float, float]:
    """Mean and binned standard error of a series."""
    s = np.asarray(samples, dtype=np.float64)
    if len(s) < 2:
        return float(s.mean()) if len(s) else float("nan"), float("nan")
    bins = _reliable_bins(s.reshape(-1, 1))[:, 0]
    return float(s.mean()), float(np.std(bins, ddof=1) / np.sqrt(len(bins)))
