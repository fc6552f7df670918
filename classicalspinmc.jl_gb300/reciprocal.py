"""Reciprocal-space helpers, mirroring reciprocal.jl: reciprocal lattice
vectors and the wavevectors passed to the structure factor
(``compute_equal_time_correlations`` and ``MonteCarlo(corr=True, ks=...)``).

Wavevector sets are D x N_k arrays (one wavevector per column), as in the
reference.  Comparisons round to 6 decimals (5 for the path-end check) as
the reference does with ``round(x, digits=...)``.
"""
from __future__ import annotations

import itertools
import math

import numpy as np


def reciprocal(*a) -> tuple:
    """reciprocal(a1, a2) / reciprocal(a1, a2, a3) (reciprocal.jl:3-16):
    b_i with a_i . b_j = 2 pi delta_ij."""
    a = [np.asarray(v, dtype=np.float64) for v in a]
    if len(a) == 2:
        a1, a2 = a
        mag = 2 * math.pi / (a1[0] * a2[1] - a1[1] * a2[0])
        return (mag * np.array([a2[1], -a2[0]]), mag * np.array([-a1[1], a1[0]]))
    if len(a) == 3:
        a1, a2, a3 = a
        mag = 2 * math.pi / float(np.dot(a1, np.cross(a2, a3)))
        return (mag * np.cross(a2, a3), mag * np.cross(a3, a1), mag * np.cross(a1, a2))
    raise ValueError("reciprocal needs two or three lattice vectors")


def get_allowed_wavevectors(uc, shape, min: int = 0, max: int = 1) -> np.ndarray:
    """get_allowed_wavevectors (reciprocal.jl:23-29): sum_d (n_d / L_d) b_d for
    n_d = min*L_d .. max*L_d (both ends included), the first dimension
    varying fastest; D x prod(L_d*(max-min)+1)."""
    B = np.stack(reciprocal(*uc.lattice_vectors), axis=1)  # columns = b_d
    rs = [np.arange(min * L, max * L + 1) / L for L in shape]
    steps = np.array([t[::-1] for t in itertools.product(*rs[::-1])]).T  # first dimension fastest
    return B @ steps.reshape(len(shape), -1)


def _round(x, d: int = 6):
    return np.round(x, d)


def _in_box(ks: np.ndarray, lo, hi) -> np.ndarray:
    lo, hi = np.broadcast_to(lo, (ks.shape[0],)), np.broadcast_to(hi, (ks.shape[0],))
    r = _round(ks)
    return np.all((_round(lo)[:, None] <= r) & (r <= _round(hi)[:, None]), axis=0)


def get_k_plane(uc, shape, min: int = -2, max: int = 2) -> np.ndarray:
    """get_k_plane (reciprocal.jl:32-41): the allowed wavevectors of
    min..max copies whose every component lies in [2 pi min, 2 pi max]."""
    ks = get_allowed_wavevectors(uc, shape, min=min, max=max)
    return ks[:, _in_box(ks, min * 2 * math.pi, max * 2 * math.pi)]


def _parallel(ks: np.ndarray, line: np.ndarray, origin: np.ndarray) -> np.ndarray:
    d = ks - origin[:, None]
    with np.errstate(invalid="ignore", divide="ignore"):
        c = np.abs(line @ (d / np.linalg.norm(d, axis=0)))
    return _round(c) == 1.0


def get_k_path(uc, a, b, c=None, d=None):
    """get_k_path, both methods of reciprocal.jl:43-101.

    ``get_k_path(uc, direction, shape, min=-2, max=2)``: the allowed
    wavevectors k of min..max copies with k - direction parallel to direction
    and every component in [2 pi min, 2 pi max].  As in the reference, a
    float ``direction`` array is normalised in place.

    ``get_k_path(uc, hsp, path, shape)``: the path through the named
    high-symmetry points ``hsp[path[0]] -> hsp[path[1]] -> ...``; returns
    (point_count, kpath) with point_count[i] the number of points after the
    i-th corner and kpath starting with the first corner."""
    if isinstance(a, dict):
        return _k_path_points(uc, a, b, c)
    direction, shape = a, b
    lo = -2 if c is None else c
    hi = 2 if d is None else d
    ks = get_allowed_wavevectors(uc, shape, min=lo, max=hi)
    if isinstance(direction, np.ndarray) and direction.dtype == np.float64:
        direction /= np.linalg.norm(direction)
        line = direction
    else:
        line = np.asarray(direction, dtype=np.float64)
        line = line / np.linalg.norm(line)
    temp = ks[:, _parallel(ks, line, line)]
    return temp[:, _in_box(temp, lo * 2 * math.pi, hi * 2 * math.pi)]


def _k_path_points(uc, hsp: dict, path: list, shape):
    ks = get_allowed_wavevectors(uc, shape)
    kpath = np.asarray(hsp[path[0]], dtype=np.float64).reshape(-1, 1)
    point_count = np.zeros(len(path), dtype=np.int64)
    for ind, point in enumerate(path[:-1]):
        p1 = np.asarray(hsp[point], dtype=np.float64)
        p2 = np.asarray(hsp[path[ind + 1]], dtype=np.float64)
        line = (p2 - p1) / np.linalg.norm(p2 - p1)
        temp = ks[:, _parallel(ks, line, p1)]
        new_path = temp[:, _in_box(temp, np.minimum(p1, p2), np.maximum(p1, p2))]
        if new_path.shape[1] == 0:
            raise IndexError(f"no allowed wavevector between {point} and {path[ind + 1]}")
        if not np.array_equal(_round(new_path[:, -1], 5), _round(p2, 5)):
            new_path = new_path[:, ::-1]
        kpath = np.hstack([kpath, new_path])
        point_count[ind + 1] = new_path.shape[1] + point_count[ind]
    return point_count, kpath
