"""reciprocal.jl (reciprocal lattice vectors, allowed wavevectors, k planes
and paths) and the configuration split of spin_correlations.jl:63-79; no
GPU.  The reference has no tests for these: the checks are the defining
properties."""
import importlib
import math

import numpy as np
import pytest


@pytest.mark.parametrize("cell", ["Square", "Triangular", "Honeycomb", "FCC", "Pyrochlore"])
def test_reciprocal_vectors(m, cell):
    uc = getattr(m, cell)()
    A = np.stack(uc.lattice_vectors)
    B = np.stack(m.reciprocal(*uc.lattice_vectors))
    assert np.allclose(A @ B.T, 2 * math.pi * np.eye(len(A)), atol=1e-12)


def test_allowed_wavevectors_order_and_count(m):
    uc = m.Square()
    ks = m.get_allowed_wavevectors(uc, (2, 3))
    assert ks.shape == (2, 3 * 4)  # n_d = 0..L_d, both ends
    # the first dimension varies fastest (Iterators.product order)
    want = [2 * math.pi * np.array([i / 2, j / 3]) for j in range(4) for i in range(3)]
    assert np.allclose(ks, np.stack(want, axis=1))
    ks = m.get_allowed_wavevectors(m.FCC(), (2, 2, 2), min=-1, max=1)
    assert ks.shape == (3, 5 ** 3)
    B = np.stack(m.reciprocal(*m.FCC().lattice_vectors), axis=1)
    assert np.allclose(ks[:, 0], B @ [-1, -1, -1]) and np.allclose(ks[:, 1], B @ [-0.5, -1, -1])


def test_k_plane_and_direction_path(m):
    uc = m.Square()
    ks = m.get_k_plane(uc, (4, 4), min=-1, max=1)
    r = np.round(ks, 6)
    assert np.all((r >= round(-2 * math.pi, 6)) & (r <= round(2 * math.pi, 6)))
    assert ks.shape[1] == 9 * 9
    d = np.array([2.0, 0.0])
    path = m.get_k_path(uc, d, (4, 4), -1, 1)
    assert np.array_equal(d, [1.0, 0.0])  # normalised in place, as the reference does
    assert np.allclose(path[1], 0.0) and path.shape[1] == 9  # the k_x axis, 2 pi n / 4 for n = -4..4


def test_high_symmetry_path(m):
    uc = m.Square()
    hsp = {"G": np.array([0.0, 0.0]), "X": np.array([math.pi, 0.0]), "M": np.array([math.pi, math.pi])}
    count, kpath = m.get_k_path(uc, hsp, ["G", "X", "M", "G"], (4, 4))
    # each leg holds the allowed points after its start (the start itself has
    # no direction: 0/0): G->X pi/2, pi; X->M (pi, pi/2), (pi, pi); M->G
    # (pi/2, pi/2), 0, reversed to end at G
    assert count.tolist() == [0, 2, 4, 6] and kpath.shape == (2, 7)
    assert np.allclose(kpath[:, 0], 0) and np.allclose(kpath[:, 2], hsp["X"]) and np.allclose(kpath[:, 4], hsp["M"])
    assert np.allclose(kpath[:, 5], [math.pi / 2, math.pi / 2]) and np.allclose(kpath[:, -1], hsp["G"])
    with pytest.raises(IndexError):
        m.get_k_path(uc, {"A": np.array([0.1, 0.1]), "B": np.array([0.2, 0.15])}, ["A", "B"], (4, 4))


@pytest.mark.parametrize("n,world", [(0, 1), (7, 1), (7, 2), (7, 3), (2, 4), (16, 4)])
def test_rank_share(m, n, world):
    sc = importlib.import_module(m.__name__ + ".spin_correlations")
    shares = [sc.rank_share(n, r, world) for r in range(world)]
    assert sum(c for _, c in shares) == n
    assert [s for s, _ in shares] == [sum(c for _, c in shares[:r]) for r in range(world)]
    assert max(c for _, c in shares) - min(c for _, c in shares) <= 1
    assert shares == sorted(shares) and all(c >= shares[-1][1] for _, c in shares)
    with pytest.raises(ValueError):
        sc.rank_share(n, world, world)
