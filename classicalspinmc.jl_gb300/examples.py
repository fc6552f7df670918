"""Unit cells of the benchmark models (the reference's examples/ define the
Kitaev honeycomb and the pyrochlore in the same way).

Each builder returns a fresh UnitCell:
  square_heisenberg   -- square lattice, J=-I on 4 neighbours, h=(0,0,0.1)
  honeycomb_kitaev    -- honeycomb K-J-Gamma-Gamma' bonds of test/mctests.jl:14-29
  sc_heisenberg       -- simple cubic, J=+I on 6 neighbours, onsite diag(0,0,D)
  triangular_afm      -- triangular, J=+I on the 6 bonds, h=(0,0,h)
  pyrochlore_ckq      -- pyrochlore J1=I on the 12 nearest-neighbour bonds, cubic
                         kappa*eps_abc on the 8 tetrahedron faces, quartic
                         q*delta_ab*delta_cd over the 3 pairings of both
                         tetrahedra, h=(0.1,0.1,0.1)/sqrt(3)
"""
from __future__ import annotations

import math

import numpy as np

from . import unit_cell as m


def square_heisenberg(J=-1.0, h=(0.0, 0.0, 0.1)):
    uc = m.Square()
    for off in [(1, 0), (-1, 0), (0, 1), (0, -1)]:
        m.addBilinear(uc, 1, 1, J * np.eye(3), off)
    m.addZeemanCoupling(uc, 1, list(h))
    return uc


def kitaev_bonds(K=-1.0, J=0.0, G=0.0, Gp=0.0):
    Jx = np.array([[K + J, Gp, Gp], [Gp, J, G], [Gp, G, J]])
    Jy = np.array([[J, Gp, G], [Gp, K + J, Gp], [G, Gp, J]])
    Jz = np.array([[J, G, Gp], [G, J, Gp], [Gp, Gp, K + J]])
    return Jx, Jy, Jz


def honeycomb_kitaev(K=-1.0, J=0.0, G=0.0, Gp=0.0, h=0.0, hdir=(1, 1, 1)):
    uc = m.Honeycomb()
    Jx, Jy, Jz = kitaev_bonds(K, J, G, Gp)
    m.addBilinear(uc, 1, 2, Jx, (0, -1))
    m.addBilinear(uc, 1, 2, Jy, (1, -1))
    m.addBilinear(uc, 1, 2, Jz, (0, 0))
    hv = h * np.asarray(hdir, dtype=np.float64) / np.linalg.norm(hdir)
    m.addZeemanCoupling(uc, 1, hv)
    m.addZeemanCoupling(uc, 2, hv)
    return uc


def sc_heisenberg(J=1.0, D=0.2):
    uc = m.UnitCell([1.0, 0, 0], [0, 1.0, 0], [0, 0, 1.0])
    for off in [(1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1)]:
        m.addBilinear(uc, 1, 1, J * np.eye(3), off)
    m.addOnSite(uc, 1, np.diag([0.0, 0.0, D]))
    return uc


def triangular_afm(h=0.0, J=1.0):
    uc = m.Triangular()
    for off in [(1, 0), (-1, 0), (0, 1), (0, -1), (1, -1), (-1, 1)]:
        m.addBilinear(uc, 1, 1, J * np.eye(3), off)
    m.addZeemanCoupling(uc, 1, [0.0, 0.0, h])
    return uc


def levi_civita():
    e = np.zeros((3, 3, 3))
    for a, b, c, s in [(0, 1, 2, 1), (1, 2, 0, 1), (2, 0, 1, 1), (0, 2, 1, -1), (2, 1, 0, -1), (1, 0, 2, -1)]:
        e[a, b, c] = s
    return e


# down tetrahedron of the pyrochlore (FCC primitive cells, bravais.jl:18-34):
# basis 1 in cell n, 2 in n+(1,0,0), 3 in n+(0,1,0), 4 in n+(0,0,1)
DOWN = {1: (0, 0, 0), 2: (1, 0, 0), 3: (0, 1, 0), 4: (0, 0, 1)}


def _rel(b, c):
    return tuple(DOWN[c][k] - DOWN[b][k] for k in range(3))


def pyrochlore_ckq(J1=1.0, kappa=0.02, q=0.05, h=0.1, bonds=True, cubic=True, quartic=True):
    uc = m.Pyrochlore()
    Jm = J1 * np.eye(3)
    pairs = [(1, 2), (1, 3), (1, 4), (2, 3), (2, 4), (3, 4)]
    if bonds:
        for b1, b2 in pairs:  # up tetrahedron
            m.addBilinear(uc, b1, b2, Jm, (0, 0, 0))
        for b1, b2 in pairs:  # down tetrahedron
            m.addBilinear(uc, b1, b2, Jm, _rel(b1, b2))
    if cubic:
        eps = kappa * levi_civita()
        for face in [(1, 2, 3), (1, 2, 4), (1, 3, 4), (2, 3, 4)]:
            m.addCubic(uc, *face, eps, (0, 0, 0), (0, 0, 0))
        for b1, b2, b3 in [(1, 2, 3), (1, 2, 4), (1, 3, 4), (2, 3, 4)]:
            m.addCubic(uc, b1, b2, b3, eps, _rel(b1, b2), _rel(b1, b3))
    if quartic:
        dd = q * np.einsum("ab,cd->abcd", np.eye(3), np.eye(3))
        for b in [(1, 2, 3, 4), (1, 3, 2, 4), (1, 4, 2, 3)]:
            m.addQuartic(uc, *b, dd, (0, 0, 0), (0, 0, 0), (0, 0, 0))
            m.addQuartic(uc, *b, dd, _rel(b[0], b[1]), _rel(b[0], b[2]), _rel(b[0], b[3]))
    hv = h * np.ones(3) / math.sqrt(3)
    for b in range(1, 5):
        m.addZeemanCoupling(uc, b, hv)
    return uc


def random_spins(n, S=1.0, seed=0):
    rng = np.random.default_rng(seed)
    v = rng.normal(size=(3, n))
    v /= np.linalg.norm(v, axis=0)
    return np.asfortranarray(S * v)
