"""UnitCell and its builders, mirroring unit_cell.jl and bravais.jl.

Julia's mutating names end in ``!``; here the ``!`` is dropped
(``addBilinear!`` -> ``addBilinear``).  Arguments have the reference's meaning:
basis indices are 1-based, matrices are 3x3 (``M[a, b]``), cubic tensors
3x3x3 and quartic tensors 3x3x3x3 indexed as in Julia, offsets are tuples of
length D.  As in the reference, all-zero couplings are dropped on insertion.
"""
from __future__ import annotations

import math
import numpy as np


class UnitCell:
    """UnitCell{D} (unit_cell.jl:3-18): lattice vectors, basis and term lists.

    field:    (b, h[3])
    onsite:   (b, M[3,3])
    bilinear: (b1, b2, M[3,3], offset)
    cubic:    (b1, b2, b3, C[3,3,3], o2, o3)
    quartic:  (b1, b2, b3, b4, R[3,3,3,3], o2, o3, o4)
    """

    def __init__(self, *vectors):
        self.lattice_vectors = tuple(np.asarray(v, dtype=np.float64) for v in vectors)
        self.basis, self.field, self.onsite = [], [], []
        self.bilinear, self.cubic, self.quartic = [], [], []

    @property
    def D(self) -> int:
        return len(self.lattice_vectors)


def _offset(uc: UnitCell, o) -> tuple:
    if o is None:
        return (0,) * uc.D
    o = tuple(int(x) for x in o)
    if len(o) != uc.D:
        raise ValueError(f"offset {o} must have {uc.D} entries")
    return o


def addBasisSite(uc: UnitCell, site) -> None:
    """addBasisSite! (unit_cell.jl:23-25)."""
    uc.basis.append(np.asarray(site, dtype=np.float64))


def addZeemanCoupling(uc: UnitCell, b1: int, h) -> None:
    """addZeemanCoupling! (unit_cell.jl:30-32)."""
    uc.field.append((int(b1), np.asarray(h, dtype=np.float64).reshape(3)))


def addOnSite(uc: UnitCell, b1: int, M) -> None:
    """addOnSite! (unit_cell.jl:37-41): dropped if M is all zeros."""
    M = np.asarray(M, dtype=np.float64).reshape(3, 3)
    if np.any(M != 0):
        uc.onsite.append((int(b1), M))


def addBilinear(uc: UnitCell, b1: int, b2: int, M, offset=None) -> None:
    """addBilinear! (unit_cell.jl:46-52)."""
    M = np.asarray(M, dtype=np.float64).reshape(3, 3)
    if np.any(M != 0):
        uc.bilinear.append((int(b1), int(b2), M, _offset(uc, offset)))


def addCubic(uc: UnitCell, b1: int, b2: int, b3: int, M, o2=None, o3=None) -> None:
    """addCubic! (unit_cell.jl:57-63)."""
    M = np.asarray(M, dtype=np.float64).reshape(3, 3, 3)
    if np.any(M != 0):
        uc.cubic.append((int(b1), int(b2), int(b3), M, _offset(uc, o2), _offset(uc, o3)))


def addQuartic(uc: UnitCell, b1: int, b2: int, b3: int, b4: int, M, o2=None, o3=None, o4=None) -> None:
    """addQuartic! (unit_cell.jl:68-75)."""
    M = np.asarray(M, dtype=np.float64).reshape(3, 3, 3, 3)
    if np.any(M != 0):
        uc.quartic.append((int(b1), int(b2), int(b3), int(b4), M, _offset(uc, o2), _offset(uc, o3),
                           _offset(uc, o4)))


# ---------------------------------------------------------------- bravais.jl

def Triangular() -> UnitCell:
    """bravais.jl:1-8."""
    a1 = [1.0, 0.0]
    a2 = [math.cos(math.pi / 3), math.sin(math.pi / 3)]
    return UnitCell(a1, a2)


def Square() -> UnitCell:
    """bravais.jl:10-16."""
    return UnitCell([1.0, 0.0], [0.0, 1.0])


def FCC() -> UnitCell:
    """bravais.jl:18-25."""
    return UnitCell(0.5 * np.array([0, 1, 1.0]), 0.5 * np.array([1, 0, 1.0]), 0.5 * np.array([1, 1, 0.0]))


def Pyrochlore() -> UnitCell:
    """bravais.jl:27-34: FCC with four basis sites."""
    uc = FCC()
    for s in ([1, 1, 1], [1, -1, -1], [-1, 1, -1], [-1, -1, 1]):
        addBasisSite(uc, np.array(s, dtype=np.float64) / 8)
    return uc


def BreathingPyrochlore(a: float = 1.01) -> UnitCell:
    """bravais.jl:36-43."""
    uc = FCC()
    for s in ([1, 1, 1], [1, -1, -1], [-1, 1, -1], [-1, -1, 1]):
        addBasisSite(uc, a * np.array(s, dtype=np.float64) / 8)
    return uc


def Honeycomb() -> UnitCell:
    """bravais.jl:45-51: triangular Bravais lattice with two basis sites."""
    uc = Triangular()
    addBasisSite(uc, [0.0, 0.0])
    addBasisSite(uc, np.array([0.0, 1.0]) / math.sqrt(3))
    return uc
