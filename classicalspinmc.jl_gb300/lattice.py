"""Lattice, mirroring lattice.jl, backed by the native flattener of libcsmc.so.

A ``Lattice`` holds the unit cell, the shape, S, the boundary condition and
the spins as the reference's 3 x N column-major Float64 array (numpy shape
(3, N), Fortran order, so memory is x,y,z interleaved per site exactly as in
Julia).  Its per-site interaction tables are built by the C++ flattener
(``csmc_lattice_tables``) with index arithmetic instead of the reference's
O(N^2) ``findfirst`` scan; they are exported on demand in the reference's
layout (``bilinear_sites`` etc., 1-based, 0 = absent).

Site arguments named ``point`` are 1-based, as in the reference.
"""
from __future__ import annotations

import copy
import ctypes as C
import math

import numpy as np

from . import _lib
from .unit_cell import UnitCell, addBasisSite


def random_spin_orientation(S: float, rng=None) -> tuple:
    """random_spin_orientation (lattice.jl:306-311)."""
    rng = np.random.default_rng() if rng is None else rng
    phi = 2.0 * math.pi * rng.random()
    z = 2.0 * rng.random() - 1.0
    r = math.sqrt(1.0 - z * z)
    return (S * (r * math.cos(phi)), S * (r * math.sin(phi)), S * z)


def set_spin(spins: np.ndarray, newspin, point: int) -> None:
    """set_spin! (lattice.jl:297-301); point is 1-based."""
    spins[:, point - 1] = newspin


def get_spin(spins: np.ndarray, point: int) -> tuple:
    """get_spin (lattice.jl:293-295); point is 1-based."""
    return tuple(float(v) for v in spins[:, point - 1])


class Description:
    """A csmc_lattice_desc with the numpy buffers it points into kept alive."""

    def __init__(self, uc: UnitCell, shape: tuple, S: float, bc: str):
        D = uc.D
        if bc not in ("periodic", "open"):
            raise ValueError("Invalid boundary condition option")  # lattice.jl:107
        if len(shape) != D:
            raise ValueError(f"shape {shape} must have {D} entries")
        self.keep = []
        d = _lib.LatticeDesc()
        d.dim = D
        d.n_basis = len(uc.basis)
        for k in range(3):
            d.shape[k] = int(shape[k]) if k < D else 1
        d.periodic = 1 if bc == "periodic" else 0
        d.spin_length = float(S)

        def i32(rows, width):
            a = np.ascontiguousarray(np.asarray(rows, dtype=np.int32).reshape(-1, width) if rows else
                                     np.zeros((0, width), np.int32))
            self.keep.append(a)
            return a.ctypes.data_as(_lib.i32p)

        def f64(rows, width):
            a = np.ascontiguousarray(np.asarray(rows, dtype=np.float64).reshape(-1, width) if rows else
                                     np.zeros((0, width), np.float64))
            self.keep.append(a)
            return a.ctypes.data_as(_lib.f64p)

        d.n_field = len(uc.field)
        d.field_basis = i32([b for b, _ in uc.field], 1)
        d.field_vec = f64([h for _, h in uc.field], 3)
        d.n_onsite = len(uc.onsite)
        d.onsite_basis = i32([b for b, _ in uc.onsite], 1)
        d.onsite_mat = f64([m.reshape(9) for _, m in uc.onsite], 9)
        d.n_bilinear = len(uc.bilinear)
        d.bilinear_basis = i32([(t[0], t[1]) for t in uc.bilinear], 2)
        d.bilinear_mat = f64([t[2].reshape(9) for t in uc.bilinear], 9)
        d.bilinear_offset = i32([t[3] for t in uc.bilinear], D)
        d.n_cubic = len(uc.cubic)
        d.cubic_basis = i32([t[:3] for t in uc.cubic], 3)
        d.cubic_tensor = f64([t[3].reshape(27) for t in uc.cubic], 27)
        d.cubic_offset = i32([t[4] + t[5] for t in uc.cubic], 2 * D)
        d.n_quartic = len(uc.quartic)
        d.quartic_basis = i32([t[:4] for t in uc.quartic], 4)
        d.quartic_tensor = f64([t[4].reshape(81) for t in uc.quartic], 81)
        d.quartic_offset = i32([t[5] + t[6] + t[7] for t in uc.quartic], 3 * D)
        self.desc = d

    def ref(self):
        return C.byref(self.desc)


class Lattice:
    """Lattice(shape, uc, S=1/2; bc="periodic", initialCondition=:random) (lattice.jl:65-291)."""

    def __init__(self, shape, uc: UnitCell, S: float = 0.5, bc: str = "periodic",
                 initialCondition: str = "random", rng=None):
        shape = tuple(int(s) for s in shape)
        if len(uc.basis) == 0:  # lattice.jl:68-70
            addBasisSite(uc, np.zeros(uc.D))
        self.unit_cell = uc
        self.S = S
        self.bc = bc
        self.shape = shape
        nb = len(uc.basis)
        self.size = int(np.prod(shape)) * nb
        self._desc = Description(uc, shape, S, bc)
        info = _lib.LatticeInfo()
        _lib.call("csmc_lattice_plan", self._desc.ref(), C.byref(info))
        self.info = info
        rng = np.random.default_rng() if rng is None else rng
        self.spins = np.zeros((3, self.size), dtype=np.float64, order="F")
        if initialCondition in ("random", ":random"):
            for i in range(self.size):
                self.spins[:, i] = random_spin_orientation(S, rng)
        elif initialCondition in ("fm", ":fm"):
            s = random_spin_orientation(S, rng)
            for i in range(self.size):
                self.spins[:, i] = s
        self.site_positions = self._positions()
        self._tables = None

    @property
    def desc(self) -> Description:
        return self._desc

    @property
    def spins(self) -> np.ndarray:
        """lattice.spins (lattice.jl:73), 3 x N.  A MonteCarlo that swept this
        lattice on the device leaves a pending read here (``_pull``); the
        configuration is copied back on first access, not after every sweep."""
        pull = self.__dict__.get("_pull")
        if pull is not None:
            self.__dict__["_pull"] = None
            self.__dict__["_spins"] = pull()
        return self.__dict__["_spins"]

    @spins.setter
    def spins(self, value) -> None:
        self.__dict__["_pull"] = None
        self.__dict__["_spins"] = value

    def __deepcopy__(self, memo):
        """deepcopy(lattice) (monte_carlo.jl:74): the ctypes description is rebuilt, not copied."""
        new = Lattice.__new__(Lattice)
        memo[id(self)] = new
        _ = self.spins  # a pending device read is resolved before copying
        for k, v in self.__dict__.items():
            if k in ("_desc", "_ctx", "_tables", "info", "_pull"):
                continue
            setattr(new, k, copy.deepcopy(v, memo))
        new._desc = Description(new.unit_cell, new.shape, new.S, new.bc)
        info = _lib.LatticeInfo()
        _lib.call("csmc_lattice_plan", new._desc.ref(), C.byref(info))
        new.info = info
        new._tables = None
        return new

    def _positions(self) -> np.ndarray:
        """compute_site_positions (lattice.jl:38-51)."""
        uc = self.unit_cell
        D = uc.D
        nb = len(uc.basis)
        pos = np.zeros((D, self.size))
        cells = int(np.prod(self.shape))
        idx = np.stack(np.unravel_index(np.arange(cells), self.shape), axis=0)  # last dim fastest
        A = np.stack(uc.lattice_vectors, axis=1)  # D x D, columns = vectors
        base = A @ idx
        for b in range(nb):
            pos[:, b * cells:(b + 1) * cells] = base + uc.basis[b].reshape(D, 1)
        return pos

    def tables(self) -> dict:
        """Per-site tables in the layout of the Lattice struct (lattice.jl:15-22)."""
        if self._tables is None:
            N, n2, n3, n4 = self.size, self.info.n_bilinear, self.info.n_cubic, self.info.n_quartic
            t = dict(
                bilinear_sites=np.zeros((N, n2), np.int64), bilinear_matrices=np.zeros((N, n2, 3, 3)),
                cubic_sites=np.zeros((N, n3, 2), np.int64), cubic_tensors=np.zeros((N, n3, 3, 3, 3)),
                quartic_sites=np.zeros((N, n4, 3), np.int64), quartic_tensors=np.zeros((N, n4, 3, 3, 3, 3)),
                field=np.zeros((N, 3)), onsite=np.zeros((N, 3, 3)))
            _lib.call("csmc_lattice_tables", self._desc.ref(),
                      _lib.ptr(t["bilinear_sites"], C.c_int64), _lib.ptr(t["bilinear_matrices"], C.c_double),
                      _lib.ptr(t["cubic_sites"], C.c_int64), _lib.ptr(t["cubic_tensors"], C.c_double),
                      _lib.ptr(t["quartic_sites"], C.c_int64), _lib.ptr(t["quartic_tensors"], C.c_double),
                      _lib.ptr(t["field"], C.c_double), _lib.ptr(t["onsite"], C.c_double))
            self._tables = t
        return self._tables

    def colouring(self):
        """Colour of each site, device order (reference site per device slot, -1 = padding), class starts."""
        info = self.info
        col = np.zeros(self.size, np.int32)
        order = np.zeros(info.padded_sites, np.int64)
        starts = np.zeros(info.n_colours + 1, np.int64)
        _lib.call("csmc_lattice_colouring", self._desc.ref(), _lib.ptr(col, C.c_int32), _lib.ptr(order, C.c_int64),
                  _lib.ptr(starts, C.c_int64))
        return col, order, starts
