"""Output files in the layout of hdf5.jl (hdf5.jl:1-270), written through the
package's own HDF5 format implementation (``h5format``).

Files and their content, as the reference writes them through HDF5.jl:

  ``<outpath><outprefix>.h5.params``  (create_params_file, hdf5.jl:142-147)
      root attributes: the SimulationParameters fields (Int64) and any
      ``inparams``; ``unit_cell/{lattice_vectors, basis, field/<b>,
      onsite/<b>, bilinear/"(b1,b2),(o..)", cubic/..., quartic/...}``;
      ``lattice/{size, S, bc}``.
  ``<outpath><outprefix>_<r>.h5``  one per replica r (initialize_hdf5,
      hdf5.jl:164-171): attributes ``T`` and ``paramsfile``, datasets
      ``spins`` and ``site_positions``; after the run ``observables/...``
      (write_final_observables, hdf5.jl:204-239) and, with ``corr``,
      ``spin_correlations/{SSF, SSF_momentum}``.
  ``IC_<r>/IC_<t>.h5``  (write_initial_configuration, hdf5.jl:185-194).

Julia arrays are column-major and HDF5.jl writes them with their dimensions
reversed, so a 3 x N spin matrix is an (N, 3) dataset whose bytes are x, y, z
per site; every array here is stored as the transpose of its Julia-order
numpy array and transposed back on reading.  Basis indices in key names are
1-based as in the reference, offsets print as Julia tuples ("(1, 0)",
"(1,)").  HDF5.jl iterates a group's keys in name order, so read_unit_cell
adds the terms in that order, as the reference does.

The ranks of the reference are the replicas (slots) of one MonteCarlo here:
``mc.outpath`` is the file of slot 0 for one replica and the list of the
slots' files for several.
"""
from __future__ import annotations

import ast
import dataclasses
import os

import numpy as np

from . import h5format as _h5
from .h5format import Dataset, Group, H5FormatError  # noqa: F401


class File:
    """h5open(filename, mode): "r" reads, "w" creates (truncating), "r+"
    reads and writes the file back on close.  Indexing, ``attrs``,
    ``create_group`` and ``keys`` act on the root group."""

    def __init__(self, filename: str, mode: str = "r"):
        if mode not in ("r", "w", "r+"):
            raise ValueError(f"unsupported mode {mode!r}")
        self.filename, self.mode = str(filename), mode
        self.root = Group() if mode == "w" else _h5.read(self.filename)
        self._open = True

    def __getitem__(self, path):
        return self.root[path]

    def __setitem__(self, path, value):
        self._writable()
        self.root[path] = value

    def __delitem__(self, path):
        self._writable()
        del self.root[path]

    def __contains__(self, path):
        return path in self.root

    def create_group(self, path) -> Group:
        self._writable()
        return self.root.create_group(path)

    def keys(self):
        return self.root.keys()

    @property
    def attrs(self) -> dict:
        return self.root.attrs

    def _writable(self):
        if self.mode == "r":
            raise PermissionError(f"{self.filename} is open read-only")

    def close(self) -> None:
        if self._open and self.mode != "r":
            _h5.write(self.filename, self.root)
        self._open = False

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        if exc[0] is None:
            self.close()
        self._open = False


def h5open(filename: str, mode: str = "r") -> File:
    return File(filename, mode)


def write_attribute(obj, name: str, value) -> None:
    """HDF5.jl write_attribute: creates the attribute; an existing name is an error."""
    attrs = obj.attrs
    if name in attrs:
        raise KeyError(f"attribute {name!r} already exists")
    attrs[name] = _h5._normalise(value)


def dump_attributes_hdf5(fid, obj) -> None:
    """dump_attributes_hdf5! (hdf5.jl:6-22): a struct's fields (in declaration
    order) or a dictionary's entries as attributes."""
    items = obj.items() if isinstance(obj, dict) else \
        ((f.name, getattr(obj, f.name)) for f in dataclasses.fields(obj))
    for k, v in items:
        write_attribute(fid, str(k), v)


def write_attributes(filename: str, d: dict) -> None:
    """write_attributes (hdf5.jl:27-31)."""
    with h5open(filename, "r+") as f:
        dump_attributes_hdf5(f, d)


def _jl_tuple(t) -> str:
    """Julia's string() of an Int64 tuple."""
    t = tuple(int(x) for x in t)
    return "(" + ", ".join(str(x) for x in t) + ("," if len(t) == 1 else "") + ")"


def _jl(a) -> np.ndarray:
    """A Julia-order array as HDF5.jl stores it (dimensions reversed)."""
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64).T)


def dump_unit_cell(fid, uc) -> None:
    """dump_unit_cell! (hdf5.jl:36-76)."""
    g = fid.create_group("unit_cell")
    D = uc.D
    lv = np.column_stack([np.asarray(v, dtype=np.float64) for v in uc.lattice_vectors])  # D x D, columns = vectors
    g["lattice_vectors"] = _jl(lv)
    basis = np.vstack([np.asarray(b, dtype=np.float64).reshape(1, D) for b in uc.basis]) if uc.basis \
        else np.zeros((0, D))
    g["basis"] = _jl(basis)
    h = g.create_group("field")
    for b, vec in uc.field:
        h[str(b)] = np.asarray(vec, dtype=np.float64)
    o = g.create_group("onsite")
    for b, M in uc.onsite:
        o[str(b)] = _jl(M)
    bl = g.create_group("bilinear")
    for b1, b2, M, off in uc.bilinear:
        bl[f"({b1},{b2}),{_jl_tuple(off)}"] = _jl(M)
    c = g.create_group("cubic")
    for b1, b2, b3, T, o2, o3 in uc.cubic:
        c[f"({b1},{b2},{b3}),{_jl_tuple(o2)},{_jl_tuple(o3)}"] = _jl(T)
    q = g.create_group("quartic")
    for b1, b2, b3, b4, T, o2, o3, o4 in uc.quartic:
        q[f"({b1},{b2},{b3},{b4}),{_jl_tuple(o2)},{_jl_tuple(o3)},{_jl_tuple(o4)}"] = _jl(T)


def _read_jl(ds) -> np.ndarray:
    return np.asarray(ds.read(), dtype=np.float64).T


def _parse_key(key: str) -> tuple:
    """eval(Meta.parse(key)) of a term key: a tuple of integer tuples."""
    try:
        v = ast.literal_eval(key)
    except (ValueError, SyntaxError) as e:
        raise H5FormatError(f"bad term key {key!r}") from e
    if not isinstance(v, tuple) or not all(isinstance(x, tuple) for x in v):
        raise H5FormatError(f"bad term key {key!r}")
    return v


def read_unit_cell(fid):
    """read_unit_cell (hdf5.jl:81-120)."""
    from .unit_cell import (UnitCell, addBasisSite, addBilinear, addCubic, addOnSite, addQuartic,
                            addZeemanCoupling)
    g = fid["unit_cell"]
    lv = _read_jl(g["lattice_vectors"])
    uc = UnitCell(*[lv[:, k] for k in range(lv.shape[1])])
    basis = _read_jl(g["basis"])
    for row in basis.reshape(-1, uc.D):
        addBasisSite(uc, row)
    for key in g["field"].keys():
        addZeemanCoupling(uc, int(key), np.asarray(g["field"][key].read(), dtype=np.float64))
    for key in g["onsite"].keys():
        addOnSite(uc, int(key), _read_jl(g["onsite"][key]))
    for key in g["bilinear"].keys():
        bs, off = _parse_key(key)
        addBilinear(uc, *bs, _read_jl(g["bilinear"][key]), off)
    for key in g["cubic"].keys():
        bs, o2, o3 = _parse_key(key)
        addCubic(uc, *bs, _read_jl(g["cubic"][key]), o2, o3)
    for key in g["quartic"].keys():
        bs, o2, o3, o4 = _parse_key(key)
        addQuartic(uc, *bs, _read_jl(g["quartic"][key]), o2, o3, o4)
    return uc


def dump_metadata(fid, mc) -> None:
    """dump_metadata! (hdf5.jl:125-137)."""
    lat = mc.lattice
    dump_unit_cell(fid, lat.unit_cell)
    l = fid.create_group("lattice")  # noqa: E741
    l["size"] = np.asarray(lat.shape, dtype=np.int64)
    l["S"] = float(lat.S)
    l["bc"] = str(lat.bc)
    dump_attributes_hdf5(fid, mc.parameters)


def create_params_file(mc, filename: str) -> str:
    """create_params_file (hdf5.jl:142-147)."""
    with h5open(filename, "w") as f:
        dump_metadata(f, mc)
    return filename


def read_lattice(fid):
    """read_lattice (hdf5.jl:152-159)."""
    from .lattice import Lattice
    l = fid["lattice"]  # noqa: E741
    size = tuple(int(x) for x in np.atleast_1d(l["size"].read()))
    uc = read_unit_cell(fid)
    return Lattice(size, uc, float(l["S"].read()), bc=l["bc"].read())


def _slot_files(mc) -> list:
    return list(mc.outpaths)


def initialize_hdf5(mc, paramsfile: str, slot: int = 0) -> None:
    """initialize_hdf5 (hdf5.jl:164-171) for one replica."""
    with h5open(_slot_files(mc)[slot], "w") as f:
        write_attribute(f, "T", float(mc.temperatures[slot]))
        write_attribute(f, "paramsfile", paramsfile)
        f["spins"] = _jl(mc.spins(slot))
        f["site_positions"] = _jl(mc.lattice.site_positions)


def write_MC_checkpoint(mc, spins=None) -> None:
    """write_MC_checkpoint (hdf5.jl:176-180): every replica's current spins
    overwrite the ``spins`` dataset of its file (``spins``: the slots' 3 x N
    arrays if already downloaded)."""
    for r, fn in enumerate(_slot_files(mc)):
        with h5open(fn, "r+") as f:
            f["spins"][...] = _jl(mc.spins(r) if spins is None else spins[r])


def write_initial_configuration(filename: str, mc, slot: int = 0, spins=None) -> None:
    """write_initial_configuration (hdf5.jl:185-194): T, the params file named
    by the replica's own file, and the spins."""
    with h5open(_slot_files(mc)[slot], "r") as p:
        paramsfile = p.attrs["paramsfile"]
    with h5open(filename, "w") as f:
        write_attribute(f, "T", float(mc.temperatures[slot]))
        write_attribute(f, "paramsfile", paramsfile)
        f["spins"] = _jl(mc.spins(slot) if spins is None else spins)


def write_final_observables(mc, verbose: bool = True) -> None:
    """write_final_observables (hdf5.jl:204-239) for every replica.  As in the
    reference, specific_heat_err and susceptibility_err are relative errors
    (|error / value|), magnetization_err and energy_err standard errors."""
    from .observables import mean_and_error, specific_heat, susceptibility
    N = mc.lattice.size
    for r, fn in enumerate(_slot_files(mc)):
        ob = mc.observables[r]
        T = float(mc.temperatures[r])
        with h5open(fn, "r+") as f:
            f["spins"][...] = _jl(mc.spins(r))
            heat, dheat = specific_heat(np.asarray(ob.energy), T, N)
            chi, dchi = susceptibility(np.asarray(ob.magnetization), T, N)
            if "observables" in f:
                g = f["observables"]
                for key in g.keys():
                    del g.children[key]
                if verbose:
                    print(f"Overwriting observables in {fn}")
            else:
                g = f.create_group("observables")
            with np.errstate(divide="ignore", invalid="ignore"):
                g["specific_heat"] = heat
                g["specific_heat_err"] = abs(np.float64(dheat) / heat)
                g["susceptibility"] = chi
                g["susceptibility_err"] = abs(np.float64(dchi) / chi)
            m, dm = mean_and_error(ob.magnetization)
            e, de = mean_and_error(ob.energy)
            g["magnetization"] = m
            g["magnetization_err"] = dm
            g["energy"] = e
            g["energy_err"] = de
            if mc.corr:
                d = f["spin_correlations"] if "spin_correlations" in f else f.create_group("spin_correlations")
                ssf = ob.mean_correlations()
                overwrite_keys(d, {"SSF": _jl(ssf if ssf is not None else np.zeros((9, 0))),
                                   "SSF_momentum": _jl(mc.momentum_vectors)}, verbose)
                if verbose:
                    print(f"Writing spin correlations to {fn}")


def overwrite_keys(fid, d: dict, verbose: bool = True) -> None:
    """overwrite_keys! (hdf5.jl:244-252)."""
    for key, value in d.items():
        if key in fid:
            del fid[key]
            if verbose:
                print(f"Overwriting parameter {key}")
        fid[key] = value


def attributes_to_dict(f) -> dict:
    """attributes_to_dict (hdf5.jl:254-261)."""
    return dict(f.attrs)


def read_spin_configuration(lat, filename: str) -> None:
    """read_spin_configuration! (hdf5.jl:266-270)."""
    with h5open(filename, "r") as f:
        s = _read_jl(f["spins"])
    if s.shape != lat.spins.shape:
        raise ValueError(f"spins of shape {s.shape} in {filename}, lattice has {lat.spins.shape}")
    lat.spins[:, :] = s
