"""A self-contained writer and reader for the subset of the HDF5 file format
that the reference's output files use.

The reference writes its files through HDF5.jl 0.17.2 (libhdf5).  Neither
libhdf5 nor h5py exists on the machines this package targets, so the files
are written here from the published HDF5 File Format Specification, in the
layout libhdf5 produces with its default ("earliest") library-version bounds
-- the layout h5py also writes by default:

  * superblock version 0, 8-byte addresses and lengths, group leaf-node K = 4,
    group internal-node K = 16, no free-space manager, no driver block;
  * version-1 object headers: a 16-byte prefix, then messages whose sizes are
    multiples of 8 bytes;
  * groups stored as symbol tables: a version-1 B-tree of group nodes (node
    type 0) whose leaves are symbol-table nodes of 2K = 8 entries sorted by
    name, and one local heap holding the names;
  * datasets: dataspace message version 1, datatype message version 1 (IEEE
    little-endian float64, two's-complement int64, fixed-length strings),
    contiguous storage through a version-3 layout message;
  * attributes: version-1 attribute messages in the object header.

The reader accepts these structures plus the variants a libhdf5-written file
of the same content may hold (continuation messages, version-2 object headers,
compact-storage link messages, compact data layout, big-endian and other-width
numbers); it rejects what it does not implement (chunked or filtered data,
dense link or attribute storage, variable-length strings) with H5FormatError.

Arrays are stored in C order with the shape given: HDF5.jl stores a Julia
array with its dimensions reversed, so callers that mirror Julia pass arr.T.
"""
from __future__ import annotations

import os
import struct

import numpy as np

SIGNATURE = b"\x89HDF\r\n\x1a\n"
UNDEF = 0xFFFFFFFFFFFFFFFF
LEAF_K, NODE_K = 4, 16
SNOD_SIZE = 8 + 2 * LEAF_K * 40              # symbol-table node: header + 2K entries
TREE_SIZE = 24 + 2 * NODE_K * 8 + (2 * NODE_K + 1) * 8  # group B-tree node: header + 2K children + 2K+1 keys
HEAP_PREFIX = 32
FREE_NULL = 1                                # end-of-free-list marker of a local heap

# object header message types
M_NIL, M_DATASPACE, M_LINKINFO, M_DATATYPE, M_FILL_OLD, M_FILL, M_LINK = 0x0, 0x1, 0x2, 0x3, 0x4, 0x5, 0x6
M_LAYOUT, M_GROUPINFO, M_FILTERS, M_ATTRIBUTE, M_CONT, M_STAB, M_ATTRINFO = 0x8, 0xA, 0xB, 0xC, 0x10, 0x11, 0x15


class H5FormatError(ValueError):
    """A file, or a part of one, outside the implemented subset of the format."""


def _pad8(b: bytes) -> bytes:
    return b + b"\0" * (-len(b) % 8)


# ----------------------------------------------------------------------------- tree

class Dataset:
    """A dataset: a numpy array (float64 or int64, any shape, scalars as
    0-d arrays) or a string, with attributes."""

    def __init__(self, data, attrs=None):
        self.data = _normalise(data)
        self.attrs = dict(attrs or {})

    def __getitem__(self, key):
        return self.data[key]

    def __setitem__(self, key, value):
        """In-place write, as ``file["spins"][:, :] = spins`` (hdf5.jl:178)."""
        if isinstance(self.data, str):
            raise TypeError("string datasets are replaced, not written in place")
        self.data[key] = value

    def read(self):
        return self.data.copy() if isinstance(self.data, np.ndarray) else self.data

    @property
    def shape(self):
        return () if isinstance(self.data, str) else self.data.shape


class Group:
    """A group: named children (Group or Dataset) and attributes.  Paths with
    '/' address nested members."""

    def __init__(self):
        self.children: dict[str, Group | Dataset] = {}
        self.attrs: dict = {}

    def _walk(self, path: str, create: bool = False):
        parts = [p for p in path.split("/") if p]
        g = self
        for p in parts[:-1]:
            if p not in g.children:
                if not create:
                    raise KeyError(path)
                g.children[p] = Group()
            g = g.children[p]
            if not isinstance(g, Group):
                raise KeyError(f"{path}: {p} is a dataset")
        if not parts:
            raise KeyError("empty path")
        return g, parts[-1]

    def __getitem__(self, path: str):
        g, name = self._walk(path)
        return g.children[name]

    def __contains__(self, path: str) -> bool:
        try:
            self[path]
            return True
        except KeyError:
            return False

    def __setitem__(self, path: str, value):
        """``g[name] = value`` creates a dataset; like HDF5.jl it refuses to replace one."""
        g, name = self._walk(path, create=True)
        _check_name(name)
        if name in g.children:
            raise KeyError(f"object {path!r} already exists")
        g.children[name] = value if isinstance(value, (Dataset, Group)) else Dataset(value)

    def __delitem__(self, path: str):
        g, name = self._walk(path)
        del g.children[name]

    def create_group(self, path: str) -> "Group":
        g, name = self._walk(path, create=True)
        _check_name(name)
        if name in g.children:
            raise KeyError(f"object {path!r} already exists")
        g.children[name] = Group()
        return g.children[name]

    def keys(self) -> list[str]:
        """Member names in the order libhdf5 iterates a symbol table (byte order)."""
        return sorted(self.children, key=lambda s: s.encode())


def _check_name(name: str) -> None:
    if not name or "/" in name or "\0" in name or name == ".":
        raise ValueError(f"invalid HDF5 link name {name!r}")


def _normalise(v):
    if isinstance(v, bytes):
        return v.decode("utf-8")
    if isinstance(v, str):
        return v
    a = np.asarray(v)
    if a.dtype.kind == "b":
        a = a.astype(np.int64)
    if a.dtype.kind in "iu":
        return np.array(a, dtype=np.int64)
    if a.dtype.kind == "f":
        return np.array(a, dtype=np.float64)
    raise TypeError(f"cannot store {type(v).__name__} of dtype {a.dtype} (float64, int64 and str are supported)")


# ----------------------------------------------------------------------------- encoding

def _dtype_msg(v) -> bytes:
    """Datatype message version 1 (class in the low nibble of the first byte)."""
    if isinstance(v, str):
        n = max(1, len(v.encode("utf-8")))
        return struct.pack("<BBBBI", 0x13, 0x10, 0, 0, n)  # null-terminated padding, UTF-8
    if v.dtype == np.float64:
        # little-endian, implied mantissa MSB, sign bit 63; offset 0, precision 64,
        # exponent at bit 52 (11 bits), mantissa at 0 (52 bits), bias 1023
        return struct.pack("<BBBBI", 0x11, 0x20, 63, 0, 8) + struct.pack("<HHBBBBI", 0, 64, 52, 11, 0, 52, 1023)
    # little-endian signed two's complement, offset 0, precision 64
    return struct.pack("<BBBBI", 0x10, 0x08, 0, 0, 8) + struct.pack("<HH", 0, 64)


def _dspace_msg(shape) -> bytes:
    """Dataspace message version 1: rank 0 is a scalar."""
    return struct.pack("<BBBBI", 1, len(shape), 0, 0, 0) + b"".join(struct.pack("<Q", int(d)) for d in shape)


def _raw(v) -> bytes:
    if isinstance(v, str):
        b = v.encode("utf-8")
        return b if b else b"\0"
    return np.ascontiguousarray(v, dtype=v.dtype.newbyteorder("<")).tobytes()


def _shape(v) -> tuple:
    return () if isinstance(v, str) else v.shape


def _attr_msg(name: str, value) -> bytes:
    v = _normalise(value)
    nb = name.encode("utf-8") + b"\0"
    dt, ds = _dtype_msg(v), _dspace_msg(_shape(v))
    body = struct.pack("<BBHHH", 1, 0, len(nb), len(dt), len(ds)) + _pad8(nb) + _pad8(dt) + _pad8(ds) + _raw(v)
    if len(body) > 0xFFF0:
        raise ValueError(f"attribute {name!r} is too large for an object-header message")
    return body


def _msg(mtype: int, body: bytes, flags: int = 0) -> bytes:
    body = _pad8(body)
    return struct.pack("<HHB3x", mtype, len(body), flags) + body


def _header(msgs: list[bytes]) -> bytes:
    """Version-1 object header: version, reserved, #messages, reference count,
    size of the message area, 4 bytes of alignment padding, messages."""
    area = b"".join(msgs)
    return struct.pack("<BBHII4x", 1, 0, len(msgs), 1, len(area)) + area


def _entry(name_off: int, header: int, stab=None) -> bytes:
    """Symbol-table entry: name offset, header address, cache type, scratch pad."""
    if stab is None:
        return struct.pack("<QQI4x16x", name_off, header, 0)
    return struct.pack("<QQI4xQQ", name_off, header, 1, stab[0], stab[1])


# ----------------------------------------------------------------------------- writer

class _Out:
    """The file image: allocations are appended (8-byte aligned) and filled in later."""

    def __init__(self):
        self.b = bytearray(96)  # the superblock

    def alloc(self, n: int) -> int:
        self.b += b"\0" * (-len(self.b) % 8)
        a = len(self.b)
        self.b += b"\0" * n
        return a

    def put(self, addr: int, data: bytes) -> None:
        self.b[addr:addr + len(data)] = data


def _emit_btree(out: _Out, leaves: list[tuple[int, int]], root: int | None = None) -> int:
    """Group B-tree over the symbol-table nodes ``leaves`` = [(address, heap
    offset of the node's last name)]; returns the root node's address.  Node
    i at a level holds keys k_0..k_n: k_0 is the previous node's last key (the
    empty name, heap offset 0, for the first) and k_{j+1} the last name under
    child j.  Siblings are linked at every level.  ``root``: space already
    allocated for a tree of one node."""
    level, nodes = 0, leaves
    while True:
        groups = [nodes[i:i + 2 * NODE_K] for i in range(0, len(nodes), 2 * NODE_K)] or [[]]
        if root is not None and len(groups) == 1 and level == 0:
            addrs = [root]
        else:
            addrs = [out.alloc(TREE_SIZE) for _ in groups]
        up, left_key = [], 0
        for i, (grp, a) in enumerate(zip(groups, addrs)):
            left = addrs[i - 1] if i > 0 else UNDEF
            right = addrs[i + 1] if i + 1 < len(addrs) else UNDEF
            body = bytearray(b"TREE" + struct.pack("<BBHQQ", 0, level, len(grp), left, right))
            body += struct.pack("<Q", left_key)
            for child, key in grp:
                body += struct.pack("<QQ", child, key)
            out.put(a, bytes(body))
            if grp:
                left_key = grp[-1][1]
            up.append((a, left_key))
        if len(addrs) == 1:
            return addrs[0]
        level, nodes = level + 1, up


def _emit_group(out: _Out, g: Group) -> tuple[int, int, int]:
    """Object header, local heap, symbol-table nodes and B-tree of a group,
    then its members; returns (header, B-tree, heap) addresses."""
    names = g.keys()
    attrs = [_msg(M_ATTRIBUTE, _attr_msg(k, v)) for k, v in g.attrs.items()]
    hdr = out.alloc(len(_header([_msg(M_STAB, bytes(16))] + attrs)))
    chunks = [names[i:i + 2 * LEAF_K] for i in range(0, len(names), 2 * LEAF_K)]
    # a one-node B-tree sits between the header and the heap, as libhdf5 places it
    root = out.alloc(TREE_SIZE) if len(chunks) <= 2 * NODE_K else None
    # local heap: the empty name at offset 0, then the member names, each
    # null-terminated and padded to 8 bytes; no free block
    heap_data, offs = bytearray(8), {}
    for n in names:
        offs[n] = len(heap_data)
        heap_data += _pad8(n.encode("utf-8") + b"\0")
    heap = out.alloc(HEAP_PREFIX)
    data = out.alloc(len(heap_data))
    out.put(heap, b"HEAP" + struct.pack("<B3xQQQ", 0, len(heap_data), FREE_NULL, data))
    out.put(data, bytes(heap_data))
    snods = [out.alloc(SNOD_SIZE) for _ in chunks]
    btree = _emit_btree(out, [(a, offs[c[-1]]) for a, c in zip(snods, chunks)], root)
    entries = {}
    for n in names:
        child = g.children[n]
        if isinstance(child, Group):
            a, bt, hp = _emit_group(out, child)
            entries[n] = _entry(offs[n], a, (bt, hp))
        else:
            entries[n] = _entry(offs[n], _emit_dataset(out, child))
    for a, c in zip(snods, chunks):
        out.put(a, b"SNOD" + struct.pack("<BBH", 1, 0, len(c)) + b"".join(entries[n] for n in c))
    out.put(hdr, _header([_msg(M_STAB, struct.pack("<QQ", btree, heap))] + attrs))
    return hdr, btree, heap


def _emit_dataset(out: _Out, d: Dataset) -> int:
    v = d.data
    raw = _raw(v)
    attrs = [_msg(M_ATTRIBUTE, _attr_msg(k, x)) for k, x in d.attrs.items()]
    head = [_msg(M_DATASPACE, _dspace_msg(_shape(v))), _msg(M_DATATYPE, _dtype_msg(v), flags=1)]
    hdr = out.alloc(len(_header(head + [_msg(M_LAYOUT, bytes(18))] + attrs)))
    addr = out.alloc(len(raw)) if raw else UNDEF
    if raw:
        out.put(addr, raw)
    layout = _msg(M_LAYOUT, struct.pack("<BBQQ", 3, 1, addr, len(raw)))  # version 3, contiguous
    out.put(hdr, _header(head + [layout] + attrs))
    return hdr


def encode(root: Group) -> bytes:
    """The HDF5 file image of ``root``."""
    out = _Out()
    hdr, btree, heap = _emit_group(out, root)
    sb = SIGNATURE + struct.pack("<BBBBBBBBHHI", 0, 0, 0, 0, 0, 8, 8, 0, LEAF_K, NODE_K, 0)
    # base address, superblock extension (free-space) address, end of file, driver block
    sb += struct.pack("<QQQQ", 0, UNDEF, len(out.b), UNDEF)
    sb += _entry(0, hdr, (btree, heap))
    assert len(sb) == 96
    out.put(0, sb)
    return bytes(out.b)


def write(path: str, root: Group) -> None:
    """Write ``root`` to ``path`` (through a temporary file and a rename, so a
    reader never sees a partly written file)."""
    img = encode(root)
    tmp = f"{path}.tmp{os.getpid()}"
    with open(tmp, "wb") as f:
        f.write(img)
    os.replace(tmp, path)


# ----------------------------------------------------------------------------- reader

class _In:
    def __init__(self, data: bytes):
        self.d = data

    def u(self, fmt: str, at: int):
        try:
            return struct.unpack_from("<" + fmt, self.d, at)
        except struct.error as e:
            raise H5FormatError(f"truncated file at {at}: {e}") from None

    def cstr(self, at: int) -> str:
        end = self.d.find(b"\0", at)
        if end < 0:
            raise H5FormatError(f"unterminated name at {at}")
        return self.d[at:end].decode("utf-8")


def _messages(f: _In, addr: int) -> list[tuple[int, bytes]]:
    """(type, body) of every message of the object header at ``addr``, over
    all its chunks (continuation messages followed)."""
    out, chunks = [], []
    if f.d[addr:addr + 4] == b"OHDR":  # version-2 header
        ver, flags = f.u("BB", addr + 4)
        if ver != 2:
            raise H5FormatError(f"object header version {ver}")
        p = addr + 6 + (16 if flags & 0x20 else 0) + (4 if flags & 0x10 else 0)
        w = 1 << (flags & 3)
        size = int.from_bytes(f.d[p:p + w], "little")
        chunks.append((p + w, p + w + size, 2, flags))
    else:
        ver, _, nmsg, _, size = f.u("BBHII", addr)
        if ver != 1:
            raise H5FormatError(f"object header version {ver} at {addr}")
        chunks.append((addr + 16, addr + 16 + size, 1, 0))
    while chunks:
        p, end, ver, flags = chunks.pop(0)
        while p + (8 if ver == 1 else 4) <= end:
            if ver == 1:
                mtype, msize, mflags = f.u("HHB", p)
                p += 8
            else:
                mtype, msize, mflags = f.u("BHB", p)
                p += 4 + (2 if flags & 0x04 else 0)
            body = f.d[p:p + msize]
            if len(body) != msize or p + msize > end:
                raise H5FormatError(f"object header message overruns its chunk at {p}")
            p += msize
            if mflags & 0x02:
                raise H5FormatError("shared object header messages are not supported")
            if mtype == M_CONT:
                caddr, clen = struct.unpack_from("<QQ", body)
                if ver == 1:
                    chunks.append((caddr, caddr + clen, 1, 0))
                else:
                    if f.d[caddr:caddr + 4] != b"OCHK":
                        raise H5FormatError("bad continuation chunk signature")
                    chunks.append((caddr + 4, caddr + clen - 4, 2, flags))
            elif mtype != M_NIL:
                out.append((mtype, body))
        if ver == 2:
            pass  # the gap and the checksum close a version-2 chunk
    return out


def _parse_dtype(b: bytes, at: int = 0):
    """A numpy dtype, or ('str', size) for a fixed-length string."""
    cv, b0, b1, b2, size = struct.unpack_from("<BBBBI", b, at)
    cls = cv & 0x0F
    be = bool(b0 & 1)
    if cls == 0:
        kind = "i" if b0 & 0x08 else "u"
        if size not in (1, 2, 4, 8):
            raise H5FormatError(f"integer of {size} bytes")
        return np.dtype((">" if be else "<") + kind + str(size))
    if cls == 1:
        if size not in (2, 4, 8):
            raise H5FormatError(f"float of {size} bytes")
        return np.dtype((">" if be else "<") + "f" + str(size))
    if cls == 3:
        return ("str", size, b0 & 0x0F)
    raise H5FormatError(f"datatype class {cls} is not supported")


def _parse_dspace(b: bytes, at: int = 0) -> tuple:
    ver, rank, flags = struct.unpack_from("<BBB", b, at)
    if ver == 1:
        p = at + 8
    elif ver == 2:
        if b[at + 3] == 2:
            return None  # null dataspace
        p = at + 4
    else:
        raise H5FormatError(f"dataspace version {ver}")
    return tuple(struct.unpack_from("<" + "Q" * rank, b, p))


def _decode(raw: bytes, dt, shape):
    n = int(np.prod(shape)) if shape else 1
    if isinstance(dt, tuple):
        _, size, pad = dt
        if n != 1:
            raise H5FormatError("string arrays are not supported")
        s = raw[:size]
        if pad in (0, 1):
            s = s.split(b"\0", 1)[0]
        else:
            s = s.rstrip(b" ")
        return s.decode("utf-8")
    a = np.frombuffer(raw, dtype=dt, count=n).astype(dt.newbyteorder("="))
    a = a.reshape(shape) if shape else a.reshape(())
    if a.dtype.kind in "iu":
        return a.astype(np.int64)
    return a.astype(np.float64)


def _parse_attr(b: bytes):
    ver = b[0]
    if ver == 1:
        nlen, dlen, slen = struct.unpack_from("<HHH", b, 2)
        p = 8
        al = lambda n: (n + 7) // 8 * 8  # noqa: E731
    elif ver in (2, 3):
        if b[1] & 0x03:
            raise H5FormatError("shared attribute datatypes are not supported")
        nlen, dlen, slen = struct.unpack_from("<HHH", b, 2)
        p = 8 + (1 if ver == 3 else 0)
        al = lambda n: n  # noqa: E731
    else:
        raise H5FormatError(f"attribute message version {ver}")
    name = b[p:p + nlen].split(b"\0", 1)[0].decode("utf-8")
    p += al(nlen)
    dt = _parse_dtype(b, p)
    p += al(dlen)
    shape = _parse_dspace(b, p)
    p += al(slen)
    v = _decode(b[p:], dt, shape)
    if isinstance(v, np.ndarray) and v.ndim == 0:
        v = v[()]  # a scalar attribute reads as a numpy scalar
    return name, v


def _read_symbol_table(f: _In, btree: int, heap: int) -> dict[str, int]:
    if f.d[heap:heap + 4] != b"HEAP":
        raise H5FormatError("bad local heap signature")
    _, dsize, _, daddr = f.u("B3xQQQ", heap + 4)
    out = {}

    def node(a):
        if f.d[a:a + 4] != b"TREE":
            raise H5FormatError("bad B-tree node signature")
        ntype, level, n = f.u("BBH", a + 4)
        if ntype != 0:
            raise H5FormatError(f"B-tree node type {ntype} in a group")
        p = a + 24 + 8
        for _ in range(n):
            (child,) = f.u("Q", p)
            p += 16
            if level > 0:
                node(child)
            else:
                if f.d[child:child + 4] != b"SNOD":
                    raise H5FormatError("bad symbol-table node signature")
                (cnt,) = f.u("H", child + 6)
                for k in range(cnt):
                    name_off, header = f.u("QQ", child + 8 + 40 * k)
                    if name_off >= dsize:
                        raise H5FormatError("link name outside the local heap")
                    out[f.cstr(daddr + name_off)] = header

    node(btree)
    return out


def _parse_link(b: bytes) -> tuple[str, int] | None:
    ver, flags = b[0], b[1]
    if ver != 1:
        raise H5FormatError(f"link message version {ver}")
    p = 2
    ltype = 0
    if flags & 0x08:
        ltype = b[p]
        p += 1
    if flags & 0x04:
        p += 8
    if flags & 0x10:
        p += 1
    w = 1 << (flags & 3)
    nlen = int.from_bytes(b[p:p + w], "little")
    p += w
    name = b[p:p + nlen].decode("utf-8")
    p += nlen
    if ltype != 0:
        return None  # soft and external links are skipped
    return name, struct.unpack_from("<Q", b, p)[0]


def _read_object(f: _In, addr: int, depth: int = 0):
    if depth > 64:
        raise H5FormatError("group nesting too deep (a cycle?)")
    msgs = _messages(f, addr)
    types = {t for t, _ in msgs}
    attrs = {}
    for t, b in msgs:
        if t == M_ATTRIBUTE:
            k, v = _parse_attr(b)
            attrs[k] = v
        elif t == M_ATTRINFO and struct.unpack_from("<Q", b, 2 + (2 if b[1] & 1 else 0))[0] != UNDEF:
            raise H5FormatError("dense attribute storage is not supported")
    if M_LAYOUT in types:
        shape = dt = layout = None
        for t, b in msgs:
            if t == M_DATASPACE:
                shape = _parse_dspace(b)
            elif t == M_DATATYPE:
                dt = _parse_dtype(b)
            elif t == M_LAYOUT:
                layout = b
            elif t == M_FILTERS:
                raise H5FormatError("filtered datasets are not supported")
        if layout[0] != 3:
            raise H5FormatError(f"layout message version {layout[0]}")
        if layout[1] == 0:
            (n,) = struct.unpack_from("<H", layout, 2)
            raw = layout[4:4 + n]
        elif layout[1] == 1:
            a, n = struct.unpack_from("<QQ", layout, 2)
            raw = b"" if a == UNDEF else f.d[a:a + n]
            if a != UNDEF and len(raw) != n:
                raise H5FormatError("dataset storage beyond the end of the file")
        else:
            raise H5FormatError("chunked datasets are not supported")
        if shape is None:
            raise H5FormatError("dataset without a dataspace")
        if isinstance(dt, tuple):
            data = _decode(raw, dt, shape)
        elif not raw:
            data = np.zeros(shape, dtype=np.int64 if dt.kind in "iu" else np.float64)
        else:
            data = _decode(raw, dt, shape)
        return Dataset(data, attrs)
    g = Group()
    g.attrs = attrs
    members = {}
    for t, b in msgs:
        if t == M_STAB:
            members.update(_read_symbol_table(f, *struct.unpack_from("<QQ", b)))
        elif t == M_LINK:
            lk = _parse_link(b)
            if lk:
                members[lk[0]] = lk[1]
        elif t == M_LINKINFO:
            off = 2 + (8 if b[1] & 1 else 0)
            if struct.unpack_from("<Q", b, off)[0] != UNDEF:
                raise H5FormatError("dense link storage is not supported")
    for name, a in members.items():
        g.children[name] = _read_object(f, a, depth + 1)
    return g


def decode(data: bytes) -> Group:
    """The tree of an HDF5 file image (superblock at offset 0)."""
    f = _In(data)
    if data[:8] != SIGNATURE:
        raise H5FormatError("not an HDF5 file (no signature at offset 0)")
    ver = data[8]
    if ver in (0, 1):
        so, sl = f.u("BB", 13)
        if (so, sl) != (8, 8):
            raise H5FormatError(f"{so}-byte addresses / {sl}-byte lengths are not supported")
        p = 24 + (4 if ver == 1 else 0)
        base, _, eof, _ = f.u("QQQQ", p)
        _, root = f.u("QQ", p + 32)
    elif ver in (2, 3):
        so, sl = f.u("BB", 9)
        if (so, sl) != (8, 8):
            raise H5FormatError(f"{so}-byte addresses / {sl}-byte lengths are not supported")
        base, _, eof, root = f.u("QQQQ", 12)
    else:
        raise H5FormatError(f"superblock version {ver}")
    if base != 0:
        raise H5FormatError("a user block / nonzero base address is not supported")
    if eof > len(data):
        raise H5FormatError(f"truncated file: end of file {eof} > size {len(data)}")
    return _read_object(f, root)


def read(path: str) -> Group:
    with open(path, "rb") as fh:
        return decode(fh.read())
