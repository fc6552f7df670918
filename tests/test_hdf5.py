"""HDF5 output in the layout of hdf5.jl (no GPU).

There is no libhdf5 or h5py on these machines to read the files back, so
the format is checked three ways: (1) the empty file's bytes against the
layout libhdf5 gives an empty file with default settings (superblock
version 0; root object header at 96, its B-tree at 136, its local heap at
680 -- libhdf5's heap then carries an 80-byte free block this writer leaves
out); (2) an independent walk of every file written here that checks the
invariants of the published format (alignment, message sizes, sorted symbol
nodes, B-tree keys, heap names, storage sizes, no overlapping structures);
(3) round trips through the package's reader.  The hdf5.jl functions are
tested as test/h5tests.jl tests them (dump_metadata! then read_unit_cell and
read_lattice), on more models."""
import ast
import struct
import types

import numpy as np
import pytest

UNDEF = 0xFFFFFFFFFFFFFFFF


@pytest.fixture(scope="module")
def h5(m):
    import importlib
    return importlib.import_module(m.__name__ + ".hdf5")


@pytest.fixture(scope="module")
def fmt(m):
    import importlib
    return importlib.import_module(m.__name__ + ".h5format")


# ------------------------------------------------------------------ an independent format walk

def validate(img: bytes) -> dict:
    """Walk a file image as the format specification describes it; return
    {path: ("group"|"dataset", header address)}.  Asserts every invariant."""
    assert img[:8] == b"\x89HDF\r\n\x1a\n"
    assert img[8:16] == bytes([0, 0, 0, 0, 0, 8, 8, 0])  # versions, reserved, 8-byte offsets/lengths
    leaf_k, node_k, flags = struct.unpack_from("<HHI", img, 16)
    assert (leaf_k, node_k, flags) == (4, 16, 0)
    base, ext, eof, drv = struct.unpack_from("<QQQQ", img, 24)
    assert base == 0 and ext == UNDEF and drv == UNDEF and eof == len(img)
    used = []  # [start, end) of every structure

    def claim(a, n):
        assert a % 8 == 0 and a + n <= len(img), (a, n)
        used.append((a, a + n))

    def entry(at):
        off, hdr, cache = struct.unpack_from("<QQI", img, at)
        assert img[at + 20:at + 24] == b"\0" * 4
        scratch = struct.unpack_from("<QQ", img, at + 24) if cache == 1 else None
        assert cache in (0, 1)
        return off, hdr, scratch

    claim(0, 96)
    off, root, scratch = entry(56)
    assert off == 0
    out = {}

    def header(a, peek=False):
        ver, res, n, refc, size = struct.unpack_from("<BBHII", img, a)
        assert (ver, res, refc) == (1, 0, 1) and img[a + 12:a + 16] == b"\0" * 4
        if not peek:
            claim(a, 16 + size)
        p, msgs = a + 16, []
        while p < a + 16 + size:
            t, s, fl = struct.unpack_from("<HHB", img, p)
            assert s % 8 == 0 and img[p + 5:p + 8] == b"\0" * 3 and fl in (0, 1)
            msgs.append((t, img[p + 8:p + 8 + s]))
            p += 8 + s
        assert p == a + 16 + size and len(msgs) == n
        return msgs

    def heap_name(data, dsize, o):
        assert 0 <= o < dsize
        return img[data + o:img.index(b"\0", data + o)]

    def group(a, path, cached):
        msgs = header(a)
        stab = [b for t, b in msgs if t == 0x11]
        assert len(stab) == 1 and all(t in (0x11, 0xC) for t, _ in msgs)
        btree, heap = struct.unpack_from("<QQ", stab[0])
        if cached is not None:
            assert tuple(cached) == (btree, heap)
        assert img[heap:heap + 8] == b"HEAP\0\0\0\0"
        dsize, free, data = struct.unpack_from("<QQQ", img, heap + 8)
        claim(heap, 32)
        claim(data, dsize)
        assert dsize % 8 == 0 and free == 1 and img[data:data + 8] == b"\0" * 8
        names = []

        def node(b, lo, hi, level_expected=None):
            assert img[b:b + 5] == b"TREE\0"
            level, n = struct.unpack_from("<BH", img, b + 5)
            if level_expected is not None:
                assert level == level_expected
            claim(b, 544)
            assert n <= 32
            keys = [struct.unpack_from("<Q", img, b + 24 + 16 * i)[0] for i in range(n + 1)]
            kids = [struct.unpack_from("<Q", img, b + 32 + 16 * i)[0] for i in range(n)]
            kn = [heap_name(data, dsize, k) for k in keys]
            if n:
                assert kn[0] == lo and kn[-1] == hi
                assert all(x < y for x, y in zip(kn, kn[1:]))
            for i, c in enumerate(kids):
                if level > 0:
                    node(c, kn[i], kn[i + 1], level - 1)
                else:
                    assert img[c:c + 6] == b"SNOD\x01\0"
                    (cnt,) = struct.unpack_from("<H", img, c + 6)
                    claim(c, 8 + 8 * 40)
                    assert 1 <= cnt <= 8
                    ents = [entry(c + 8 + 40 * j) for j in range(cnt)]
                    nm = [heap_name(data, dsize, e[0]) for e in ents]
                    assert all(x < y for x, y in zip(nm, nm[1:]))
                    assert kn[i] < nm[0] and nm[-1] == kn[i + 1]
                    for name, (_, h, sc) in zip(nm, ents):
                        names.append(name)
                        sub = path + "/" + name.decode()
                        t = {t for t, _ in header(h, peek=True)}
                        if 0x11 in t:
                            assert sc is not None
                            group(h, sub, sc)
                        else:
                            dataset(h, sub)
            return n

        # the root node's key range: "" .. the last name overall
        assert img[btree:btree + 4] == b"TREE"
        level, n = struct.unpack_from("<BH", img, btree + 5)
        if n:
            last = struct.unpack_from("<Q", img, btree + 24 + 16 * n)[0]
            node(btree, b"", heap_name(data, dsize, last))
        else:
            node(btree, b"", b"")
        assert names == sorted(names)
        out[path or "/"] = ("group", a)

    def dataset(a, path):
        msgs = dict((t, b) for t, b in header(a))
        assert set(msgs) <= {0x1, 0x3, 0x8, 0xC}
        ds, dt, lay = msgs[0x1], msgs[0x3], msgs[0x8]
        assert ds[0] == 1 and ds[2] == 0
        dims = struct.unpack_from("<" + "Q" * ds[1], ds, 8)
        cls, size = dt[0], struct.unpack_from("<I", dt, 4)[0]
        assert cls in (0x10, 0x11, 0x13)
        if cls == 0x11:
            assert dt[1:4] == bytes([0x20, 63, 0]) and struct.unpack_from("<HHBBBBI", dt, 8) == (0, 64, 52, 11, 0, 52, 1023)
        if cls == 0x10:
            assert dt[1] == 0x08 and struct.unpack_from("<HH", dt, 8) == (0, 64)
        assert lay[:2] == b"\x03\x01"
        addr, n = struct.unpack_from("<QQ", lay, 2)
        assert n == int(np.prod(dims)) * size
        if n:
            claim(addr, n)
        else:
            assert addr == UNDEF
        out[path] = ("dataset", a)

    group(root, "", scratch)
    used.sort()
    for (a0, a1), (b0, b1) in zip(used, used[1:]):
        assert a1 <= b0, f"structures overlap: [{a0},{a1}) and [{b0},{b1})"
    return out


# ------------------------------------------------------------------ format

def test_empty_file_matches_libhdf5_layout(fmt):
    img = fmt.encode(fmt.Group())
    assert len(img) == 720  # libhdf5: 800, with an 80-byte free block in the 88-byte heap
    sb = (b"\x89HDF\r\n\x1a\n" + bytes([0, 0, 0, 0, 0, 8, 8, 0]) + struct.pack("<HHI", 4, 16, 0)
          + struct.pack("<QQQQ", 0, UNDEF, 720, UNDEF)
          + struct.pack("<QQI4xQQ", 0, 96, 1, 136, 680))
    assert img[:96] == sb
    # root object header: one symbol-table message (B-tree 136, heap 680)
    assert img[96:136] == struct.pack("<BBHII4x", 1, 0, 1, 1, 24) + struct.pack("<HHB3xQQ", 0x11, 16, 0, 136, 680)
    assert img[136:144] == b"TREE\0\0\0\0" and img[144:160] == b"\xff" * 16
    assert img[680:712] == b"HEAP\0\0\0\0" + struct.pack("<QQQ", 8, 1, 712)
    validate(img)


def _tree(fmt, n_many):
    g = fmt.Group()
    g.attrs.update(T=0.25, paramsfile="out/configuration.h5.params", n=7, v=np.arange(3.0))
    g["spins"] = np.random.default_rng(1).normal(size=(10, 3))
    g["a/b/c"] = np.arange(5)
    g["s"] = "periodic"
    g["empty"] = np.zeros((0, 3))
    g["scalar"] = 1.5
    g.create_group("nothing")
    g.create_group("many")
    for i in range(n_many):
        g[f"many/k{i:04d}"] = float(i)
    g["many"].attrs["count"] = n_many
    return g


@pytest.mark.parametrize("n_many", [0, 1, 8, 9, 256, 257, 1000])
def test_round_trip_and_format_invariants(fmt, n_many):
    g = _tree(fmt, n_many)
    img = fmt.encode(g)
    objs = validate(img)
    assert objs["/spins"][0] == "dataset" and objs["/many"][0] == "group" and objs["/nothing"][0] == "group"
    h = fmt.decode(img)
    assert h.attrs["T"] == 0.25 and h.attrs["paramsfile"] == "out/configuration.h5.params" and h.attrs["n"] == 7
    assert np.array_equal(h.attrs["v"], np.arange(3.0))
    assert np.array_equal(h["spins"].read(), g["spins"].read())
    assert h["a/b/c"].read().dtype == np.int64 and list(h["a/b/c"].read()) == [0, 1, 2, 3, 4]
    assert h["s"].read() == "periodic" and h["empty"].shape == (0, 3) and float(h["scalar"].read()) == 1.5
    assert h["nothing"].keys() == []
    assert h["many"].keys() == [f"k{i:04d}" for i in range(n_many)] and h["many"].attrs["count"] == n_many
    assert all(float(h[f"many/k{i:04d}"].read()) == i for i in range(n_many))


def test_names_sort_by_bytes_and_bad_inputs(fmt):
    g = fmt.Group()
    for k in ["b", "B", "a10", "a2", "(2,1),(0, 0)", "(1,2),(1, 0)", "ü"]:
        g[k] = 1.0
    img = fmt.encode(g)
    validate(img)
    assert fmt.decode(img).keys() == sorted(g.children, key=lambda s: s.encode())
    with pytest.raises(KeyError):
        g["b"] = 2.0  # HDF5.jl refuses to overwrite a dataset
    for bad in ["", "."]:
        with pytest.raises((ValueError, KeyError)):
            g[bad] = 1.0
    with pytest.raises(TypeError):
        g["obj"] = np.array([object()])
    with pytest.raises(fmt.H5FormatError):
        fmt.decode(b"not an hdf5 file" * 8)
    with pytest.raises(fmt.H5FormatError):
        fmt.decode(img[:-16])  # truncated: end-of-file address beyond the data


# ------------------------------------------------------------------ hdf5.jl

def _fake_mc(m, lat, T, params=None, corr=False, ks=None, seed=3):
    """The fields of a MonteCarlo that hdf5.jl reads, with host spins (no device)."""
    rng = np.random.default_rng(seed)
    spins = [rng.normal(size=(3, lat.size)) for _ in T]
    obs = []
    for _ in T:
        o = m.observables.Observables()
        for _ in range(100):
            o.push(rng.normal(-1.0, 0.1), abs(rng.normal(0.5, 0.1)))
        if corr:
            for _ in range(3):
                o.push_correlations(rng.random((9, ks.shape[1])))
        obs.append(o)
    mc = types.SimpleNamespace(lattice=lat, temperatures=np.asarray(T, dtype=np.float64), outpaths=[],
                               parameters=m.MCParamsBuffer(params or {"t_thermalization": 10000,
                                                                      "overrelaxation_rate": 10,
                                                                      "t_deterministic": 10000000}),
                               observables=obs, corr=corr, momentum_vectors=ks)
    mc.spins = lambda r: spins[r]
    return mc, spins


def _terms(uc):
    """A unit cell's terms as comparable tuples, in their order."""
    f = lambda a: tuple(np.asarray(a, dtype=np.float64).ravel().tolist())  # noqa: E731
    return dict(field=[(b, f(h)) for b, h in uc.field], onsite=[(b, f(M)) for b, M in uc.onsite],
                bilinear=[(b1, b2, f(M), tuple(o)) for b1, b2, M, o in uc.bilinear],
                cubic=[(a, b, c, f(M), tuple(o2), tuple(o3)) for a, b, c, M, o2, o3 in uc.cubic],
                quartic=[(a, b, c, d, f(M), tuple(o2), tuple(o3), tuple(o4))
                         for a, b, c, d, M, o2, o3, o4 in uc.quartic])


def test_dumping_metadata_square(m, h5, fmt, tmp_path):
    """test/h5tests.jl:5-46: dump_metadata! then read_unit_cell / read_lattice
    give back the unit cell and the lattice tables."""
    U = m.Square()
    lat = m.Lattice((2, 2), U, 1.0)
    mc, _ = _fake_mc(m, lat, [1.0])
    fn = str(tmp_path / ".test.h5")
    with h5.h5open(fn, "w") as f:
        h5.dump_metadata(f, mc)
    validate(open(fn, "rb").read())
    with h5.h5open(fn, "r") as f:
        R = h5.read_unit_cell(f)
        assert all(np.array_equal(a, b) for a, b in zip(U.lattice_vectors, R.lattice_vectors))
        assert all(np.array_equal(a, b) for a, b in zip(U.basis, R.basis)) and len(U.basis) == len(R.basis)
        assert _terms(U) == _terms(R)
        L = h5.read_lattice(f)
        assert (L.S, L.bc, L.size, tuple(L.shape)) == (lat.S, lat.bc, lat.size, tuple(lat.shape))
        assert np.array_equal(L.site_positions, lat.site_positions)
        for k, v in lat.tables().items():
            assert np.array_equal(L.tables()[k], v), k
        # root attributes: the SimulationParameters fields, Int64
        assert f.keys() == ["lattice", "unit_cell"]
        assert list(f.attrs) == ["t_thermalization", "t_deterministic", "t_measurement", "probe_rate",
                                 "swap_rate", "overrelaxation_rate", "report_interval", "checkpoint_rate"]
        assert f.attrs["t_thermalization"] == 10000 and f.attrs["t_deterministic"] == 10000000
        assert f.attrs["overrelaxation_rate"] == 10 and f.attrs["t_measurement"] == 1
        assert isinstance(f.attrs["probe_rate"], np.int64)


def _sorted_cell(m, uc):
    """The unit cell read_unit_cell rebuilds: terms added in key-name order."""
    from_file = m.UnitCell(*uc.lattice_vectors)
    for b in uc.basis:
        m.addBasisSite(from_file, b)
    h5 = __import__(m.__name__ + ".hdf5", fromlist=["x"])
    key = lambda s: s.encode()  # noqa: E731
    for b, h in sorted(uc.field, key=lambda t: key(str(t[0]))):
        m.addZeemanCoupling(from_file, b, h)
    for b, M in sorted(uc.onsite, key=lambda t: key(str(t[0]))):
        m.addOnSite(from_file, b, M)
    for b1, b2, M, o in sorted(uc.bilinear, key=lambda t: key(f"({t[0]},{t[1]}),{h5._jl_tuple(t[3])}")):
        m.addBilinear(from_file, b1, b2, M, o)
    for t in sorted(uc.cubic, key=lambda t: key(f"({t[0]},{t[1]},{t[2]}),{h5._jl_tuple(t[4])},{h5._jl_tuple(t[5])}")):
        m.addCubic(from_file, *t)
    for t in sorted(uc.quartic, key=lambda t: key(f"({t[0]},{t[1]},{t[2]},{t[3]}),{h5._jl_tuple(t[5])},"
                                                   f"{h5._jl_tuple(t[6])},{h5._jl_tuple(t[7])}")):
        m.addQuartic(from_file, *t)
    return from_file


@pytest.mark.parametrize("name", ["honeycomb", "sc", "triangular", "pyrochlore", "chain"])
def test_params_file_round_trip(m, h5, name, tmp_path):
    """create_params_file then read_lattice on models with every kind of term:
    the unit cell comes back with its terms in key-name order (HDF5.jl's
    iteration order) and the lattice tables equal those of that cell."""
    E = m.examples
    rng = np.random.default_rng(5)
    if name == "honeycomb":
        uc, shape, bc = E.honeycomb_kitaev(K=-1, J=0.1, G=0.05, h=0.1), (4, 3), "open"
        m.addOnSite(uc, 1, rng.normal(size=(3, 3)))
        m.addOnSite(uc, 2, rng.normal(size=(3, 3)))
    elif name == "sc":
        uc, shape, bc = E.sc_heisenberg(), (3, 3, 3), "periodic"
    elif name == "triangular":
        uc, shape, bc = E.triangular_afm(h=0.5), (4, 4), "periodic"
    elif name == "pyrochlore":
        uc, shape, bc = E.pyrochlore_ckq(), (2, 2, 2), "periodic"
        m.addCubic(uc, 1, 2, 3, rng.normal(size=(3, 3, 3)), (0, 0, 0), (1, 0, 0))
        m.addQuartic(uc, 4, 3, 2, 1, rng.normal(size=(3, 3, 3, 3)), (0, 0, 0), (-1, 1, 0), (0, 0, 1))
    else:
        uc = m.UnitCell([1.0])
        m.addBasisSite(uc, [0.0])
        m.addBilinear(uc, 1, 1, np.diag([1.0, 2.0, 3.0]), (1,))
        m.addZeemanCoupling(uc, 1, [0.0, 0.0, 0.3])
        shape, bc = (7,), "periodic"
    lat = m.Lattice(shape, uc, 1.5, bc=bc)
    mc, _ = _fake_mc(m, lat, [0.5])
    fn = h5.create_params_file(mc, str(tmp_path / "configuration.h5.params"))
    validate(open(fn, "rb").read())
    with h5.h5open(fn) as f:
        R = h5.read_unit_cell(f)
        L = h5.read_lattice(f)
    want = _sorted_cell(m, uc)
    assert _terms(R) == _terms(want)
    ref = m.Lattice(shape, want, 1.5, bc=bc)
    assert (L.S, L.bc, tuple(L.shape)) == (1.5, bc, tuple(shape))
    for k, v in ref.tables().items():
        assert np.array_equal(L.tables()[k], v), k
    # with terms in key order to begin with, the tables are the original lattice's
    if [t[:2] + t[3:] for t in _terms(uc)["bilinear"]] == [t[:2] + t[3:] for t in _terms(want)["bilinear"]]:
        assert np.array_equal(L.tables()["bilinear_sites"], lat.tables()["bilinear_sites"])


def test_key_names_and_array_layout(m, h5, tmp_path):
    """Key names print as Julia's string() does; arrays are Julia arrays with
    the dimensions reversed (spins (N, 3), lattice_vectors rows = vectors,
    basis (D, n_basis), a 3x3 coupling M stored as M^T)."""
    uc = m.Honeycomb()
    M = np.arange(9.0).reshape(3, 3) + 1
    m.addBilinear(uc, 1, 2, M, (1, -1))
    C3 = np.arange(27.0).reshape(3, 3, 3) + 1
    m.addCubic(uc, 1, 2, 1, C3, (0, 0), (1, 0))
    lat = m.Lattice((2, 2), uc, 1.0)
    mc, spins = _fake_mc(m, lat, [0.7])
    fn = h5.create_params_file(mc, str(tmp_path / "p.h5.params"))
    with h5.h5open(fn) as f:
        assert f["unit_cell/bilinear"].keys() == ["(1,2),(1, -1)"]
        assert f["unit_cell/cubic"].keys() == ["(1,2,1),(0, 0),(1, 0)"]
        assert np.array_equal(f["unit_cell/bilinear/(1,2),(1, -1)"].read(), M.T)
        assert np.array_equal(f["unit_cell/cubic/(1,2,1),(0, 0),(1, 0)"].read(), C3.transpose(2, 1, 0))
        lv = f["unit_cell/lattice_vectors"].read()
        assert np.array_equal(lv[0], uc.lattice_vectors[0]) and np.array_equal(lv[1], uc.lattice_vectors[1])
        assert f["unit_cell/basis"].shape == (2, 2) and np.array_equal(f["unit_cell/basis"].read()[:, 1], uc.basis[1])
        assert f["lattice/size"].read().tolist() == [2, 2] and f["lattice/bc"].read() == "periodic"
        assert f["lattice/S"].shape == ()
    assert h5._jl_tuple((1,)) == "(1,)" and h5._jl_tuple((0, -1, 2)) == "(0, -1, 2)"
    assert ast.literal_eval("(1,2),(1, -1)") == ((1, 2), (1, -1))


def test_configuration_files(m, h5, tmp_path):
    """initialize_hdf5, write_MC_checkpoint, write_final_observables,
    write_initial_configuration and read_spin_configuration on two replicas."""
    lat = m.Lattice((3, 2), m.examples.honeycomb_kitaev(K=-1, J=0.1), 1.0)
    ks = np.random.default_rng(2).random((2, 4))
    mc, spins = _fake_mc(m, lat, [0.5, 0.9], corr=True, ks=ks)
    out = str(tmp_path) + "/"
    pf = h5.create_params_file(mc, out + "configuration.h5.params")
    mc.outpaths = [out + f"configuration_{r}.h5" for r in range(2)]
    for r in range(2):
        h5.initialize_hdf5(mc, pf, r)
    with h5.h5open(mc.outpaths[1]) as f:
        assert f.attrs["T"] == 0.9 and f.attrs["paramsfile"] == pf
        assert f["spins"].shape == (lat.size, 3) and np.array_equal(f["spins"].read(), spins[1].T)
        assert np.array_equal(f["site_positions"].read(), lat.site_positions.T)
    new = [s * 2.0 for s in spins]
    h5.write_MC_checkpoint(mc, new)
    with h5.h5open(mc.outpaths[0]) as f:
        assert np.array_equal(f["spins"].read(), new[0].T)
    h5.write_initial_configuration(out + "IC_1.h5", mc, 1, new[1])
    with h5.h5open(out + "IC_1.h5") as f:
        assert f.keys() == ["spins"] and f.attrs["paramsfile"] == pf and f.attrs["T"] == 0.9
    h5.write_final_observables(mc, verbose=False)
    h5.write_final_observables(mc, verbose=False)  # the second call replaces the group
    for r in range(2):
        img = open(mc.outpaths[r], "rb").read()
        validate(img)
        with h5.h5open(mc.outpaths[r]) as f:
            assert np.array_equal(f["spins"].read(), spins[r].T)
            g = f["observables"]
            assert g.keys() == sorted(["specific_heat", "specific_heat_err", "susceptibility", "susceptibility_err",
                                       "magnetization", "magnetization_err", "energy", "energy_err"])
            ob, T = mc.observables[r], mc.temperatures[r]
            c, dc = m.specific_heat(np.asarray(ob.energy), T, lat.size)
            x, dx = m.susceptibility(np.asarray(ob.magnetization), T, lat.size)
            assert float(g["specific_heat"].read()) == c and float(g["specific_heat_err"].read()) == abs(dc / c)
            assert float(g["susceptibility"].read()) == x and float(g["susceptibility_err"].read()) == abs(dx / x)
            assert float(g["energy"].read()) == np.mean(ob.energy)
            assert float(g["magnetization"].read()) == np.mean(ob.magnetization)
            assert np.allclose(f["spin_correlations/SSF"].read(), ob.mean_correlations().T)
            assert np.array_equal(f["spin_correlations/SSF_momentum"].read(), ks.T)
    lat2 = m.Lattice((3, 2), m.examples.honeycomb_kitaev(K=-1, J=0.1), 1.0)
    h5.read_spin_configuration(lat2, mc.outpaths[1])
    assert np.array_equal(lat2.spins, spins[1])
    h5.write_attributes(pf, {"J": 0.1, "model": "Kitaev"})
    with h5.h5open(pf) as f:
        assert f.attrs["J"] == 0.1 and f.attrs["model"] == "Kitaev" and f.attrs["swap_rate"] == 1
    with pytest.raises(KeyError):
        h5.write_attributes(pf, {"J": 0.2})  # an existing attribute is an error, as in HDF5.jl
