"""Host-side flattening and colouring of libcsmc.so against the oracle's
restatement of Lattice() (lattice.jl:65-291).  No GPU needed."""
import ctypes as C

import numpy as np
import pytest


def _models(m):
    E = m.examples
    asym = np.arange(9.0).reshape(3, 3) - 3.0
    uc_b = m.Honeycomb()  # asymmetric couplings exercise transposeJ
    m.addBilinear(uc_b, 1, 2, asym, (0, -1))
    m.addBilinear(uc_b, 2, 1, asym.T * 0.5, (1, 0))
    m.addBilinear(uc_b, 1, 1, np.eye(3), (1, 1))  # b1 == b2: b1 role only
    m.addOnSite(uc_b, 1, np.diag([0.1, 0.2, 0.3]))
    m.addOnSite(uc_b, 2, np.diag([0.3, 0.2, 0.1]))
    m.addZeemanCoupling(uc_b, 1, [0.1, 0.0, 0.0])
    m.addZeemanCoupling(uc_b, 2, [0.0, 0.2, 0.0])
    rng = np.random.default_rng(4)
    uc_c = m.Pyrochlore()  # generic tensors exercise permutedims of every role
    m.addCubic(uc_c, 1, 2, 3, rng.normal(size=(3, 3, 3)), (0, 0, 0), (1, 0, 0))
    m.addCubic(uc_c, 2, 4, 1, rng.normal(size=(3, 3, 3)), (0, 1, 0), (0, 0, -1))
    m.addQuartic(uc_c, 1, 2, 3, 4, rng.normal(size=(3, 3, 3, 3)), (1, 0, 0), (0, 1, 0), (0, 0, 1))
    m.addQuartic(uc_c, 4, 3, 2, 1, rng.normal(size=(3, 3, 3, 3)), (0, 0, 0), (-1, 1, 0), (0, 0, 1))
    return [
        ("square", E.square_heisenberg(), (6, 4), "periodic"),
        ("square_open", E.square_heisenberg(), (5, 3), "open"),
        ("honeycomb", E.honeycomb_kitaev(K=-1, J=0.1, G=0.05, h=0.1), (4, 6), "periodic"),
        ("honeycomb_asym", uc_b, (3, 4), "periodic"),
        ("honeycomb_asym_open", uc_b, (3, 4), "open"),
        ("sc", E.sc_heisenberg(), (4, 4, 4), "periodic"),
        ("triangular", E.triangular_afm(h=0.5), (6, 6), "periodic"),
        ("pyrochlore", E.pyrochlore_ckq(), (2, 2, 2), "periodic"),
        ("pyrochlore_open", E.pyrochlore_ckq(), (2, 3, 2), "open"),
        ("generic_tensors", uc_c, (2, 2, 3), "periodic"),
        ("generic_tensors_open", uc_c, (3, 2, 2), "open"),
        ("square_L1_selfloops", E.square_heisenberg(), (1, 1), "periodic"),
        ("square_L2_double_partners", E.square_heisenberg(), (2, 2), "periodic"),
    ]


@pytest.mark.parametrize("idx", range(13))
def test_tables_match_oracle(m, orc, idx):
    name, uc, shape, bc = _models(m)[idx]
    lat = m.Lattice(shape, uc, 1.0, bc=bc)
    ol = orc.OracleLattice(uc, shape, 1.0, bc=bc)
    a, b = lat.tables(), ol.tables()
    for k in a:
        assert np.array_equal(a[k], b[k]), (name, k)


@pytest.mark.parametrize("idx", range(13))
def test_colouring_is_valid(m, idx):
    """No site reads a partner of its own colour (the concurrency invariant)."""
    name, uc, shape, bc = _models(m)[idx]
    lat = m.Lattice(shape, uc, 1.0, bc=bc)
    col, order, starts = lat.colouring()
    t = lat.tables()
    N = lat.size
    for i in range(N):
        partners = list(t["bilinear_sites"][i]) + list(t["cubic_sites"][i].ravel()) + list(t["quartic_sites"][i].ravel())
        for j in partners:
            if j > 0 and j - 1 != i:
                assert col[j - 1] != col[i], (name, i, j - 1)
    # device order: every site exactly once, classes contiguous, padded to 32
    real = order[order >= 0]
    assert sorted(real.tolist()) == list(range(N))
    assert all(s % 32 == 0 for s in starts)
    for c in range(len(starts) - 1):
        seg = order[starts[c]:starts[c + 1]]
        assert all(col[i] == c for i in seg[seg >= 0])


def test_expected_colour_counts(m):
    E = m.examples
    assert m.Lattice((8, 8), E.square_heisenberg(), 1.0).info.n_colours == 2
    assert m.Lattice((24, 24, 24), E.sc_heisenberg(), 1.0).info.n_colours == 2
    assert m.Lattice((48, 48), E.honeycomb_kitaev(), 1.0).info.n_colours == 2
    assert m.Lattice((12, 12), E.triangular_afm(), 1.0).info.n_colours == 3
    assert m.Lattice((4, 4, 4), E.pyrochlore_ckq(), 1.0).info.n_colours == 4
    # odd periodic extent: no 2-colouring exists
    assert m.Lattice((5, 5), E.square_heisenberg(), 1.0).info.n_colours == 3


def test_deduplicated_couplings(m):
    info = m.Lattice((48, 48), m.examples.honeycomb_kitaev(K=-1, J=0.1, G=0.05), 1.0).info
    assert info.n_matrices == 1 + 3  # zero matrix + the symmetric x/y/z bond matrices
    info = m.Lattice((4, 4, 4), m.examples.pyrochlore_ckq(), 1.0).info
    assert info.width_bilinear == 6 and info.width_cubic == 6 and info.width_quartic == 6


def test_isotropic_tensor_forms(m):
    """kappa eps_abc and the delta pairings are recognised after the role
    permutations (lattice.jl:241-291); other tensors keep the dense form."""
    info = m.Lattice((2, 2, 2), m.examples.pyrochlore_ckq(), 1.0).info
    assert info.n_isotropic_cubic == info.n_cubic_tensors  # zero tensor, +kappa eps, -kappa eps
    assert info.n_isotropic_quartic == info.n_quartic_tensors
    assert info.n_cubic_tensors == 3
    uc = m.examples.pyrochlore_ckq(cubic=False, quartic=False)
    rng = np.random.default_rng(1)
    m.addCubic(uc, 1, 2, 3, rng.normal(size=(3, 3, 3)), (0, 0, 0), (0, 0, 0))
    iso = 0.3 * np.einsum("ab,cd->abcd", np.eye(3), np.eye(3)) - 0.1 * np.einsum("ac,bd->abcd", np.eye(3), np.eye(3))
    m.addQuartic(uc, 1, 2, 3, 4, iso, (0, 0, 0), (0, 0, 0), (0, 0, 0))
    info = m.Lattice((2, 2, 2), uc, 1.0).info
    assert info.n_isotropic_cubic == 1  # only the zero tensor
    assert info.n_isotropic_quartic == info.n_quartic_tensors


def test_field_assignment_rule(m, orc):
    """lattice.jl:128-139 assigns the i-th field entry to column f_indices[i]."""
    uc = m.Honeycomb()
    m.addZeemanCoupling(uc, 2, [0.0, 0.0, 2.0])
    m.addZeemanCoupling(uc, 1, [0.0, 0.0, 1.0])
    lat = m.Lattice((2, 2), uc, 1.0)
    ol = orc.OracleLattice(uc, (2, 2), 1.0)
    assert np.array_equal(lat.tables()["field"], ol.tables()["field"])
    # only basis 2 has a field: the reference indexes past the list (BoundsError)
    uc = m.Honeycomb()
    m.addZeemanCoupling(uc, 2, [0.0, 0.0, 2.0])
    with pytest.raises(m.CSMCError) as e:
        m.Lattice((2, 2), uc, 1.0)
    assert e.value.code == 1
    with pytest.raises(ValueError):
        orc.OracleLattice(uc, (2, 2), 1.0)


def test_invalid_descriptions(m):
    uc = m.Square()
    m.addBilinear(uc, 1, 2, np.eye(3), (1, 0))  # basis 2 does not exist
    with pytest.raises(m.CSMCError) as e:
        m.Lattice((4, 4), uc, 1.0)
    assert e.value.code == 1
    with pytest.raises(ValueError):
        m.Lattice((4, 4), m.Square(), 1.0, bc="twisted")
    # cubic term whose partner is the site itself: valid in the reference,
    # rejected by the colour-sweep kernels
    uc = m.Square()
    m.addCubic(uc, 1, 1, 1, np.ones((3, 3, 3)), (0, 0), (1, 0))
    with pytest.raises(m.CSMCError) as e:
        m.Lattice((4, 4), uc, 1.0)
    assert e.value.code == 6


def test_empty_and_single_site(m, orc):
    uc = m.Square()  # no basis site, no terms: Lattice adds one at the origin
    lat = m.Lattice((1, 1), uc, 0.5)
    assert lat.size == 1 and len(uc.basis) == 1
    assert lat.info.n_colours == 1
    assert lat.tables()["bilinear_sites"].shape == (1, 0)


def test_site_positions(m):
    """compute_site_positions (lattice.jl:38-51)."""
    lat = m.Lattice((2, 3), m.Honeycomb(), 1.0)
    uc = lat.unit_cell
    i = 0
    for b in range(2):
        for n1 in range(2):
            for n2 in range(3):
                exp = n1 * uc.lattice_vectors[0] + n2 * uc.lattice_vectors[1] + uc.basis[b]
                assert np.allclose(lat.site_positions[:, i], exp)
                i += 1
