"""Bit-exact integer work: connectivity, face codes, Dirichlet masks and
element colouring, for the product (numpy generator + libvdr.so host
colouring) against the oracle and against fixtures produced by the
reference's own colouring code."""
import ctypes
import os

import numpy as np
import pytest

from helpers import GOLDEN

MESHES = [(2, 2, 2), (3, 2, 2), (4, 5, 3), (7, 20, 20), (33, 33, 17), (6, 3, 9)]


@pytest.fixture(scope="module")
def golden_colors():
    return np.load(os.path.join(GOLDEN, "ref_colors.npz"))


@pytest.mark.parametrize("dims", MESHES)
def test_connectivity_and_face_codes(vdr, oracle, dims):
    P = vdr.problems
    assert np.array_equal(P.connectivity(*dims), oracle.w_el(*dims))
    assert np.array_equal(P.face_codes(*dims), oracle.kod_el_dr(*dims))


@pytest.mark.parametrize("dims", MESHES)
@pytest.mark.parametrize("mode", [0, 1])
def test_face_dirichlet_masks(vdr, oracle, dims, mode):
    P = vdr.problems
    m = P.structured_mesh(dims[0] - 1, dims[1] - 1, dims[2] - 1)
    assert np.array_equal(P.face_dirichlet(m, mode),
                          oracle.build_bc_nodes(*dims, m.iss, m.kod, mode))


def test_ot_mask_quirk_marks_interior_rows(vdr):
    """OT's faces 5/6 mark the node rows y=1 and y=nay-2 (not y=0, nay-1)."""
    P = vdr.problems
    m = P.structured_mesh(4, 5, 3)
    nax, nay = m.nax, m.nay
    bc = P.face_dirichlet(m, P.MASK_OT).reshape(m.naz, nay, nax)
    bcv = P.face_dirichlet(m, P.MASK_VF).reshape(m.naz, nay, nax)
    inner = slice(1, -1)
    assert bc[inner, 1, 0:nax - 1].all() and bc[inner, nay - 2, 0:nax - 1].all()
    assert bcv[inner, 0, 0:nax - 1].all() and bcv[inner, nay - 1, 0:nax - 1].all()


@pytest.mark.parametrize("dims", MESHES)
def test_oracle_colors_match_reference(oracle, golden_colors, dims):
    key = "%d_%d_%d" % dims
    ref = golden_colors["colors_" + key]
    assert np.array_equal(oracle.parity_colors(*dims), ref)
    ce, co = oracle.color_lists(ref, 8)
    assert np.array_equal(ce, golden_colors["elems_" + key])
    assert np.array_equal(co, golden_colors["offsets_" + key])


@pytest.mark.parametrize("dims", MESHES)
def test_greedy_equals_parity_on_structured(vdr, oracle, golden_colors, dims):
    iss = vdr.problems.connectivity(*dims)
    c, nc = oracle.greedy_colors(iss, dims[0] * dims[1] * dims[2])
    ref = golden_colors["colors_%d_%d_%d" % dims]
    assert np.array_equal(c, ref)


@pytest.mark.parametrize("dims", MESHES)
def test_product_colors_match_reference(vdr, golden_colors, dims):
    lib = vdr.load_library()
    iss = vdr.problems.connectivity(*dims)
    E = len(iss) // 8
    col = np.empty(E, dtype=np.int32)
    IP = ctypes.POINTER(ctypes.c_int)
    nc = lib.vdr_color_elements(dims[0] * dims[1] * dims[2], E,
                                iss.ctypes.data_as(IP), col.ctypes.data_as(IP))
    assert nc == 8
    assert np.array_equal(col, golden_colors["colors_%d_%d_%d" % dims])


def test_product_greedy_on_permuted_numbering(vdr, oracle):
    """Non-canonical numbering: the product falls back to greedy first-fit,
    which must equal the oracle's and be a valid colouring."""
    lib = vdr.load_library()
    dims = (5, 4, 3)
    iss = vdr.problems.connectivity(*dims).reshape(8, -1)
    E = iss.shape[1]
    perm = np.random.default_rng(3).permutation(E)
    iss = np.ascontiguousarray(iss[:, perm]).ravel()
    col = np.empty(E, dtype=np.int32)
    IP = ctypes.POINTER(ctypes.c_int)
    nc = lib.vdr_color_elements(60, E, iss.ctypes.data_as(IP),
                                col.ctypes.data_as(IP))
    ref, nref = oracle.greedy_colors(iss, 60)
    assert nc == nref and np.array_equal(col, ref)
    nodes = iss.reshape(8, E)
    for c in range(nc):
        sel = nodes[:, col == c].ravel()
        assert len(np.unique(sel)) == len(sel)
