"""CPU oracle checks: pinned against the reference's own tiler (golden
fixtures, and the live reference build where its checkout exists) and against
an independent structural/numeric product (scipy)."""
import glob
import os

import numpy as np
import pytest
import scipy.sparse as sp

import oracle
from oracle import ref
from gpu_spgemm_gb300 import synth
from gpu_spgemm_gb300.synth import CSR
import cases

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "tiles_*.npz")))
A_KEYS = ["tile_ptr", "tile_columnidx", "tile_nnz", "tile_csr_Ptr", "mask", "tile_csr_Val", "tile_csr_Col"]
B_KEYS = A_KEYS + ["csc_tile_ptr", "csc_tile_rowidx", "tile_csc_Ptr", "tile_csc_Row", "tile_csc_Val"]


def _csr_from_npz(z):
    return CSR(int(z["in_m"]), int(z["in_n"]), z["in_row_ptr"], z["in_col_idx"], z["in_val"])


def test_golden_fixtures_present():
    assert len(GOLDEN) >= 10


@pytest.mark.parametrize("path", GOLDEN, ids=lambda p: os.path.basename(p)[6:-4])
def test_oracle_tiler_matches_reference_golden(path):
    z = np.load(path)
    csr = _csr_from_npz(z)
    TA = oracle.csr2tile(csr)
    for k in A_KEYS:
        np.testing.assert_array_equal(TA[k], z["A_" + k], err_msg=k)
    TB = oracle.build_csc_tiles(csr, with_tile_csc=True)
    for k in B_KEYS:
        np.testing.assert_array_equal(TB[k], z["B_" + k], err_msg=k)
    # B keeps its row-major tile-level arrays (read by step 1)
    np.testing.assert_array_equal(TB["tile_ptr"], z["A_tile_ptr"])
    np.testing.assert_array_equal(TB["tile_columnidx"], z["A_tile_columnidx"])


@pytest.mark.skipif(not ref.available(), reason="reference checkout not present")
@pytest.mark.parametrize("name,csr", [
    ("rmat_12", synth.rmat(12, 8, dtype=np.float64)),
    ("stencil27_6", synth.stencil27_dof3(6, dtype=np.float64)),
    ("rand_333x257", cases.random_csr(333, 257, 0.03, 21, empty_row_frac=0.3)),
    ("poisson3d_10", synth.poisson3d(10, dtype=np.float64)),
])
def test_oracle_tiler_matches_live_reference(name, csr):
    TA = oracle.csr2tile(csr)
    RA = ref.ref_tiles(csr, csc=False)
    for k in A_KEYS:
        np.testing.assert_array_equal(TA[k], RA[k], err_msg=k)
    TB = oracle.build_csc_tiles(csr, with_tile_csc=True)
    RB = ref.ref_tiles(csr, csc=True)
    for k in B_KEYS:
        np.testing.assert_array_equal(TB[k], RB[k], err_msg=k)


def _pattern(m):
    m = m.tocsr().copy()
    m.data[:] = 1.0
    return m


@pytest.mark.parametrize("name,a,b", cases.product_cases(), ids=[c[0] for c in cases.product_cases()])
def test_oracle_product_matches_scipy(name, a, b):
    S = oracle.spgemm_tiles(a, b)
    A, B = a.to_scipy(), b.to_scipy()
    # structure: mask-expanded C equals the structural product pattern
    P = (_pattern(A) @ _pattern(B)).tocsr()
    P.sort_indices()
    rp, cols, vals = oracle.tiles_to_csr(a.m, b.n, S)
    np.testing.assert_array_equal(rp, P.indptr)
    np.testing.assert_array_equal(cols, P.indices)
    # values: FP64 tile oracle equals scipy's product on the same pattern
    Cv = (A @ B).tocsr()
    Ct = sp.csr_matrix((vals, cols, rp), shape=(a.m, b.n))
    diff = abs(Ct - Cv)
    assert (diff.max() if diff.nnz else 0.0) <= 1e-12 * max(1.0, abs(Cv).max() if Cv.nnz else 1.0)
    # step 1: tile set equals the tile-level pattern product
    TA = oracle.csr2tile(a)
    TB = oracle.build_csc_tiles(b, with_tile_csc=False)
    ta = sp.csr_matrix((np.ones(TA["numtile"]), TA["tile_columnidx"], TA["tile_ptr"]),
                       shape=(TA["tilem"], max(TA["tilen"], 1)))
    tb = sp.csr_matrix((np.ones(TB["numtile"]), TB["tile_columnidx"], TB["tile_ptr"]),
                       shape=(max(TB["tilem"], 1), TB["tilen"]))
    if ta.shape[1] == tb.shape[0]:
        tc = (ta @ tb).tocsr()
        tc.sort_indices()
        np.testing.assert_array_equal(S["tile_ptrC"], tc.indptr)
        np.testing.assert_array_equal(S["tile_colidxC"], tc.indices)
    # nnz prefix and per-row offsets agree with the masks
    pc = np.array([bin(int(x)).count("1") for x in S["maskC"]], np.int64).reshape(-1, 16)
    np.testing.assert_array_equal(np.diff(S["tile_nnzC"]), pc.sum(1))
    excl = (np.cumsum(pc, 1) - pc).astype(np.uint8).ravel()
    np.testing.assert_array_equal(S["ptrRowC"], excl)


@pytest.mark.parametrize("name,a,b", cases.product_cases()[:5], ids=[c[0] for c in cases.product_cases()[:5]])
def test_gustavson_matches_scipy(name, a, b):
    rp, cols, vals = oracle.gustavson(a, b)
    P = (_pattern(a.to_scipy()) @ _pattern(b.to_scipy())).tocsr()
    P.sort_indices()
    np.testing.assert_array_equal(rp, P.indptr)
    np.testing.assert_array_equal(cols, P.indices)
    rp2, cols2, vals2 = oracle.tiles_to_csr(a.m, b.n, oracle.spgemm_tiles(a, b))
    np.testing.assert_allclose(vals, vals2, rtol=1e-12, atol=1e-12)


def test_gustavson_rows_counts():
    a = synth.poisson2d(16)
    tot = oracle.gustavson_rows(a, a, 0, a.m, np.float32)
    rp, _, _ = oracle.gustavson(a, a)
    assert tot == rp[-1]


CSTRUCT = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "cstruct_*.npz")))
C_KEYS = ["tile_ptrC", "tile_rowidxC", "tile_colidxC", "maskC", "tile_nnzC", "ptrRowC", "tile_colC"]


def _ab_from_npz(z):
    a = CSR(int(z["in_a_m"]), int(z["in_a_n"]), z["in_a_row_ptr"], z["in_a_col_idx"], z["in_a_val"])
    b = CSR(int(z["in_b_m"]), int(z["in_b_n"]), z["in_b_row_ptr"], z["in_b_col_idx"], z["in_b_val"])
    return a, b


def test_reference_kernel_fixtures_present():
    assert len(CSTRUCT) >= 10, "run tests/golden/make_cstruct_golden.py on a GPU host"


@pytest.mark.parametrize("path", CSTRUCT, ids=lambda p: os.path.basename(p)[8:-4])
def test_oracle_c_structure_matches_reference_kernels(path):
    """C's tile arrays from the reference's own step-1/2/3 kernels (recorded on
    a GB300) equal the oracle's bit for bit; values agree to FP64 rounding."""
    z = np.load(path)
    a, b = _ab_from_npz(z)
    S = oracle.spgemm_tiles(a, b)
    assert S["numtileC"] == int(z["numtileC"]) and S["nnzC"] == int(z["nnzC"])
    for k in C_KEYS:
        np.testing.assert_array_equal(S[k], z[k].astype(S[k].dtype), err_msg=k)
    ref = z["tile_valC"]
    den = np.linalg.norm(ref) or 1.0
    assert np.linalg.norm(S["tile_valC"] - ref) / den <= 1e-12


@pytest.mark.parametrize("name,a,b", cases.product_cases(), ids=[c[0] for c in cases.product_cases()])
def test_tilerow_checker_accepts_the_oracle_and_catches_planted_errors(name, a, b):
    """oracle.check_tilerows (the FP64 row Gustavson compared entry by entry
    with C's tiles, used on the full-size GPU products) reports no error on
    the tiled oracle's own C, and catches a value and a mask bit changed in
    a copy of it."""
    S = oracle.spgemm_tiles(a, b)
    tilem = S["tilem"]
    tp = S["tile_ptrC"].astype(np.int64)
    for i0, i1 in ((0, tilem), (tilem // 3, tilem)):
        t0, t1 = tp[i0], tp[i1]
        v0, v1 = S["tile_nnzC"][t0], S["tile_nnzC"][t1]
        d = dict(tile_ptr=tp[i0:i1 + 1] - t0, tile_colidxC=S["tile_colidxC"][t0:t1], tile_nnzC=S["tile_nnzC"][t0:t1 + 1],
                 maskC=S["maskC"][t0 * 16:t1 * 16], ptrRowC=S["ptrRowC"][t0 * 16:t1 * 16],
                 tile_colC=S["tile_colC"][v0:v1], tile_valC=S["tile_valC"][v0:v1])
        r = oracle.check_tilerows(a, b, i0, i1, d)
        assert r["mismatches"] == 0 and r["rel_frob"] <= 1e-14, r
        if v1 > v0:
            bad = dict(d, tile_valC=d["tile_valC"].copy())
            bad["tile_valC"][(v1 - v0) // 2] += 1.0
            assert oracle.check_tilerows(a, b, i0, i1, bad)["rel_frob"] > 0
            bad = dict(d, maskC=d["maskC"].copy())
            k = int(np.flatnonzero(bad["maskC"])[0])
            mk = int(bad["maskC"][k])
            bad["maskC"][k] = np.uint16(mk & (mk - 1))  # one entry dropped from the mask
            assert oracle.check_tilerows(a, b, i0, i1, bad)["mismatches"] > 0
