"""Device conversions: CSR transpose (the --aat path), tile->CSR export, and the
Galerkin triple product P^T (A P) chained on the device."""
import os

import numpy as np
import pytest

import oracle
from gpu_spgemm_gb300 import api, synth
import cases

pytestmark = pytest.mark.gpu

STRUCT_KEYS = ["tile_ptrC", "tile_rowidxC", "tile_colidxC", "maskC", "tile_nnzC", "ptrRowC", "tile_colC"]


def rel(x, y):
    x = np.asarray(x, np.float64); y = np.asarray(y, np.float64)
    return np.linalg.norm(x - y) / (np.linalg.norm(y) or 1.0)


@pytest.mark.parametrize("name,a", [("rmat_12", synth.rmat(12, 16)), ("rect", cases.random_csr(300, 170, 0.03, 3,
                                                                                                  dtype=np.float32)),
                                    ("empty", cases.empty_csr(40, 50, np.float32))])
def test_transpose_matches_host(handle, name, a):
    T = api.csr2tile(handle, a)
    Tt = api.transpose(handle, T, layout="row").to_host()
    ref = oracle.csr2tile(synth.transpose(a))
    for k in ("tile_ptr", "tile_columnidx", "tile_nnz", "tile_csr_Ptr", "mask", "tile_csr_Col"):
        np.testing.assert_array_equal(Tt[k], ref[k], err_msg=k)
    np.testing.assert_array_equal(Tt["tile_csr_Val"], ref["tile_csr_Val"].astype(np.float32))


@pytest.mark.parametrize("algo", ["plain", "rowwise"])
def test_a_times_a_transpose(handle, algo):
    """C = A * A^T with B built by the device transpose (reference --aat)."""
    a = synth.rmat(11, 16)
    A = api.csr2tile(handle, a)
    B = api.transpose(handle, A, layout="b_csc")
    got = api.spgemm(handle, A, B, algo=algo).to_host()
    S = oracle.spgemm_tiles(a, synth.transpose(a))
    for k in STRUCT_KEYS:
        np.testing.assert_array_equal(got[k], S[k].astype(got[k].dtype), err_msg=k)
    assert rel(got["tile_valC"], S["tile_valC"]) <= 1e-6


@pytest.mark.parametrize("name,a,b", cases.product_cases()[:6], ids=[c[0] for c in cases.product_cases()[:6]])
def test_ctiles_to_csr(handle, name, a, b):
    A = api.csr2tile(handle, a)
    B = api.build_csc_tiles(handle, b)
    Cm = api.spgemm(handle, A, B)
    rp, ci, v = api.ctiles_to_csr(handle, Cm)
    S = oracle.spgemm_tiles(a, b)
    orp, oci, ov = oracle.tiles_to_csr(a.m, b.n, S)
    np.testing.assert_array_equal(rp, orp)
    np.testing.assert_array_equal(ci, oci)
    assert rel(v, ov) <= 1e-12


@pytest.mark.parametrize("g", [8, 16])
def test_galerkin_matches_oracle(handle, g):
    a = synth.poisson3d(g)
    p0 = synth.aggregation_p0(g)
    p = synth.smoothed_aggregation(a, p0)
    C, prods = api.galerkin(handle, a, p)
    got = C.to_host()
    # oracle: A P, expanded to CSR, then P^T (A P)
    S1 = oracle.spgemm_tiles(a, p)
    rp, ci, v = oracle.tiles_to_csr(a.m, p.n, S1)
    ap = synth.CSR(a.m, p.n, rp.astype(np.int32), ci, v)
    pt = synth.transpose(p)
    S = oracle.spgemm_tiles(pt, ap)
    for k in STRUCT_KEYS:
        np.testing.assert_array_equal(got[k], S[k].astype(got[k].dtype), err_msg=k)
    assert rel(got["tile_valC"], S["tile_valC"]) <= 1e-6
    assert prods == synth.products(a, p) + synth.products(pt, ap)
    # and against scipy's triple product on the expanded result
    R = (p.to_scipy().T.astype(np.float64) @ (a.to_scipy().astype(np.float64) @ p.to_scipy().astype(np.float64))).tocsr()
    grp, gci, gv = oracle.tiles_to_csr(p.n, p.n, got)
    import scipy.sparse as sp
    G = sp.csr_matrix((gv, gci, grp), shape=R.shape)
    assert abs(G - R).max() <= 1e-5 * abs(R).max()


@pytest.mark.skipif(not os.path.exists(api.SIZING_MODEL_PATH), reason="no trained sizing model shipped")
def test_galerkin_with_learned_sizing_same_structure(handle):
    """The Galerkin triple product with the trained sizing model attached
    (learned per-row slots in both products' step 1) equals the exact run."""
    g = 16
    a = synth.poisson3d(g)
    p = synth.smoothed_aggregation(a, synth.aggregation_p0(g))
    ref, _ = api.galerkin(handle, a, p)
    ref_h = ref.to_host()
    model = api.SizingModel.load(handle)
    model.attach()
    try:
        C, _ = api.galerkin(handle, a, p)
        got = C.to_host()
    finally:
        model.detach()
        model.free()
    for k in STRUCT_KEYS:
        np.testing.assert_array_equal(got[k], ref_h[k], err_msg=k)
    assert rel(got["tile_valC"], ref_h["tile_valC"]) <= 1e-6
