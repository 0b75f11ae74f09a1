"""Parity at the benchmark configurations' full sizes.

* R-MAT 2^20 (deg 16, FP32), the headline product, on the default path
  (learned sizing + row-wise windows): C's structure totals against the
  oracle's full-size counts (C tiles from its step 1, nonzeros from its
  Gustavson row counts, tile pairs from A's tiling), and C's structure and
  values on the hub tile-rows and a middle band against the FP64 oracle,
  entry by entry.
* 27-point stencil 64^3 x 3 dof (FP32), the dense-tile product: the whole C,
  bit-exact structure, values <= 1e-6 (FP32 registers and the mixed-precision
  tensor path).
* The Galerkin triple product on the 128^3 Poisson problem: the whole RAP,
  bit-exact structure, values <= 1e-6, with and without the sizing model.
* The 512-problem Erdos-Renyi batch: every 16th problem in full.

Tolerances: relative Frobenius error against the FP64 oracle <= 1e-6 for FP32
data (the reference's own criterion is rel_frob < 1e-5,
src/spgemm_raw_v2.cu:355)."""
import os

import numpy as np
import pytest

import oracle
from gpu_spgemm_gb300 import api, synth

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
STRUCT_KEYS = ["tile_ptrC", "tile_rowidxC", "tile_colidxC", "maskC", "tile_nnzC", "ptrRowC", "tile_colC"]
TOL32 = 1e-6


def rel(x, y):
    x = np.asarray(x, np.float64)
    y = np.asarray(y, np.float64)
    return np.linalg.norm(x - y) / (np.linalg.norm(y) or 1.0)


def oracle_counts(a, b):
    """C's tile count (step 1, src/spgemm_raw_kernels.cuh:23-57), nonzero count
    (structural Gustavson, src/spgemm_raw_v2.cu:289-338), tile pairs and
    products of A*B, from the CPU oracle."""
    l = oracle.lib()
    TA = oracle.csr2tile(a)
    TB = TA if b is a else oracle.csr2tile(b)
    tp = np.zeros(TA["tilem"] + 1, np.int64)
    ntc = l.orc_step1_count(TA["tilem"], TB["tilen"], oracle._p(TA["tile_ptr"]), oracle._p(TA["tile_columnidx"]),
                            oracle._p(TB["tile_ptr"]), oracle._p(TB["tile_columnidx"]), oracle._p(tp))
    arp, aci = oracle._i32(a.row_ptr), oracle._i32(a.col_idx)
    brp, bci = oracle._i32(b.row_ptr), oracle._i32(b.col_idx)
    rn = np.zeros(a.m, np.int64)
    nnz = l.orc_gustavson_rowcounts(a.m, b.n, oracle._p(arp), oracle._p(aci), oracle._p(brp), oracle._p(bci),
                                    oracle._p(rn))
    btiles = np.diff(TB["tile_ptr"]).astype(np.int64)
    return {"numtileC": int(ntc), "nnzC": int(nnz), "tile_pairs": int(btiles[TA["tile_columnidx"]].sum()),
            "products": synth.products(a, b)}


def check_tile_rows(handle, a, b, Cm, i0, i1):
    """C tile-rows [i0, i1) from the device against the FP64 Gustavson oracle."""
    import ctypes as C
    h = handle
    tp = np.zeros(Cm.tilem + 1, np.int32)
    h.check(h.lib.spg_ctiles_to_host(h.h, C.byref(Cm.c), tp.ctypes.data, None, None, None, None, None, None, None))
    s, e = int(tp[i0]), int(tp[i1])
    nt = e - s
    d = dict(tile_colidxC=np.zeros(max(nt, 1), np.int32), maskC=np.zeros(max(nt, 1) * 16, np.uint16),
             tile_nnzC=np.zeros(nt + 1, np.int64), ptrRowC=np.zeros(max(nt, 1) * 16, np.uint8))
    h.check(h.lib.spg_ctiles_to_host_range(h.h, C.byref(Cm.c), s, e, None, d["tile_colidxC"].ctypes.data,
                                           d["maskC"].ctypes.data, d["tile_nnzC"].ctypes.data,
                                           d["ptrRowC"].ctypes.data, None, None, 0, None))
    nv = int(d["tile_nnzC"][-1] - d["tile_nnzC"][0])
    d["tile_valC"] = np.zeros(max(nv, 1), a.val.dtype)
    d["tile_colC"] = np.zeros(max(nv, 1), np.uint8)
    got = C.c_int64()
    h.check(h.lib.spg_ctiles_to_host_range(h.h, C.byref(Cm.c), s, e, None, None, None, None, None,
                                           d["tile_valC"].ctypes.data, d["tile_colC"].ctypes.data, max(nv, 1),
                                           C.byref(got)))
    d["tile_ptr"] = tp[i0:i1 + 1].astype(np.int64) - s
    return oracle.check_tilerows(a, b, i0, i1, d), nv


@pytest.fixture(scope="module")
def rmat20():
    a = synth.rmat(20, 16)
    return a, oracle_counts(a, a)


@pytest.mark.parametrize("sizing", [True, False], ids=["learned-sizing", "exact-two-pass"])
def test_rmat20_default_path_structure_and_hub_values(handle, rmat20, sizing):
    a, ref = rmat20
    A = api.csr2tile(handle, a)
    B = api.build_csc_tiles(handle, a)
    model = None
    if sizing:
        model = api.SizingModel.load(handle)
        model.attach(1.0)
    try:
        assert api.products(handle, A, B) == ref["products"]
        Cm = api.spgemm(handle, A, B)
        st = handle.stats()
    finally:
        if model is not None:
            model.detach()
            model.free()
    assert st["algo_used"] == 2  # row-wise windows
    assert Cm.numtileC == ref["numtileC"]
    assert Cm.nnzC == ref["nnzC"]
    assert Cm.pairs == ref["tile_pairs"]
    # the hub tile-rows (up to 146,674 A nonzeros a tile-row) and a middle band
    for i0, i1 in ((0, 512), (Cm.tilem // 2, Cm.tilem // 2 + 2048)):
        r, nv = check_tile_rows(handle, a, a, Cm, i0, i1)
        assert nv > 0
        assert r["mismatches"] == 0, (i0, i1, r)
        assert r["rel_frob"] <= TOL32, (i0, i1, r)
    Cm.free()


@pytest.fixture(scope="module")
def stencil27_64():
    a = synth.stencil27_dof3(64)
    return a, oracle.spgemm_tiles(a, a)


@pytest.mark.parametrize("prec", ["f32", "mixed"])
def test_stencil27_64_whole_product(handle, stencil27_64, prec):
    a, S = stencil27_64
    A = api.csr2tile(handle, a)
    B = api.build_csc_tiles(handle, a)
    Cm = api.spgemm(handle, A, B, algo="auto", prec=prec)
    st = handle.stats()
    got = Cm.to_host()
    Cm.free()
    assert got["numtileC"] == S["numtileC"] and got["nnzC"] == S["nnzC"]
    for k in STRUCT_KEYS:
        np.testing.assert_array_equal(got[k], S[k].astype(got[k].dtype), err_msg=k)
    assert rel(got["tile_valC"], S["tile_valC"]) <= TOL32
    if prec == "mixed":
        assert st["tensor_pairs"] > 0


@pytest.fixture(scope="module")
def galerkin128():
    g = 128
    a = synth.poisson3d(g)
    p = synth.smoothed_aggregation(a, synth.aggregation_p0(g))
    S1 = oracle.spgemm_tiles(a, p)
    rp, ci, v = oracle.tiles_to_csr(a.m, p.n, S1)
    ap = synth.CSR(a.m, p.n, rp.astype(np.int32), ci, v)
    pt = synth.transpose(p)
    return a, p, oracle.spgemm_tiles(pt, ap), synth.products(a, p) + synth.products(pt, ap)


@pytest.mark.parametrize("sizing", [True, False], ids=["learned-sizing", "exact-two-pass"])
@pytest.mark.parametrize("algo", ["auto", "plain", "rowwise"])
def test_galerkin_128_whole_product(handle, galerkin128, algo, sizing):
    """The Galerkin configuration at full size (n = 2,097,152, 262,144
    aggregates), both products chained on the device, exact in structure.
    The reference's step 1 gives each warp a bitmap of B's tile columns (4
    warps x tilenB/32 words of dynamic shared memory,
    src/spgemm_raw_v2.cu:119-128): 8 KB for these two products, whose B has
    16,384 tile columns, but 64 KB -- above the 48 KB default, so no launch --
    for a product whose B has this n's 131,072 tile columns, such as A*A.  The
    span-limited bitmap here has no such limit."""
    a, p, S, prods = galerkin128
    model = None
    if sizing:
        model = api.SizingModel.load(handle)
        model.attach(1.0)
    try:
        Cm, got_prods = api.galerkin(handle, a, p, algo=algo)
    finally:
        if model is not None:
            model.detach()
            model.free()
    got = Cm.to_host()
    Cm.free()
    assert got_prods == prods
    for k in STRUCT_KEYS:
        np.testing.assert_array_equal(got[k], S[k].astype(got[k].dtype), err_msg=k)
    assert rel(got["tile_valC"], S["tile_valC"]) <= TOL32


def test_er_batch_512(handle):
    """All 512 problems of the batch configuration in one batched product:
    every 16th problem checked in full (tile count from the oracle's step 1,
    every entry against the FP64 Gustavson), the product count of all."""
    pairs = synth.er_batch(512)
    bt = api.Batch(handle, pairs)
    bt.tune()
    bt.spgemm()
    assert bt.products() == sum(synth.products(a, b) for a, b in pairs)
    for p in range(0, 512, 16):
        a, b = pairs[p]
        got = bt.result(p)
        assert got["numtileC"] == oracle_counts(a, b)["numtileC"], p
        d = dict(tile_ptr=got["tile_ptrC"].astype(np.int64), tile_colidxC=got["tile_colidxC"],
                 tile_nnzC=got["tile_nnzC"], maskC=got["maskC"], ptrRowC=got["ptrRowC"], tile_colC=got["tile_colC"],
                 tile_valC=got["tile_valC"])
        r = oracle.check_tilerows(a, b, 0, (a.m + 15) // 16, d)
        assert r["mismatches"] == 0 and r["rel_frob"] <= TOL32, (p, r)
    bt.free()


def test_poisson3d_128_squared_beyond_the_reference_step1_limit(handle):
    """A*A on the 128^3 Poisson matrix (n = 2,097,152, 131,072 tile columns):
    the reference's step 1 would need 4 x 4,096 words = 64 KB of dynamic
    shared memory per block here, above the 48 KB default, and could not
    launch (src/spgemm_raw_v2.cu:119-128).  The span-limited bitmap has no
    such bound; the whole C matches the oracle."""
    a = synth.poisson3d(128)
    S = oracle.spgemm_tiles(a, a)
    A = api.csr2tile(handle, a)
    B = api.build_csc_tiles(handle, a)
    got = api.spgemm(handle, A, B).to_host()
    for k in STRUCT_KEYS:
        np.testing.assert_array_equal(got[k], S[k].astype(got[k].dtype), err_msg=k)
    assert rel(got["tile_valC"], S["tile_valC"]) <= TOL32
