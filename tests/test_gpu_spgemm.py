"""SpGEMM parity on the GPU: C's structure arrays bit-exact against the CPU
oracle (itself pinned to the reference), values within the relative Frobenius
tolerance against the FP64 oracle (FP64 path: 1e-12, FP32 path: 1e-6)."""
import os

import numpy as np
import pytest

import oracle
from gpu_spgemm_gb300 import api, synth
import cases

pytestmark = pytest.mark.gpu

STRUCT_KEYS = ["tile_ptrC", "tile_rowidxC", "tile_colidxC", "maskC", "tile_nnzC", "ptrRowC", "tile_colC"]
TOL = {np.float64: 1e-12, np.float32: 1e-6}


def rel_frob(x, ref):
    x = np.asarray(x, np.float64)
    ref = np.asarray(ref, np.float64)
    den = np.linalg.norm(ref)
    return np.linalg.norm(x - ref) / (den if den > 0 else 1.0)


def check_product(handle, a, b, algo, dtype, prec="f32"):
    a = a.astype(dtype)
    b = b.astype(dtype)
    A = api.csr2tile(handle, a)
    B = api.build_csc_tiles(handle, b)
    C = api.spgemm(handle, A, B, algo=algo, prec=prec)
    got = C.to_host()
    S = oracle.spgemm_tiles(a, b)
    assert got["numtileC"] == S["numtileC"]
    assert got["nnzC"] == S["nnzC"]
    for k in STRUCT_KEYS:
        np.testing.assert_array_equal(got[k], S[k].astype(got[k].dtype), err_msg=k)
    err = rel_frob(got["tile_valC"], S["tile_valC"])
    # FP64 data: FP64 rounding; FP32 data: <= 1e-6, and <= 1e-7 (output rounding
    # only) when the accumulation runs in FP64
    tol = TOL[np.float64] if dtype == np.float64 else (1e-7 if prec == "f64" else TOL[np.float32])
    assert err <= tol, (err, tol)
    assert got["pairs"] == S["pairs"]
    return got, S


@pytest.mark.parametrize("algo", ["plain", "rowwise"])
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("name,a,b", cases.product_cases(), ids=[c[0] for c in cases.product_cases()])
def test_spgemm_small_cases(handle, name, a, b, dtype, algo):
    check_product(handle, a, b, algo, dtype)


@pytest.mark.parametrize("algo", ["plain", "rowwise"])
def test_poisson2d_256_fp64_full_config(handle, algo):
    a = synth.poisson2d(256)
    got, S = check_product(handle, a, a, algo, np.float64)
    assert got["numtileC"] == 50532 and got["nnzC"] == 846852


@pytest.mark.parametrize("algo", ["plain", "rowwise"])
@pytest.mark.parametrize("name,a", [("rmat_14", synth.rmat(14, 16)), ("stencil27_12", synth.stencil27_dof3(12)),
                                    ("poisson3d_32", synth.poisson3d(32))])
def test_medium_fp32(handle, name, a, algo):
    check_product(handle, a, a, algo, np.float32)


def test_pair_cache_overflow_rerun(handle, monkeypatch):
    # shrink the matched-pair cache so step 2 overflows and re-runs; results unchanged
    monkeypatch.setenv("SPG_SPEC_CAP_DIV", "64")
    a = synth.stencil27_dof3(4, dtype=np.float64)
    check_product(handle, a, a, "plain", np.float64)
    assert handle.stats()["overflow_reruns"] >= 1


def test_products_matches_host(handle):
    a = synth.rmat(12, 8)
    A = api.csr2tile(handle, a)
    B = api.build_csc_tiles(handle, a)
    assert api.products(handle, A, B) == synth.products(a, a)


def test_dimension_mismatch_rejected(handle):
    from gpu_spgemm_gb300._lib import SpgError
    a = cases.random_csr(20, 30, 0.1, 1)
    A = api.csr2tile(handle, a)
    B = api.build_csc_tiles(handle, a)
    with pytest.raises(SpgError):
        api.spgemm(handle, A, B)


def regions_case():
    """A tile-row with > 16384 C tiles (several row-wise work items) and more
    than 2048 A nonzeros (cursors in global scratch): a dense row in a
    2^19-column matrix."""
    n = 1 << 19
    rng = np.random.Generator(np.random.PCG64(17))
    rows = rng.integers(0, n, size=2 * n)
    cols = rng.integers(0, n, size=2 * n)
    rows = np.concatenate([rows, np.zeros(n, np.int64)])
    cols = np.concatenate([cols, np.arange(n)])
    key = np.unique(rows * n + cols)
    r, c = key // n, key % n
    rp = np.zeros(n + 1, np.int64)
    np.cumsum(np.bincount(r, minlength=n), out=rp[1:])
    return synth.CSR(n, n, rp.astype(np.int32), c.astype(np.int32), (rng.random(r.size) * 2 - 1).astype(np.float32))


@pytest.mark.parametrize("algo", ["rowwise", "plain"])
def test_multi_region_tile_row(handle, algo):
    a = regions_case()
    got, S = check_product(handle, a, a, algo, np.float32)
    assert np.diff(S["tile_ptrC"]).max() > 16384


@pytest.mark.parametrize("name,a", [("rmat_13", synth.rmat(13, 16)), ("stencil27_6", synth.stencil27_dof3(6))])
def test_rowwise_fp64_accumulation_of_fp32(handle, name, a):
    got, S = check_product(handle, a, a, "rowwise", np.float32, prec="f64")


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_rowwise_numeric_after_plain_symbolic(handle, dtype):
    """A C whose symbolic phase ran on the plain kernels (27-point stencil
    26^3 x 3 dof) takes the row-wise numeric kernels when asked: their plan is
    built at numeric time.  Same values as the plain numeric phase, and FP64
    accumulation of FP32 data runs row-wise after a plain symbolic phase."""
    a = synth.stencil27_dof3(26).astype(dtype)
    S = oracle.spgemm_tiles(a, a)
    A = api.csr2tile(handle, a)
    B = api.build_csc_tiles(handle, a)
    runs = [("auto", "f32", 1), ("rowwise", "f32", 2)] + ([("auto", "f64", 2)] if dtype == np.float32 else [])
    for algo, prec, want in runs:
        Cm = api.symbolic(handle, A, B, algo="plain")
        api.numeric(handle, A, B, Cm, algo=algo, prec=prec)
        assert handle.stats()["numeric_algo"] == want, (algo, prec)
        got = Cm.to_host()
        for k in STRUCT_KEYS:
            np.testing.assert_array_equal(got[k], S[k].astype(got[k].dtype), err_msg=k)
        tol = TOL[np.float64] if dtype == np.float64 else (1e-7 if prec == "f64" else TOL[np.float32])
        assert rel_frob(got["tile_valC"], S["tile_valC"]) <= tol, (algo, prec)
        Cm.free()


@pytest.mark.parametrize("sizing", [False, True], ids=["exact-two-pass", "learned-sizing"])
def test_step1_saturation_exit_er(handle, sizing):
    """Erdos-Renyi 32,768 x 32,768, degree 16 (493,562 A tiles, one nonzero
    a tile): every C tile-row holds all 2,048 tile columns, which its tile
    pairs (about 57,000 a row) reach long before the last one, so step 1
    stops probing early.  C's tile set, tile pairs and the rest of the
    structure still equal the oracle's full step 1."""
    if sizing and not os.path.exists(api.SIZING_MODEL_PATH):
        pytest.skip("no trained sizing model shipped")
    rng = np.random.Generator(np.random.PCG64(7))
    a = synth.erdos_renyi(32768, 16.0, rng)
    model = None
    if sizing:
        model = api.SizingModel.load(handle)
        model.attach(1.0)
    try:
        got, S = check_product(handle, a, a, "rowwise", np.float32)
    finally:
        if model is not None:
            model.detach()
            model.free()
    assert got["numtileC"] == 2048 * 2048


def test_host_range_copy_matches_full(handle):
    import ctypes as C
    from gpu_spgemm_gb300 import _lib as L
    a = synth.rmat(12, 16)
    A = api.csr2tile(handle, a)
    B = api.build_csc_tiles(handle, a)
    Cm = api.spgemm(handle, A, B)
    full = Cm.to_host()
    nt = Cm.numtileC
    tb, te = nt // 3, (2 * nt) // 3
    v0, v1 = full["tile_nnzC"][tb], full["tile_nnzC"][te]
    o = dict(r=np.zeros(te - tb, np.int32), c=np.zeros(te - tb, np.int32), m=np.zeros((te - tb) * 16, np.uint16),
             p=np.zeros(te - tb + 1, np.int64), pr=np.zeros((te - tb) * 16, np.uint8),
             v=np.zeros(v1 - v0, np.float32), cc=np.zeros(v1 - v0, np.uint8))
    nv = C.c_int64()
    P = lambda x: x.ctypes.data_as(C.c_void_p)
    handle.check(handle.lib.spg_ctiles_to_host_range(handle.h, C.byref(Cm.c), tb, te, P(o["r"]), P(o["c"]),
                                                     P(o["m"]), P(o["p"]), P(o["pr"]), P(o["v"]), P(o["cc"]),
                                                     int(v1 - v0), C.byref(nv)))
    assert nv.value == v1 - v0
    np.testing.assert_array_equal(o["r"], full["tile_rowidxC"][tb:te])
    np.testing.assert_array_equal(o["m"], full["maskC"][tb * 16:te * 16])
    np.testing.assert_array_equal(o["p"], full["tile_nnzC"][tb:te + 1])
    np.testing.assert_array_equal(o["v"], full["tile_valC"][v0:v1])
    np.testing.assert_array_equal(o["cc"], full["tile_colC"][v0:v1])
    st = handle.lib.spg_ctiles_to_host_range(handle.h, C.byref(Cm.c), tb, te, None, None, None, None, None,
                                             P(o["v"]), None, int(v1 - v0) - 1, C.byref(nv))
    assert st == L.SPG_ERR_INVALID


CSTRUCT = sorted(__import__("glob").glob(os.path.join(os.path.dirname(__file__), "golden", "cstruct_*.npz")))


@pytest.mark.parametrize("algo", ["plain", "rowwise"])
@pytest.mark.parametrize("path", CSTRUCT, ids=lambda p: os.path.basename(p)[8:-4])
def test_matches_reference_kernels_fixture(handle, path, algo):
    """Bit-exact C structure and FP64 values against the reference's own kernels."""
    z = np.load(path)
    a = synth.CSR(int(z["in_a_m"]), int(z["in_a_n"]), z["in_a_row_ptr"], z["in_a_col_idx"], z["in_a_val"])
    b = synth.CSR(int(z["in_b_m"]), int(z["in_b_n"]), z["in_b_row_ptr"], z["in_b_col_idx"], z["in_b_val"])
    A = api.csr2tile(handle, a)
    B = api.build_csc_tiles(handle, b)
    got = api.spgemm(handle, A, B, algo=algo).to_host()
    for k in STRUCT_KEYS:
        np.testing.assert_array_equal(got[k], z[k].astype(got[k].dtype), err_msg=k)
    assert rel_frob(got["tile_valC"], z["tile_valC"]) <= 1e-12


@pytest.mark.parametrize("name,a", [("stencil27_8", synth.stencil27_dof3(8)), ("dense_tile", cases.dense_tile_csr(np.float32)),
                                    ("rmat_12", synth.rmat(12, 16)), ("poisson2d_64", synth.poisson2d(64, np.float32))])
def test_mixed_precision_tensor_path(handle, name, a):
    """Dense tile pairs on tensor cores (FP16 hi+lo, FP32 accumulation): exact
    structure, <= 1e-6 relative Frobenius error against the FP64 oracle."""
    got, S = check_product(handle, a, a, "plain", np.float32, prec="mixed")
    st = handle.stats()
    if name in ("stencil27_8", "dense_tile"):
        assert st["tensor_pairs"] > 0


def test_long_tile_scan_is_exact(handle):
    """C with more than 2^22 tiles takes the two-pass streaming scan for
    tile_nnzC: every prefix step must equal the popcount of its tile's mask."""
    a = synth.rmat(16, 16)
    A = api.csr2tile(handle, a)
    B = api.build_csc_tiles(handle, a)
    C = api.symbolic(handle, A, B, algo="rowwise")
    assert C.numtileC >= (1 << 22)
    got = C.to_host(values=False)
    pc = np.unpackbits(got["maskC"].view(np.uint8)).reshape(-1, 256).sum(1, dtype=np.int64)
    assert got["tile_nnzC"][0] == 0
    np.testing.assert_array_equal(np.diff(got["tile_nnzC"]), pc)
    assert got["tile_nnzC"][-1] == got["nnzC"]


def test_mixed_params_threshold_and_validation(handle):
    """spg_set_mixed_params: out-of-range arguments are rejected; a lower
    tensor-core threshold routes more pairs to the tensor cores and the
    result stays within the FP32 tolerance with exact structure."""
    from gpu_spgemm_gb300 import _lib as L
    for bad in ((0, 1e-6), (257, 1e-6), (32, -1.0), (32, 1.0)):
        with pytest.raises(L.SpgError):
            handle.set_mixed_params(*bad)
    a = synth.stencil27_dof3(8)
    try:
        handle.set_mixed_params(200)  # above any tile's nonzeros: no tensor-core pairs
        check_product(handle, a, a, "plain", np.float32, prec="mixed")
        assert handle.stats()["tensor_pairs"] == 0
        handle.set_mixed_params(8)
        check_product(handle, a, a, "plain", np.float32, prec="mixed")
        assert handle.stats()["tensor_pairs"] > 0
    finally:
        handle.set_mixed_params(32, 2.0 ** -20)


@pytest.mark.parametrize("algo", ["plain", "rowwise"])
def test_split_symbolic_matches_one_call(handle, algo):
    """spg_symbolic_tiles then spg_symbolic_masks give the product spg_symbolic
    gives.  C's tile indices copy out between the two calls; the prefix and
    the values cannot, spg_numeric refuses a C without masks, and a second
    spg_symbolic_masks on the same C is refused without freeing it."""
    import ctypes as C
    from gpu_spgemm_gb300 import _lib as L
    lib = handle.lib
    a = synth.rmat(12, 16).astype(np.float32)
    A = api.csr2tile(handle, a)
    B = api.build_csc_tiles(handle, a)
    S = oracle.spgemm_tiles(a, a)
    Cm = api.symbolic_tiles(handle, A, B, algo=algo)
    nt = Cm.numtileC
    assert nt == S["numtileC"]
    P = lambda x: x.ctypes.data_as(C.c_void_p)
    r, c = np.zeros(nt, np.int32), np.zeros(nt, np.int32)
    handle.check(lib.spg_ctiles_to_host_range(handle.h, C.byref(Cm.c), 0, nt, P(r), P(c), None, None, None,
                                              None, None, 0, None))
    np.testing.assert_array_equal(r, S["tile_rowidxC"])
    np.testing.assert_array_equal(c, S["tile_colidxC"])
    nv = C.c_int64()
    assert lib.spg_ctiles_to_host_range(handle.h, C.byref(Cm.c), 0, nt, None, None, None, None, None, None, None,
                                        0, C.byref(nv)) == L.SPG_ERR_INVALID
    assert lib.spg_numeric(handle.h, C.byref(A.t), C.byref(B.t), api._ALGOS[algo], api._PRECS["f32"],
                           C.byref(Cm.c)) == L.SPG_ERR_INVALID
    api.symbolic_masks(handle, A, B, Cm)
    assert lib.spg_symbolic_masks(handle.h, C.byref(A.t), C.byref(B.t), C.byref(Cm.c)) == L.SPG_ERR_INVALID
    api.numeric(handle, A, B, Cm, algo=algo)
    got = Cm.to_host()
    assert got["nnzC"] == S["nnzC"]
    for k in STRUCT_KEYS:
        np.testing.assert_array_equal(got[k], S[k].astype(got[k].dtype), err_msg=k)
    assert rel_frob(got["tile_valC"], S["tile_valC"]) <= TOL[np.float32]


@pytest.mark.parametrize("algo,prec,name,a", [
    ("rowwise", "f32", "rmat_12", synth.rmat(12, 16)),
    ("plain", "f32", "rmat_12", synth.rmat(12, 16)),
    ("rowwise", "f64", "rmat_11", synth.rmat(11, 16)),
    ("plain", "mixed", "stencil27_6", synth.stencil27_dof3(6)),
], ids=["rowwise-f32", "plain-f32", "rowwise-f64acc", "plain-mixed"])
def test_numeric_rows_bands_match_whole(handle, algo, prec, name, a):
    """spg_numeric_rows over uneven tile-row bands (one of them empty) gives
    the product one spg_numeric gives; bad ranges are refused."""
    from gpu_spgemm_gb300 import _lib as L
    a = a.astype(np.float32)
    A = api.csr2tile(handle, a)
    B = api.build_csc_tiles(handle, a)
    S = oracle.spgemm_tiles(a, a)
    Cm = api.symbolic(handle, A, B, algo=algo)
    tm = Cm.tilem
    for bad in ((-1, 1), (2, 1), (0, tm + 1)):
        with pytest.raises(L.SpgError):
            api.numeric_rows(handle, A, B, Cm, *bad, algo=algo, prec=prec)
    bounds = [0, 1, 1, max(2, tm // 3), max(3, (3 * tm) // 4), tm]
    for r0, r1 in zip(bounds[:-1], bounds[1:]):
        api.numeric_rows(handle, A, B, Cm, r0, r1, algo=algo, prec=prec)
    got = Cm.to_host()
    for k in STRUCT_KEYS:
        np.testing.assert_array_equal(got[k], S[k].astype(got[k].dtype), err_msg=k)
    tol = 1e-7 if prec == "f64" else TOL[np.float32]
    assert rel_frob(got["tile_valC"], S["tile_valC"]) <= tol


@pytest.mark.parametrize("algo,prec,a", [
    ("rowwise", "f32", synth.rmat(13, 16)),
    ("rowwise", "f64", synth.rmat(11, 16)),
    ("plain", "f32", synth.rmat(11, 16)),
    ("plain", "mixed", synth.stencil27_dof3(6)),
], ids=["rowwise-f32", "rowwise-f64acc", "plain-f32", "plain-mixed"])
@pytest.mark.parametrize("last_first", [False, True], ids=["first-to-last", "last-to-first"])
def test_numeric_bands_report_final_values(handle, algo, prec, a, last_first):
    """spg_numeric_bands reports every band once, and a band's values and
    column bytes, copied by a second handle on another stream inside the
    callback (while the numeric launch may still run), already match the
    oracle.  Bad band bounds are refused."""
    import ctypes as C
    import torch
    from gpu_spgemm_gb300 import _lib as L
    a = a.astype(np.float32)
    A = api.csr2tile(handle, a)
    B = api.build_csc_tiles(handle, a)
    S = oracle.spgemm_tiles(a, a)
    Cm = api.symbolic(handle, A, B, algo=algo)
    tm = Cm.tilem
    tp, pre = S["tile_ptrC"], S["tile_nnzC"]
    for bad in ([1, tm], [0, tm - 1], [0, 3, 2, tm]):
        with pytest.raises(L.SpgError):
            api.numeric_bands(handle, A, B, Cm, bad, lambda *x: None, algo=algo, prec=prec)
    rows_ok = np.array([0, tm], np.int32)
    assert handle.lib.spg_numeric_bands(handle.h, C.byref(A.t), C.byref(B.t), api._ALGOS[algo], api._PRECS[prec],
                                        C.byref(Cm.c), 1, rows_ok.ctypes.data, 2, L.BAND_FN(lambda *x: None),
                                        None) == L.SPG_ERR_INVALID
    bounds = sorted({0, 1, tm // 5, tm // 2, (4 * tm) // 5, tm}) + [tm]  # the last band is empty
    side = api.Handle(0, torch.cuda.Stream())
    seen = []
    P = lambda x: x.ctypes.data_as(C.c_void_p)
    try:
        def on_band(k, r0, r1):
            t0, t1 = int(tp[r0]), int(tp[r1])
            v0, v1 = int(pre[t0]), int(pre[t1])
            v = np.zeros(max(1, v1 - v0), np.float32)
            cc = np.zeros(max(1, v1 - v0), np.uint8)
            nv = C.c_int64()
            side.check(side.lib.spg_ctiles_to_host_range(side.h, C.byref(Cm.c), t0, t1, None, None, None, None,
                                                         None, P(v), P(cc), v.size, C.byref(nv)))
            assert nv.value == v1 - v0
            seen.append((k, r0, r1, rel_frob(v[:v1 - v0], S["tile_valC"][v0:v1]),
                         bool(np.array_equal(cc[:v1 - v0], S["tile_colC"][v0:v1]))))

        api.numeric_bands(handle, A, B, Cm, bounds, on_band, algo=algo, prec=prec, last_first=last_first)
    finally:
        side.close()
    assert sorted(s[0] for s in seen) == list(range(len(bounds) - 1))
    for k, r0, r1, err, cols in seen:
        assert (r0, r1) == (bounds[k], bounds[k + 1])
        assert cols, k
        assert err <= (1e-7 if prec == "f64" else TOL[np.float32]), (k, err)
    got = Cm.to_host()
    assert rel_frob(got["tile_valC"], S["tile_valC"]) <= TOL[np.float32]


def wide_span_case():
    """A: 256 rows of 64 columns spread over ~1.05 M columns; B: Erdős–Rényi
    of that size, degree 2.  C's tile-rows span the whole width sparsely
    (2,056 rank-bitmap words, most C tiles empty), so row-wise windows are
    bounded by the span they cover rather than by their values."""
    rng = np.random.Generator(np.random.PCG64(11))
    n = (1 << 20) + 4096
    b = synth.erdos_renyi(n, 2.0, rng)
    m = 256
    rows = np.repeat(np.arange(m), 64)
    cols = rng.integers(0, n, size=m * 64)
    a = synth._assemble(m, n, [rows], [cols], [rng.random(m * 64) * 2 - 1], np.float32)
    return a, b


@pytest.mark.parametrize("algo", ["rowwise", "plain"])
def test_wide_sparse_span(handle, algo):
    a, b = wide_span_case()
    check_product(handle, a, b, algo, np.float32)
