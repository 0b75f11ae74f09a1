"""Per-tile-row binning (SPG_ALGO_BINNED, the AUTO default): each C tile-row
goes to the plain per-C-tile kernels or to the row-wise windows, decided
from its products per tile pair and, with the sizing model attached, from
the model's predicted C nonzeros per C tile.  A block-diagonal matrix of a
stencil beside a power-law graph gets both bins in one product; the result
must equal the oracle's exactly in structure and within the value tolerance
on every path that consumes a binned C (whole, tile-row ranges, bands, FP64
accumulation, mixed precision)."""
import os

import numpy as np
import pytest

import oracle
from gpu_spgemm_gb300 import api, synth

pytestmark = pytest.mark.gpu
KEYS = ["tile_ptrC", "tile_rowidxC", "tile_colidxC", "maskC", "tile_nnzC", "ptrRowC", "tile_colC"]
PLAIN, ROWWISE, BINNED = 1, 2, 3


def rel(x, y):
    x = np.asarray(x, np.float64)
    y = np.asarray(y, np.float64)
    return np.linalg.norm(x - y) / (np.linalg.norm(y) or 1.0)


def mixed(dtype=np.float32):
    return synth.block_diag(synth.stencil27_dof3(6), synth.rmat(11, 16)).astype(dtype)


def check(got, S, tol):
    assert got["numtileC"] == S["numtileC"] and got["nnzC"] == S["nnzC"]
    for k in KEYS:
        np.testing.assert_array_equal(got[k], S[k].astype(got[k].dtype), err_msg=k)
    assert rel(got["tile_valC"], S["tile_valC"]) <= tol


@pytest.fixture(scope="module")
def mixed32():
    a = mixed()
    return a, oracle.spgemm_tiles(a, a)


@pytest.mark.parametrize("algo", ["binned", "auto"])
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_binned_mixed_matrix(handle, algo, dtype):
    """AUTO bins an A of at least 65,536 tiles (the larger mixed matrix)."""
    a = mixed(dtype) if algo == "binned" else \
        synth.block_diag(synth.stencil27_dof3(8), synth.rmat(14, 16)).astype(dtype)
    S = oracle.spgemm_tiles(a, a)
    A = api.csr2tile(handle, a)
    B = api.build_csc_tiles(handle, a)
    Cm = api.spgemm(handle, A, B, algo=algo)
    assert handle.stats()["algo_used"] == BINNED
    check(Cm.to_host(), S, 1e-12 if dtype == np.float64 else 1e-6)


@pytest.mark.skipif(not os.path.exists(api.SIZING_MODEL_PATH), reason="no trained sizing model shipped")
def test_learned_bins_with_the_sizing_model(handle, mixed32):
    a, S = mixed32
    model = api.SizingModel.load(handle)
    model.attach(1.0)
    try:
        A = api.csr2tile(handle, a)
        B = api.build_csc_tiles(handle, a)
        Cm = api.spgemm(handle, A, B, algo="binned")
        st = handle.stats()
    finally:
        model.detach()
        model.free()
    assert st["algo_used"] == BINNED and st["predicted_tiles"] > 0
    check(Cm.to_host(), S, 1e-6)


def test_pure_matrices_run_one_algorithm(handle):
    rng = np.random.Generator(np.random.PCG64(5))
    for a, want in ((synth.erdos_renyi(4096, 8.0, rng), ROWWISE), (synth.stencil27_dof3(5), PLAIN)):
        A = api.csr2tile(handle, a)
        B = api.build_csc_tiles(handle, a)
        Cm = api.spgemm(handle, A, B, algo="binned")
        assert handle.stats()["algo_used"] == want
        check(Cm.to_host(), oracle.spgemm_tiles(a, a), 1e-6)


def test_bin_thresholds_move_rows(handle, mixed32):
    """pp_thr above every tile-row's products per pair sends all to the
    row-wise windows; 0 sends all to the plain kernels; results unchanged."""
    a, S = mixed32
    A = api.csr2tile(handle, a)
    B = api.build_csc_tiles(handle, a)
    try:
        for pp, want in ((1e6, ROWWISE), (0.0, PLAIN)):
            handle.set_bin_params(pp, 0.0)
            Cm = api.spgemm(handle, A, B, algo="binned")
            assert handle.stats()["algo_used"] == want
            check(Cm.to_host(), S, 1e-6)
        from gpu_spgemm_gb300 import _lib as L
        for bad in ((-1.0, 1.0), (1.0, -1.0), (1.0, 300.0)):
            with pytest.raises(L.SpgError):
                handle.set_bin_params(*bad)
    finally:
        handle.set_bin_params()


@pytest.mark.parametrize("prec,tol", [("f64", 1e-7), ("mixed", 1e-6)])
def test_binned_c_other_precisions(handle, mixed32, prec, tol):
    """FP64 accumulation runs the row-wise kernels over every tile-row of a
    binned C; mixed precision runs the plain kernels over every tile (the
    pair cache holds the binned tiles' pairs, the rest intersect)."""
    a, S = mixed32
    A = api.csr2tile(handle, a)
    B = api.build_csc_tiles(handle, a)
    Cm = api.symbolic(handle, A, B, algo="binned")
    api.numeric(handle, A, B, Cm, prec=prec)
    check(Cm.to_host(), S, tol)


def test_binned_rows_and_bands(handle, mixed32):
    a, S = mixed32
    A = api.csr2tile(handle, a)
    B = api.build_csc_tiles(handle, a)
    Cm = api.symbolic(handle, A, B, algo="binned")
    tm = Cm.tilem
    stencil_rows = (3 * 6 ** 3 + 15) // 16
    bounds = [0, 3, stencil_rows, stencil_rows + 5, tm]   # bands across the bin boundary
    for r0, r1 in zip(bounds[:-1], bounds[1:]):
        api.numeric_rows(handle, A, B, Cm, r0, r1)
    check(Cm.to_host(), S, 1e-6)
    Cm2 = api.symbolic(handle, A, B, algo="binned")
    seen = []
    api.numeric_bands(handle, A, B, Cm2, bounds, lambda k, r0, r1: seen.append(k), last_first=True)
    assert sorted(seen) == list(range(len(bounds) - 1))
    check(Cm2.to_host(), S, 1e-6)
