"""The synthetic workloads have the documented shapes; the Matrix Market
reader follows the reference's load_mtx (src/tile_format.h:51-90)."""
import glob
import os

import numpy as np
import pytest

from gpu_spgemm_gb300 import synth


def test_poisson2d_256():
    a = synth.poisson2d(256)
    assert (a.m, a.nnz) == (65536, 326656)
    assert synth.products(a, a) == 1629192
    assert a.val.dtype == np.float64


def test_stencil27_dof3_small_matches_formula():
    g = 6
    a = synth.stencil27_dof3(g)
    assert a.m == 3 * g ** 3
    assert a.nnz == (g + 2 * (g - 1)) ** 3 * 9
    d = np.diff(a.col_idx.astype(np.int64))
    starts = np.zeros(a.nnz, bool)
    starts[a.row_ptr[:-1][np.diff(a.row_ptr) > 0]] = True
    assert np.all(d[~starts[1:]] > 0)


def test_poisson3d_small():
    g = 8
    a = synth.poisson3d(g)
    assert a.nnz == 7 * g ** 3 - 6 * g ** 2


def test_rmat_small_canonical_and_deterministic():
    a = synth.rmat(10, 8)
    b = synth.rmat(10, 8)
    assert np.array_equal(a.col_idx, b.col_idx) and np.array_equal(a.val, b.val)
    assert a.nnz <= 8 * 1024
    assert np.all(np.abs(a.val) <= 1)


def test_er_batch_sizes():
    pairs = synth.er_batch(6, 1024, 4096)
    for A, B in pairs:
        assert 1024 <= A.m <= 4096 and A.m == A.n == B.m == B.n
        assert 2 <= A.nnz / A.m <= 40


def test_transpose_roundtrip():
    a = synth.rmat(8, 4)
    t = synth.transpose(synth.transpose(a))
    assert np.array_equal(t.row_ptr, a.row_ptr) and np.array_equal(t.col_idx, a.col_idx)


def test_smoothed_aggregation_shapes():
    a = synth.poisson3d(8)
    p0 = synth.aggregation_p0(8)
    p = synth.smoothed_aggregation(a, p0)
    assert (p.m, p.n) == (512, 64)
    assert p0.nnz == 512


MTX_DIR = os.path.join(os.path.dirname(__file__), "golden")
MTX = sorted(glob.glob(os.path.join(MTX_DIR, "mtx", "*.mtx")))


def _rows_as_sets(rp, ci, val):
    return [sorted(zip(ci[rp[i]:rp[i + 1]].tolist(), val[rp[i]:rp[i + 1]].tolist())) for i in range(len(rp) - 1)]


def test_mtx_fixtures_present():
    assert len(MTX) >= 5


@pytest.mark.parametrize("path", MTX, ids=lambda p: os.path.basename(p)[:-4])
def test_load_mtx_matches_reference_reader(path):
    """synth.load_mtx against the reference's own load_mtx
    (src/tile_format.h:51-90) recorded in mtx_<name>.npz: with merge=False the
    same rows, columns and values, duplicates included (compared per row as
    multisets: the reference's sort leaves duplicates in no set order); with
    merge=True the duplicates summed and every row strictly ascending."""
    z = np.load(os.path.join(MTX_DIR, "mtx_" + os.path.basename(path)[:-4] + ".npz"))
    a = synth.load_mtx(path, merge=False)
    assert (a.m, a.n) == (int(z["m"]), int(z["n"]))
    np.testing.assert_array_equal(a.row_ptr, z["row_ptr"])
    assert _rows_as_sets(a.row_ptr, a.col_idx, a.val) == _rows_as_sets(z["row_ptr"], z["col_idx"], z["val"])
    b = synth.load_mtx(path)
    for i in range(b.m):
        c = b.col_idx[b.row_ptr[i]:b.row_ptr[i + 1]]
        assert np.all(np.diff(c) > 0)
        want = {}
        for col, v in zip(z["col_idx"][z["row_ptr"][i]:z["row_ptr"][i + 1]], z["val"][z["row_ptr"][i]:z["row_ptr"][i + 1]]):
            want[int(col)] = want.get(int(col), 0.0) + float(v)
        got = dict(zip(c.tolist(), b.val[b.row_ptr[i]:b.row_ptr[i + 1]].tolist()))
        assert got == want, i


def test_load_mtx_product_through_the_oracle():
    """A loaded matrix goes through the tiled oracle like any other input."""
    import oracle
    a = synth.load_mtx(os.path.join(MTX_DIR, "mtx", "symmetric.mtx"))
    S = oracle.spgemm_tiles(a, a)
    d = a.to_scipy().toarray()
    rp, ci, v = oracle.tiles_to_csr(a.m, a.n, S)
    got = np.zeros_like(d)
    for i in range(a.m):
        got[i, ci[rp[i]:rp[i + 1]]] = v[rp[i]:rp[i + 1]]
    np.testing.assert_allclose(got, d @ d, rtol=1e-12)
