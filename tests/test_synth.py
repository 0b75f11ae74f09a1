"""The synthetic workloads have the documented shapes."""
import numpy as np

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
