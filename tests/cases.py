"""Seeded small matrices shared by the CPU and GPU parity tests and by the
golden-fixture generator.  Sizes are chosen so the CPU oracle finishes in
milliseconds; together they cover the edge cases of the tile format: sizes not
a multiple of 16, empty rows, columns and matrices, a fully dense 16x16 tile
(256 nonzeros, the uint8 offsets' limit), hub rows/columns, rectangular
shapes and single-row / single-column matrices."""
from __future__ import annotations

import numpy as np

from gpu_spgemm_gb300 import synth
from gpu_spgemm_gb300.synth import CSR


def random_csr(m, n, density, seed, dtype=np.float64, empty_row_frac=0.0) -> CSR:
    rng = np.random.Generator(np.random.PCG64(seed))
    mask = rng.random((m, n)) < density
    if empty_row_frac > 0:
        mask[rng.random(m) < empty_row_frac, :] = False
    r, c = np.nonzero(mask)
    vals = (rng.random(r.size) * 2 - 1).astype(dtype)
    rp = np.zeros(m + 1, np.int64)
    np.cumsum(np.bincount(r, minlength=m), out=rp[1:])
    return CSR(m, n, rp.astype(np.int32), c.astype(np.int32), vals)


def dense_tile_csr(dtype=np.float64) -> CSR:
    """40x40: a full 16x16 tile at (0,0), a full tile row segment, scattered rest."""
    rng = np.random.Generator(np.random.PCG64(7))
    d = np.zeros((40, 40), bool)
    d[:16, :16] = True
    d[16:32, 16:32] = rng.random((16, 16)) < 0.9
    d[32:40, :] = rng.random((8, 40)) < 0.2
    d[:, 33] = True
    r, c = np.nonzero(d)
    rp = np.zeros(41, np.int64)
    np.cumsum(np.bincount(r, minlength=40), out=rp[1:])
    return CSR(40, 40, rp.astype(np.int32), c.astype(np.int32), rng.standard_normal(r.size).astype(dtype))


def hub_csr(n=300, seed=3, dtype=np.float64) -> CSR:
    """Random sparse square matrix plus a dense row and a dense column."""
    rng = np.random.Generator(np.random.PCG64(seed))
    d = rng.random((n, n)) < 0.01
    d[5, :] = True
    d[:, 200] = True
    r, c = np.nonzero(d)
    rp = np.zeros(n + 1, np.int64)
    np.cumsum(np.bincount(r, minlength=n), out=rp[1:])
    return CSR(n, n, rp.astype(np.int32), c.astype(np.int32), (rng.random(r.size) * 2 - 1).astype(dtype))


def empty_csr(m, n, dtype=np.float64) -> CSR:
    return CSR(m, n, np.zeros(m + 1, np.int32), np.zeros(0, np.int32), np.zeros(0, dtype))


def tiler_cases():
    """(name, csr) pairs for tiling tests (any shape)."""
    return [
        ("poisson2d_8", synth.poisson2d(8)),
        ("poisson2d_13", synth.poisson2d(13)),
        ("rand_50x37", random_csr(50, 37, 0.1, 1, empty_row_frac=0.2)),
        ("rand_70x40", random_csr(70, 40, 0.05, 2)),
        ("dense_tile", dense_tile_csr()),
        ("hub_300", hub_csr()),
        ("empty_20", empty_csr(20, 20)),
        ("rmat_8", synth.rmat(8, 8, dtype=np.float64)),
        ("stencil27_4", synth.stencil27_dof3(4, dtype=np.float64)),
        ("row_1x100", random_csr(1, 100, 0.3, 4)),
        ("col_100x1", random_csr(100, 1, 0.3, 5)),
    ]


def product_cases():
    """(name, A, B) pairs with A.n == B.m for SpGEMM parity tests."""
    p = synth.poisson2d(13)
    s27 = synth.stencil27_dof3(4, dtype=np.float64)
    rm = synth.rmat(9, 8, dtype=np.float64)
    dt = dense_tile_csr()
    hub = hub_csr()
    a_rect = random_csr(50, 70, 0.05, 11, empty_row_frac=0.1)
    b_rect = random_csr(70, 45, 0.06, 12, empty_row_frac=0.1)
    e = empty_csr(20, 20)
    return [
        ("poisson2d_13^2", p, p),
        ("stencil27_4^2", s27, s27),
        ("rmat_9^2", rm, rm),
        ("dense_tile^2", dt, dt),
        ("hub_300^2", hub, hub),
        ("rect_50x70*70x45", a_rect, b_rect),
        ("empty^2", e, e),
        ("poisson*empty", synth.poisson2d(4), empty_csr(16, 16)),
        ("rmat_9*transpose", rm, synth.transpose(rm)),
    ]


def reference_kernel_extra_cases():
    """Extra cases for the reference-kernel fixtures: C tiles with more than 32
    matched tile pairs (the merge fallback of src/spgemm_raw_kernels.cuh:189-194
    and src/spgemm_raw_kernels_v2.cuh:100-109)."""
    a = random_csr(600, 600, 0.015, 31)
    return [("rand_600_many_pairs^2", a, a)]
