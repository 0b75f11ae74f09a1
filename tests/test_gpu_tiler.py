"""CUDA tiler parity: bit-exact against the reference's tiler (golden fixtures)
and the CPU oracle."""
import glob
import os

import numpy as np
import pytest

import oracle
from gpu_spgemm_gb300 import api, synth
from gpu_spgemm_gb300._lib import SpgError, SPG_ERR_INVALID
from gpu_spgemm_gb300.synth import CSR
import cases

pytestmark = pytest.mark.gpu

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "tiles_*.npz")))
A_KEYS = ["tile_ptr", "tile_columnidx", "tile_nnz", "tile_csr_Ptr", "mask", "tile_csr_Col"]
B_KEYS = A_KEYS + ["csc_tile_ptr", "csc_tile_rowidx", "tile_csc_Ptr", "tile_csc_Row"]


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("path", GOLDEN, ids=lambda p: os.path.basename(p)[6:-4])
def test_tiler_matches_reference_golden(handle, path, dtype):
    z = np.load(path)
    csr = CSR(int(z["in_m"]), int(z["in_n"]), z["in_row_ptr"], z["in_col_idx"], z["in_val"].astype(dtype))
    A = api.csr2tile(handle, csr).to_host()
    for k in A_KEYS:
        np.testing.assert_array_equal(A[k], z["A_" + k], err_msg=k)
    np.testing.assert_array_equal(A["tile_csr_Val"], z["A_tile_csr_Val"].astype(dtype))
    B = api.build_csc_tiles(handle, csr, with_tile_csc=True).to_host()
    for k in B_KEYS:
        np.testing.assert_array_equal(B[k], z["B_" + k], err_msg=k)
    np.testing.assert_array_equal(B["tile_csr_Val"], z["B_tile_csr_Val"].astype(dtype))
    np.testing.assert_array_equal(B["tile_csc_Val"], z["B_tile_csc_Val"].astype(dtype))


@pytest.mark.parametrize("name,csr", [
    ("rmat_14", synth.rmat(14, 16)),
    ("stencil27_10", synth.stencil27_dof3(10)),
    ("poisson3d_24", synth.poisson3d(24)),
    ("rand_1000x777", cases.random_csr(1000, 777, 0.01, 9, dtype=np.float32, empty_row_frac=0.3)),
])
def test_tiler_matches_oracle_larger(handle, name, csr):
    A = api.csr2tile(handle, csr).to_host()
    OA = oracle.csr2tile(csr)
    for k in A_KEYS:
        np.testing.assert_array_equal(A[k], OA[k], err_msg=k)
    np.testing.assert_array_equal(A["tile_csr_Val"], OA["tile_csr_Val"].astype(np.float32))
    B = api.build_csc_tiles(handle, csr).to_host()
    OB = oracle.build_csc_tiles(csr, with_tile_csc=False)
    for k in A_KEYS + ["csc_tile_ptr", "csc_tile_rowidx"]:
        np.testing.assert_array_equal(B[k], OB[k], err_msg=k)
    np.testing.assert_array_equal(B["tile_csr_Val"], OB["tile_csr_Val"].astype(np.float32))


def test_tiler_rejects_unsorted_columns(handle):
    bad = CSR(2, 20, np.array([0, 2, 3], np.int32), np.array([5, 3, 1], np.int32), np.ones(3))
    with pytest.raises(SpgError) as e:
        api.csr2tile(handle, bad)
    assert e.value.status == SPG_ERR_INVALID


def test_tiler_rejects_out_of_range_column(handle):
    bad = CSR(2, 20, np.array([0, 1, 2], np.int32), np.array([5, 20], np.int32), np.ones(2))
    with pytest.raises(SpgError) as e:
        api.build_csc_tiles(handle, bad)
    assert e.value.status == SPG_ERR_INVALID
    # handle stays usable
    ok = api.csr2tile(handle, synth.poisson2d(4)).to_host()
    assert ok["numtile"] == 1
