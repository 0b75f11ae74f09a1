"""ctypes binding of libspgemm_gb300.so (C ABI in include/spgemm_gb300.h).

Loading fails loudly when the library has not been built: there is no CPU
fallback anywhere in the product path.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libspgemm_gb300.so")

SPG_OK, SPG_ERR_INVALID, SPG_ERR_OOM, SPG_ERR_OVERFLOW_RERUN, SPG_ERR_TIMEOUT, SPG_ERR_CUDA, \
    SPG_ERR_UNSUPPORTED = range(7)
STATUS_NAMES = {0: "SPG_OK", 1: "SPG_ERR_INVALID", 2: "SPG_ERR_OOM", 3: "SPG_ERR_OVERFLOW_RERUN",
                4: "SPG_ERR_TIMEOUT", 5: "SPG_ERR_CUDA", 6: "SPG_ERR_UNSUPPORTED"}
SPG_F32, SPG_F64 = 0, 1
SPG_LAYOUT_ROW, SPG_LAYOUT_B_CSC = 0, 1
SPG_TILE_WITH_TILE_CSC = 1
SPG_TILE = 16  # tile edge
SPG_ALGO_AUTO, SPG_ALGO_PLAIN, SPG_ALGO_ROWWISE, SPG_ALGO_BINNED = 0, 1, 2, 3
SPG_PREC_F32, SPG_PREC_MIXED, SPG_PREC_F64 = 0, 1, 2
SPG_BANDS_FIRST_TO_LAST, SPG_BANDS_LAST_TO_FIRST = 0, 1

P = C.c_void_p
I32 = C.c_int
I64 = C.c_int64


class SpgTiles(C.Structure):
    _fields_ = [("m", I32), ("n", I32), ("nnz", I64), ("tilem", I32), ("tilen", I32), ("numtile", I64),
                ("dtype", I32), ("layout", I32),
                ("tile_ptr", P), ("tile_columnidx", P), ("tile_nnz", P), ("tile_csr_Ptr", P), ("mask", P),
                ("tile_csr_Val", P), ("tile_csr_Col", P), ("csc_tile_ptr", P), ("csc_tile_rowidx", P),
                ("csc_to_row", P), ("tile_csc_Ptr", P), ("tile_csc_Row", P), ("tile_csc_Val", P),
                ("row_ptr", P), ("col_idx", P), ("row_val", P), ("priv", P)]


class SpgCTiles(C.Structure):
    _fields_ = [("m", I32), ("n", I32), ("tilem", I32), ("tilen", I32), ("numtileC", I64), ("nnzC", I64),
                ("dtype", I32), ("tile_ptrC", P), ("tile_rowidxC", P), ("tile_colidxC", P), ("maskC", P),
                ("tile_nnzC", P), ("ptrRowC", P), ("tile_valC", P), ("tile_colC", P), ("pairs", I64),
                ("priv", P)]


class SpgStats(C.Structure):
    _fields_ = [("ms_step1", C.c_float), ("ms_step2", C.c_float), ("ms_step3", C.c_float),
                ("products", I64), ("overflow_reruns", I64), ("work_items", I64), ("tensor_pairs", I64),
                ("fp64_tiles", I64), ("algo_used", I32), ("sizing_fallbacks", I32), ("predicted_tiles", I64),
                ("numeric_algo", I32), ("reserved", I32)]


# spg_band_fn: (user, band, row_begin, row_end)
BAND_FN = C.CFUNCTYPE(None, C.c_void_p, C.c_int, C.c_int, C.c_int)

# name -> (restype, argtypes); every symbol the header declares
SIGNATURES = {
    "spg_create": (I32, [C.POINTER(P), I32, P]),
    "spg_destroy": (I32, [P]),
    "spg_set_stream": (I32, [P, P]),
    "spg_last_error": (C.c_char_p, [P]),
    "spg_get_stats": (I32, [P, C.POINTER(SpgStats)]),
    "spg_kernel_launches": (I32, [P, C.POINTER(I64)]),
    "spg_tile_from_csr": (I32, [P, I32, I32, I64, P, P, P, I32, I32, I32, C.POINTER(SpgTiles)]),
    "spg_tile_from_csr_host": (I32, [P, I32, I32, I64, P, P, P, I32, I32, I32, C.POINTER(SpgTiles)]),
    "spg_tiles_free": (I32, [P, C.POINTER(SpgTiles)]),
    "spg_symbolic": (I32, [P, C.POINTER(SpgTiles), C.POINTER(SpgTiles), I32, C.POINTER(SpgCTiles)]),
    "spg_numeric": (I32, [P, C.POINTER(SpgTiles), C.POINTER(SpgTiles), I32, I32, C.POINTER(SpgCTiles)]),
    "spg_spgemm": (I32, [P, C.POINTER(SpgTiles), C.POINTER(SpgTiles), I32, I32, C.POINTER(SpgCTiles)]),
    "spg_ctiles_to_host": (I32, [P, C.POINTER(SpgCTiles), P, P, P, P, P, P, P, P]),
    "spg_ctiles_to_host_range": (I32, [P, C.POINTER(SpgCTiles), I64, I64, P, P, P, P, P, P, P, I64,
                                       C.POINTER(I64)]),
    "spg_tiles_to_host": (I32, [P, C.POINTER(SpgTiles), P, P, P, P, P, P, P, P, P, P, P, P]),
    "spg_ctiles_free": (I32, [P, C.POINTER(SpgCTiles)]),
    "spg_products": (I32, [P, C.POINTER(SpgTiles), C.POINTER(SpgTiles), C.POINTER(I64)]),
    "spg_csr_transpose": (I32, [P, I32, I32, I64, P, P, P, I32, P, P, P]),
    "spg_ctiles_to_csr": (I32, [P, C.POINTER(SpgCTiles), P, P, P, C.POINTER(I64)]),
    "spg_ctiles_to_csr_noalloc": (I32, [P, C.POINTER(SpgCTiles), P, P, P, C.POINTER(I64)]),
    "spg_batch_create_host": (I32, [P, I32, P, P, P, P, P, P, P, P, P, P, P, I32, C.POINTER(P)]),
    "spg_batch_free": (I32, [P, P]),
    "spg_batch_spgemm": (I32, [P, P, I32, I32]),
    "spg_batch_info": (I32, [P, P, I32, C.POINTER(I64), C.POINTER(I64), C.POINTER(I64)]),
    "spg_batch_to_host": (I32, [P, P, I32, P, P, P, P, P, P, P, P]),
    "spg_batch_set_values_host": (I32, [P, P, P, P]),
    "spg_batch_numeric": (I32, [P, P, I32]),
    "spg_batch_graph_capture": (I32, [P, P, P, P, P, I32]),
    "spg_batch_graph_launch": (I32, [P, P]),
    "spg_batch_bin_count": (I32, [P, P, C.POINTER(I32), P]),
    "spg_batch_tune": (I32, [P, P, I32, C.POINTER(I32), P, P]),
    "spg_batch_set_bins": (I32, [P, P, I32, P, P]),
    "spg_mlp_num_params": (I32, []),
    "spg_mlp_num_features": (I32, []),
    "spg_mlp_create": (I32, [P, P, P, C.POINTER(P)]),
    "spg_mlp_free": (I32, [P, P]),
    "spg_mlp_get_params": (I32, [P, P, P, P]),
    "spg_mlp_set_norm": (I32, [P, P, P]),
    "spg_mlp_features": (I32, [P, C.POINTER(SpgTiles), C.POINTER(SpgTiles), P]),
    "spg_mlp_forward": (I32, [P, P, P, I64, P]),
    "spg_mlp_gradient": (I32, [P, P, P, P, I64, P, P]),
    "spg_mlp_train": (I32, [P, P, P, P, I64, P, I32, I32, C.c_float, P]),
    "spg_set_sizing_model": (I32, [P, P, C.c_float]),
    "spg_set_mixed_params": (I32, [P, C.c_int, C.c_float]),
    "spg_set_bin_params": (I32, [P, C.c_float, C.c_float]),
    "spg_symbolic_tiles": (I32, [P, P, P, C.c_int, P]),
    "spg_symbolic_masks": (I32, [P, P, P, P]),
    "spg_numeric_rows": (I32, [P, P, P, I32, I32, P, I32, I32]),
    "spg_numeric_bands": (I32, [P, P, P, I32, I32, P, I32, P, I32, BAND_FN, P]),
    "spg_galerkin": (I32, [P, I32, I32, I64, P, P, P, I64, P, P, P, I32, I32, I32, C.POINTER(SpgCTiles),
                           C.POINTER(I64)]),
}

_lib = None


class SpgError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


def load(path: str = LIB_PATH):
    """Load the CUDA library.  Raises if it is missing -- build it first with
    ``__graft_entry__.build()`` or ``python gpu_spgemm_gb300/build.py``."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"libspgemm_gb300.so not found at {path}; the CUDA extension must be built "
                           "(python -c 'import __graft_entry__ as g; g.build()')")
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def check(h, status: int):
    if status != SPG_OK:
        msg = load().spg_last_error(h)
        raise SpgError(status, msg.decode() if msg else "")
