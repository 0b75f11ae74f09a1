"""Host-side mirror of jianjianh1/GPU_SPGEMM's interface over the C ABI.

The reference's interface is source level: ``csr2tile`` and ``build_csc_tiles``
(src/tile_format.h:93,424) build a ``TileMatrix``; ``upload_tiles``
(src/spgemm_raw_v2.cu:25) copies it to the GPU; ``main`` (src/spgemm_raw_v2.cu:101-243)
runs step 1 (tile structure), step 2 (bitmask symbolic) and step 3 (numeric).
Here the same names build device-resident tiles directly on the GPU and the
steps run through ``libspgemm_gb300.so``.  Array names and meanings follow
``TileMatrix``; ``to_host()`` returns them as numpy arrays with the same keys the
CPU oracle uses, so tests compare them one to one.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L

TS = 16
_ALGOS = {"auto": L.SPG_ALGO_AUTO, "plain": L.SPG_ALGO_PLAIN, "rowwise": L.SPG_ALGO_ROWWISE}
_PRECS = {"f32": L.SPG_PREC_F32, "mixed": L.SPG_PREC_MIXED, "f64": L.SPG_PREC_F64}


def _dtype_code(dt) -> int:
    dt = np.dtype(dt)
    if dt == np.float32:
        return L.SPG_F32
    if dt == np.float64:
        return L.SPG_F64
    raise ValueError(f"unsupported value dtype {dt}")


def _np_dtype(code: int):
    return np.float64 if code == L.SPG_F64 else np.float32


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


class Handle:
    """Library handle bound to one device and one CUDA stream (an int
    ``cudaStream_t`` or an object with a ``cuda_stream`` attribute)."""

    def __init__(self, device: int = 0, stream=None):
        self.lib = L.load()
        s = getattr(stream, "cuda_stream", stream)
        self.h = C.c_void_p()
        st = self.lib.spg_create(C.byref(self.h), device, C.c_void_p(s or 0))
        if st != L.SPG_OK:
            raise L.SpgError(st, "spg_create failed")

    def check(self, status):
        L.check(self.h, status)

    def set_stream(self, stream):
        s = getattr(stream, "cuda_stream", stream)
        self.check(self.lib.spg_set_stream(self.h, C.c_void_p(s or 0)))

    def stats(self) -> dict:
        st = L.SpgStats()
        self.check(self.lib.spg_get_stats(self.h, C.byref(st)))
        return {k: getattr(st, k) for k, _ in L.SpgStats._fields_}

    def close(self):
        if self.h:
            self.lib.spg_destroy(self.h)
            self.h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


class TileMatrix:
    """Device-resident tile matrix (the reference's ``TileMatrix``)."""

    def __init__(self, handle: Handle, t: L.SpgTiles):
        self.handle = handle
        self.t = t

    def __getattr__(self, k):
        if k in ("m", "n", "nnz", "tilem", "tilen", "numtile", "dtype", "layout"):
            return getattr(self.t, k)
        raise AttributeError(k)

    @property
    def value_dtype(self):
        return _np_dtype(self.t.dtype)

    def to_host(self) -> dict:
        t = self.t
        nt, nz = t.numtile, t.nnz
        vd = _np_dtype(t.dtype)
        out = dict(m=t.m, n=t.n, nnz=nz, tilem=t.tilem, tilen=t.tilen, numtile=nt,
                   tile_ptr=np.zeros(t.tilem + 1, np.int32), tile_columnidx=np.zeros(nt, np.int32),
                   tile_nnz=np.zeros(nt + 1, np.int32), tile_csr_Ptr=np.zeros(nt * TS, np.uint8),
                   mask=np.zeros(nt * TS, np.uint16), tile_csr_Val=np.zeros(nz, vd),
                   tile_csr_Col=np.zeros(nz, np.uint8))
        csc = t.layout == L.SPG_LAYOUT_B_CSC
        if csc:
            out.update(csc_tile_ptr=np.zeros(t.tilen + 1, np.int32), csc_tile_rowidx=np.zeros(nt, np.int32),
                       numtileB_csc=nt)
        has_tcsc = bool(t.tile_csc_Ptr)
        if has_tcsc:
            out.update(tile_csc_Ptr=np.zeros(nt * TS, np.uint8), tile_csc_Row=np.zeros(nz, np.uint8),
                       tile_csc_Val=np.zeros(nz, vd))
        g = out.get
        self.handle.check(self.handle.lib.spg_tiles_to_host(
            self.handle.h, C.byref(t), _ptr(out["tile_ptr"]), _ptr(out["tile_columnidx"]), _ptr(out["tile_nnz"]),
            _ptr(out["tile_csr_Ptr"]), _ptr(out["mask"]), _ptr(out["tile_csr_Val"]), _ptr(out["tile_csr_Col"]),
            _ptr(g("csc_tile_ptr")), _ptr(g("csc_tile_rowidx")), _ptr(g("tile_csc_Ptr")), _ptr(g("tile_csc_Row")),
            _ptr(g("tile_csc_Val"))))
        return out

    def free(self):
        if self.t.tile_ptr or self.t.row_ptr:
            self.handle.check(self.handle.lib.spg_tiles_free(self.handle.h, C.byref(self.t)))

    def __del__(self):
        try:
            if self.handle.h:
                self.free()
        except Exception:
            pass


def tile_from_csr(handle: Handle, csr, layout: int, flags: int = 0) -> TileMatrix:
    """Tile a host CSR (anything with m, n, row_ptr, col_idx, val)."""
    rp = np.ascontiguousarray(csr.row_ptr, np.int32)
    ci = np.ascontiguousarray(csr.col_idx, np.int32)
    val = np.ascontiguousarray(csr.val)
    code = _dtype_code(val.dtype)
    t = L.SpgTiles()
    handle.check(handle.lib.spg_tile_from_csr_host(handle.h, int(csr.m), int(csr.n), int(rp[-1]), _ptr(rp),
                                                   _ptr(ci), _ptr(val), code, layout, flags, C.byref(t)))
    return TileMatrix(handle, t)


def tile_from_device_csr(handle: Handle, m: int, n: int, nnz: int, row_ptr: int, col_idx: int, val: int,
                         dtype, layout: int, flags: int = 0) -> TileMatrix:
    """Tile a CSR already in device memory (raw device pointers)."""
    t = L.SpgTiles()
    handle.check(handle.lib.spg_tile_from_csr(handle.h, m, n, nnz, C.c_void_p(row_ptr), C.c_void_p(col_idx),
                                              C.c_void_p(val), _dtype_code(dtype), layout, flags, C.byref(t)))
    return TileMatrix(handle, t)


def csr2tile(handle: Handle, csr) -> TileMatrix:
    """Row-major tiling of A (src/tile_format.h:93-222), built on the GPU."""
    return tile_from_csr(handle, csr, L.SPG_LAYOUT_ROW)


def build_csc_tiles(handle: Handle, csr, with_tile_csc: bool = False) -> TileMatrix:
    """B in CSC tile order (src/tile_format.h:424-585), built on the GPU."""
    return tile_from_csr(handle, csr, L.SPG_LAYOUT_B_CSC, L.SPG_TILE_WITH_TILE_CSC if with_tile_csc else 0)


class CTileMatrix:
    """Device-resident C tiles as steps 1-3 produce them."""

    def __init__(self, handle: Handle, c: L.SpgCTiles):
        self.handle = handle
        self.c = c

    def __getattr__(self, k):
        if k in ("m", "n", "tilem", "tilen", "numtileC", "nnzC", "pairs", "dtype"):
            return getattr(self.c, k)
        raise AttributeError(k)

    def to_host(self, values: bool = True) -> dict:
        c = self.c
        nt, nz = c.numtileC, c.nnzC
        out = dict(tilem=c.tilem, tilen=c.tilen, numtileC=nt, nnzC=nz, pairs=c.pairs,
                   tile_ptrC=np.zeros(c.tilem + 1, np.int32), tile_rowidxC=np.zeros(nt, np.int32),
                   tile_colidxC=np.zeros(nt, np.int32), maskC=np.zeros(nt * TS, np.uint16),
                   tile_nnzC=np.zeros(nt + 1, np.int64), ptrRowC=np.zeros(nt * TS, np.uint8))
        if values:
            out.update(tile_valC=np.zeros(nz, _np_dtype(c.dtype)), tile_colC=np.zeros(nz, np.uint8))
        g = out.get
        self.handle.check(self.handle.lib.spg_ctiles_to_host(
            self.handle.h, C.byref(c), _ptr(out["tile_ptrC"]), _ptr(out["tile_rowidxC"]), _ptr(out["tile_colidxC"]),
            _ptr(out["maskC"]), _ptr(out["tile_nnzC"]), _ptr(out["ptrRowC"]), _ptr(g("tile_valC")),
            _ptr(g("tile_colC"))))
        return out

    def free(self):
        if self.c.tile_ptrC or self.c.priv:
            self.handle.check(self.handle.lib.spg_ctiles_free(self.handle.h, C.byref(self.c)))

    def __del__(self):
        try:
            if self.handle.h:
                self.free()
        except Exception:
            pass


def symbolic(handle: Handle, A: TileMatrix, B: TileMatrix, algo: str = "auto") -> CTileMatrix:
    """Steps 1 and 2 (src/spgemm_raw_v2.cu:111-221)."""
    c = L.SpgCTiles()
    handle.check(handle.lib.spg_symbolic(handle.h, C.byref(A.t), C.byref(B.t), _ALGOS[algo], C.byref(c)))
    return CTileMatrix(handle, c)


def numeric(handle: Handle, A: TileMatrix, B: TileMatrix, Cm: CTileMatrix, algo: str = "auto",
            prec: str = "f32") -> CTileMatrix:
    """Step 3 (src/spgemm_raw_v2.cu:223-243)."""
    handle.check(handle.lib.spg_numeric(handle.h, C.byref(A.t), C.byref(B.t), _ALGOS[algo], _PRECS[prec],
                                        C.byref(Cm.c)))
    return Cm


def spgemm(handle: Handle, A: TileMatrix, B: TileMatrix, algo: str = "auto", prec: str = "f32") -> CTileMatrix:
    """Steps 1-3 in one call."""
    c = L.SpgCTiles()
    handle.check(handle.lib.spg_spgemm(handle.h, C.byref(A.t), C.byref(B.t), _ALGOS[algo], _PRECS[prec],
                                       C.byref(c)))
    return CTileMatrix(handle, c)


def products(handle: Handle, A: TileMatrix, B: TileMatrix) -> int:
    """Intermediate products (src/spgemm_raw_v2.cu:95-99)."""
    out = C.c_int64()
    handle.check(handle.lib.spg_products(handle.h, C.byref(A.t), C.byref(B.t), C.byref(out)))
    return out.value
