"""ctypes access to oracle/_ref/libreftile.so: the reference project's own
csr2tile / build_csc_tiles (src/tile_format.h:93,424) compiled from its source.
TEST INFRASTRUCTURE ONLY; present only where the reference checkout exists."""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_ref", "libreftile.so")
TS = 16


def available() -> bool:
    if not os.path.exists(LIB):
        try:
            subprocess.run(["sh", os.path.join(HERE, "build_ref.sh")], check=True, capture_output=True)
        except Exception:
            return False
    return os.path.exists(LIB)


def _lib():
    l = C.CDLL(LIB)
    l.ref_build.restype = C.c_int
    l.ref_build.argtypes = [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]
    l.ref_get.restype = None
    l.ref_get.argtypes = [C.c_void_p] * 12
    return l


def ref_tiles(csr, csc: bool) -> dict:
    """Run the reference tiler on a host CSR; returns its arrays."""
    l = _lib()
    rp = np.ascontiguousarray(csr.row_ptr, np.int32)
    ci = np.ascontiguousarray(csr.col_idx, np.int32)
    val = np.ascontiguousarray(csr.val, np.float64)
    nt = l.ref_build(csr.m, csr.n, int(rp[-1]), rp.ctypes.data, ci.ctypes.data, val.ctypes.data, int(csc))
    tilem, tilen = (csr.m + TS - 1) // TS, (csr.n + TS - 1) // TS
    nz = int(rp[-1])
    o = dict(tile_ptr=np.zeros(tilem + 1, np.int32), tile_columnidx=np.zeros(nt, np.int32),
             tile_nnz=np.zeros(nt + 1, np.int32), tile_csr_Ptr=np.zeros(nt * TS, np.uint8),
             mask=np.zeros(nt * TS, np.uint16), tile_csr_Val=np.zeros(nz, np.float64),
             tile_csr_Col=np.zeros(nz, np.uint8))
    if csc:
        o.update(csc_tile_ptr=np.zeros(tilen + 1, np.int32), csc_tile_rowidx=np.zeros(nt, np.int32),
                 tile_csc_Ptr=np.zeros(nt * TS, np.uint8), tile_csc_Row=np.zeros(nz, np.uint8),
                 tile_csc_Val=np.zeros(nz, np.float64))
    z = None
    g = o.get
    l.ref_get(o["tile_ptr"].ctypes.data, o["tile_columnidx"].ctypes.data, o["tile_nnz"].ctypes.data,
              o["tile_csr_Ptr"].ctypes.data, o["mask"].ctypes.data, o["tile_csr_Val"].ctypes.data,
              o["tile_csr_Col"].ctypes.data,
              *(g(k).ctypes.data if g(k) is not None else z for k in
                ("csc_tile_ptr", "csc_tile_rowidx", "tile_csc_Ptr", "tile_csc_Row", "tile_csc_Val")))
    return o


def ref_load_mtx(path: str):
    """The reference's load_mtx (src/tile_format.h:51-90) on a file: returns
    (m, n, row_ptr, col_idx, val) with duplicates kept."""
    l = C.CDLL(LIB)
    l.ref_mtx_load.restype = C.c_int
    l.ref_mtx_load.argtypes = [C.c_char_p, C.c_void_p, C.c_void_p, C.c_void_p]
    l.ref_mtx_get.restype = None
    l.ref_mtx_get.argtypes = [C.c_void_p] * 3
    m, n, nz = C.c_int(), C.c_int(), C.c_int()
    l.ref_mtx_load(path.encode(), C.byref(m), C.byref(n), C.byref(nz))
    rp = np.zeros(m.value + 1, np.int32)
    ci = np.zeros(nz.value, np.int32)
    val = np.zeros(nz.value, np.float64)
    l.ref_mtx_get(rp.ctypes.data, ci.ctypes.data, val.ctypes.data)
    return m.value, n.value, rp, ci, val
