"""CPU oracle for the tiled SpGEMM -- TEST INFRASTRUCTURE ONLY.

Wraps ``spgemm_oracle.c`` (a plain-C restatement of jianjianh1/GPU_SPGEMM's
tile format, bitmask symbolic phase, numeric phase and Gustavson check; see the
file header for the per-function source citations) with ctypes.  Only the test
suite, ``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` use
this module, and only as a checker / reported baseline -- never as the product.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libspgemm_oracle.so")
SRC = os.path.join(HERE, "spgemm_oracle.c")
TS = 16

_lib = None


def build(force: bool = False) -> str:
    """Compile the oracle shared library with gcc + OpenMP (portable flags only)."""
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(SRC):
        subprocess.check_call(["gcc", "-O2", "-fopenmp", "-fPIC", "-shared", "-std=c11",
                               "-o", LIB_PATH, SRC])
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(LIB_PATH)
        _declare(_lib)
    return _lib


P = C.c_void_p
I = C.c_int
L = C.c_int64


def _declare(l):
    sig = {
        "orc_tile_count": (L, [I, I, P, P, P]),
        "orc_csr2tile": (None, [I, I, P, P, P, P, P, P, P, P, P, P]),
        "orc_build_csc_tiles": (None, [I, I, P, P, P, P, P, P, P, P, P, P, P, P, P]),
        "orc_step1_count": (L, [I, I, P, P, P, P, P]),
        "orc_step1_fill": (None, [I, I, P, P, P, P, P, P, P]),
        "orc_step2_symbolic": (L, [L, P, P, P, P, P, P, P, P, P, P, P, P, P, P]),
        "orc_step3_numeric": (None, [L, P, P, P, P, P, P, P, P, P, P, P, P, P, P, P, P, P, P, P]),
        "orc_tiles_to_csr": (None, [I, I, L, P, P, P, P, P, P, P, P]),
        "orc_gustavson_rowcounts": (L, [I, I, P, P, P, P, P]),
        "orc_gustavson_fill_f64": (None, [I, I, P, P, P, P, P, P, P, P, P]),
        "orc_gustavson_fill_f32": (None, [I, I, P, P, P, P, P, P, P, P, P]),
        "orc_gustavson_range_f64": (L, [I, I, I, P, P, P, P, P, P, P]),
        "orc_gustavson_range_f32": (L, [I, I, I, P, P, P, P, P, P, P]),
        "orc_check_tilerows_f64": (None, [I, I, I, I, P, P, P, P, P, P, P, P, P, P, P, P, P, P]),
        "orc_check_tilerows_f32": (None, [I, I, I, I, P, P, P, P, P, P, P, P, P, P, P, P, P, P]),
        "orc_max_threads": (I, []),
        "orc_set_threads": (None, [I]),
    }
    for name, (res, args) in sig.items():
        f = getattr(l, name)
        f.restype = res
        f.argtypes = args


def _p(a: np.ndarray):
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def csr2tile(csr) -> dict:
    """Row-major tiling (src/tile_format.h:93-222).  Values are float64."""
    l = lib()
    m, n = csr.m, csr.n
    tilem, tilen = (m + TS - 1) // TS, (n + TS - 1) // TS
    rp, ci = _i32(csr.row_ptr), _i32(csr.col_idx)
    val = np.ascontiguousarray(csr.val, dtype=np.float64)
    tile_ptr = np.zeros(tilem + 1, np.int32)
    nt = l.orc_tile_count(m, n, _p(rp), _p(ci), _p(tile_ptr))
    nnz = csr.nnz
    T = dict(m=m, n=n, nnz=nnz, tilem=tilem, tilen=tilen, numtile=int(nt), tile_ptr=tile_ptr,
             tile_columnidx=np.zeros(nt, np.int32), tile_nnz=np.zeros(nt + 1, np.int32),
             tile_csr_Val=np.zeros(nnz, np.float64), tile_csr_Col=np.zeros(nnz, np.uint8),
             tile_csr_Ptr=np.zeros(nt * TS, np.uint8), mask=np.zeros(nt * TS, np.uint16))
    l.orc_csr2tile(m, n, _p(rp), _p(ci), _p(val), _p(tile_ptr), _p(T["tile_columnidx"]),
                   _p(T["tile_nnz"]), _p(T["tile_csr_Val"]), _p(T["tile_csr_Col"]),
                   _p(T["tile_csr_Ptr"]), _p(T["mask"]))
    return T


def build_csc_tiles(csr, with_tile_csc: bool = True) -> dict:
    """CSC tile order for B (src/tile_format.h:424-585).  Returns the B-side
    arrays: tile_ptr / tile_columnidx keep the row-major tiling (step 1 reads
    them), the rest is in CSC tile order -- the same split the reference's
    TileMatrix for B has after build_csc_tiles."""
    l = lib()
    T = csr2tile(csr)
    m, n = csr.m, csr.n
    rp, ci = _i32(csr.row_ptr), _i32(csr.col_idx)
    val = np.ascontiguousarray(csr.val, dtype=np.float64)
    nt, nnz = T["numtile"], csr.nnz
    out = dict(T)
    out.update(csc_tile_ptr=np.zeros(T["tilen"] + 1, np.int32), csc_tile_rowidx=np.zeros(nt, np.int32),
               tile_nnz=np.zeros(nt + 1, np.int32), tile_csr_Ptr=np.zeros(nt * TS, np.uint8),
               tile_csr_Val=np.zeros(nnz, np.float64), tile_csr_Col=np.zeros(nnz, np.uint8),
               mask=np.zeros(nt * TS, np.uint16), numtileB_csc=nt)
    if with_tile_csc:
        out.update(tile_csc_Ptr=np.zeros(nt * TS, np.uint8), tile_csc_Row=np.zeros(nnz, np.uint8),
                   tile_csc_Val=np.zeros(nnz, np.float64))
        tcp, tcr, tcv = _p(out["tile_csc_Ptr"]), _p(out["tile_csc_Row"]), _p(out["tile_csc_Val"])
    else:
        tcp = tcr = tcv = None
    l.orc_build_csc_tiles(m, n, _p(rp), _p(ci), _p(val), _p(out["csc_tile_ptr"]),
                          _p(out["csc_tile_rowidx"]), _p(out["tile_nnz"]), _p(out["tile_csr_Ptr"]),
                          _p(out["tile_csr_Val"]), _p(out["tile_csr_Col"]), _p(out["mask"]),
                          tcp, tcr, tcv)
    return out


def symbolic(TA: dict, TB: dict) -> dict:
    """Steps 1 and 2 (src/spgemm_raw_kernels.cuh:23-215)."""
    l = lib()
    tilemA, tilenB = TA["tilem"], TB["tilen"]
    tile_ptrC = np.zeros(tilemA + 1, np.int64)
    ntc = l.orc_step1_count(tilemA, tilenB, _p(TA["tile_ptr"]), _p(TA["tile_columnidx"]),
                            _p(TB["tile_ptr"]), _p(TB["tile_columnidx"]), _p(tile_ptrC))
    ntc = int(ntc)
    rowidx = np.zeros(ntc, np.int32)
    colidx = np.zeros(ntc, np.int32)
    l.orc_step1_fill(tilemA, tilenB, _p(TA["tile_ptr"]), _p(TA["tile_columnidx"]),
                     _p(TB["tile_ptr"]), _p(TB["tile_columnidx"]), _p(tile_ptrC), _p(rowidx), _p(colidx))
    maskC = np.zeros(ntc * TS, np.uint16)
    tile_nnzC = np.zeros(ntc + 1, np.int64)
    ptrRowC = np.zeros(ntc * TS, np.uint8)
    pairs = np.zeros(1, np.int64)
    nnzC = l.orc_step2_symbolic(ntc, _p(rowidx), _p(colidx), _p(TA["tile_ptr"]), _p(TA["tile_columnidx"]),
                                _p(TA["tile_nnz"]), _p(TA["tile_csr_Col"]), _p(TA["tile_csr_Ptr"]),
                                _p(TB["csc_tile_ptr"]), _p(TB["csc_tile_rowidx"]), _p(TB["mask"]),
                                _p(maskC), _p(tile_nnzC), _p(ptrRowC), _p(pairs))
    return dict(tilem=tilemA, tilen=tilenB, numtileC=ntc, nnzC=int(nnzC), tile_ptrC=tile_ptrC,
                tile_rowidxC=rowidx, tile_colidxC=colidx, maskC=maskC, tile_nnzC=tile_nnzC,
                ptrRowC=ptrRowC, pairs=int(pairs[0]))


def numeric(TA: dict, TB: dict, S: dict) -> dict:
    """Step 3 in FP64 (src/spgemm_raw_kernels_v2.cuh:10-139)."""
    l = lib()
    valC = np.zeros(S["nnzC"], np.float64)
    colC = np.zeros(S["nnzC"], np.uint8)
    # converted copies are bound to names so they outlive the C call
    a_val = np.ascontiguousarray(TA["tile_csr_Val"], np.float64)
    b_val = np.ascontiguousarray(TB["tile_csr_Val"], np.float64)
    l.orc_step3_numeric(S["numtileC"], _p(S["tile_rowidxC"]), _p(S["tile_colidxC"]),
                        _p(TA["tile_ptr"]), _p(TA["tile_columnidx"]), _p(TA["tile_nnz"]),
                        _p(a_val), _p(TA["tile_csr_Col"]),
                        _p(TA["tile_csr_Ptr"]), _p(TB["csc_tile_ptr"]), _p(TB["csc_tile_rowidx"]),
                        _p(TB["tile_nnz"]), _p(b_val),
                        _p(TB["tile_csr_Col"]), _p(TB["tile_csr_Ptr"]), _p(S["tile_nnzC"]),
                        _p(S["maskC"]), _p(S["ptrRowC"]), _p(valC), _p(colC))
    return dict(tile_valC=valC, tile_colC=colC)


def spgemm_tiles(a, b) -> dict:
    """Full oracle: tile A and B, steps 1-3.  Returns the C tile arrays."""
    TA = csr2tile(a)
    TB = build_csc_tiles(b, with_tile_csc=False)
    S = symbolic(TA, TB)
    S.update(numeric(TA, TB, S))
    return S


def tiles_to_csr(m: int, n: int, S: dict):
    """Expand C tiles to CSR (src/spgemm_raw_v2.cu:268-284)."""
    l = lib()
    # converted copies are bound to names so they outlive the C calls
    rowidx = np.ascontiguousarray(S["tile_rowidxC"], np.int32)
    colidx = np.ascontiguousarray(S["tile_colidxC"], np.int32)
    nnzc = np.ascontiguousarray(S["tile_nnzC"], np.int64)
    colc = np.ascontiguousarray(S["tile_colC"], np.uint8)
    valc = np.ascontiguousarray(S["tile_valC"], np.float64)
    rp = np.zeros(m + 1, np.int64)
    l.orc_tiles_to_csr(m, n, int(S["numtileC"]), _p(rowidx), _p(colidx), _p(nnzc), _p(colc), _p(valc), _p(rp),
                       None, None)
    cols = np.zeros(int(rp[-1]), np.int32)
    vals = np.zeros(int(rp[-1]), np.float64)
    l.orc_tiles_to_csr(m, n, int(S["numtileC"]), _p(rowidx), _p(colidx), _p(nnzc), _p(colc), _p(valc), _p(rp),
                       _p(cols), _p(vals))
    return rp, cols, vals


def gustavson(a, b, dtype=np.float64):
    """Structural row-wise Gustavson (src/spgemm_raw_v2.cu:289-338)."""
    l = lib()
    arp, aci, brp, bci = _i32(a.row_ptr), _i32(a.col_idx), _i32(b.row_ptr), _i32(b.col_idx)
    rn = np.zeros(a.m, np.int64)
    tot = l.orc_gustavson_rowcounts(a.m, b.n, _p(arp), _p(aci), _p(brp), _p(bci), _p(rn))
    rp = np.zeros(a.m + 1, np.int64)
    np.cumsum(rn, out=rp[1:])
    cols = np.zeros(int(tot), np.int32)
    vals = np.zeros(int(tot), dtype)
    av = np.ascontiguousarray(a.val, dtype)
    bv = np.ascontiguousarray(b.val, dtype)
    f = l.orc_gustavson_fill_f64 if dtype == np.float64 else l.orc_gustavson_fill_f32
    f(a.m, b.n, _p(arp), _p(aci), _p(av), _p(brp), _p(bci), _p(bv), _p(rp), _p(cols), _p(vals))
    return rp, cols, vals


def gustavson_rows(a, b, r0: int, r1: int, dtype=np.float32) -> int:
    """Timed CPU baseline kernel: Gustavson over rows [r0, r1) with every
    available OpenMP thread; returns the nnz formed."""
    l = lib()
    arp, aci, brp, bci = _i32(a.row_ptr), _i32(a.col_idx), _i32(b.row_ptr), _i32(b.col_idx)
    av = np.ascontiguousarray(a.val, dtype)
    bv = np.ascontiguousarray(b.val, dtype)
    rn = np.zeros(max(r1 - r0, 1), np.int64)
    f = l.orc_gustavson_range_f64 if dtype == np.float64 else l.orc_gustavson_range_f32
    return int(f(r0, r1, b.n, _p(arp), _p(aci), _p(av), _p(brp), _p(bci), _p(bv), _p(rn)))


def check_tilerows(a, b, i0: int, i1: int, tiles: dict) -> dict:
    """Compare C tile-rows [i0, i1) of A*B given as tiles (keys ``tile_ptr``:
    i1-i0+1 tile offsets from 0, ``tile_colidxC``, ``tile_nnzC``: absolute
    nonzero prefix of those tiles, ``maskC``, ``ptrRowC``, ``tile_colC``,
    ``tile_valC`` starting at the first tile's first value) with the FP64
    Gustavson of the same rows (src/spgemm_raw_v2.cu:289-338).  Returns the
    relative Frobenius error and the count of structural mismatches."""
    l = lib()
    vt = np.float64 if np.dtype(tiles["tile_valC"].dtype) == np.float64 else np.float32
    arp, aci, brp, bci = _i32(a.row_ptr), _i32(a.col_idx), _i32(b.row_ptr), _i32(b.col_idx)
    av = np.ascontiguousarray(a.val, vt)
    bv = np.ascontiguousarray(b.val, vt)
    ctp = np.ascontiguousarray(tiles["tile_ptr"], np.int64)
    ccol = _i32(tiles["tile_colidxC"])
    cnz = np.ascontiguousarray(tiles["tile_nnzC"], np.int64)
    cmask = np.ascontiguousarray(tiles["maskC"], np.uint16)
    cptr = np.ascontiguousarray(tiles["ptrRowC"], np.uint8)
    ccolb = np.ascontiguousarray(tiles["tile_colC"], np.uint8)
    cval = np.ascontiguousarray(tiles["tile_valC"], vt)
    out = np.zeros(3, np.float64)
    f = l.orc_check_tilerows_f64 if vt == np.float64 else l.orc_check_tilerows_f32
    f(int(i0), int(i1), int(a.m), int(b.n), _p(arp), _p(aci), _p(av), _p(brp), _p(bci), _p(bv), _p(ctp), _p(ccol),
      _p(cnz), _p(cmask), _p(cptr), _p(ccolb), _p(cval), _p(out))
    return {"rel_frob": float(np.sqrt(out[0]) / (np.sqrt(out[1]) or 1.0)), "mismatches": int(out[2]),
            "ref_frob": float(np.sqrt(out[1]))}


def max_threads() -> int:
    return int(lib().orc_max_threads())
