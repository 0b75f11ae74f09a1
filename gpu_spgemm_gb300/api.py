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
_ALGOS = {"auto": L.SPG_ALGO_AUTO, "plain": L.SPG_ALGO_PLAIN, "rowwise": L.SPG_ALGO_ROWWISE,
          "binned": L.SPG_ALGO_BINNED}
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

    def set_mixed_params(self, dense_thr: int = 32, cancel_eps: float = 2.0 ** -20):
        """SPG_PREC_MIXED: tensor-core threshold (nonzeros in both tiles) and
        the cancellation bound that sends a C tile to FP64."""
        self.check(self.lib.spg_set_mixed_params(self.h, int(dense_thr), float(cancel_eps)))

    def set_bin_params(self, pp_thr: float = 12.0, fill_thr: float = 16.0):
        """SPG_ALGO_BINNED / AUTO: a tile-row runs the plain kernels when its
        products per tile pair reach pp_thr and (with a sizing model) its
        predicted C nonzeros per C tile reach fill_thr."""
        self.check(self.lib.spg_set_bin_params(self.h, float(pp_thr), float(fill_thr)))

    def stats(self) -> dict:
        st = L.SpgStats()
        self.check(self.lib.spg_get_stats(self.h, C.byref(st)))
        return {k: getattr(st, k) for k, _ in L.SpgStats._fields_}

    def launches(self) -> int:
        """Kernels launched through this handle so far (a running count)."""
        n = C.c_int64()
        self.check(self.lib.spg_kernel_launches(self.h, C.byref(n)))
        return n.value

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


def symbolic_tiles(handle: Handle, A: TileMatrix, B: TileMatrix, algo: str = "auto") -> CTileMatrix:
    """Step 1 alone (src/spgemm_raw_v2.cu:111-158): C's tile structure."""
    c = L.SpgCTiles()
    handle.check(handle.lib.spg_symbolic_tiles(handle.h, C.byref(A.t), C.byref(B.t), _ALGOS[algo], C.byref(c)))
    return CTileMatrix(handle, c)


def symbolic_masks(handle: Handle, A: TileMatrix, B: TileMatrix, Cm: CTileMatrix) -> CTileMatrix:
    """Step 2 on a C from symbolic_tiles (src/spgemm_raw_v2.cu:160-221)."""
    handle.check(handle.lib.spg_symbolic_masks(handle.h, C.byref(A.t), C.byref(B.t), C.byref(Cm.c)))
    return Cm


def numeric(handle: Handle, A: TileMatrix, B: TileMatrix, Cm: CTileMatrix, algo: str = "auto",
            prec: str = "f32") -> CTileMatrix:
    """Step 3 (src/spgemm_raw_v2.cu:223-243)."""
    handle.check(handle.lib.spg_numeric(handle.h, C.byref(A.t), C.byref(B.t), _ALGOS[algo], _PRECS[prec],
                                        C.byref(Cm.c)))
    return Cm


def numeric_rows(handle: Handle, A: TileMatrix, B: TileMatrix, Cm: CTileMatrix, row_begin: int, row_end: int,
                 algo: str = "auto", prec: str = "f32") -> CTileMatrix:
    """Step 3 on C tile-rows [row_begin, row_end) (src/spgemm_raw_v2.cu:223-243)."""
    handle.check(handle.lib.spg_numeric_rows(handle.h, C.byref(A.t), C.byref(B.t), _ALGOS[algo], _PRECS[prec],
                                             C.byref(Cm.c), int(row_begin), int(row_end)))
    return Cm


def numeric_bands(handle: Handle, A: TileMatrix, B: TileMatrix, Cm: CTileMatrix, band_rows, on_band,
                  algo: str = "auto", prec: str = "f32", last_first: bool = False) -> CTileMatrix:
    """Step 3 (src/spgemm_raw_v2.cu:223-243) reporting bands of C tile-rows:
    on_band(k, row_begin, row_end) runs as soon as band k's values are final
    (band k = tile-rows [band_rows[k], band_rows[k+1])); last_first works on
    the last band first."""
    rows = np.ascontiguousarray(np.asarray(band_rows, dtype=np.int32))
    errs = []

    def cb(_user, k, r0, r1):
        try:
            on_band(k, r0, r1)
        except Exception as e:  # raised again after the call
            errs.append(e)

    fn = L.BAND_FN(cb)
    handle.check(handle.lib.spg_numeric_bands(handle.h, C.byref(A.t), C.byref(B.t), _ALGOS[algo], _PRECS[prec],
                                              C.byref(Cm.c), len(rows) - 1, _ptr(rows),
                                              L.SPG_BANDS_LAST_TO_FIRST if last_first else L.SPG_BANDS_FIRST_TO_LAST,
                                              fn, None))
    if errs:
        raise errs[0]
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


# ---------------------------------------------------------------------------
# conversions and chained products (device memory for outputs comes from torch,
# used only as a device allocator here)
# ---------------------------------------------------------------------------
def _torch_empty(n, dtype):
    import torch
    return torch.empty(max(int(n), 1), dtype=dtype, device="cuda")


def transpose(handle: Handle, T: TileMatrix, layout: str = "b_csc") -> TileMatrix:
    """Tile the transpose of T (from T's device row view): the device form of
    the reference's --aat transpose (src/spgemm_raw_v2.cu:79-90)."""
    import torch
    t = T.t
    vt = torch.float64 if t.dtype == L.SPG_F64 else torch.float32
    rp = _torch_empty(t.n + 1, torch.int32)
    ci = _torch_empty(t.nnz, torch.int32)
    vv = _torch_empty(t.nnz, vt)
    handle.check(handle.lib.spg_csr_transpose(handle.h, t.m, t.n, t.nnz, C.c_void_p(t.row_ptr), C.c_void_p(t.col_idx),
                                              C.c_void_p(t.row_val), t.dtype, C.c_void_p(rp.data_ptr()),
                                              C.c_void_p(ci.data_ptr()), C.c_void_p(vv.data_ptr())))
    lay = L.SPG_LAYOUT_B_CSC if layout == "b_csc" else L.SPG_LAYOUT_ROW
    out = L.SpgTiles()
    handle.check(handle.lib.spg_tile_from_csr(handle.h, t.n, t.m, t.nnz, C.c_void_p(rp.data_ptr()),
                                              C.c_void_p(ci.data_ptr()), C.c_void_p(vv.data_ptr()), t.dtype, lay, 0,
                                              C.byref(out)))
    return TileMatrix(handle, out)


def ctiles_to_csr(handle: Handle, Cm: CTileMatrix):
    """C's tiles -> host CSR arrays (row_ptr int32, col_idx int32, values),
    expanded on the device (src/spgemm_raw_v2.cu:268-284)."""
    import torch
    c = Cm.c
    nnz = C.c_int64()
    handle.check(handle.lib.spg_ctiles_to_csr(handle.h, C.byref(c), None, None, None, C.byref(nnz)))
    vt = torch.float64 if c.dtype == L.SPG_F64 else torch.float32
    rp = _torch_empty(c.m + 1, torch.int32)
    ci = _torch_empty(nnz.value, torch.int32)
    vv = _torch_empty(nnz.value, vt)
    handle.check(handle.lib.spg_ctiles_to_csr(handle.h, C.byref(c), C.c_void_p(rp.data_ptr()),
                                              C.c_void_p(ci.data_ptr()), C.c_void_p(vv.data_ptr()), C.byref(nnz)))
    torch.cuda.synchronize()
    n = nnz.value
    return rp.cpu().numpy()[:c.m + 1], ci.cpu().numpy()[:n], vv.cpu().numpy()[:n]


def galerkin(handle: Handle, a, p, algo: str = "auto", prec: str = "f32"):
    """RAP = P^T (A P) for host CSR A (m x m) and P (m x nc); returns
    (CTileMatrix, intermediate products of both SpGEMMs)."""
    import torch
    dev = lambda x: torch.from_numpy(np.ascontiguousarray(x)).cuda()
    ar, ac, av = dev(a.row_ptr.astype(np.int32)), dev(a.col_idx.astype(np.int32)), dev(a.val)
    pr_, pc, pv = dev(p.row_ptr.astype(np.int32)), dev(p.col_idx.astype(np.int32)), dev(p.val)
    return galerkin_device(handle, a.m, p.n, a.nnz, ar.data_ptr(), ac.data_ptr(), av.data_ptr(), p.nnz,
                           pr_.data_ptr(), pc.data_ptr(), pv.data_ptr(), a.val.dtype, algo, prec, keep=(ar, ac, av, pr_, pc, pv))


def galerkin_device(handle: Handle, m, nc, nnza, a_rp, a_ci, a_val, nnzp, p_rp, p_ci, p_val, dtype,
                    algo="auto", prec="f32", keep=None):
    c = L.SpgCTiles()
    prod = C.c_int64()
    handle.check(handle.lib.spg_galerkin(handle.h, m, nc, nnza, C.c_void_p(a_rp), C.c_void_p(a_ci), C.c_void_p(a_val),
                                         nnzp, C.c_void_p(p_rp), C.c_void_p(p_ci), C.c_void_p(p_val),
                                         _dtype_code(dtype), _ALGOS[algo], _PRECS[prec], C.byref(c), C.byref(prod)))
    return CTileMatrix(handle, c), prod.value


class Batch:
    """Many independent products C_p = A_p * B_p, one launch per phase per bin
    (block-diagonal assembly on the device).  ``pairs`` is a list of (A, B)
    host CSRs with A.n == B.m."""

    def __init__(self, handle: Handle, pairs):
        self.handle = handle
        self.pairs = pairs
        n = len(pairs)
        dt = np.dtype(pairs[0][0].val.dtype)
        self.dtype = dt
        self._keep = []

        def arr(xs, ct):
            a = (ct * n)(*xs)
            self._keep.append(a)
            return a

        def hold(x, dtype):
            x = np.ascontiguousarray(x, dtype)
            self._keep.append(x)
            return x.ctypes.data

        m = arr([a.m for a, b in pairs], C.c_int)
        k = arr([a.n for a, b in pairs], C.c_int)
        nn = arr([b.n for a, b in pairs], C.c_int)
        na = arr([a.nnz for a, b in pairs], C.c_int64)
        nb = arr([b.nnz for a, b in pairs], C.c_int64)
        arp = arr([hold(a.row_ptr, np.int32) for a, b in pairs], C.c_void_p)
        aci = arr([hold(a.col_idx, np.int32) for a, b in pairs], C.c_void_p)
        av = arr([hold(a.val, dt) for a, b in pairs], C.c_void_p)
        brp = arr([hold(b.row_ptr, np.int32) for a, b in pairs], C.c_void_p)
        bci = arr([hold(b.col_idx, np.int32) for a, b in pairs], C.c_void_p)
        bv = arr([hold(b.val, dt) for a, b in pairs], C.c_void_p)
        self.b = C.c_void_p()
        handle.check(handle.lib.spg_batch_create_host(handle.h, n, m, k, nn, na, arp, aci, av, nb, brp, bci, bv,
                                                      _dtype_code(dt), C.byref(self.b)))

    def spgemm(self, algo: str = "auto", prec: str = "f32"):
        self.handle.check(self.handle.lib.spg_batch_spgemm(self.handle.h, self.b, _ALGOS[algo], _PRECS[prec]))

    def numeric(self, prec: str = "f32"):
        self.handle.check(self.handle.lib.spg_batch_numeric(self.handle.h, self.b, _PRECS[prec]))

    def products(self) -> int:
        p = C.c_int64()
        self.handle.check(self.handle.lib.spg_batch_info(self.handle.h, self.b, -1, None, None, C.byref(p)))
        return p.value

    def tune(self, prec: str = "f32"):
        nt = C.c_int()
        thr = (C.c_int * 4)()
        alg = (C.c_int * 4)()
        self.handle.check(self.handle.lib.spg_batch_tune(self.handle.h, self.b, _PRECS[prec], C.byref(nt), thr, alg))
        return list(thr[:nt.value]), list(alg[:nt.value + 1])

    def set_bins(self, thresholds, algos=None):
        t = (C.c_int * max(1, len(thresholds)))(*thresholds)
        a = (C.c_int * (len(thresholds) + 1))(*[_ALGOS[x] if isinstance(x, str) else x for x in algos]) \
            if algos else None
        self.handle.check(self.handle.lib.spg_batch_set_bins(self.handle.h, self.b, len(thresholds), t, a))

    def set_values(self, a_vals=None, b_vals=None):
        n = len(self.pairs)
        keep = []

        def arr(vs):
            if vs is None:
                return None
            xs = [np.ascontiguousarray(v, self.dtype) for v in vs]
            keep.extend(xs)
            return (C.c_void_p * n)(*[x.ctypes.data for x in xs])
        self.handle.check(self.handle.lib.spg_batch_set_values_host(self.handle.h, self.b, arr(a_vals), arr(b_vals)))

    def result(self, p: int, values: bool = True) -> dict:
        nt, nz = C.c_int64(), C.c_int64()
        self.handle.check(self.handle.lib.spg_batch_info(self.handle.h, self.b, p, C.byref(nt), C.byref(nz), None))
        a, b = self.pairs[p]
        tilem = (a.m + TS - 1) // TS
        out = dict(numtileC=nt.value, nnzC=nz.value, tile_ptrC=np.zeros(tilem + 1, np.int32),
                   tile_rowidxC=np.zeros(nt.value, np.int32), tile_colidxC=np.zeros(nt.value, np.int32),
                   maskC=np.zeros(nt.value * TS, np.uint16), tile_nnzC=np.zeros(nt.value + 1, np.int64),
                   ptrRowC=np.zeros(nt.value * TS, np.uint8))
        if values:
            out.update(tile_valC=np.zeros(nz.value, self.dtype), tile_colC=np.zeros(nz.value, np.uint8))
        g = out.get
        self.handle.check(self.handle.lib.spg_batch_to_host(
            self.handle.h, self.b, p, _ptr(out["tile_ptrC"]), _ptr(out["tile_rowidxC"]), _ptr(out["tile_colidxC"]),
            _ptr(out["maskC"]), _ptr(out["tile_nnzC"]), _ptr(out["ptrRowC"]), _ptr(g("tile_valC")),
            _ptr(g("tile_colC"))))
        return out

    def bins(self):
        nb = C.c_int()
        self.handle.check(self.handle.lib.spg_batch_bin_count(self.handle.h, self.b, C.byref(nb), None))
        nz = (C.c_int64 * nb.value)()
        self.handle.check(self.handle.lib.spg_batch_bin_count(self.handle.h, self.b, C.byref(nb), nz))
        return list(nz)

    def graph_capture(self, a_vals, b_vals, host_outs, prec: str = "f32"):
        """host_outs: one pinned numpy buffer per bin (C values, block order)."""
        n = len(self.pairs)
        self._gkeep = [np.ascontiguousarray(v, self.dtype) for v in a_vals] + \
                      [np.ascontiguousarray(v, self.dtype) for v in b_vals]
        av = (C.c_void_p * n)(*[x.ctypes.data for x in self._gkeep[:n]])
        bv = (C.c_void_p * n)(*[x.ctypes.data for x in self._gkeep[n:]])
        ho = (C.c_void_p * len(host_outs))(*[x.ctypes.data if x is not None else None for x in host_outs])
        self._gkeep += [av, bv, ho]
        self.handle.check(self.handle.lib.spg_batch_graph_capture(self.handle.h, self.b, av, bv, ho, _PRECS[prec]))

    def graph_launch(self):
        self.handle.check(self.handle.lib.spg_batch_graph_launch(self.handle.h, self.b))

    def free(self):
        if self.b:
            self.handle.lib.spg_batch_free(self.handle.h, self.b)
            self.b = C.c_void_p()

    def __del__(self):
        try:
            if self.handle.h:
                self.free()
        except Exception:
            pass


import os as _os

SIZING_MODEL_PATH = _os.path.join(_os.path.dirname(_os.path.abspath(__file__)), "sizing_mlp.npz")


class SizingModel:
    """Learned sizing of C (8 -> 32 -> 32 -> 2 MLP on per-tile-row features),
    trained and evaluated by the library's own CUDA kernels."""

    NF, NO, NNORM = 8, 2, 20

    def __init__(self, handle: Handle, params=None, norm=None):
        self.handle = handle
        self.nparam = handle.lib.spg_mlp_num_params()
        self.m = C.c_void_p()
        p = None if params is None else np.ascontiguousarray(params, np.float32)
        n = None if norm is None else np.ascontiguousarray(norm, np.float32)
        handle.check(handle.lib.spg_mlp_create(handle.h, _ptr(p), _ptr(n), C.byref(self.m)))

    @classmethod
    def load(cls, handle: Handle, path: str = SIZING_MODEL_PATH):
        z = np.load(path)
        return cls(handle, z["params"], z["norm"])

    def params(self):
        p = np.zeros(self.nparam, np.float32)
        n = np.zeros(self.NNORM, np.float32)
        self.handle.check(self.handle.lib.spg_mlp_get_params(self.handle.h, self.m, _ptr(p), _ptr(n)))
        return p, n

    def set_norm(self, norm):
        n = np.ascontiguousarray(norm, np.float32)
        self.handle.check(self.handle.lib.spg_mlp_set_norm(self.handle.h, self.m, _ptr(n)))

    def features(self, A: TileMatrix, B: TileMatrix):
        import torch
        f = torch.zeros((max(A.tilem, 1), self.NF), dtype=torch.float32, device="cuda")
        self.handle.check(self.handle.lib.spg_mlp_features(self.handle.h, C.byref(A.t), C.byref(B.t),
                                                           C.c_void_p(f.data_ptr())))
        return f[:A.tilem]

    def predict(self, feat):
        import torch
        out = torch.zeros((max(feat.shape[0], 1), self.NO), dtype=torch.float32, device="cuda")
        self.handle.check(self.handle.lib.spg_mlp_forward(self.handle.h, self.m, C.c_void_p(feat.data_ptr()),
                                                          feat.shape[0], C.c_void_p(out.data_ptr())))
        return out[:feat.shape[0]]

    def gradient(self, feat, target):
        import torch
        g = torch.zeros(self.nparam, dtype=torch.float32, device="cuda")
        loss = C.c_float()
        self.handle.check(self.handle.lib.spg_mlp_gradient(self.handle.h, self.m, C.c_void_p(feat.data_ptr()),
                                                           C.c_void_p(target.data_ptr()), feat.shape[0],
                                                           C.c_void_p(g.data_ptr()), C.byref(loss)))
        return g.cpu().numpy(), loss.value

    def train(self, feat, target, epochs=20, batch=8192, lr=3e-3, seed=0):
        import torch
        n = feat.shape[0]
        gen = torch.Generator(device="cpu").manual_seed(seed)
        perm = torch.cat([torch.randperm(n, generator=gen) for _ in range(epochs)]).to(torch.int32).cuda()
        loss = C.c_float()
        self.handle.check(self.handle.lib.spg_mlp_train(self.handle.h, self.m, C.c_void_p(feat.data_ptr()),
                                                        C.c_void_p(target.data_ptr()), n,
                                                        C.c_void_p(perm.data_ptr()), epochs, batch, lr,
                                                        C.byref(loss)))
        return loss.value

    def attach(self, margin: float = 1.0):
        self.handle.check(self.handle.lib.spg_set_sizing_model(self.handle.h, self.m, margin))

    def detach(self):
        self.handle.check(self.handle.lib.spg_set_sizing_model(self.handle.h, None, 0.0))

    def save(self, path: str, **meta):
        p, n = self.params()
        np.savez(path, params=p, norm=n, **meta)

    def free(self):
        if self.m:
            self.handle.lib.spg_mlp_free(self.handle.h, self.m)
            self.m = C.c_void_p()


def sizing_targets(Cm: CTileMatrix):
    """Per C tile-row: log1p(C tiles), log1p(C nonzeros) as a (tilem, 2) float32
    device tensor (from the exact symbolic phase)."""
    import torch
    h = Cm.to_host(values=False)
    tp = h["tile_ptrC"].astype(np.int64)
    ntc = np.diff(tp)
    nz = h["tile_nnzC"][tp[1:]] - h["tile_nnzC"][tp[:-1]]
    t = np.stack([np.log1p(ntc), np.log1p(nz)], axis=1).astype(np.float32)
    return torch.from_numpy(t).cuda()
