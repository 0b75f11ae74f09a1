"""spg_ctiles_to_csr_noalloc: exporting C's tiles to a CSR held in the caller's
own device buffers while the library allocates no device memory.  It exists
for callers that cannot let a library allocate -- a process or framework that
owns all of HBM through its own pool, code where an allocation could block or
fail mid-run, a plugin given only a stream and buffers -- and works out of a
fixed area inside the library, so C may have at most 2^20 rows.

The result must equal the allocating export (spg_ctiles_to_csr) exactly, on
two calls in a row (a larger C, then a smaller one, so the shared working
area's leftover contents from the first call would show up in the second).
This file is collected last on purpose."""
import ctypes as C

import numpy as np
import pytest
import torch

from gpu_spgemm_gb300 import _lib as L
from gpu_spgemm_gb300 import api, synth

pytestmark = pytest.mark.gpu

MAX_ROWS = 1 << 20


@pytest.fixture(scope="module")
def h():
    with api.Handle(0) as handle:
        yield handle


def _export_noalloc(h, Cm):
    c = Cm.c
    vt = torch.float64 if c.dtype == L.SPG_F64 else torch.float32
    rp = torch.full((c.m + 1,), -1, dtype=torch.int32, device="cuda")
    ci = torch.full((max(c.nnzC, 1),), -1, dtype=torch.int32, device="cuda")
    val = torch.full((max(c.nnzC, 1),), -7.0, dtype=vt, device="cuda")
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    nnz = C.c_int64()
    h.check(h.lib.spg_ctiles_to_csr_noalloc(h.h, C.byref(c), C.c_void_p(rp.data_ptr()), C.c_void_p(ci.data_ptr()),
                                            C.c_void_p(val.data_ptr()), C.byref(nnz)))
    torch.cuda.synchronize()
    free1 = torch.cuda.mem_get_info()[0]
    n = nnz.value
    return rp.cpu().numpy(), ci[:n].cpu().numpy(), val[:n].cpu().numpy(), free0 - free1


def test_noalloc_export_matches_allocating_export_twice(h):
    grabbed = []
    for a in (synth.rmat(13, 16), synth.poisson2d(40, np.float32)):
        A = api.csr2tile(h, a)
        B = api.build_csc_tiles(h, a)
        Cm = api.spgemm(h, A, B)
        rp0, ci0, v0 = api.ctiles_to_csr(h, Cm)
        rp1, ci1, v1, grabbed_bytes = _export_noalloc(h, Cm)
        np.testing.assert_array_equal(rp1, rp0)
        np.testing.assert_array_equal(ci1, ci0)
        np.testing.assert_array_equal(v1, v0)   # same values, copied: tolerance 0
        grabbed.append(grabbed_bytes)
    # after the first call (which may load the library's device code) no call
    # takes device memory
    assert grabbed[1] == 0


def test_noalloc_export_fp64_twice(h):
    """FP64 values take the double fill; again a larger C, then a smaller one."""
    for a in (synth.poisson2d(64), synth.rmat(11, 16, dtype=np.float64)):
        A = api.csr2tile(h, a)
        B = api.build_csc_tiles(h, a)
        Cm = api.spgemm(h, A, B)
        rp0, ci0, v0 = api.ctiles_to_csr(h, Cm)
        rp1, ci1, v1, _ = _export_noalloc(h, Cm)
        assert v1.dtype == np.float64
        np.testing.assert_array_equal(rp1, rp0)
        np.testing.assert_array_equal(ci1, ci0)
        np.testing.assert_array_equal(v1, v0)


@pytest.mark.parametrize("m,n", [(0, 16), (40, 24)], ids=["no-rows", "rows-without-nonzeros"])
def test_noalloc_export_of_an_empty_c(h, m, n):
    """A C with no rows, and a C whose rows hold nothing: the row pointer is
    all zeros (m+1 entries), nothing else is written, nnz is 0."""
    a = synth.CSR(m, n, np.zeros(m + 1, np.int32), np.zeros(0, np.int32), np.zeros(0, np.float32))
    rng = np.random.Generator(np.random.PCG64(3))
    b = synth.erdos_renyi(n, 4.0, rng)  # B has entries; A reaches none of them
    A = api.csr2tile(h, a)
    B = api.build_csc_tiles(h, b)
    Cm = api.spgemm(h, A, B)
    assert Cm.nnzC == 0
    rp0, _, _ = api.ctiles_to_csr(h, Cm)
    rp1, ci1, v1, _ = _export_noalloc(h, Cm)
    np.testing.assert_array_equal(rp1, np.zeros(m + 1, np.int32))
    np.testing.assert_array_equal(rp1, rp0)
    assert ci1.size == 0 and v1.size == 0


def test_noalloc_rejects_more_rows_than_its_area(h):
    m = MAX_ROWS + 16
    a = synth.CSR(m, 16, np.zeros(m + 1, np.int32), np.zeros(0, np.int32), np.zeros(0, np.float32))
    b = synth.CSR(16, 16, np.zeros(17, np.int32), np.zeros(0, np.int32), np.zeros(0, np.float32))
    A = api.csr2tile(h, a)
    B = api.build_csc_tiles(h, b)
    Cm = api.spgemm(h, A, B)
    rp = torch.zeros(m + 1, dtype=torch.int32, device="cuda")
    nnz = C.c_int64()
    st = h.lib.spg_ctiles_to_csr_noalloc(h.h, C.byref(Cm.c), C.c_void_p(rp.data_ptr()), None, None, C.byref(nnz))
    assert st == L.SPG_ERR_INVALID
    assert b"1,048,576" in h.lib.spg_last_error(h.h)
