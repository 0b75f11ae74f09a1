"""Writes cstruct_<case>.npz: C = A*B computed by the reference project's OWN
GPU kernels (step1_count/fill, step2_symbolic, step2_build_ptrRowC,
step3_numeric_kernel_v2 from src/spgemm_raw_kernels.cuh and
src/spgemm_raw_kernels_v2.cuh), compiled from the reference source into
oracle/_ref/ref_kernels.cubin by oracle/build_ref.sh and driven here through the
CUDA driver API in the order of src/spgemm_raw_v2.cu:111-243.

Inputs are tiled by the CPU oracle, whose tiling is pinned bit-exactly to the
reference's own tile_format.h by tiles_*.npz.  The matched-pair cache is sized
from the oracle's pair count (the reference sizes it 8*numtileC and only checks
for overflow after writing past it), and every case keeps B's tile-column count
small enough for step 1's default 48 KB of dynamic shared memory, so every
launch stays inside its buffers.

Run on a GPU host from the repository root (writes to the given directory):
    python tests/golden/make_cstruct_golden.py OUT_DIR
With --time instead it times those kernels on the benchmark configurations
they can run (see time_reference).
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

import oracle  # noqa: E402
import cases  # noqa: E402

CUBIN = os.path.join(ROOT, "oracle", "_ref", "ref_kernels.cubin")
NAMES = {
    "step1_count": "_Z18step1_count_kernelPKiS0_iS0_S0_iPi",
    "step1_fill": "_Z17step1_fill_kernelPKiS0_iS0_S0_iS0_PiS1_",
    "step2_symbolic": "_Z21step2_symbolic_kernelPKiS0_S0_PKhS2_PKtS0_S0_S0_S0_iPiPtS5_S5_S5_S5_S5_",
    "step2_ptrRowC": "_Z26step2_build_ptrRowC_kernelPKtPhi",
    "step3_numeric_v2": "_Z23step3_numeric_kernel_v2PKiS0_S0_PKdPKhS4_S0_S0_S0_S2_S4_S4_S0_S0_S0_PKtS4_PdPhS0_S0_S0_S0_i",
}


class Driver:
    def __init__(self):
        import torch
        self.torch = torch
        torch.cuda.init()
        torch.zeros(1, device="cuda")  # make the primary context current
        self.cu = C.CDLL("libcuda.so.1")
        self.mod = C.c_void_p()
        self._ck(self.cu.cuModuleLoad(C.byref(self.mod), CUBIN.encode()), "cuModuleLoad")
        self.fn = {}
        for k, name in NAMES.items():
            f = C.c_void_p()
            self._ck(self.cu.cuModuleGetFunction(C.byref(f), self.mod, name.encode()), name)
            self.fn[k] = f

    @staticmethod
    def _ck(r, what):
        if r != 0:
            raise RuntimeError(f"{what} failed with CUresult {r}")

    timings = None  # name -> list of ms, when timing

    def launch(self, name, grid, block, smem, args):
        holders = []
        for a in args:
            if isinstance(a, int):
                holders.append(C.c_int(a))
            else:  # torch tensor or None
                holders.append(C.c_void_p(a.data_ptr() if a is not None else 0))
        arr = (C.c_void_p * len(holders))(*[C.cast(C.pointer(h), C.c_void_p) for h in holders])
        ev = None
        if self.timings is not None:
            ev = [self.torch.cuda.Event(enable_timing=True) for _ in range(2)]
            self.torch.cuda.synchronize()
            ev[0].record()
        self._ck(self.cu.cuLaunchKernel(self.fn[name], grid, 1, 1, block, 1, 1, smem, None, arr, None), name)
        if ev is not None:
            ev[1].record()
        self._ck(self.cu.cuCtxSynchronize(), name + " sync")
        if ev is not None:
            self.timings.setdefault(name, []).append(ev[0].elapsed_time(ev[1]))

    def dev(self, x):
        x = np.ascontiguousarray(x)
        if x.dtype == np.uint16:
            x = x.view(np.int16)
        t = self.torch.from_numpy(x.copy() if x.size else np.zeros(1, x.dtype)).cuda()
        return t

    def zeros(self, n, dtype):
        return self.torch.zeros(max(int(n), 1), dtype=dtype, device="cuda")


def run_case(d: Driver, a, b):
    torch = d.torch
    TA = oracle.csr2tile(a)
    TB = oracle.build_csc_tiles(b, with_tile_csc=False)
    S = oracle.spgemm_tiles(a, b)
    tilemA, tilenB = TA["tilem"], TB["tilen"]
    nmasks = (tilenB + 31) // 32
    assert 4 * nmasks * 4 <= 48 * 1024
    A = {k: d.dev(TA[k]) for k in ("tile_ptr", "tile_columnidx", "tile_nnz", "tile_csr_Val", "tile_csr_Col",
                                   "tile_csr_Ptr")}
    B = {k: d.dev(TB[k]) for k in ("tile_ptr", "tile_columnidx", "tile_nnz", "tile_csr_Val", "tile_csr_Col",
                                   "tile_csr_Ptr", "mask", "csc_tile_ptr", "csc_tile_rowidx")}
    out = {}
    # ---- step 1 (src/spgemm_raw_v2.cu:111-158)
    tp = d.zeros(tilemA + 1, torch.int32)
    blocks = (tilemA + 3) // 4
    smem = 4 * nmasks * 4
    if tilemA > 0:
        d.launch("step1_count", blocks, 128, smem, [A["tile_ptr"], A["tile_columnidx"], tilemA, B["tile_ptr"],
                                                   B["tile_columnidx"], tilenB, tp])
    cnt = tp[:tilemA].to(torch.int64)
    pre = torch.zeros(tilemA + 1, dtype=torch.int64, device="cuda")
    pre[1:] = torch.cumsum(cnt, 0)
    tp = pre.to(torch.int32).contiguous()
    numtileC = int(pre[-1].item())
    rowidx = d.zeros(numtileC, torch.int32)
    colidx = d.zeros(numtileC, torch.int32)
    if tilemA > 0:
        d.launch("step1_fill", blocks, 128, smem, [A["tile_ptr"], A["tile_columnidx"], tilemA, B["tile_ptr"],
                                                  B["tile_columnidx"], tilenB, tp, rowidx, colidx])
    out["tile_ptrC"] = tp.cpu().numpy()
    out["tile_rowidxC"] = rowidx.cpu().numpy()[:numtileC]
    out["tile_colidxC"] = colidx.cpu().numpy()[:numtileC]
    # ---- step 2 (:160-221)
    nnzc_cnt = d.zeros(numtileC + 1, torch.int32)
    maskC = d.zeros(numtileC * 16, torch.int16)
    spec_cnt = d.zeros(numtileC, torch.int32)
    spec_off = d.zeros(numtileC, torch.int32)
    alloc = d.zeros(1, torch.int32)
    cap = S["pairs"] + 16
    posa = d.zeros(cap, torch.int32)
    posb = d.zeros(cap, torch.int32)
    if numtileC > 0:
        hw = (numtileC + 7) // 8
        d.launch("step2_symbolic", (hw + 7) // 8, 128, 0,
                 [A["tile_ptr"], A["tile_columnidx"], A["tile_nnz"], A["tile_csr_Col"], A["tile_csr_Ptr"], B["mask"],
                  B["csc_tile_ptr"], B["csc_tile_rowidx"], rowidx, colidx, numtileC, nnzc_cnt, maskC, spec_cnt,
                  spec_off, posa, posb, alloc])
    assert int(alloc.item()) <= cap
    nz = torch.zeros(numtileC + 1, dtype=torch.int64, device="cuda")
    nz[1:] = torch.cumsum(nnzc_cnt[:numtileC].to(torch.int64), 0)
    nnzC = int(nz[-1].item())
    nz32 = nz.to(torch.int32).contiguous()
    ptrRowC = d.zeros(numtileC * 16, torch.uint8)
    if numtileC > 0:
        d.launch("step2_ptrRowC", (numtileC + 255) // 256, 256, 0, [maskC, ptrRowC, numtileC])
    out["maskC"] = maskC.cpu().numpy()[:numtileC * 16].view(np.uint16)
    out["tile_nnzC"] = nz.cpu().numpy()
    out["ptrRowC"] = ptrRowC.cpu().numpy()[:numtileC * 16]
    # ---- step 3 (:223-243)
    valC = d.zeros(nnzC, torch.float64)
    colC = d.zeros(nnzC, torch.uint8)
    if numtileC > 0:
        d.launch("step3_numeric_v2", (numtileC + 7) // 8, 256, 0,
                 [A["tile_ptr"], A["tile_columnidx"], A["tile_nnz"], A["tile_csr_Val"], A["tile_csr_Col"],
                  A["tile_csr_Ptr"], B["csc_tile_ptr"], B["csc_tile_rowidx"], B["tile_nnz"], B["tile_csr_Val"],
                  B["tile_csr_Col"], B["tile_csr_Ptr"], rowidx, colidx, nz32, maskC, ptrRowC, valC, colC,
                  spec_cnt, spec_off, posa, posb, numtileC])
    out["tile_valC"] = valC.cpu().numpy()[:nnzC]
    out["tile_colC"] = colC.cpu().numpy()[:nnzC]
    out["numtileC"] = np.int64(numtileC)
    out["nnzC"] = np.int64(nnzC)
    return out


def time_reference(reps: int = 5):
    """Kernel times of the reference's own steps 1-3 on the two benchmark
    configurations they can run (FP64, their only value type): the 2-D
    5-point Poisson 256^2 and the 27-point stencil 64^3 x 3 dof.  Each kernel
    is bracketed by CUDA events on the default stream (host scans, copies and
    allocations between them are not counted, so the sum is a lower bound on
    the reference's step time).  Prints one JSON line per configuration."""
    import json
    from gpu_spgemm_gb300 import synth
    d = Driver()
    for name, a in (("poisson2d_256_f64", synth.poisson2d(256)),
                    ("stencil27_64_dof3_f64", synth.stencil27_dof3(64, dtype=np.float64))):
        d.timings = None
        run_case(d, a, a)  # warm-up, and the oracle's pair count sizes the cache
        d.timings = {}
        for _ in range(reps):
            run_case(d, a, a)
        per = {k: float(np.median(v)) for k, v in d.timings.items()}
        steps = {"step1": per.get("step1_count", 0) + per.get("step1_fill", 0),
                 "step2": per.get("step2_symbolic", 0) + per.get("step2_ptrRowC", 0),
                 "step3": per.get("step3_numeric_v2", 0)}
        ms = sum(steps.values())
        prods = synth.products(a, a)
        print(json.dumps({"reference_kernels": name, "products": prods, "kernel_ms": per, "step_ms": steps,
                          "ms_steps_1_3": ms, "gflops": 2.0 * prods / (ms * 1e-3) / 1e9, "reps": reps}), flush=True)


def main():
    if len(sys.argv) > 1 and sys.argv[1] == "--time":
        time_reference()
        return
    out_dir = sys.argv[1] if len(sys.argv) > 1 else os.path.dirname(os.path.abspath(__file__))
    os.makedirs(out_dir, exist_ok=True)
    d = Driver()
    for name, a, b in cases.product_cases() + cases.reference_kernel_extra_cases():
        o = run_case(d, a, b)
        o.update({"in_a_m": np.int64(a.m), "in_a_n": np.int64(a.n), "in_a_row_ptr": a.row_ptr,
                  "in_a_col_idx": a.col_idx, "in_a_val": a.val.astype(np.float64), "in_b_m": np.int64(b.m),
                  "in_b_n": np.int64(b.n), "in_b_row_ptr": b.row_ptr, "in_b_col_idx": b.col_idx,
                  "in_b_val": b.val.astype(np.float64)})
        safe = name.replace("^", "_sq").replace("*", "_x_")
        np.savez_compressed(os.path.join(out_dir, f"cstruct_{safe}.npz"), **o)
        print(name, int(o["numtileC"]), int(o["nnzC"]), flush=True)


if __name__ == "__main__":
    main()
