"""Benchmark: tiled SpGEMM GFLOP/s and HBM-roofline fraction on one GB300.

Default workload: C = A*A, A = R-MAT scale 20 (n = 2^20, 16 edges per vertex
before merging, (a,b,c,d) = (.57,.19,.19,.05), duplicates merged), FP32 values
U[-1,1] -- the configuration the metric is quoted on.  A "step" is one full
SpGEMM (C tile structure + bitmask symbolic + numeric, with every allocation
of C) on tiles already resident in HBM; GFLOP/s = 2 * products / step time,
products = sum over A's nonzeros of nnz(B row) (src/spgemm_raw_v2.cu:95-99,250).
Other workloads (--workload): poisson2d, stencil27, galerkin128 (the Galerkin
triple product P^T (A P) on a 128^3 Poisson problem, one step = one
spg_galerkin call), rmatNN, erbatch.

Printed JSON (rank 0, one line) carries:
  value      GFLOP/s of the device-resident steps (max over ranks of the time)
  e2e        the same metric through the public C ABI with host buffers: each
             step copies the CSR inputs host->device, tiles them, multiplies and
             copies C's result arrays back to pinned host memory
  roofline   the dominant kernel's algorithmic bytes / its CUDA-event time
  accuracy   C checked against the FP64 oracle: exact structure and relative
             Frobenius error on sampled tile-rows (the hub rows first)
  vs_plain   the same product by the plain per-C-tile kernels (the reference's
             method, exact two-pass step 1, no sizing model) and by the default
             path without the sizing model, timed in the same run
  cpu_baseline  OpenMP Gustavson (the CPU oracle's port of the reference's
             check, src/spgemm_raw_v2.cu:289-338) on a seeded row sample

`config` holds only what identifies the workload, so both arms print the same
one.  `--impl reference` times the reference's CPU implementation of the path
(that Gustavson port) on all host threads for the same workload and metric.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from gpu_spgemm_gb300 import synth  # noqa: E402

L2_BYTES = 129 * 1024 * 1024
TS = 16

# DRAM traffic of the numeric kernel per algorithmic byte, from an ncu capture
# (dram__bytes_read.sum + dram__bytes_write.sum of rw_numeric_kernel) on the
# R-MAT 2^17 product, where the capture holds a few GB: 2.881 + 2.418 GB
# against 5.309 GB of algorithmic bytes.  A full-size launch's traffic is
# reported as this ratio times its algorithmic bytes: a lower bound once B's
# entries outgrow L2 (R-MAT 2^20: 134 MB).
TRAFFIC_PER_ALGO_BYTE = {"rw_numeric_kernel": (2.880523e9 + 2.418124e9) / 5.308991570e9}

# A tiles from which the bench attaches the learned sizing model (step 1's
# slotted pass); the library's AUTO bins tile-rows from the same size on.
SIZING_MIN_TILES = 65536


# ---------------------------------------------------------------------------
# workloads
# ---------------------------------------------------------------------------
def workload(name: str) -> dict:
    """kind "product": C = A*B; kind "galerkin": RAP = P^T (A P)."""
    if name == "rmat20":
        a = synth.rmat(20, 16)
        return dict(kind="product", a=a, b=a, desc="C=A*A, A=R-MAT scale 20, edge factor 16, "
                                                   "(a,b,c,d)=(.57,.19,.19,.05), duplicates merged, FP32 U[-1,1]")
    if name == "poisson2d":
        a = synth.poisson2d(256)
        return dict(kind="product", a=a, b=a, desc="C=A*A, A=2-D 5-point Poisson 256x256, FP64")
    if name == "stencil27":
        a = synth.stencil27_dof3(64)
        return dict(kind="product", a=a, b=a, desc="C=A*A, A=27-point stencil 64^3 x 3 dof, FP32 N(0,1)")
    if name == "stencil27f64":  # the reference's value type, for the comparison with its own kernels
        a = synth.stencil27_dof3(64, dtype=np.float64)
        return dict(kind="product", a=a, b=a, desc="C=A*A, A=27-point stencil 64^3 x 3 dof, FP64 N(0,1)")
    if name.startswith("stencil27_"):  # smaller grids of the same stencil (profiling cases)
        g = int(name[10:])
        a = synth.stencil27_dof3(g)
        return dict(kind="product", a=a, b=a, desc=f"C=A*A, A=27-point stencil {g}^3 x 3 dof, FP32 N(0,1)")
    if name == "mixed":
        a = synth.block_diag(synth.stencil27_dof3(40), synth.rmat(18, 16))
        return dict(kind="product", a=a, b=a, desc="C=A*A, A=block diagonal of a 27-point stencil 40^3 x 3 dof "
                                                   "(FP32 N(0,1)) and R-MAT scale 18, edge factor 16")
    if name.startswith("galerkin"):
        g = int(name[8:] or 128)
        a = synth.poisson3d(g)
        p = synth.smoothed_aggregation(a, synth.aggregation_p0(g))
        return dict(kind="galerkin", a=a, p=p,
                    desc=f"RAP=P^T(A P), A=3-D 7-point Poisson {g}^3, P=2x2x2 aggregation smoothed by one "
                         "weighted-Jacobi step (omega=2/3), FP32")
    if name.startswith("rmat"):
        s = int(name[4:])
        a = synth.rmat(s, 16)
        return dict(kind="product", a=a, b=a, desc=f"C=A*A, A=R-MAT scale {s}, edge factor 16, FP32")
    raise SystemExit(f"unknown workload {name}")


def galerkin_operands(w: dict):
    """P^T and A*P as host CSR (structure and FP32 values from scipy), for the
    product count and the CPU legs."""
    if "pt" not in w:
        a, p = w["a"], w["p"]
        ap = (a.to_scipy().astype(np.float64) @ p.to_scipy().astype(np.float64)).tocsr()
        w["pt"] = synth.transpose(p)
        w["ap"] = synth.CSR.from_scipy(ap, dtype=np.float32)
    return w["pt"], w["ap"]


def structural_products(w: dict) -> int:
    if w["kind"] == "product":
        return synth.products(w["a"], w["b"])
    pt, ap = galerkin_operands(w)
    # A*P keeps every structural product (cancellations included), as the tiled
    # product does; scipy's A@P drops exact zeros, so count on |A| |P|
    a, p = w["a"], w["p"]
    return synth.products(a, p) + synth.products(pt, structural_ap(w))


def structural_ap(w: dict):
    if "ap_struct" not in w:
        a, p = w["a"], w["p"]
        sa = a.to_scipy().astype(np.float64)
        sp_ = p.to_scipy().astype(np.float64)
        sa.data[:] = 1.0
        sp_.data[:] = 1.0
        w["ap_struct"] = synth.CSR.from_scipy((sa @ sp_).tocsr(), dtype=np.float32)
    return w["ap_struct"]


def workload_config(w: dict, products: int) -> dict:
    """The workload's identity, the same in both arms' lines."""
    if w["kind"] == "product":
        a, b = w["a"], w["b"]
        vbytes = a.val.dtype.itemsize
        inputs = (a.nnz + b.nnz) * (4 + vbytes) + 4 * (a.m + b.m + 2)
        cfg = {"workload": w["desc"], "n": a.m, "nnz": a.nnz, "products": int(products)}
    else:
        a, p = w["a"], w["p"]
        inputs = (a.nnz + p.nnz) * 8 + 4 * (a.m + p.m + 2)
        cfg = {"workload": w["desc"], "n": a.m, "nnz": a.nnz, "nnzP": p.nnz, "nc": p.n,
               "products": int(products)}
    cfg["l2"] = ("inputs exceed L2 (%.0f MB of CSR > 129 MB), no flush between steps" % (inputs / 1e6)
                 if inputs > L2_BYTES else "L2 flushed between timed steps (256 MB write outside the timing)")
    return cfg


def needs_flush(w: dict) -> bool:
    return "flushed" in workload_config(w, 0)["l2"]


def tile_bytes(numtile, nnz, tilem, v, b_side=False):
    """Compulsory bytes of one tile matrix: tile_ptr, per tile colidx + nnz
    prefix + 16 row offsets + 16 row masks, per nonzero value + column byte;
    B additionally its CSC tile pointer/rowidx arrays."""
    b = 4 * (tilem + 1) + numtile * (4 + 4 + 16 + 32) + nnz * (v + 1)
    if b_side:
        b += 4 * (tilem + 1) + 4 * numtile
    return b


def c_bytes(numtileC, nnzC, tilem, v):
    return 4 * (tilem + 1) + numtileC * (4 + 4 + 8 + 32 + 16) + nnzC * (v + 1)


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except Exception:
            self.proc.kill()
            out, _ = self.proc.communicate()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax = float(p[2])
            except ValueError:
                continue
            for nm, flag in zip(names, p[5:9]):
                if flag.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def job_time_and_value(ms_local: float, flops_local: float, world: int, device) -> tuple:
    """Whole-job figures of a replicas-only run: every rank multiplies its own
    copy of the workload between two barriers, so the job's step time is the
    slowest rank's and its work is the sum of the ranks' work.  Returns
    (ms per step, GFLOP/s of the whole job).  Works on any process-group
    backend (NCCL on the GPUs, gloo on CPU)."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([ms_local], dtype=torch.float64, device=device)
    f = torch.tensor([flops_local], dtype=torch.float64, device=device)
    if world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        dist.all_reduce(f, op=dist.ReduceOp.SUM)
        dist.barrier()
    ms = float(t.item())
    return ms, float(f.item()) / (ms * 1e-3) / 1e9


# ---------------------------------------------------------------------------
# CPU legs (the oracle's OpenMP Gustavson: a reported baseline, never the product)
# ---------------------------------------------------------------------------
def _row_sample(a, k, off):
    rows = np.arange(off, a.m, k, dtype=np.int64)
    lens = np.diff(a.row_ptr)[rows]
    rp = np.zeros(rows.size + 1, np.int64)
    np.cumsum(lens, out=rp[1:])
    starts = a.row_ptr[rows].astype(np.int64)
    idx = np.repeat(starts - rp[:-1], lens) + np.arange(int(rp[-1]), dtype=np.int64) if rows.size else \
        np.zeros(0, np.int64)
    return synth.CSR(rows.size, a.n, rp.astype(np.int32), a.col_idx[idx], a.val[idx])


def cpu_gflops(w: dict, target_s: float = 12.0):
    """OpenMP Gustavson on a seeded stride sample of the left operand's rows,
    sized to about target_s seconds; returns (GFLOP/s, threads, sample text).
    For the Galerkin workload both products are sampled alike."""
    import oracle
    threads = oracle.max_threads()
    rng = np.random.Generator(np.random.PCG64(0xC0FFEE))
    if w["kind"] == "product":
        legs = [(w["a"], w["b"])]
    else:
        pt, ap = galerkin_operands(w)
        legs = [(w["a"], w["p"]), (pt, ap)]
    dtype = np.float64 if legs[0][0].val.dtype == np.float64 else np.float32

    def run(frac):
        k = max(1, int(round(1.0 / frac)))
        off = int(rng.integers(0, k))
        prods, dt = 0, 0.0
        for left, right in legs:
            s = _row_sample(left, k, off)
            prods += synth.products(s, right)
            t0 = time.perf_counter()
            oracle.gustavson_rows(s, right, 0, s.m, dtype)
            dt += time.perf_counter() - t0
        return k, prods, max(dt, 1e-4)

    k, p, dt = run(0.01)
    frac = min(1.0, 0.01 * target_s / dt)
    k, p, dt = run(frac)
    what = "left operand" if w["kind"] == "product" else "left operand of each product"
    return 2.0 * p / dt / 1e9, threads, f"every {k}-th row of the {what} ({p} products), {dt:.1f} s"


def run_reference(args):
    world, rank, _ = dist_setup()
    if rank != 0:
        return
    w = workload(args.workload)
    import oracle
    products = structural_products(w)
    dtype = np.float64 if w["a"].val.dtype == np.float64 else np.float32
    vals = []
    desc = ""
    threads = oracle.max_threads()
    for i in range(args.warmup + args.steps):
        g, threads, desc = cpu_gflops(w, target_s=args.ref_step_s)
        if i >= args.warmup:
            vals.append(g)
    v = statistics.mean(vals)
    line = {"impl": "reference", "metric": "SpGEMM GFLOP/s", "value": v, "unit": "GFLOP/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "dtype": np.dtype(dtype).name,
            "data": "synthetic", "config": workload_config(w, products), "vs_baseline": None,
            "cpu_baseline": {"value": v, "unit": "GFLOP/s", "cores": threads, "kind": "port",
                             "sample": "OpenMP row-parallel Gustavson (CPU oracle's restatement of "
                                       "src/spgemm_raw_v2.cu:289-338), " + desc},
            "e2e": {"value": v, "unit": "GFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
class Timer:
    """CUDA-event timing of K steps on the library's stream: one bracket when
    the inputs exceed L2, else one bracket per step with an L2 flush (a 256 MB
    write on the same stream) between steps, outside the brackets."""

    def __init__(self, stream, flush: bool):
        import torch
        self.torch = torch
        self.stream = stream
        self.flush_buf = torch.empty(256 << 20, dtype=torch.uint8, device="cuda") if flush else None

    def run(self, fn, steps: int) -> float:
        torch = self.torch
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        if self.flush_buf is None:
            torch.cuda.synchronize()
            ev[0].record(self.stream)
            for _ in range(steps):
                fn()
            ev[1].record(self.stream)
            torch.cuda.synchronize()
            return ev[0].elapsed_time(ev[1]) / steps
        tot = 0.0
        for _ in range(steps):
            with torch.cuda.stream(self.stream):
                self.flush_buf.fill_(1)
            torch.cuda.synchronize()
            ev[0].record(self.stream)
            fn()
            ev[1].record(self.stream)
            torch.cuda.synchronize()
            tot += ev[0].elapsed_time(ev[1])
        return tot / steps


def load_peaks():
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        peaks = {}
    if "hbm_gbs" in peaks:
        return float(peaks["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def step_roofline(args, A, B, numtileC, nnzC, v, s1, s2, s3, rowwise, sized, numeric_algo=None):
    """Roofline of the dominant step's kernel: its algorithmic bytes (each
    array it must touch, read or written once) over its CUDA-event time."""
    hbm_peak, peak_src = load_peaks()
    a_b = tile_bytes(A.numtile, A.nnz, A.tilem, v)
    b_b = tile_bytes(B.numtile, B.nnz, B.tilem, v, b_side=True)
    # numeric: reads A and B (tiles and row views alike: the same bytes once),
    # C's structure; writes C's values and column bytes
    num_bytes = a_b + b_b + 4 * (A.tilem + 1) + numtileC * (4 + 4 + 8 + 32 + 16) + nnzC * (v + 1)
    sym_bytes = (4 * (A.tilem + 1) + A.numtile * (4 + 4 + 16) + A.nnz + B.numtile * (4 + 32) + 4 * (B.tilen + 1)
                 + numtileC * (4 + 4 + 32 + 16 + 4))
    st1_bytes = 4 * (A.tilem + 1) * 2 + 4 * A.numtile + 4 * B.numtile + 8 * numtileC
    steps_ms = {"step1": s1, "step2": s2, "step3": s3}
    dom = max(steps_ms, key=steps_ms.get)
    dom_bytes = {"step1": st1_bytes, "step2": sym_bytes, "step3": num_bytes}[dom]
    names = {"step1": "c1_slot_kernel + c1_compact_kernel" if sized else "c1_count_kernel + c1_fill_kernel",
             "step2": "rw_symbolic_kernel" if rowwise else "c2_symbolic_kernel",
             "step3": {2: "rw_numeric_kernel", 3: "rw_numeric_kernel + c3_numeric_kernel (binned)"}.get(
                 numeric_algo if numeric_algo is not None else (2 if rowwise else 1), "c3_numeric_kernel")}
    if args.prec == "mixed" and names["step3"] == "c3_numeric_kernel":
        names["step3"] = "c3_numeric_kernel + c3_tensor_kernel"
    achieved = dom_bytes / (steps_ms[dom] * 1e-3) / 1e9
    traffic = args.traffic
    traffic_src = "--traffic" if traffic is not None else None
    ratio = TRAFFIC_PER_ALGO_BYTE.get(names[dom])
    if traffic is None and ratio is not None:
        traffic = ratio * dom_bytes
        traffic_src = ("ncu DRAM bytes per algorithmic byte of the R-MAT 2^17 launch (%.3f), times this launch's "
                       "algorithmic bytes; a lower bound where B's entries exceed L2" % ratio)
    return {"bound": "hbm", "kernel": names[dom], "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
            "frac": achieved / hbm_peak, "peak_source": peak_src, "algorithmic_bytes": dom_bytes,
            "ms": steps_ms[dom], "traffic": traffic, "traffic_source": traffic_src}, a_b + b_b


def check_ranges(tilem, which="default"):
    """Tile-rows checked against the oracle: the first 512 (the hub rows of a
    power-law matrix, the worst case for accumulation order) and 2,048 from
    the middle."""
    r = [(0, min(tilem, 512))]
    mid = tilem // 2
    if mid + 2048 <= tilem and mid >= 512:
        r.append((mid, mid + 2048))
    return r


def value_check(h, api, w, Cm):
    """C's structure and values on sampled tile-rows against the FP64 oracle
    (each C tile-row depends only on the same 16 rows of A and all of B): the
    oracle forms those rows by Gustavson in FP64 and compares entry by entry.
    Returns the relative Frobenius error, the structural mismatches and what
    was checked."""
    import ctypes as C
    import oracle
    a, b = w["a"], w["b"]
    vd = np.float64 if a.val.dtype == np.float64 else np.float32
    tp = np.zeros(Cm.tilem + 1, np.int32)
    h.check(h.lib.spg_ctiles_to_host(h.h, C.byref(Cm.c), tp.ctypes.data, None, None, None, None, None, None, None))
    err2 = ref2 = 0.0
    bad = 0
    nvals = 0
    rows = 0
    t0 = time.perf_counter()
    for i0, i1 in check_ranges(Cm.tilem):
        s, e = int(tp[i0]), int(tp[i1])
        nt = e - s
        d = dict(tile_colidxC=np.zeros(max(nt, 1), np.int32), maskC=np.zeros(max(nt, 1) * 16, np.uint16),
                 tile_nnzC=np.zeros(nt + 1, np.int64), ptrRowC=np.zeros(max(nt, 1) * 16, np.uint8))
        h.check(h.lib.spg_ctiles_to_host_range(h.h, C.byref(Cm.c), s, e, None, d["tile_colidxC"].ctypes.data,
                                               d["maskC"].ctypes.data, d["tile_nnzC"].ctypes.data,
                                               d["ptrRowC"].ctypes.data, None, None, 0, None))
        nv = int(d["tile_nnzC"][-1] - d["tile_nnzC"][0])
        d["tile_valC"] = np.zeros(max(nv, 1), vd)
        d["tile_colC"] = np.zeros(max(nv, 1), np.uint8)
        got = C.c_int64()
        h.check(h.lib.spg_ctiles_to_host_range(h.h, C.byref(Cm.c), s, e, None, None, None, None, None,
                                               d["tile_valC"].ctypes.data, d["tile_colC"].ctypes.data, max(nv, 1),
                                               C.byref(got)))
        d["tile_ptr"] = tp[i0:i1 + 1].astype(np.int64) - s
        r = oracle.check_tilerows(a, b, i0, i1, d)
        err2 += (r["rel_frob"] * r["ref_frob"]) ** 2
        ref2 += r["ref_frob"] ** 2
        bad += r["mismatches"]
        nvals += nv
        rows += i1 - i0
    return {"tile_rows_checked": rows, "ranges": check_ranges(Cm.tilem), "c_values_checked": nvals,
            "rel_frob_vs_fp64": float(np.sqrt(err2) / (np.sqrt(ref2) or 1.0)), "structure_mismatches": bad,
            "cols_equal": bad == 0, "oracle": "FP64 Gustavson per row (src/spgemm_raw_v2.cu:289-338)",
            "check_s": round(time.perf_counter() - t0, 1)}


def run_ours(args):
    import torch
    import torch.distributed as dist
    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl")
    w = workload(args.workload)
    if w["kind"] == "galerkin":
        return run_galerkin(args, w, world, rank, local)
    from gpu_spgemm_gb300 import api
    a, b = w["a"], w["b"]
    dtype = a.val.dtype
    v = 8 if dtype == np.float64 else 4
    stream = torch.cuda.Stream()
    h = api.Handle(local, stream)
    A = api.csr2tile(h, a)
    B = api.build_csc_tiles(h, b)
    products = api.products(h, A, B)
    flops = 2.0 * products
    h.set_mixed_params(args.dense_thr)
    sizing = None
    # the learned step 1 pays three read-backs where the exact one pays one:
    # it is attached for an A of at least 65,536 tiles, where its single
    # bitmap pass saves more than they cost
    if args.sizing and os.path.exists(api.SIZING_MODEL_PATH) and A.numtile >= SIZING_MIN_TILES:
        sizing = api.SizingModel.load(h)
        sizing.attach(args.sizing_margin)
    timer = Timer(stream, needs_flush(w))

    last = {}

    def step(algo=args.algo, prec=args.prec):
        C = api.spgemm(h, A, B, algo=algo, prec=prec)
        last["stats"] = h.stats()
        last["info"] = (C.numtileC, C.nnzC, C.pairs)
        C.free()

    stats = []

    def timed_step():
        step()
        stats.append(last["stats"])

    for _ in range(args.warmup):
        step()
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    l0 = h.launches()
    ms_local = timer.run(timed_step, args.steps)
    launches = h.launches() - l0
    clk = clocks.stop()
    ms, value = job_time_and_value(ms_local, flops, world, "cuda")
    numtileC, nnzC, pairs = last["info"]
    s1 = statistics.mean(s["ms_step1"] for s in stats)
    s2 = statistics.mean(s["ms_step2"] for s in stats)
    s3 = statistics.mean(s["ms_step3"] for s in stats)
    rowwise = stats[-1].get("algo_used", 1) in (2, 3)
    roofline, ab_bytes = step_roofline(args, A, B, numtileC, nnzC, v, s1, s2, s3, rowwise, sizing is not None,
                                       stats[-1].get("numeric_algo"))
    c_b = c_bytes(numtileC, nnzC, A.tilem, v)

    accuracy = None
    if not args.no_check:
        Cm = api.spgemm(h, A, B, algo=args.algo, prec=args.prec)
        accuracy = value_check(h, api, w, Cm)
        accuracy.update(numtileC=Cm.numtileC, nnzC=Cm.nnzC, tensor_pairs=h.stats()["tensor_pairs"],
                        fp64_tiles=h.stats()["fp64_tiles"])
        Cm.free()

    # ---- end to end (before the comparison legs, whose allocations would
    # leave the memory pool shaped for other products)
    e2e = None
    if not args.no_e2e:
        small = numtileC < E2E_STREAM_MIN_TILES if args.e2e_mode == "auto" else args.e2e_mode == "whole"
        e2e = measure_e2e(h, api, a, b, args, flops, stream, small_c=small)

    # ---- the same product by the plain kernels and without the sizing model
    vs_plain = None
    if not args.no_compare:
        vs_plain = {}
        if sizing is not None:
            sizing.detach()
        step(algo="plain", prec="f32")  # warm-up
        pms = timer.run(lambda: step(algo="plain", prec="f32"), args.plain_steps)
        ps = last["stats"]
        vs_plain["plain"] = {"gflops": flops / (pms * 1e-3) / 1e9, "ms_step": pms, "ms_step1": ps["ms_step1"],
                             "ms_step2": ps["ms_step2"], "ms_step3": ps["ms_step3"],
                             "what": "per-C-tile kernels (tile-list intersection, register accumulation; the "
                                     "reference's method), exact two-pass step 1, no sizing model, FP32 registers"}
        if sizing is not None:
            step()
            nms = timer.run(step, max(1, args.steps // 2))
            ns = last["stats"]
            vs_plain["default_without_sizing_model"] = {
                "gflops": flops / (nms * 1e-3) / 1e9, "ms_step": nms, "ms_step1": ns["ms_step1"],
                "ms_step2": ns["ms_step2"], "ms_step3": ns["ms_step3"]}
            vs_plain["sizing_model_gain"] = nms / ms_local
            sizing.attach(args.sizing_margin)
        vs_plain["speedup_vs_plain"] = pms / ms_local

    cpu = None
    if rank == 0 and not args.no_cpu:
        g, thr, desc = cpu_gflops(w, target_s=args.cpu_s)
        cpu = {"value": g, "unit": "GFLOP/s", "cores": thr, "kind": "port",
               "sample": "OpenMP row-parallel Gustavson (CPU oracle's restatement of "
                         "src/spgemm_raw_v2.cu:289-338), " + desc}

    if rank == 0:
        hbm_peak = roofline["peak"]
        hbm_steps = (ab_bytes + c_b) / (ms * 1e-3) / 1e9
        details = {"numtileC": numtileC, "nnzC": nnzC, "tile_pairs": pairs, "algo": args.algo, "prec": args.prec,
                   "algo_used": {0: "auto", 1: "plain", 2: "rowwise", 3: "binned"}.get(stats[-1].get("algo_used"), "?"),
                   "ms_step1": s1, "ms_step2": s2, "ms_step3": s3,
                   "tile_bytes": {"A+B": ab_bytes, "C": c_b},
                   "hbm_gbs_steps": hbm_steps, "hbm_frac_steps": hbm_steps / hbm_peak,
                   "tensor_pairs": stats[-1].get("tensor_pairs", 0), "fp64_tiles": stats[-1].get("fp64_tiles", 0),
                   "learned_sizing": "not attached: A has fewer than %d tiles" % SIZING_MIN_TILES
                   if sizing is None and args.sizing else None if sizing is None else {
                       "model": os.path.relpath(api.SIZING_MODEL_PATH, ROOT), "margin": args.sizing_margin,
                       "predicted_tiles": stats[-1].get("predicted_tiles", 0), "actual_tiles": numtileC,
                       "overflow_reruns": stats[-1].get("overflow_reruns", 0),
                       "fallbacks": stats[-1].get("sizing_fallbacks", 0),
                       "step1": "one bitmap pass into predicted per-row slots, then compaction; "
                                "rows that outgrow their slot re-run the exact fill"}}
        line = {"metric": "SpGEMM GFLOP/s", "value": value, "unit": "GFLOP/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": np.dtype(dtype).name, "data": "synthetic",
                "config": workload_config(w, products), "details": details, "accuracy": accuracy,
                "vs_plain": vs_plain, "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "clocks": clk,
                "gpu_launches": launches}
        print(json.dumps(line), flush=True)
    h.close()
    if world > 1:
        dist.destroy_process_group()


def run_galerkin(args, w, world, rank, local):
    """RAP = P^T (A P) through spg_galerkin: A and P resident as device CSR;
    one step tiles A and P, forms A*P, expands it to CSR and re-tiles it as
    the B operand, transposes P, tiles P^T and forms P^T (A P).  GFLOP/s
    counts both products."""
    import torch
    import torch.distributed as dist
    from gpu_spgemm_gb300 import api
    import oracle
    a, p = w["a"], w["p"]
    stream = torch.cuda.Stream()
    h = api.Handle(local, stream)
    dev = lambda x: torch.from_numpy(np.ascontiguousarray(x)).cuda()
    ar, ac, av = dev(a.row_ptr), dev(a.col_idx), dev(a.val)
    pr_, pc, pv = dev(p.row_ptr), dev(p.col_idx), dev(p.val)
    sizing = None
    if args.sizing and os.path.exists(api.SIZING_MODEL_PATH):
        sizing = api.SizingModel.load(h)
        sizing.attach(args.sizing_margin)
    timer = Timer(stream, needs_flush(w))
    last = {}

    def step(algo=args.algo, prec=args.prec):
        Cm, prods = api.galerkin_device(h, a.m, p.n, a.nnz, ar.data_ptr(), ac.data_ptr(), av.data_ptr(), p.nnz,
                                        pr_.data_ptr(), pc.data_ptr(), pv.data_ptr(), a.val.dtype, algo, prec)
        last.update(prods=prods, stats=h.stats(), info=(Cm.numtileC, Cm.nnzC))
        return Cm

    stats = []

    def timed_step():
        step().free()
        stats.append(last["stats"])

    for _ in range(args.warmup):
        step().free()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    l0 = h.launches()
    ms_local = timer.run(timed_step, args.steps)
    launches = h.launches() - l0
    clk = clocks.stop()
    products = last["prods"]
    flops = 2.0 * products
    ms, value = job_time_and_value(ms_local, flops, world, "cuda")
    st = stats[-1]
    hbm_peak, peak_src = load_peaks()

    accuracy = None
    if not args.no_check:
        Cm = step()
        got = Cm.to_host()
        Cm.free()
        t0 = time.perf_counter()
        S1 = oracle.spgemm_tiles(a, p)
        rp, ci, vv = oracle.tiles_to_csr(a.m, p.n, S1)
        ap = synth.CSR(a.m, p.n, rp.astype(np.int32), ci, vv)
        S = oracle.spgemm_tiles(synth.transpose(p), ap)
        bad = sum(int(not np.array_equal(got[k], S[k].astype(got[k].dtype)))
                  for k in ("tile_ptrC", "tile_rowidxC", "tile_colidxC", "maskC", "tile_nnzC", "ptrRowC",
                            "tile_colC"))
        ref = S["tile_valC"]
        err = float(np.linalg.norm(got["tile_valC"].astype(np.float64) - ref) / (np.linalg.norm(ref) or 1.0))
        accuracy = {"rel_frob_vs_fp64": err, "structure_arrays_differing": bad, "cols_equal": bad == 0,
                    "numtileC": int(got["numtileC"]), "nnzC": int(got["nnzC"]),
                    "oracle": "tiled FP64 oracle: A*P, expanded to CSR, then P^T (A P)",
                    "check_s": round(time.perf_counter() - t0, 1)}

    vs_plain = None
    if not args.no_compare:
        if sizing is not None:
            sizing.detach()
        step(algo="plain", prec="f32").free()
        pms = timer.run(lambda: step(algo="plain", prec="f32").free(), max(1, args.steps // 2))
        vs_plain = {"plain": {"gflops": flops / (pms * 1e-3) / 1e9, "ms_step": pms,
                              "what": "both products on the per-C-tile kernels, exact two-pass step 1, "
                                      "no sizing model"},
                    "speedup_vs_plain": pms / ms_local}
        if sizing is not None:
            step().free()
            nms = timer.run(lambda: step().free(), max(1, args.steps // 2))
            vs_plain["default_without_sizing_model"] = {"gflops": flops / (nms * 1e-3) / 1e9, "ms_step": nms}
            vs_plain["sizing_model_gain"] = nms / ms_local
            sizing.attach(args.sizing_margin)

    e2e = None
    if not args.no_e2e:
        e2e = galerkin_e2e(h, api, w, args, flops, stream)

    cpu = None
    if rank == 0 and not args.no_cpu:
        g, thr, desc = cpu_gflops(w, target_s=args.cpu_s)
        cpu = {"value": g, "unit": "GFLOP/s", "cores": thr, "kind": "port",
               "sample": "OpenMP row-parallel Gustavson (CPU oracle's restatement of "
                         "src/spgemm_raw_v2.cu:289-338) of A*P and P^T (A P), " + desc}
    if rank == 0:
        s123 = st["ms_step1"] + st["ms_step2"] + st["ms_step3"]
        details = {"numtileC": last["info"][0], "nnzC": last["info"][1], "algo": args.algo, "prec": args.prec,
                   "ms_steps_of_both_products": {"step1": st["ms_step1"], "step2": st["ms_step2"],
                                                 "step3": st["ms_step3"]},
                   "ms_tiling_and_conversions": ms_local - s123,
                   "learned_sizing": "not attached: A has fewer than %d tiles" % SIZING_MIN_TILES
                   if sizing is None and args.sizing else None if sizing is None else {"margin": args.sizing_margin,
                                                                  "overflow_reruns": st["overflow_reruns"]}}
        steps_ms = {"step1": st["ms_step1"], "step2": st["ms_step2"], "step3": st["ms_step3"],
                    "tiling and conversions": ms_local - s123}
        dom = max(steps_ms, key=steps_ms.get)
        roofline = {"bound": "hbm", "kernel": f"galerkin {dom}", "achieved": None, "peak": hbm_peak,
                    "unit": "GB/s", "frac": None, "peak_source": peak_src, "ms": steps_ms[dom], "traffic": None}
        line = {"metric": "SpGEMM GFLOP/s", "value": value, "unit": "GFLOP/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": np.dtype(a.val.dtype).name, "data": "synthetic",
                "config": workload_config(w, products), "details": details, "accuracy": accuracy,
                "vs_plain": vs_plain, "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "clocks": clk,
                "gpu_launches": launches}
        print(json.dumps(line), flush=True)
    h.close()
    if world > 1:
        dist.destroy_process_group()


def galerkin_e2e(h, api, w, args, flops, stream):
    """spg_galerkin end to end: A and P copied from pinned host memory to the
    device each step, RAP's result arrays (the ones the reference reads back,
    src/spgemm_raw_v2.cu:257-266) copied to pinned host memory."""
    import ctypes as C
    import torch
    a, p = w["a"], w["p"]
    pin = lambda x: torch.from_numpy(np.ascontiguousarray(x)).pin_memory()
    host = [pin(x) for x in (a.row_ptr, a.col_idx, a.val, p.row_ptr, p.col_idx, p.val)]
    devs = [torch.empty_like(x, device="cuda") for x in host]
    h2d = sum(x.numel() * x.element_size() for x in host)
    out = {}

    def one():
        with torch.cuda.stream(stream):
            for d, x in zip(devs, host):
                d.copy_(x, non_blocking=True)
        ar, ac, av, pr_, pc, pv = devs
        Cm, _ = api.galerkin_device(h, a.m, p.n, a.nnz, ar.data_ptr(), ac.data_ptr(), av.data_ptr(), p.nnz,
                                    pr_.data_ptr(), pc.data_ptr(), pv.data_ptr(), a.val.dtype, args.algo, args.prec)
        c = Cm.c
        nt, nz = c.numtileC, c.nnzC
        if out.get("nt") != nt or out.get("nz") != nz:
            out.update(nt=nt, nz=nz, tp=pin(np.zeros(c.tilem + 1, np.int32)), r=pin(np.zeros(max(nt, 1), np.int32)),
                       c=pin(np.zeros(max(nt, 1), np.int32)), p=pin(np.zeros(nt + 1, np.int64)),
                       v=pin(np.zeros(max(nz, 1), np.float32)), cc=pin(np.zeros(max(nz, 1), np.uint8)))
        g = lambda k: C.c_void_p(out[k].data_ptr())
        h.check(h.lib.spg_ctiles_to_host(h.h, C.byref(c), g("tp"), g("r"), g("c"), None, g("p"), None, g("v"),
                                         g("cc")))
        Cm.free()
        return (c.tilem + 1) * 4 + nt * 8 + (nt + 1) * 8 + nz * 5

    try:
        one()
        torch.cuda.synchronize()
        steps = max(1, args.e2e_steps)
        t0 = time.perf_counter()
        d2h = 0
        for _ in range(steps):
            d2h = one()
        torch.cuda.synchronize()
        dt = (time.perf_counter() - t0) / steps
        return {"value": flops / dt / 1e9, "unit": "GFLOP/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "ms_per_step": dt * 1e3, "steps": steps,
                "path": "pinned host CSR A and P -> device, spg_galerkin, spg_ctiles_to_host of tile_ptrC, "
                        "tile_rowidxC, tile_colidxC, tile_nnzC, tile_valC, tile_colC to pinned host memory"}
    except Exception as e:  # report instead of dying
        return {"value": None, "unit": "GFLOP/s", "error": str(e)[:200], "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": None}


def e2e_tile_inputs(h, a, b, ha, hb, code):
    """The step's inputs, host CSR -> device tiles: A row-major, B in CSC tile
    order.  For A*A (b is a) the CSR crosses once: B is tiled from A's device
    row view, the copy of the CSR that A's tiles keep."""
    import ctypes as C
    from gpu_spgemm_gb300 import _lib as L
    lib = h.lib
    ta, tb = L.SpgTiles(), L.SpgTiles()
    h.check(lib.spg_tile_from_csr_host(h.h, a.m, a.n, a.nnz, ha[0][1].ctypes.data, ha[1][1].ctypes.data,
                                       ha[2][1].ctypes.data, code, L.SPG_LAYOUT_ROW, 0, C.byref(ta)))
    if b is a:
        h.check(lib.spg_tile_from_csr(h.h, a.m, a.n, a.nnz, ta.row_ptr, ta.col_idx, ta.row_val, code,
                                      L.SPG_LAYOUT_B_CSC, 0, C.byref(tb)))
    else:
        h.check(lib.spg_tile_from_csr_host(h.h, b.m, b.n, b.nnz, hb[0][1].ctypes.data, hb[1][1].ctypes.data,
                                           hb[2][1].ctypes.data, code, L.SPG_LAYOUT_B_CSC, 0, C.byref(tb)))
    return ta, tb


def e2e_whole(h, api, a, b, args, flops, pin, code, vd, h2d, ha, hb):
    """End to end for a C small enough to copy whole: per step the CSR inputs
    go host->device and are tiled, spg_spgemm runs steps 1-3, and C's result
    arrays come back to pinned host buffers in one spg_ctiles_to_host call
    (the streaming of the large path would only add its bookkeeping)."""
    import ctypes as C
    from gpu_spgemm_gb300 import _lib as L
    lib = h.lib
    out = {}

    def one():
        c = L.SpgCTiles()
        ta, tb = e2e_tile_inputs(h, a, b, ha, hb, code)
        h.check(lib.spg_spgemm(h.h, C.byref(ta), C.byref(tb), api._ALGOS[args.algo], api._PRECS[args.prec],
                               C.byref(c)))
        nt, nz = c.numtileC, c.nnzC
        if out.get("nt") != nt or out.get("nz") != nz:
            out.update(nt=nt, nz=nz, tp=pin(np.zeros(c.tilem + 1, np.int32)), r=pin(np.zeros(max(nt, 1), np.int32)),
                       c=pin(np.zeros(max(nt, 1), np.int32)), p=pin(np.zeros(nt + 1, np.int64)),
                       v=pin(np.zeros(max(nz, 1), vd)), cc=pin(np.zeros(max(nz, 1), np.uint8)))
        g = lambda k: out[k][1].ctypes.data
        h.check(lib.spg_ctiles_to_host(h.h, C.byref(c), g("tp"), g("r"), g("c"), None, g("p"), None, g("v"),
                                       g("cc")))
        lib.spg_ctiles_free(h.h, C.byref(c))
        lib.spg_tiles_free(h.h, C.byref(ta))
        lib.spg_tiles_free(h.h, C.byref(tb))
        return (c.tilem + 1) * 4 + nt * 8 + (nt + 1) * 8 + nz * (np.dtype(vd).itemsize + 1)

    try:
        one()
        steps = max(5, args.e2e_steps)
        t0 = time.perf_counter()
        d2h = 0
        for _ in range(steps):
            d2h = one()
        dt = (time.perf_counter() - t0) / steps
        return {"value": flops / dt / 1e9, "unit": "GFLOP/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "ms_per_step": dt * 1e3, "steps": steps,
                "path": "spg_tile_from_csr_host (A, and B unless B is A) + spg_tile_from_csr of B from A's row view when B is A + spg_spgemm + spg_ctiles_to_host of tile_ptrC, tile_rowidxC, "
                        "tile_colidxC, tile_nnzC, tile_valC, tile_colC into pinned host buffers"}
    except Exception as e:  # report instead of dying
        return {"value": None, "unit": "GFLOP/s", "error": str(e)[:200], "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": None}


# C tiles below which the e2e copies C whole after the product instead of
# streaming it while the product runs
E2E_STREAM_MIN_TILES = 1 << 22


def measure_e2e(h, api, a, b, args, flops, stream, small_c=False):
    """End to end through the C ABI with host buffers, per step: the CSR inputs
    are copied from pinned host memory to the device and tiled, C = A*B is
    computed, and C's result is copied back to pinned host memory: the arrays
    the reference reads back for its result (src/spgemm_raw_v2.cu:257-266):
    tile_ptrC, tile_rowidxC, tile_colidxC, the nonzero prefix tile_nnzC, the
    column bytes tile_colC and the values tile_valC.  (maskC and ptrRowC are
    intermediates that tile_colC restates; they stay on the device.)  C can
    exceed host memory (R-MAT 2^20: ~77 GB of result), so it streams through
    fixed pinned staging in tile ranges (spg_ctiles_to_host_range) on copy
    workers, each with its own handle, stream and staging, fed from one FIFO
    as the arrays become final: the tile indices when spg_symbolic_tiles
    returns (copied while spg_symbolic_masks runs), the prefix when the masks
    are done, and each band of tile-rows' values as spg_numeric_bands reports
    the band complete (copied while the numeric launch goes on)."""
    import queue
    import threading
    import ctypes as C
    import torch
    from gpu_spgemm_gb300 import _lib as L

    def pin(x):
        t = torch.from_numpy(np.ascontiguousarray(x)).pin_memory()
        return t, t.numpy()

    ha = [pin(a.row_ptr), pin(a.col_idx), pin(a.val)]
    hb = ha if b is a else [pin(b.row_ptr), pin(b.col_idx), pin(b.val)]
    code = L.SPG_F64 if a.val.dtype == np.float64 else L.SPG_F32
    vd = np.float64 if code == L.SPG_F64 else np.float32
    vsz = np.dtype(vd).itemsize
    h2d = sum(x[1].nbytes for x in (ha if b is a else ha + hb))
    CT = max(1 << 16, args.e2e_range_tiles)  # C tiles per staged range
    VC = 1 << 27            # values per staged range (ranges halve when a range holds more)
    NW = max(1, args.e2e_copy_workers)
    NB = max(1, args.e2e_bands)
    lib = h.lib

    class Worker:
        def __init__(self):
            self.stream = torch.cuda.Stream()
            self.h = api.Handle(torch.cuda.current_device(), self.stream)
            self.st = dict(r=pin(np.zeros(CT, np.int32)), c=pin(np.zeros(CT, np.int32)),
                           p=pin(np.zeros(CT + 1, np.int64)), v=pin(np.zeros(VC, vd)),
                           cc=pin(np.zeros(VC, np.uint8)))

    if small_c:
        return e2e_whole(h, api, a, b, args, flops, pin, code, vd, h2d, ha, hb)
    workers = [Worker() for _ in range(NW)]
    tstat = {}

    def copy_range(wk, c, kind, t0, t1):
        """One staged copy of C tiles [t0, t1): "index" (tile row and column
        indices), "prefix" (tile_nnzC) or "value" (values and column bytes,
        split in halves while a range holds more than VC values)."""
        nv = C.c_int64()
        g = lambda k: wk.st[k][1].ctypes.data
        nb = 0
        while t0 < t1:
            step = t1 - t0
            while True:
                e = min(t1, t0 + step)
                if kind == "index":
                    s_ = lib.spg_ctiles_to_host_range(wk.h.h, C.byref(c), t0, e, g("r"), g("c"), None, None, None,
                                                      None, None, VC, None)
                elif kind == "prefix":
                    s_ = lib.spg_ctiles_to_host_range(wk.h.h, C.byref(c), t0, e, None, None, None, g("p"), None,
                                                      None, None, VC, None)
                else:
                    s_ = lib.spg_ctiles_to_host_range(wk.h.h, C.byref(c), t0, e, None, None, None, None, None,
                                                      g("v"), g("cc"), VC, C.byref(nv))
                if s_ == L.SPG_ERR_INVALID and kind == "value" and step > 1:
                    step //= 2
                    continue
                wk.h.check(s_)
                break
            nb += {"index": (e - t0) * 8, "prefix": (e - t0 + 1) * 8}.get(kind, 0) + \
                (nv.value * (vsz + 1) if kind == "value" else 0)
            t0 = e
        return nb

    def one():
        c = L.SpgCTiles()
        ta, tb = e2e_tile_inputs(h, a, b, ha, hb, code)
        h.check(lib.spg_symbolic_tiles(h.h, C.byref(ta), C.byref(tb), api._ALGOS[args.algo], C.byref(c)))
        tp = np.zeros(c.tilem + 1, np.int32)
        h.check(lib.spg_ctiles_to_host(h.h, C.byref(c), tp.ctypes.data, None, None, None, None, None, None, None))
        q = queue.Queue()
        nbytes = [tp.nbytes]
        errs = []
        lock = threading.Lock()
        done_at = {}

        def work(wk):
            while True:
                task = q.get()
                if task is None:
                    return
                kind, t0, t1 = task
                try:
                    if not errs:
                        ts = time.perf_counter()
                        nb = copy_range(wk, c, kind, t0, t1)
                        te = time.perf_counter()
                        with lock:
                            nbytes[0] += nb
                            done_at.setdefault(kind, []).append((ts, te, nb))
                except Exception as ex:  # reported after the join
                    errs.append(ex)

        def push(kind, t0, t1):
            for x in range(t0, t1, CT):
                q.put((kind, x, min(t1, x + CT)))

        ths = [threading.Thread(target=work, args=(wk,)) for wk in workers]
        for th in ths:
            th.start()
        t = time.perf_counter()
        try:
            push("index", 0, c.numtileC)
            h.check(lib.spg_symbolic_masks(h.h, C.byref(ta), C.byref(tb), C.byref(c)))
            t_msk = time.perf_counter()
            push("prefix", 0, c.numtileC)
            # tile-row bands of about equal tile counts
            cuts = np.searchsorted(tp, np.linspace(0, c.numtileC, NB + 1)[1:-1], side="left")
            bounds = [0] + sorted(set(int(x) for x in cuts if 0 < x < c.tilem)) + [c.tilem]
            rows = np.asarray(bounds, np.int32)
            band_at = []

            def on_band(_u, k, r0, r1):
                band_at.append((k, time.perf_counter()))
                push("value", int(tp[r0]), int(tp[r1]))

            fn = L.BAND_FN(on_band)
            order = L.SPG_BANDS_LAST_TO_FIRST if args.e2e_band_order == "last" else L.SPG_BANDS_FIRST_TO_LAST
            h.check(lib.spg_numeric_bands(h.h, C.byref(ta), C.byref(tb), api._ALGOS[args.algo],
                                          api._PRECS[args.prec], C.byref(c), len(bounds) - 1,
                                          rows.ctypes.data, order, fn, None))
            t_num = time.perf_counter()
        finally:
            for _ in ths:
                q.put(None)
            for th in ths:
                th.join()
        t_end = time.perf_counter()
        if errs:
            raise errs[0]
        ms = lambda x: round((x - t_msk) * 1e3, 1)
        # per worker: bytes over the time its copy calls took (workers copy side by side)
        gbs = lambda v: round(sum(b_ for _, _, b_ in v) / max(1e-9, sum(e_ - s_ for s_, e_, _ in v)) / 1e9, 1)
        tstat.update(mask_step_ms=(t_msk - t) * 1e3, numeric_bands_ms=(t_num - t_msk) * 1e3,
                     copy_tail_ms=(t_end - t_num) * 1e3, bands=len(bounds) - 1,
                     band_done_ms=[ms(x) for _, x in sorted(band_at)],
                     copy_window_ms={k: [ms(min(s_ for s_, _, _ in v)), ms(max(e_ for _, e_, _ in v))]
                                     for k, v in done_at.items()},
                     copy_gbs_per_worker={k: gbs(v) for k, v in done_at.items()})
        lib.spg_ctiles_free(h.h, C.byref(c))
        lib.spg_tiles_free(h.h, C.byref(ta))
        lib.spg_tiles_free(h.h, C.byref(tb))
        return nbytes[0]

    try:
        one()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        steps = max(1, args.e2e_steps)
        d2h = 0
        for _ in range(steps):
            d2h = one()
        torch.cuda.synchronize()
        dt = (time.perf_counter() - t0) / steps
        return {"value": flops / dt / 1e9, "unit": "GFLOP/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "ms_per_step": dt * 1e3, "steps": steps,
                "last_step": {k: (round(v, 1) if isinstance(v, float) else v) for k, v in tstat.items()},
                "path": "spg_tile_from_csr_host (A, and B unless B is A; B tiled from A's device row view when B is A) + spg_symbolic_tiles + spg_symbolic_masks + spg_numeric_bands "
                        "(%d tile-row bands, %s band first); C's result (tile_ptrC, tile_rowidxC, tile_colidxC, tile_nnzC, "
                        "tile_colC, tile_valC, as the reference reads it back) to pinned host staging by "
                        "spg_ctiles_to_host_range on %d copy handles/streams as each part becomes final "
                        "(%d tiles per range)" % (NB, args.e2e_band_order, NW, CT)}
    except Exception as e:  # report instead of dying
        return {"value": None, "unit": "GFLOP/s", "error": str(e)[:200], "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": None}
    finally:
        for wk in workers:
            wk.h.close()


def run_batch(args):
    """512 independent C = A*B (n log-uniform in [1024, 65536], Erdos-Renyi,
    average degree U[4, 32], FP32 U[-1,1]): one plain launch sequence per
    product vs the batched path (tuned bins, one launch per phase per bin) vs
    CUDA-graph replays of the numeric phase for new values."""
    import torch
    from gpu_spgemm_gb300 import api
    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    count = args.batch_count
    pairs = synth.er_batch(count)
    stream = torch.cuda.Stream()
    h = api.Handle(local, stream)
    flops = 2.0 * sum(synth.products(a, b) for a, b in pairs)

    def timed(fn, steps):
        for _ in range(args.warmup):
            fn()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True); e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / steps

    # (1) one launch sequence per product, plain kernels
    tiles = [(api.csr2tile(h, a), api.build_csc_tiles(h, b)) for a, b in pairs]

    def per_product():
        for A, B in tiles:
            api.spgemm(h, A, B, algo="plain").free()
    ms_plain = timed(per_product, max(1, args.steps // 2))
    del tiles
    # (2) batched, autotuned bins; each bin is one block-diagonal product of
    # far more than 65,536 A tiles, so the learned step 1 is attached as for a
    # single large product (one bitmap pass instead of two)
    sizing = None
    if args.sizing and os.path.exists(api.SIZING_MODEL_PATH):
        sizing = api.SizingModel.load(h)
        sizing.attach(args.sizing_margin)
    bt = api.Batch(h, pairs)
    thr, algos = bt.tune()
    clocks = ClockSampler(local)
    clocks.start()
    l0 = h.launches()
    ms_batch = timed(lambda: bt.spgemm(), args.steps)
    launches = (h.launches() - l0) * args.steps // (args.steps + args.warmup)
    clk = clocks.stop()
    ms_batch_nosz = None
    if sizing is not None and not args.no_compare:
        sizing.detach()
        ms_batch_nosz = timed(lambda: bt.spgemm(), args.steps)
        sizing.attach(args.sizing_margin)
    # (3) numeric-only graph replay with new values (same structure)
    nz = bt.bins()
    outs = [torch.empty(max(1, int(z)), dtype=torch.float32).pin_memory().numpy() for z in nz]
    rng = np.random.default_rng(1)
    new_a = [torch.from_numpy(rng.random(a.nnz, dtype=np.float32)).pin_memory().numpy() for a, b in pairs]
    new_b = [torch.from_numpy(rng.random(b.nnz, dtype=np.float32)).pin_memory().numpy() for a, b in pairs]
    bt.graph_capture(new_a, new_b, outs)
    ms_graph = timed(bt.graph_launch, args.steps)
    h2d = sum(x.nbytes for x in new_a + new_b)
    d2h = sum(int(z) * 4 for z in nz)
    ms_batch, value = job_time_and_value(ms_batch, flops, world, "cuda")
    line = {"metric": "SpGEMM GFLOP/s", "value": value, "unit": "GFLOP/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_batch, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "float32", "data": "synthetic",
            "config": {"workload": f"batch of {count} C=A*B, n log-uniform [1024,65536], Erdos-Renyi deg U[4,32], "
                                   "FP32 U[-1,1]", "products": flops / 2},
            "details": {"tuned_thresholds": thr, "tuned_algos": algos,
                        "graph_numeric_ms": ms_graph, "graph_numeric_gflops": flops / (ms_graph * 1e-3) / 1e9,
                        "learned_sizing": "attached (margin %g)" % args.sizing_margin if sizing is not None
                        else "not attached",
                        "gflops_without_sizing_model": (flops / (ms_batch_nosz * 1e-3) / 1e9
                                                        if ms_batch_nosz else None)},
            "vs_plain": {"plain": {"ms_step": ms_plain, "gflops": flops / (ms_plain * 1e-3) / 1e9,
                                   "what": "one plain launch sequence per product"},
                         "speedup_vs_plain": ms_plain / ms_batch},
            "e2e": {"value": flops / (ms_graph * 1e-3) / 1e9, "unit": "GFLOP/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "path": "CUDA graph: new values host->device, numeric, C values "
                                                       "device->host (structure fixed)"},
            "clocks": clk, "gpu_launches": launches}
    if rank == 0:
        print(json.dumps(line), flush=True)
    bt.free()
    if sizing is not None:
        sizing.detach()
        sizing.free()
    h.close()


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--workload", default="rmat20")
    p.add_argument("--algo", default="auto", choices=["auto", "plain", "rowwise", "binned"])
    p.add_argument("--prec", default="f32", choices=["f32", "mixed", "f64"])
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--no-check", action="store_true", help="skip the FP64-oracle check of C (on by default)")
    p.add_argument("--no-compare", action="store_true",
                   help="skip timing the plain kernels and the path without the sizing model (on by default)")
    p.add_argument("--plain-steps", type=int, default=1, help="timed steps of the plain-kernel comparison")
    p.add_argument("--e2e-steps", type=int, default=2)
    p.add_argument("--e2e-bands", type=int, default=8,
                   help="tile-row bands of the e2e numeric phase (a band's values copy once it is complete)")
    p.add_argument("--e2e-mode", default="auto", choices=["auto", "stream", "whole"],
                   help="e2e copy-out: C streamed out band by band while the numeric phase runs, or copied whole "
                        "after the product (auto: by C's tile count)")
    p.add_argument("--e2e-range-tiles", type=int, default=1 << 23,
                   help="C tiles per staged e2e copy range (pinned staging per copy worker scales with it)")
    p.add_argument("--e2e-band-order", choices=["last", "first"], default="last",
                   help="e2e bands worked on from the last (light rows first, hub rows last) or the first")
    p.add_argument("--e2e-copy-workers", type=int, default=2,
                   help="copy handles/streams/host threads streaming C back in the e2e measurement")
    p.add_argument("--cpu-s", type=float, default=12.0)
    p.add_argument("--ref-step-s", type=float, default=8.0)
    p.add_argument("--batch-count", type=int, default=512)
    p.add_argument("--sizing", type=int, default=1, help="attach the trained sizing MLP (1) or not (0)")
    p.add_argument("--sizing-margin", type=float, default=1.0,
                   help="slot of a tile-row = predicted tiles * (1 + margin) + 2")
    p.add_argument("--dense-thr", type=int, default=32,
                   help="--prec mixed: tile pairs with both tiles >= this many nonzeros go to tensor cores")
    p.add_argument("--traffic", type=float, default=None,
                   help="dram bytes per launch of the dominant kernel from an ncu capture")
    args = p.parse_args()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "erbatch":
        run_batch(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
