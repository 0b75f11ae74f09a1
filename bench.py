"""Benchmark: tiled SpGEMM GFLOP/s and HBM-roofline fraction on one GB300.

Default workload: C = A*A, A = R-MAT scale 20 (n = 2^20, 16 edges per vertex
before merging, (a,b,c,d) = (.57,.19,.19,.05), duplicates merged), FP32 values
U[-1,1] -- the configuration the metric is quoted on.  A "step" is one full
SpGEMM (C tile structure + bitmask symbolic + numeric, with every allocation
of C) on tiles already resident in HBM; GFLOP/s = 2 * products / step time,
products = sum over A's nonzeros of nnz(B row) (src/spgemm_raw_v2.cu:95-99,250).

Printed JSON (rank 0, one line) carries:
  value      GFLOP/s of the device-resident steps (max over ranks of the time)
  e2e        the same metric through the public C ABI with host buffers: each
             step copies the CSR inputs host->device, tiles them, multiplies and
             copies every array of C back to pinned host memory
  roofline   the dominant kernel's algorithmic bytes / its CUDA-event time
  cpu_baseline  OpenMP Gustavson (the CPU oracle's port of the reference's
             check, src/spgemm_raw_v2.cu:289-338) on a seeded row sample

`--impl reference` times the reference's CPU implementation of the path (that
Gustavson port) on all host threads for the same workload and metric.
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

# DRAM bytes per launch of the dominant kernel, from one-pass ncu captures of
# the same bench command (dram__bytes_read.sum + dram__bytes_write.sum), by
# (workload, step); profiles/traffic_rmat20.md holds the capture.
MEASURED_TRAFFIC = {("rmat20", "step3"): 279.02e9 + 65.14e9}


def workload(name: str):
    if name == "rmat20":
        a = synth.rmat(20, 16)
        return a, a, {"workload": "C=A*A, A=R-MAT scale 20, edge factor 16, (a,b,c,d)=(.57,.19,.19,.05), "
                                  "duplicates merged, FP32 U[-1,1]", "n": a.m, "nnz": a.nnz}
    if name == "poisson2d":
        a = synth.poisson2d(256)
        return a, a, {"workload": "C=A*A, A=2-D 5-point Poisson 256x256, FP64", "n": a.m, "nnz": a.nnz}
    if name == "stencil27":
        a = synth.stencil27_dof3(64)
        return a, a, {"workload": "C=A*A, A=27-point stencil 64^3 x 3 dof, FP32 N(0,1)", "n": a.m, "nnz": a.nnz}
    if name.startswith("rmat"):
        s = int(name[4:])
        a = synth.rmat(s, 16)
        return a, a, {"workload": f"C=A*A, A=R-MAT scale {s}, edge factor 16, FP32", "n": a.m, "nnz": a.nnz}
    raise SystemExit(f"unknown workload {name}")


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


def cpu_gflops(a, b, target_s: float = 12.0, dtype=np.float32):
    """OpenMP Gustavson on a seeded stride sample of A's rows, sized to about
    target_s seconds; returns (GFLOP/s, threads, sample description)."""
    import oracle
    threads = oracle.max_threads()
    rng = np.random.Generator(np.random.PCG64(0xC0FFEE))

    def sample(frac):
        k = max(1, int(round(1.0 / frac)))
        off = int(rng.integers(0, k))
        rows = np.arange(off, a.m, k, dtype=np.int64)
        lens = np.diff(a.row_ptr)[rows]
        rp = np.zeros(rows.size + 1, np.int64)
        np.cumsum(lens, out=rp[1:])
        idx = np.concatenate([np.arange(a.row_ptr[r], a.row_ptr[r + 1]) for r in rows]) if rows.size else \
            np.zeros(0, np.int64)
        s = synth.CSR(rows.size, a.n, rp.astype(np.int32), a.col_idx[idx], a.val[idx].astype(dtype))
        return s, k

    frac = 0.01
    s, k = sample(frac)
    p = synth.products(s, b)
    t0 = time.perf_counter()
    oracle.gustavson_rows(s, b, 0, s.m, dtype)
    dt = max(time.perf_counter() - t0, 1e-4)
    frac = min(1.0, frac * target_s / dt)
    s, k = sample(frac)
    p = synth.products(s, b)
    t0 = time.perf_counter()
    oracle.gustavson_rows(s, b, 0, s.m, dtype)
    dt = time.perf_counter() - t0
    return 2.0 * p / dt / 1e9, threads, f"every {k}-th row of A ({s.m} rows, {p} products), {dt:.1f} s"


def run_reference(args):
    world, rank, _ = dist_setup()
    if rank != 0:
        return
    a, b, cfg = workload(args.workload)
    import oracle
    dtype = np.float64 if a.val.dtype == np.float64 else np.float32
    vals = []
    desc = ""
    threads = oracle.max_threads()
    for i in range(args.warmup + args.steps):
        g, threads, desc = cpu_gflops(a, b, target_s=args.ref_step_s, dtype=dtype)
        if i >= args.warmup:
            vals.append(g)
    v = statistics.mean(vals)
    line = {"impl": "reference", "metric": "SpGEMM GFLOP/s", "value": v, "unit": "GFLOP/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "dtype": np.dtype(dtype).name,
            "data": "synthetic", "config": cfg, "vs_baseline": None,
            "cpu_baseline": {"value": v, "unit": "GFLOP/s", "cores": threads, "kind": "port",
                             "sample": "OpenMP row-parallel Gustavson (CPU oracle's restatement of "
                                       "src/spgemm_raw_v2.cu:289-338), " + desc},
            "e2e": {"value": v, "unit": "GFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args):
    import torch
    import torch.distributed as dist
    world, rank, local = dist_setup()
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl")
    from gpu_spgemm_gb300 import api
    a, b, cfg = workload(args.workload)
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
    if args.sizing and os.path.exists(api.SIZING_MODEL_PATH):
        sizing = api.SizingModel.load(h)
        sizing.attach(args.sizing_margin)

    def step():
        C = api.spgemm(h, A, B, algo=args.algo, prec=args.prec)
        st = h.stats()
        info = (C.numtileC, C.nnzC, C.pairs)
        C.free()
        return st, info

    for _ in range(args.warmup):
        step()
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    stats = []
    info = None
    for _ in range(args.steps):
        st, info = step()
        stats.append(st)
    ev1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms, value = job_time_and_value(ev0.elapsed_time(ev1) / args.steps, flops, world, "cuda")
    numtileC, nnzC, pairs = info

    # ---- roofline of the dominant kernel (CUDA events around it inside the library)
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
    s1 = statistics.mean(s["ms_step1"] for s in stats)
    s2 = statistics.mean(s["ms_step2"] for s in stats)
    s3 = statistics.mean(s["ms_step3"] for s in stats)
    a_b = tile_bytes(A.numtile, A.nnz, A.tilem, v)
    b_b = tile_bytes(B.numtile, B.nnz, B.tilem, v, b_side=True)
    c_b = c_bytes(numtileC, nnzC, A.tilem, v)
    # numeric kernel: reads A and B tiles and C's structure, writes C's values and column bytes
    num_bytes = (a_b + b_b + 4 * (A.tilem + 1) + numtileC * (4 + 4 + 8 + 32 + 16) + nnzC * (v + 1))
    sym_bytes = (4 * (A.tilem + 1) + A.numtile * (4 + 4 + 16) + A.nnz + B.numtile * (4 + 32) + 4 * (B.tilen + 1)
                 + numtileC * (4 + 4 + 32 + 16 + 4))
    steps_ms = {"step1": s1, "step2": s2, "step3": s3}
    dom = max(steps_ms, key=steps_ms.get)
    dom_bytes = {"step1": 4 * (A.tilem + 1) * 2 + 4 * A.numtile + 4 * B.numtile + 8 * numtileC,
                 "step2": sym_bytes, "step3": num_bytes}[dom]
    achieved = dom_bytes / (steps_ms[dom] * 1e-3) / 1e9
    rowwise = stats[-1].get("algo_used", 1) == 2
    names = {"step1": "c1_slot_kernel + c1_compact_kernel" if args.sizing else "c1_count_kernel + c1_fill_kernel",
             "step2": "rw_symbolic_kernel" if rowwise else "c2_symbolic_kernel",
             "step3": "rw_numeric_kernel" if rowwise else "c3_numeric_kernel"}
    roofline = {"bound": "hbm", "kernel": names[dom],
                "achieved": achieved, "peak": hbm_peak, "unit": "GB/s", "frac": achieved / hbm_peak,
                "peak_source": peak_src, "algorithmic_bytes": dom_bytes, "ms": steps_ms[dom],
                "traffic": args.traffic if args.traffic is not None else MEASURED_TRAFFIC.get((args.workload, dom))}
    total_bytes = a_b + b_b + c_b
    hbm_steps = total_bytes / (ms * 1e-3) / 1e9

    accuracy = value_check(h, api, a, b, args) if args.check else None

    # ---- end to end through the public API with host buffers
    e2e = None
    if not args.no_e2e:
        e2e = measure_e2e(h, api, a, b, args, flops, stream)

    # ---- CPU baseline (rank 0 only)
    cpu = None
    if rank == 0 and not args.no_cpu:
        g, thr, desc = cpu_gflops(a, b, target_s=args.cpu_s, dtype=np.float64 if v == 8 else np.float32)
        cpu = {"value": g, "unit": "GFLOP/s", "cores": thr, "kind": "port",
               "sample": "OpenMP row-parallel Gustavson (CPU oracle's restatement of "
                         "src/spgemm_raw_v2.cu:289-338), " + desc}

    if rank == 0:
        cfg = dict(cfg)
        cfg.update({"products": products, "numtileC": numtileC, "nnzC": nnzC, "tile_pairs": pairs,
                    "algo": args.algo, "prec": args.prec,
                    "l2": "inputs and outputs exceed L2 (A,B tiles %.2f GB, C %.1f GB > 129 MB)" %
                          ((a_b + b_b) / 1e9, c_b / 1e9),
                    "ms_step1": s1, "ms_step2": s2, "ms_step3": s3,
                    "hbm_gbs_steps": hbm_steps, "hbm_frac_steps": hbm_steps / hbm_peak,
                    "tensor_pairs": stats[-1].get("tensor_pairs", 0), "fp64_tiles": stats[-1].get("fp64_tiles", 0),
                    "learned_sizing": None if sizing is None else {
                        "model": os.path.relpath(api.SIZING_MODEL_PATH, ROOT), "margin": args.sizing_margin,
                        "predicted_tiles": stats[-1].get("predicted_tiles", 0), "actual_tiles": numtileC,
                        "overflow_reruns": stats[-1].get("overflow_reruns", 0),
                        "step1": "one bitmap pass into predicted per-row slots, then compaction; "
                                 "rows that outgrow their slot re-run the exact fill"},
                    "accuracy": accuracy})
        line = {"metric": "SpGEMM GFLOP/s", "value": value, "unit": "GFLOP/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": np.dtype(dtype).name, "data": "synthetic",
                "config": cfg, "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "clocks": clk,
                "gpu_launches": gpu_launches(args.algo) * args.steps}
        print(json.dumps(line), flush=True)
    h.close()
    if world > 1:
        dist.destroy_process_group()


def value_check(h, api, a, b, args, tile_rows=512):
    """Relative Frobenius error of C's values against the FP64 oracle on the
    first `tile_rows` C tile-rows (each C tile-row depends only on the same
    16 rows of A, so the oracle multiplies that row block of A by B)."""
    import ctypes as C
    import oracle
    from gpu_spgemm_gb300 import _lib as L
    rows = min(a.m, 16 * tile_rows)
    asub = synth.CSR(rows, a.n, a.row_ptr[:rows + 1].copy(), a.col_idx[:a.row_ptr[rows]].copy(),
                     a.val[:a.row_ptr[rows]].copy())
    S = oracle.spgemm_tiles(asub, b)
    A = api.csr2tile(h, a)
    B = api.build_csc_tiles(h, b)
    Cm = api.spgemm(h, A, B, algo=args.algo, prec=args.prec)
    nt = int(S["numtileC"])
    nv = int(S["nnzC"])
    vd = np.float64 if a.val.dtype == np.float64 else np.float32
    vals = np.zeros(max(nv, 1), vd)
    cols = np.zeros(max(nv, 1), np.uint8)
    got = C.c_int64()
    h.check(h.lib.spg_ctiles_to_host_range(h.h, C.byref(Cm.c), 0, nt, None, None, None, None, None,
                                           vals.ctypes.data, cols.ctypes.data, max(nv, 1), C.byref(got)))
    st = h.stats()
    Cm.free(); A.free(); B.free()
    ref = S["tile_valC"]
    err = float(np.linalg.norm(vals[:nv].astype(np.float64) - ref) / (np.linalg.norm(ref) or 1.0))
    return {"tile_rows_checked": int(rows // 16), "c_values_checked": nv, "rel_frob_vs_fp64": err,
            "cols_equal": bool(np.array_equal(cols[:nv], S["tile_colC"])), "tensor_pairs": st["tensor_pairs"],
            "fp64_tiles": st["fp64_tiles"]}


def gpu_launches(algo):
    # plain path per step: step1 count + scan + i64->i32 + fill, step2 symbolic + scan, step3 numeric
    return 7


def measure_e2e(h, api, a, b, args, flops, stream):
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
    hb = [pin(b.row_ptr), pin(b.col_idx), pin(b.val)]
    code = L.SPG_F64 if a.val.dtype == np.float64 else L.SPG_F32
    vd = np.float64 if code == L.SPG_F64 else np.float32
    vsz = np.dtype(vd).itemsize
    h2d = sum(x[1].nbytes for x in ha + hb)
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
        ta, tb, c = L.SpgTiles(), L.SpgTiles(), L.SpgCTiles()
        h.check(lib.spg_tile_from_csr_host(h.h, a.m, a.n, a.nnz, ha[0][1].ctypes.data, ha[1][1].ctypes.data,
                                           ha[2][1].ctypes.data, code, L.SPG_LAYOUT_ROW, 0, C.byref(ta)))
        h.check(lib.spg_tile_from_csr_host(h.h, b.m, b.n, b.nnz, hb[0][1].ctypes.data, hb[1][1].ctypes.data,
                                           hb[2][1].ctypes.data, code, L.SPG_LAYOUT_B_CSC, 0, C.byref(tb)))
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
                "path": "spg_tile_from_csr_host x2 + spg_symbolic_tiles + spg_symbolic_masks + spg_numeric_bands "
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
    # (2) batched, autotuned bins
    bt = api.Batch(h, pairs)
    thr, algos = bt.tune()
    clocks = ClockSampler(local)
    clocks.start()
    ms_batch = timed(lambda: bt.spgemm(), args.steps)
    clk = clocks.stop()
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
                                   "FP32 U[-1,1]", "products": flops / 2, "tuned_thresholds": thr,
                       "tuned_algos": algos, "plain_launches_ms": ms_plain,
                       "plain_launches_gflops": flops / (ms_plain * 1e-3) / 1e9,
                       "graph_numeric_ms": ms_graph, "graph_numeric_gflops": flops / (ms_graph * 1e-3) / 1e9,
                       "speedup_batched_vs_plain_launches": ms_plain / ms_batch},
            "e2e": {"value": flops / (ms_graph * 1e-3) / 1e9, "unit": "GFLOP/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "path": "CUDA graph: new values host->device, numeric, C values "
                                                       "device->host (structure fixed)"},
            "clocks": clk}
    if rank == 0:
        print(json.dumps(line), flush=True)
    bt.free()
    h.close()


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--workload", default="rmat20")
    p.add_argument("--algo", default="auto", choices=["auto", "plain", "rowwise"])
    p.add_argument("--prec", default="f32", choices=["f32", "mixed", "f64"])
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--e2e-steps", type=int, default=2)
    p.add_argument("--e2e-bands", type=int, default=8,
                   help="tile-row bands of the e2e numeric phase (a band's values copy once it is complete)")
    p.add_argument("--e2e-range-tiles", type=int, default=1 << 23,
                   help="C tiles per staged e2e copy range (pinned staging per copy worker scales with it)")
    p.add_argument("--e2e-band-order", choices=["last", "first"], default="last",
                   help="e2e bands worked on from the last (light rows first, hub rows last) or the first")
    p.add_argument("--e2e-copy-workers", type=int, default=2,
                   help="copy handles/streams/host threads streaming C back in the e2e measurement")
    p.add_argument("--cpu-s", type=float, default=12.0)
    p.add_argument("--ref-step-s", type=float, default=8.0)
    p.add_argument("--batch-count", type=int, default=512)
    p.add_argument("--check", action="store_true", help="value error vs the FP64 oracle on a prefix of C")
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
