"""Batched products: one launch per phase per bin (block-diagonal assembly),
per-problem results bit-exact in structure against the oracle; numeric-only
re-runs and CUDA-graph replays for new values; the autotuner's choice gives
the same results."""
import numpy as np
import pytest
import torch

import oracle
from gpu_spgemm_gb300 import api, synth
import cases

pytestmark = pytest.mark.gpu
KEYS = ["tile_ptrC", "tile_rowidxC", "tile_colidxC", "maskC", "tile_nnzC", "ptrRowC", "tile_colC"]


def rel(x, y):
    x = np.asarray(x, np.float64); y = np.asarray(y, np.float64)
    return np.linalg.norm(x - y) / (np.linalg.norm(y) or 1.0)


def small_batch(count=24, seed=5):
    rng = np.random.Generator(np.random.PCG64(seed))
    pairs = []
    for i in range(count):
        n = int(rng.integers(20, 900))
        a = synth.erdos_renyi(n, rng.uniform(2, 12), rng)
        b = synth.erdos_renyi(n, rng.uniform(2, 12), rng)
        pairs.append((a, b))
    # rectangular and empty members
    pairs.append((cases.random_csr(37, 53, 0.1, 7, np.float32), cases.random_csr(53, 29, 0.1, 8, np.float32)))
    pairs.append((cases.empty_csr(16, 16, np.float32), cases.empty_csr(16, 16, np.float32)))
    return pairs


def check_batch(bt, pairs, tol=1e-6):
    for p, (a, b) in enumerate(pairs):
        got = bt.result(p)
        S = oracle.spgemm_tiles(a, b)
        assert got["numtileC"] == S["numtileC"] and got["nnzC"] == S["nnzC"], p
        for k in KEYS:
            np.testing.assert_array_equal(got[k], S[k].astype(got[k].dtype), err_msg=f"{p}:{k}")
        assert rel(got["tile_valC"], S["tile_valC"]) <= tol, p


@pytest.mark.parametrize("algo", ["plain", "rowwise"])
def test_batch_matches_oracle(handle, algo):
    pairs = small_batch()
    bt = api.Batch(handle, pairs)
    bt.spgemm(algo=algo)
    check_batch(bt, pairs)
    assert bt.products() == sum(synth.products(a, b) for a, b in pairs)


def test_batch_bins_and_tuner(handle):
    pairs = small_batch(30, seed=9)
    bt = api.Batch(handle, pairs)
    thr, algos = bt.tune()
    assert len(algos) == len(thr) + 1
    bt.spgemm()
    check_batch(bt, pairs)
    bt.set_bins([200, 500], ["rowwise", "plain", "rowwise"])
    bt.spgemm()
    check_batch(bt, pairs)


def test_batch_numeric_rerun_and_graph(handle):
    stream = torch.cuda.Stream()
    handle.set_stream(stream)
    try:
        pairs = small_batch(12, seed=11)
        bt = api.Batch(handle, pairs)
        bt.spgemm(algo="rowwise")
        rng = np.random.default_rng(3)
        new_a = [rng.standard_normal(a.nnz).astype(np.float32) for a, b in pairs]
        new_b = [rng.standard_normal(b.nnz).astype(np.float32) for a, b in pairs]
        pairs2 = [(synth.CSR(a.m, a.n, a.row_ptr, a.col_idx, va), synth.CSR(b.m, b.n, b.row_ptr, b.col_idx, vb))
                  for (a, b), va, vb in zip(pairs, new_a, new_b)]
        # numeric-only re-run with new values
        bt.set_values(new_a, new_b)
        bt.numeric()
        torch.cuda.synchronize()
        check_batch(bt, pairs2)
        # graph: values H2D + numeric + C values D2H, replayed
        nz = bt.bins()
        outs = [torch.empty(max(1, int(z)), dtype=torch.float32).pin_memory().numpy() for z in nz]
        bt.graph_capture(new_a, new_b, outs)
        bt.graph_launch()
        torch.cuda.synchronize()
        ref = np.concatenate([oracle.spgemm_tiles(a, b)["tile_valC"] for a, b in pairs2])
        got = np.concatenate([o[:int(z)] for o, z in zip(outs, nz)])
        assert got.size == ref.size and rel(got, ref) <= 1e-6
        bt.graph_launch()
        torch.cuda.synchronize()
        got2 = np.concatenate([o[:int(z)] for o, z in zip(outs, nz)])
        assert rel(got2, ref) <= 1e-6
    finally:
        handle.set_stream(None)
