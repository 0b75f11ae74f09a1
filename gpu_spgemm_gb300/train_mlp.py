"""Train the sizing MLP on the GPU with the library's own kernels.

Training data: per C tile-row features and exact targets (C tiles, C nonzeros
from the exact bitmap symbolic phase) of 200 generated products -- stencils
(2-D / 3-D Poisson, 27-point x 3 dof), R-MAT graphs of scales 8-15 with varied
skew and edge factors, Erdos-Renyi pairs and smoothed-aggregation A*P products.
All matrices are seeded; the list is `training_set()`.

    python -m gpu_spgemm_gb300.train_mlp [OUT.npz]
"""
from __future__ import annotations

import sys
import time

import numpy as np

from . import api, synth


def training_set(seed: int = 2024):
    rng = np.random.Generator(np.random.PCG64(seed))
    items = []
    for g in np.linspace(16, 200, 20).astype(int):
        items.append(("poisson2d", lambda g=g: (synth.poisson2d(int(g), np.float32),) * 2))
    for g in np.linspace(8, 48, 15).astype(int):
        items.append(("poisson3d", lambda g=g: (synth.poisson3d(int(g)),) * 2))
    for g in np.linspace(4, 20, 15).astype(int):
        items.append(("stencil27", lambda g=g: (synth.stencil27_dof3(int(g)),) * 2))
    for k in range(100):
        scale = int(rng.integers(8, 16))
        ef = int(rng.integers(4, 33))
        a_ = float(rng.uniform(0.45, 0.65))
        b_ = float(rng.uniform(0.1, (1 - a_) / 2))
        s = int(rng.integers(1, 1 << 30))
        items.append(("rmat", lambda scale=scale, ef=ef, a_=a_, b_=b_, s=s:
                      (synth.rmat(scale, ef, (a_, b_, b_, 1 - a_ - 2 * b_), seed=s),) * 2))
    for k in range(30):
        n = int(np.exp(rng.uniform(np.log(1024), np.log(65536))))
        s = int(rng.integers(1, 1 << 30))
        items.append(("er", lambda n=n, s=s: tuple(synth.erdos_renyi(n, float(np.random.default_rng(s + i).uniform(4, 32)),
                                                                     np.random.default_rng(s + i)) for i in (0, 1))))
    for g in np.linspace(8, 40, 20).astype(int):
        def ap(g=int(g) // 2 * 2):
            a = synth.poisson3d(g)
            p = synth.smoothed_aggregation(a, synth.aggregation_p0(g))
            return a, p
        items.append(("galerkin_AP", ap))
    return items


def collect(handle, items, log=print):
    import torch
    model = api.SizingModel(handle)
    feats, targs = [], []
    for i, (name, make) in enumerate(items):
        a, b = make()
        A = api.csr2tile(handle, a)
        B = api.build_csc_tiles(handle, b)
        Cm = api.symbolic(handle, A, B)
        feats.append(model.features(A, B).clone())
        targs.append(api.sizing_targets(Cm))
        Cm.free(); A.free(); B.free()
        if log and i % 20 == 0:
            log(f"  [{i}/{len(items)}] {name} m={a.m} rows so far={sum(f.shape[0] for f in feats)}")
    model.free()
    return torch.cat(feats), torch.cat(targs)


def normalisation(feat, targ):
    f = feat.cpu().numpy().astype(np.float64)
    t = targ.cpu().numpy().astype(np.float64)
    fm, fs = f.mean(0), f.std(0)
    tm, ts = t.mean(0), t.std(0)
    fs[fs < 1e-6] = 1.0
    ts[ts < 1e-6] = 1.0
    return np.concatenate([fm, 1.0 / fs, tm, ts]).astype(np.float32)


def train(out_path: str = api.SIZING_MODEL_PATH, epochs: int = 40, seed: int = 2024, log=print):
    import torch
    with api.Handle(0) as h:
        t0 = time.time()
        items = training_set(seed)
        feat, targ = collect(h, items, log)
        norm = normalisation(feat, targ)
        model = api.SizingModel(h, norm=norm)
        loss = model.train(feat, targ, epochs=epochs, batch=8192, lr=3e-3, seed=seed)
        # accuracy: predicted / actual tile totals per matrix family
        pred = model.predict(feat).cpu().numpy()
        act = targ.cpu().numpy()
        ratio_t = float(np.expm1(pred[:, 0]).sum() / np.expm1(act[:, 0]).sum())
        ratio_z = float(np.expm1(pred[:, 1]).sum() / np.expm1(act[:, 1]).sum())
        model.save(out_path, matrices=len(items), samples=feat.shape[0], final_loss=loss, epochs=epochs, seed=seed,
                   ratio_tiles=ratio_t, ratio_nnz=ratio_z, seconds=time.time() - t0)
        log(f"trained on {len(items)} matrices / {feat.shape[0]} tile-rows, loss {loss:.4f}, "
            f"sum(pred)/sum(actual) tiles {ratio_t:.3f} nnz {ratio_z:.3f}, {time.time() - t0:.1f} s")
        model.free()


if __name__ == "__main__":
    train(sys.argv[1] if len(sys.argv) > 1 else api.SIZING_MODEL_PATH)
