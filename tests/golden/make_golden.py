"""Writes tests/golden/tiles_<case>.npz: the reference project's own tiler
(csr2tile and build_csc_tiles, src/tile_format.h:93,424, compiled from its
source by oracle/build_ref.sh) run on every case of tests/cases.py; and
tests/golden/mtx_<name>.npz: its Matrix Market reader (load_mtx,
src/tile_format.h:51-90) on every file under tests/golden/mtx/.

Run from the repository root:  python tests/golden/make_golden.py
The fixtures pin the CPU oracle and the CUDA tiler where the reference
checkout is absent (the GPU host)."""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

from oracle import ref  # noqa: E402
import cases  # noqa: E402


def write_mtx_fixtures(out_dir):
    """mtx_<name>.npz: the reference's own load_mtx (src/tile_format.h:51-90)
    on each tests/golden/mtx/<name>.mtx (duplicates kept, as it keeps them)."""
    import glob
    for path in sorted(glob.glob(os.path.join(out_dir, "mtx", "*.mtx"))):
        m, n, rp, ci, val = ref.ref_load_mtx(path)
        name = os.path.basename(path)[:-4]
        np.savez_compressed(os.path.join(out_dir, f"mtx_{name}.npz"), m=np.int64(m), n=np.int64(n), row_ptr=rp,
                            col_idx=ci, val=val)
        print("mtx", name, m, n, int(rp[-1]))


def main():
    if not ref.available():
        raise SystemExit("reference tiler unavailable (oracle/build_ref.sh needs the reference checkout)")
    out_dir = os.path.dirname(os.path.abspath(__file__))
    write_mtx_fixtures(out_dir)
    for name, csr in cases.tiler_cases():
        arrays = {"in_m": np.int64(csr.m), "in_n": np.int64(csr.n), "in_row_ptr": csr.row_ptr,
                  "in_col_idx": csr.col_idx, "in_val": csr.val.astype(np.float64)}
        for k, v in ref.ref_tiles(csr, csc=False).items():
            arrays["A_" + k] = v
        for k, v in ref.ref_tiles(csr, csc=True).items():
            arrays["B_" + k] = v
        np.savez_compressed(os.path.join(out_dir, f"tiles_{name}.npz"), **arrays)
        print(name, csr.m, csr.n, csr.nnz)


if __name__ == "__main__":
    main()
