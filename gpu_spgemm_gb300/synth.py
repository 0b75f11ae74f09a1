"""Seeded synthetic sparse matrices for the tiled SpGEMM workloads.

Every generator returns a :class:`CSR` with int32 ``row_ptr`` / ``col_idx``
(columns strictly ascending inside each row, duplicates merged) and values in
the requested float type.  numpy's PCG64 generator is platform independent, so
the same seed gives the same matrix on x86 and Arm hosts.

The five workloads mirror the matrices the tiled SpGEMM is measured on:

* ``poisson2d(256)``      2-D 5-point Laplacian, diag 4 / off-diag -1, FP64
* ``rmat(20, 16)``         R-MAT power-law graph, (a,b,c,d)=(.57,.19,.19,.05),
                           self-loops kept, duplicates merged, FP32 U[-1,1]
* ``stencil27_dof3(64)``  27-point stencil on 64^3 nodes x dense 3x3 dof blocks,
                           FP32 N(0,1)
* ``er_batch(512)``       pairs of Erdos-Renyi matrices, n log-uniform in
                           [1024, 65536], average degree U[4, 32], FP32 U[-1,1]
* ``poisson3d(128)`` + ``smoothed_aggregation(...)``  7-point 3-D Laplacian and
                           its 2x2x2 smoothed-aggregation prolongator
                           P = (I - 2/3 D^-1 A) P0 for the Galerkin product P^T (A P)

The reference loads Matrix Market files instead (src/tile_format.h:51-90);
:func:`load_mtx` keeps that path for external matrices and additionally merges
duplicate entries.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

SEED = 0x5EED


@dataclasses.dataclass
class CSR:
    m: int
    n: int
    row_ptr: np.ndarray  # int32 [m+1]
    col_idx: np.ndarray  # int32 [nnz]
    val: np.ndarray      # float32 / float64 [nnz]

    @property
    def nnz(self) -> int:
        return int(self.row_ptr[-1])

    def astype(self, dtype) -> "CSR":
        return CSR(self.m, self.n, self.row_ptr, self.col_idx, self.val.astype(dtype))

    def to_scipy(self):
        import scipy.sparse as sp
        return sp.csr_matrix((self.val, self.col_idx, self.row_ptr), shape=(self.m, self.n))

    @staticmethod
    def from_scipy(a, dtype=None) -> "CSR":
        a = a.tocsr()
        a.sum_duplicates()
        a.sort_indices()
        val = a.data if dtype is None else a.data.astype(dtype)
        return CSR(a.shape[0], a.shape[1], a.indptr.astype(np.int32),
                   a.indices.astype(np.int32), np.ascontiguousarray(val))


def _from_coo_sorted_unique(m: int, n: int, rows: np.ndarray, cols: np.ndarray,
                            vals: np.ndarray) -> CSR:
    """Build CSR from COO already sorted by (row, col) with no duplicates."""
    counts = np.bincount(rows, minlength=m).astype(np.int64)
    row_ptr = np.zeros(m + 1, dtype=np.int64)
    np.cumsum(counts, out=row_ptr[1:])
    if row_ptr[-1] >= 2**31:
        raise ValueError("nnz exceeds int32 CSR indexing")
    return CSR(m, n, row_ptr.astype(np.int32), cols.astype(np.int32), vals)


def _merge_keys(m: int, n: int, rows: np.ndarray, cols: np.ndarray):
    key = rows.astype(np.int64) * n + cols.astype(np.int64)
    key = np.unique(key)  # sorted, duplicates merged
    return (key // n).astype(np.int64), (key % n).astype(np.int64)


# ----------------------------------------------------------------------------
# 2-D / 3-D Poisson
# ----------------------------------------------------------------------------
def poisson2d(g: int = 256, dtype=np.float64) -> CSR:
    """5-point Laplacian on a g x g grid, natural ordering (node = x + g*y)."""
    n = g * g
    idx = np.arange(n, dtype=np.int64)
    x, y = idx % g, idx // g
    rows, cols, vals = [], [], []
    # emit per-row entries in ascending column order: -g, -1, 0, +1, +g
    for dx, dy, v in ((0, -1, -1.0), (-1, 0, -1.0), (0, 0, 4.0), (1, 0, -1.0), (0, 1, -1.0)):
        ok = (x + dx >= 0) & (x + dx < g) & (y + dy >= 0) & (y + dy < g)
        rows.append(idx[ok]); cols.append(idx[ok] + dx + g * dy)
        vals.append(np.full(int(ok.sum()), v))
    return _assemble(n, n, rows, cols, vals, dtype)


def poisson3d(g: int = 128, dtype=np.float32) -> CSR:
    """7-point Laplacian on a g^3 grid (diag 6, off-diag -1), node = x + g*(y + g*z)."""
    n = g ** 3
    idx = np.arange(n, dtype=np.int64)
    x, y, z = idx % g, (idx // g) % g, idx // (g * g)
    rows, cols, vals = [], [], []
    for dx, dy, dz, v in ((0, 0, -1, -1.0), (0, -1, 0, -1.0), (-1, 0, 0, -1.0), (0, 0, 0, 6.0),
                          (1, 0, 0, -1.0), (0, 1, 0, -1.0), (0, 0, 1, -1.0)):
        ok = ((x + dx >= 0) & (x + dx < g) & (y + dy >= 0) & (y + dy < g)
              & (z + dz >= 0) & (z + dz < g))
        rows.append(idx[ok]); cols.append(idx[ok] + dx + g * (dy + g * dz))
        vals.append(np.full(int(ok.sum()), v))
    return _assemble(n, n, rows, cols, vals, dtype)


def _assemble(m, n, rows, cols, vals, dtype) -> CSR:
    r = np.concatenate(rows); c = np.concatenate(cols); v = np.concatenate(vals)
    order = np.lexsort((c, r))
    return _from_coo_sorted_unique(m, n, r[order], c[order], v[order].astype(dtype))


# ----------------------------------------------------------------------------
# R-MAT
# ----------------------------------------------------------------------------
def rmat(scale: int = 20, edge_factor: int = 16, abcd=(0.57, 0.19, 0.19, 0.05),
         seed: int = SEED, dtype=np.float32) -> CSR:
    """R-MAT graph with 2^scale vertices and edge_factor * 2^scale edges before
    merging.  Each edge descends ``scale`` quadrant levels; self-loops are kept
    and duplicate edges merged.  Values are drawn U[-1, 1] after merging."""
    a, b, c, _ = abcd
    n = 1 << scale
    e = edge_factor * n
    rng = np.random.Generator(np.random.PCG64(seed))
    rows = np.zeros(e, dtype=np.int64)
    cols = np.zeros(e, dtype=np.int64)
    chunk = 1 << 22
    for s in range(0, e, chunk):
        t = min(e, s + chunk)
        r = np.zeros(t - s, dtype=np.int64); q = np.zeros(t - s, dtype=np.int64)
        for _lvl in range(scale):
            u = rng.random(t - s)
            rb = u >= a + b
            cb = ((u >= a) & (u < a + b)) | (u >= a + b + c)
            r = (r << 1) | rb
            q = (q << 1) | cb
        rows[s:t] = r; cols[s:t] = q
    rows, cols = _merge_keys(n, n, rows, cols)
    vals = (rng.random(rows.size) * 2.0 - 1.0).astype(dtype)
    return _from_coo_sorted_unique(n, n, rows, cols, vals)


# ----------------------------------------------------------------------------
# 27-point stencil x 3 dof
# ----------------------------------------------------------------------------
def stencil27_dof3(g: int = 64, dof: int = 3, seed: int = SEED, dtype=np.float32) -> CSR:
    """27-point stencil on a g^3 grid coupled with dense dof x dof node blocks.
    Row (node, d) = dof*node + d, node = x + g*(y + g*z).  Values N(0, 1)."""
    nn = g ** 3
    n = nn * dof
    node = np.arange(nn, dtype=np.int64)
    x, y, z = node % g, (node // g) % g, node // (g * g)
    # neighbour offsets in ascending linear order
    offs = [(dx, dy, dz) for dz in (-1, 0, 1) for dy in (-1, 0, 1) for dx in (-1, 0, 1)]
    nbr_cols = []
    nbr_ok = []
    for dx, dy, dz in offs:
        ok = ((x + dx >= 0) & (x + dx < g) & (y + dy >= 0) & (y + dy < g)
              & (z + dz >= 0) & (z + dz < g))
        nbr_ok.append(ok)
        nbr_cols.append(node + dx + g * (dy + g * dz))
    ok = np.stack(nbr_ok, axis=1)            # [nn, 27]
    nb = np.stack(nbr_cols, axis=1)          # [nn, 27], ascending per row
    deg = ok.sum(axis=1)                     # neighbours per node
    # per node-row: for each valid neighbour, dof columns
    row_len = deg * dof                      # entries per scalar row
    counts = np.repeat(row_len, dof)         # [n]
    row_ptr = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(counts, out=row_ptr[1:])
    nb_valid = nb[ok]                        # flattened valid neighbours, node-major
    seg = np.zeros(nn + 1, dtype=np.int64)
    np.cumsum(deg, out=seg[1:])
    # columns of a node's scalar rows (identical for its dof rows)
    node_cols = (nb_valid[:, None] * dof + np.arange(dof)[None, :]).reshape(-1)  # [sum deg * dof]
    # replicate node block columns dof times (one per dof row)
    starts = seg[:-1] * dof
    lens = deg * dof
    rep_start = np.repeat(starts, dof)
    rep_len = np.repeat(lens, dof)
    total = int(rep_len.sum())
    idx = np.arange(total, dtype=np.int64) - np.repeat(row_ptr[:-1], rep_len) + np.repeat(rep_start, rep_len)
    col_idx = node_cols[idx]
    rng = np.random.Generator(np.random.PCG64(seed))
    vals = rng.standard_normal(total).astype(dtype)
    if row_ptr[-1] >= 2**31:
        raise ValueError("nnz exceeds int32")
    return CSR(n, n, row_ptr.astype(np.int32), col_idx.astype(np.int32), vals)


# ----------------------------------------------------------------------------
# Erdos-Renyi batch
# ----------------------------------------------------------------------------
def erdos_renyi(n: int, avg_deg: float, rng: np.random.Generator, dtype=np.float32) -> CSR:
    """G(n, p) with p = avg_deg / n: every (i, j) present independently with
    probability p.  Drawn as a Bernoulli process over the row-major index
    i*n + j (geometric gaps, cumulative sum), so entries come out sorted and
    unique with no sort.  Values U[-1, 1]."""
    p = min(1.0, avg_deg / n)
    total = n * n
    est = int(total * p + 8 * np.sqrt(total * p) + 64)
    gaps = rng.geometric(p, size=est).astype(np.int64)
    lin = np.cumsum(gaps) - 1
    while lin[-1] < total - 1 and lin.size:  # rare: extend the process
        more = rng.geometric(p, size=max(64, est // 8)).astype(np.int64)
        lin = np.concatenate([lin, lin[-1] + np.cumsum(more)])
    lin = lin[lin < total]
    r, c = lin // n, lin % n
    vals = (rng.random(r.size) * 2.0 - 1.0).astype(dtype)
    return _from_coo_sorted_unique(n, n, r, c, vals)


def er_batch(count: int = 512, n_lo: int = 1024, n_hi: int = 65536, deg_lo: float = 4.0,
             deg_hi: float = 32.0, seed: int = SEED, dtype=np.float32):
    """``count`` independent (A, B) pairs; n = round(exp(U[ln n_lo, ln n_hi])), A and B
    drawn independently with average degree U[deg_lo, deg_hi] each."""
    rng = np.random.Generator(np.random.PCG64(seed))
    pairs = []
    for _ in range(count):
        n = int(round(math.exp(rng.uniform(math.log(n_lo), math.log(n_hi)))))
        da = rng.uniform(deg_lo, deg_hi)
        db = rng.uniform(deg_lo, deg_hi)
        pairs.append((erdos_renyi(n, da, rng, dtype), erdos_renyi(n, db, rng, dtype)))
    return pairs


# ----------------------------------------------------------------------------
# Smoothed aggregation prolongator
# ----------------------------------------------------------------------------
def aggregation_p0(g: int, agg: int = 2, dtype=np.float32) -> CSR:
    """Piecewise-constant aggregation of a g^3 grid into (g/agg)^3 aggregates of
    agg^3 nodes: one 1 per row."""
    n = g ** 3
    ga = g // agg
    idx = np.arange(n, dtype=np.int64)
    x, y, z = idx % g, (idx // g) % g, idx // (g * g)
    col = (x // agg) + ga * ((y // agg) + ga * (z // agg))
    row_ptr = np.arange(n + 1, dtype=np.int32)
    return CSR(n, ga ** 3, row_ptr, col.astype(np.int32), np.ones(n, dtype=dtype))


def smoothed_aggregation(a: CSR, p0: CSR, omega: float = 2.0 / 3.0) -> CSR:
    """P = (I - omega D^-1 A) P0, computed with scipy in float64 then cast to the
    dtype of ``a``.  Used only to build inputs."""
    import scipy.sparse as sp
    A = a.to_scipy().astype(np.float64)
    P0 = p0.to_scipy().astype(np.float64)
    dinv = 1.0 / A.diagonal()
    S = sp.identity(a.m, format="csr") - omega * sp.diags(dinv) @ A
    P = (S @ P0).tocsr()
    return CSR.from_scipy(P, dtype=a.val.dtype)


def block_diag(*blocks: CSR) -> CSR:
    """The block-diagonal matrix of the given CSR blocks (values cast to the
    first block's type): a product of it with itself is the independent
    products of its blocks side by side, each block keeping its own
    character (a stencil beside a power-law graph, for instance)."""
    dtype = blocks[0].val.dtype
    m = sum(b.m for b in blocks)
    n = sum(b.n for b in blocks)
    rps, cis, vals = [np.zeros(1, np.int64)], [], []
    r_off = c_off = nz_off = 0
    for b in blocks:
        rps.append(b.row_ptr[1:].astype(np.int64) + nz_off)
        cis.append(b.col_idx.astype(np.int64) + c_off)
        vals.append(b.val.astype(dtype))
        r_off += b.m
        c_off += b.n
        nz_off += b.nnz
    rp = np.concatenate(rps)
    if rp[-1] >= 2**31:
        raise ValueError("nnz exceeds int32 CSR indexing")
    return CSR(m, n, rp.astype(np.int32), np.concatenate(cis).astype(np.int32), np.concatenate(vals))


def transpose(a: CSR) -> CSR:
    """Host CSR transpose with stable (row-ascending) order inside each column,
    the same order the reference's ``--aat`` path builds (src/spgemm_raw_v2.cu:79-90)."""
    counts = np.bincount(a.col_idx, minlength=a.n).astype(np.int64)
    rp = np.zeros(a.n + 1, dtype=np.int64)
    np.cumsum(counts, out=rp[1:])
    rows = np.repeat(np.arange(a.m, dtype=np.int64), np.diff(a.row_ptr))
    order = np.argsort(a.col_idx, kind="stable")
    return CSR(a.n, a.m, rp.astype(np.int32), rows[order].astype(np.int32),
               np.ascontiguousarray(a.val[order]))


def products(a: CSR, b: CSR) -> int:
    """Intermediate products sum_{(i,k) in A} nnz(B(k,:)) (src/spgemm_raw_v2.cu:95-99)."""
    blen = np.diff(b.row_ptr).astype(np.int64)
    return int(blen[a.col_idx].sum())


def read_mtx_entries(path: str):
    """Matrix Market coordinate file -> (m, n, rows, cols, vals) the way the
    reference reads it (src/tile_format.h:51-90): the banner line's words
    "symmetric", "pattern" and "complex" set the mode (so a skew-symmetric
    file is mirrored like a symmetric one, with the same value), '%' lines
    are skipped, indices are 1-based, pattern entries are 1.0, complex
    entries keep their real part, and every off-diagonal entry of a
    symmetric file is mirrored.  Entries come back in file order."""
    with open(path) as f:
        banner = f.readline()
        sym, pat, cplx = "symmetric" in banner, "pattern" in banner, "complex" in banner
        line = f.readline()
        while line and line.startswith("%"):
            line = f.readline()
        m, n, nf = (int(x) for x in line.split()[:3])
        per = 2 if pat else (4 if cplx else 3)
        data = np.array(f.read().split()[:nf * per], dtype=np.float64).reshape(nf, per) if nf else \
            np.zeros((0, per))
    rows = data[:, 0].astype(np.int64) - 1
    cols = data[:, 1].astype(np.int64) - 1
    vals = np.ones(nf) if pat else data[:, 2].copy()
    if sym:
        off = rows != cols
        # the mirrored entry follows its original, as the reader pushes them
        rows = np.stack([rows, np.where(off, cols, -1)], 1).ravel()
        cols = np.stack([cols, np.where(off, data[:, 0].astype(np.int64) - 1, -1)], 1).ravel()
        vals = np.stack([vals, vals], 1).ravel()
        keep = rows >= 0
        rows, cols, vals = rows[keep], cols[keep], vals[keep]
    return m, n, rows, cols, vals


def load_mtx(path: str, dtype=np.float64, merge: bool = True) -> CSR:
    """Matrix Market reader following src/tile_format.h:51-90 (see
    read_mtx_entries), rows sorted by (row, col).  merge=True (the default)
    also sums duplicate entries, which the reference keeps: the library
    wants canonical CSR, columns strictly ascending inside each row.  With
    merge=False duplicates stay, in file order, as the reference's CSR holds
    them (its sort leaves their order unspecified)."""
    m, n, rows, cols, vals = read_mtx_entries(path)
    order = np.lexsort((cols, rows))
    rows, cols, vals = rows[order], cols[order], vals[order]
    if merge and rows.size:
        key = rows * max(n, 1) + cols
        first = np.concatenate([[True], key[1:] != key[:-1]])
        seg = np.cumsum(first) - 1
        vals = np.bincount(seg, weights=vals, minlength=int(seg[-1]) + 1)
        rows, cols = rows[first], cols[first]
    counts = np.bincount(rows, minlength=m).astype(np.int64)
    rp = np.zeros(m + 1, np.int64)
    np.cumsum(counts, out=rp[1:])
    return CSR(m, n, rp.astype(np.int32), cols.astype(np.int32), np.ascontiguousarray(vals.astype(dtype)))
