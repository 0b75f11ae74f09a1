// rowwise.cu -- row-wise (Gustavson-order) tiled SpGEMM: the bitmask symbolic
// phase and the numeric phase organised per C tile-row instead of per C tile.
//
// Same outputs as the per-C-tile kernels (plain.cu), bit for bit in the
// structure: row r of C tile (i,j) is the OR over A's nonzeros (r,k) of the
// 16-bit row mask of B's tile (k/16, j) at row k%16 -- exactly the reference's
// OR of maskB rows over matched tile pairs (src/spgemm_raw_kernels.cuh:173-184)
// -- but the pairs are enumerated from A's rows and B's rows instead of by
// intersecting A's tile-row list with B's tile-column list for every C tile.
// On a power-law matrix (R-MAT, 2^20) the intersections cost 1.1e11 probes
// against 2.1e10 products; this order touches every product once.
//
// Work decomposition (GB300: 152 SMs, 227 KB shared memory per CTA):
//   work item  = (C tile-row i, region of <= RT consecutive C tiles)
//   persistent CTAs take items from an atomic ticket (biggest tile-rows first,
//   in natural order);
//   a region is walked in shared-memory windows (symbolic: WS tiles of 16 row
//   masks; numeric: as many C tiles as fit one shared-memory arena at 64 bytes
//   of metadata a tile plus one accumulator a value, so windows of dense C
//   tiles hold more values and windows of sparse ones more tiles);
//   per A nonzero of the tile-row a cursor into its B row carries over from
//   window to window, so B's rows are read once per region, never searched
//   per window;
//   a B entry (c, v) finds its C tile by a popcount rank in a bitmap of the
//   window's tile columns, its value slot by popc of the C row mask;
//   C's arrays stream through L2 once (evict-first loads and stores), so the
//   re-read B rows keep the cache.
#include <climits>

#include "rowwise.cuh"

namespace {

constexpr int RW_THREADS = 512;
constexpr int RW_WARPS = RW_THREADS / 32;
constexpr int RT = 16384;       // C tiles per work item
constexpr int WS = 2048;        // C tiles per symbolic window
// numeric window arena (bytes): 8 B a tile + 5 B a non-empty tile row +
// sizeof(ACC) a value + 8 B per 32 tile columns the window spans (its rank
// bitmap).  These are the sizes that always fit; a launch grows its arena
// into whatever shared memory its blocks per SM leave.  Row words keep value
// offsets in 16 bits, so an arena stays below 2^16 values.
constexpr int NW_ARENA_F32 = 74752;   // two blocks per SM
constexpr int NW_ARENA_F64 = 131072;  // one block per SM
constexpr int NW_ARENA_MAX = 196608;
template <typename ACC>
constexpr int nw_arena() { return sizeof(ACC) == 4 ? NW_ARENA_F32 : NW_ARENA_F64; }
constexpr int MAXA_SMEM = 256;  // A nonzeros per tile-row whose cursors fit in shared memory
constexpr int SWU = 4;          // 32-product steps per sweep round of a warp (loads in flight)

// B's column at row-view position p, read from B's column array (the
// symbolic phase) or from the interleaved {column, value} entries the numeric
// phase reads, where one load brings a product's column and its value and
// the segment searches pull the values into L1 for the sweep that follows.
struct ColArray {
    const int* ci;
    __device__ __forceinline__ int operator()(int p) const { return __ldg(&ci[p]); }
};
template <typename V>
struct BEntry;
template <>
struct __align__(8) BEntry<float> { int c; float v; };
template <>
struct __align__(16) BEntry<double> { int c; int pad; double v; };
template <typename V>
struct ColEntries {
    const BEntry<V>* e;
    __device__ __forceinline__ int operator()(int p) const { return __ldg(&e[p].c); }
};

template <typename Cols>
__device__ __forceinline__ int lower_bound_i(Cols col, int lo, int hi, int key) {
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (col(mid) < key) lo = mid + 1; else hi = mid;
    }
    return lo;
}

template <typename V>
__global__ void bentry_fill_kernel(int64_t nnz, const int* __restrict__ ci, const V* __restrict__ val,
                                   BEntry<V>* __restrict__ out) {
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < nnz; p += (int64_t)gridDim.x * blockDim.x) {
        BEntry<V> e{};
        e.c = ci[p];
        e.v = val[p];
        out[p] = e;
    }
}

// Plan, pass 1: per C tile-row its products (sum over A's nonzeros of the B
// row lengths), the largest A nonzero count of any tile-row with C tiles, and
// the total products.  One warp per tile-row.
__global__ void rw_plan_kernel(int tilem, int m, const int* __restrict__ tile_ptrC, const int* __restrict__ a_rp,
                               const int* __restrict__ a_ci, const int* __restrict__ b_rp,
                               int64_t* __restrict__ prod, unsigned long long* __restrict__ max_na,
                               unsigned long long* __restrict__ total) {
    const int lane = threadIdx.x & 31;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < tilem; i += nw) {
        const int ntc = tile_ptrC[i + 1] - tile_ptrC[i];
        const int e0 = a_rp[i * TS], e1 = a_rp[min(i * TS + TS, m)];
        unsigned long long p = 0;
        if (ntc > 0)
            for (int e = e0 + lane; e < e1; e += 32) {
                const int k = __ldg(&a_ci[e]);
                p += (unsigned long long)(__ldg(&b_rp[k + 1]) - __ldg(&b_rp[k]));
            }
        p = warp_sum(p);
        if (lane == 0) {
            prod[i] = (int64_t)p;
            if (ntc > 0) {
                atomicMax(max_na, (unsigned long long)(e1 - e0));
                if (p) atomicAdd(total, p);
            }
        }
    }
}

// Plan, pass 2: work items per tile-row.  A tile-row is cut into regions of
// at most RT C tiles and at most ~PW products, PW = total / (SMs * 16)
// clamped to [2^16, 2^21]: hub tile-rows of a power-law matrix become many
// balanced items instead of one long one, and no item runs long enough
// (~2 M products at most) to hold up the end of a launch or of a band of
// tile-rows.  Finer items cost time: each re-seeks its A nonzeros' cursors
// (R-MAT 2^16 ran 15 % slower at total / (SMs * 64)).
__global__ void rw_plan2_kernel(int tilem, int num_sms, const int* __restrict__ tile_ptrC,
                                const int64_t* __restrict__ prod, const unsigned long long* __restrict__ total,
                                int64_t* __restrict__ nitems) {
    const unsigned long long tot = *total;
    unsigned long long pw = tot / ((unsigned long long)num_sms * 16ull);
    if (pw > (1ull << 21)) pw = 1ull << 21;
    if (pw < (1ull << 16)) pw = 1ull << 16;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < tilem; i += gridDim.x * blockDim.x) {
        const int64_t ntc = tile_ptrC[i + 1] - tile_ptrC[i];
        int64_t n = 0;
        if (ntc > 0) {
            const int64_t by_t = (ntc + RT - 1) / RT;
            const int64_t by_p = (int64_t)(((unsigned long long)prod[i] + pw - 1) / pw);
            n = by_t > by_p ? by_t : by_p;
            if (n > ntc) n = ntc;
            if (n < 1) n = 1;
        }
        nitems[i] = n;
    }
}

// Shared state of one work item.
struct ItemInfo {
    long long id;
    int i, rs, re, e0, na, q;
};

// Takes the next work item of [item_lo, item_hi); returns false when none is
// left.  All threads call.  With rev_bands > 0 (and item_lo == 0) tickets run
// through the bands of band_end from the last band to the first, each band's
// items in order: ticket x lies in band b when band_start[b] < item_hi - x <=
// band_end[b].
__device__ bool next_item(unsigned long long* ticket, const int64_t* __restrict__ item_prefix, int tilem,
                          int64_t item_lo, int64_t item_hi, const int* __restrict__ tile_ptrC,
                          const int* __restrict__ a_rp, int m, ItemInfo* s_it, int* s_rows, int rev_bands = 0,
                          const int64_t* __restrict__ band_end = nullptr) {
    __shared__ long long s_item;
    if (threadIdx.x == 0) {
        long long x = item_lo + (long long)atomicAdd(ticket, 1ull);
        if (rev_bands > 0 && x < item_hi) {
            const long long y = item_hi - x;  // in [1, item_hi]
            int lo = 0, hi = rev_bands - 1;   // first band whose end is >= y
            while (lo < hi) {
                const int mid = (lo + hi) >> 1;
                if (band_end[mid] >= y) hi = mid; else lo = mid + 1;
            }
            const long long bs = lo > 0 ? band_end[lo - 1] : 0;
            x = bs + (x - (item_hi - band_end[lo]));
        }
        s_item = x;
    }
    __syncthreads();
    const int64_t item = s_item;
    if (item >= item_hi) return false;
    if (threadIdx.x == 0) {
        int lo = 0, hi = tilem;
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (item_prefix[mid] <= item) lo = mid; else hi = mid;
        }
        const int64_t q = item - item_prefix[lo];
        const int64_t nreg = item_prefix[lo + 1] - item_prefix[lo];
        const int64_t ts = tile_ptrC[lo], ntc = tile_ptrC[lo + 1] - ts;
        s_it->id = item;
        s_it->i = lo;
        s_it->q = (int)q;
        s_it->rs = (int)(ts + (q * ntc) / nreg);
        s_it->re = (int)(ts + ((q + 1) * ntc) / nreg);
    }
    __syncthreads();
    if (threadIdx.x <= TS) {
        const int r0 = s_it->i * TS;
        s_rows[threadIdx.x] = a_rp[min(r0 + (int)threadIdx.x, m)];
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        s_it->e0 = s_rows[0];
        s_it->na = s_rows[TS] - s_rows[0];
    }
    __syncthreads();
    return true;
}

// Walk state of the A nonzeros of a tile-row, one array per field: the
// cursor into the nonzero's B row, the column there (INT_MAX past the row
// end), the row's end, and the length of the nonzero's latest segment (the
// first guess for its next one).
struct Cursors {
    int* pos;
    int* col;
    int* end;
    int* len;
};

__device__ __forceinline__ Cursors cursors_at(int* base, int stride) {
    return Cursors{base, base + stride, base + 2 * stride, base + 3 * stride};
}

// Cursor of every A nonzero of the tile-row: first B-row position whose column
// is >= the region's first column, that column, and the row's end (so later
// windows need no a_ci / b_rp loads).
template <typename Cols>
__device__ void init_cursors(const ItemInfo& it, Cursors cu, const int* __restrict__ colidxC,
                             const int* __restrict__ a_ci, const int* __restrict__ b_rp, Cols col) {
    const int cstart = colidxC[it.rs] * TS;
    for (int x = threadIdx.x; x < it.na; x += RW_THREADS) {
        const int k = __ldg(&a_ci[it.e0 + x]);
        int b = __ldg(&b_rp[k]);
        const int be = __ldg(&b_rp[k + 1]);
        if (it.q > 0) b = lower_bound_i(col, b, be, cstart);
        cu.pos[x] = b;
        cu.col[x] = b < be ? col(b) : INT_MAX;
        cu.end[x] = be;
        cu.len[x] = 0;
    }
    __syncthreads();
}

// Bitmap of a window's (sorted, distinct) tile columns with the popcount
// prefix of every word beside it (bp[w] = {bits, prefix}, one 8-byte load):
// rank(j) = index of column j among the window's tiles.
__device__ void build_window_rank(const int* __restrict__ colidxC, int t0, int nt, int wlo, int nwd, uint2* bp,
                                  int64_t* s_sh) {
    for (int x = threadIdx.x; x < nwd; x += RW_THREADS) bp[x] = make_uint2(0u, 0u);
    __syncthreads();
    for (int x = threadIdx.x; x < nt; x += RW_THREADS) {
        const int j = __ldcs(&colidxC[t0 + x]);
        atomicOr(&bp[(j >> 5) - wlo].x, 1u << (j & 31));
    }
    __syncthreads();
    const int wpt = (nwd + RW_THREADS - 1) / RW_THREADS;
    const int a = min(nwd, (int)threadIdx.x * wpt), b = min(nwd, a + wpt);
    int64_t local = 0;
    for (int x = a; x < b; x++) local += __popc(bp[x].x);
    int64_t tot;
    int64_t run = block_excl_scan<int64_t>(local, s_sh, &tot);
    for (int x = a; x < b; x++) {
        bp[x].y = (uint32_t)run;
        run += __popc(bp[x].x);
    }
    __syncthreads();
}

__device__ __forceinline__ int wrank(const uint2* bp, int wlo, int j) {
    const uint2 e = bp[(j >> 5) - wlo];
    return (int)e.y + __popc(e.x & ((1u << (j & 31)) - 1u));
}

__device__ __forceinline__ int row_of(const int* s_rows, int e) {
    int r = 0;
#pragma unroll
    for (int q = 1; q < TS; q++) r += (s_rows[q] <= e) ? 1 : 0;
    return r;
}

// Segment end of one active nonzero: the first position >= p0 + 1 whose
// column reaches `limit` (b_ci[p0] < limit is known).  The guess g (the
// nonzero's previous segment length) is probed first together with its
// successor, so a repeat of the last length costs one round of loads; a
// shorter segment is found by bisection below the guess, a longer one by
// galloping above it.  Returns the end; *nc receives the column there.
template <typename Cols>
__device__ __forceinline__ int segment_end(Cols col, int p0, int be, int g, int pa, int pb, int limit, int* nc) {
    if (pa >= limit) {  // col(p0) < limit <= col(p0 + g - 1)
        int lo = p0, hi = p0 + g - 1;
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (col(mid) < limit) lo = mid; else hi = mid;
        }
        *nc = (hi == p0 + g - 1) ? pa : col(hi);
        return hi;
    }
    if (pb >= limit) {  // exactly g entries (pb is INT_MAX at the row end)
        *nc = pb;
        return p0 + g;
    }
    int lo = p0 + g, hi = be, step = g;  // col(lo) = pb < limit
    while (true) {
        const int q = lo + step;
        if (q >= be) break;
        if (col(q) >= limit) { hi = q; break; }
        lo = q;
        step <<= 1;
    }
    while (hi - lo > 1) {  // col(lo) < limit <= col(hi) (or hi == be)
        const int mid = (lo + hi) >> 1;
        if (col(mid) < limit) lo = mid; else hi = mid;
    }
    *nc = hi < be ? col(hi) : INT_MAX;
    return hi;
}

// Runs the products of every B entry (column c < limit) that the A nonzeros
// of the tile-row reach inside the current window, and moves each nonzero's
// cursor past the window.  Warp-centric, with no block-wide barrier inside:
// a warp takes the next (up to) 32 nonzeros from the block's counter *s_fx
// (zeroed by the caller), each lane finds the window segment of its own nonzero
// (segment_end, from the cursor), a shuffle scan flattens the warp's
// segments, and the warp sweeps the products lane by lane, SWU steps of 32
// per round with all their loads in flight: consecutive lanes read
// consecutive B entries of one segment, and a slow search stalls only its
// own warp.  The caller synchronises the block afterwards.
// In the numeric walk, segments of at least LQ_MIN products are not swept by
// the warp that found them: they wait in a block queue of LQ_CAP entries that
// every warp drains together once the walk is over (drain_long).  A hub B row
// can hold thousands of products inside one window; swept by one warp, it
// kept the other warps waiting at the window's barrier (R-MAT 2^20 numeric
// 224 -> 218 ms).
constexpr int LQ_CAP = 128;
constexpr int LQ_MIN = 256;

// One entry of a warp's owner table: a segment that overlaps the products
// of the current sweep round.  A flat product index q of the warp's step maps
// to B position base + q.
template <typename Entry>
struct Owner {
    int base;  // first B position of the segment minus its first flat index
    int r;     // the A nonzero's row in its tile
    Entry e;
};

template <typename Entry>
struct LongQueue {
    int n;                 // segments offered (may pass LQ_CAP: the rest stayed with their warp)
    int next;              // drain ticket, in products
    int p0[LQ_CAP];        // first B position
    int pre[LQ_CAP + 1];   // exclusive prefix of the lengths (filled by drain_long)
    int r[LQ_CAP];         // the A nonzero's row in its tile
    Entry e[LQ_CAP];
};

template <typename Op, typename Cols>
__device__ __forceinline__ void walk_window(const ItemInfo& it, Cursors cu, const int* s_rows, int limit, Cols col,
                                            int* s_fx, Op op, LongQueue<typename Op::Entry>* lq,
                                            Owner<typename Op::Entry>* own) {
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    while (true) {
        // guided schedule: a step takes 1/RW_WARPS of what is left (at most
        // 32), so a short tile-row still spreads over every warp and the
        // window ends on small steps
        int base = 0, cnt = 0;
        if (lane == 0) {
            const int left = it.na - *reinterpret_cast<volatile int*>(s_fx);
            cnt = min(32, max(1, (left + RW_WARPS - 1) / RW_WARPS));
            base = atomicAdd(s_fx, cnt);
        }
        base = __shfl_sync(FULL, base, 0);
        cnt = __shfl_sync(FULL, cnt, 0);
        if (base >= it.na) break;
        const int x = base + lane;
        int len = 0, p0 = 0, r = 0;
        typename Op::Entry ent{};
        if (lane < cnt && x < it.na && cu.col[x] < limit) {
            p0 = cu.pos[x];
            const int be = cu.end[x];
            const int g = max(1, min(cu.len[x], be - p0));
            const int pa = g > 1 ? col(p0 + g - 1) : INT_MIN;
            const int pb = p0 + g < be ? col(p0 + g) : INT_MAX;
            ent = op.entry(x);
            r = row_of(s_rows, it.e0 + x);
            int nc;
            const int hi = segment_end(col, p0, be, g, pa, pb, limit, &nc);
            len = hi - p0;
            cu.pos[x] = hi;
            cu.col[x] = nc;
            cu.len[x] = len;
            if (lq && len >= LQ_MIN) {  // leave it to the whole block
                const int k = atomicAdd(&lq->n, 1);
                if (k < LQ_CAP) {
                    lq->p0[k] = p0;
                    lq->pre[k] = len;
                    lq->r[k] = r;
                    lq->e[k] = ent;
                    len = 0;
                }
            }
        }
        int inc = len;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const int o = __shfl_up_sync(FULL, inc, d);
            if (lane >= d) inc += o;
        }
        const int P = __shfl_sync(FULL, inc, 31);
        const int off = inc - len;  // exclusive offset of this lane's segment
        for (int q0 = 0; q0 < P; q0 += 32 * SWU) {
            // the segments overlapping products [q0, q0 + 32 SWU), in lane
            // order, go to the warp's owner table; each marks its first
            // product in the round (the one carried in: the round's first) in
            // SWU words of start bits.  A product's owner is the last segment
            // starting at or before it: its index is the count of start bits
            // up to the product's position, less one.
            const bool ov = len > 0 && off < q0 + 32 * SWU && off + len > q0;
            const int slot = max(off - q0, 0);
            const unsigned ovm = __ballot_sync(FULL, ov);
            if (ov) own[__popc(ovm & lanemask_lt())] = Owner<typename Op::Entry>{p0 - off, r, ent};
            unsigned sb[SWU];
#pragma unroll
            for (int u = 0; u < SWU; u++)
                sb[u] = __reduce_or_sync(FULL, (ov && (slot >> 5) == u) ? 1u << (slot & 31) : 0u);
            __syncwarp();
            int pp[SWU], rr[SWU];
            typename Op::Entry ee[SWU];
            int before = 0;  // start bits in the words of earlier u
#pragma unroll
            for (int u = 0; u < SWU; u++) {
                const int q = q0 + u * 32 + lane;
                // (2 << lane) - 1: positions 0..lane of this word (all 32 for lane 31)
                const int k = before + __popc(sb[u] & ((2u << lane) - 1u)) - 1;  // >= 0: position q0 is covered
                before += __popc(sb[u]);
                const Owner<typename Op::Entry> o = own[k];
                pp[u] = q < P ? o.base + q : -1;
                rr[u] = o.r;
                ee[u] = o.e;
            }
            __syncwarp();  // every lane has read the table before the next round writes it
            typename Op::Loaded ld[SWU];
            int cc[SWU];
#pragma unroll
            for (int u = 0; u < SWU; u++) op.fetch(pp[u], &cc[u], &ld[u]);
#pragma unroll
            for (int u = 0; u < SWU; u++)
                if (pp[u] >= 0) op.apply(rr[u], cc[u], ee[u], ld[u]);
        }
    }
}

// Sweeps the queued long segments with every warp of the block: the lengths
// become an exclusive prefix, then warps take 32 * SWU products at a time
// from a ticket and find each product's segment by bisection of the prefix.
// Called by all threads after the block's walk (a barrier ahead of it); the
// caller synchronises afterwards.  Resets the queue.
template <typename Op, typename Cols>
__device__ __forceinline__ void drain_long(LongQueue<typename Op::Entry>* lq, Cols col, Op op) {
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nq = min(lq->n, LQ_CAP);
    if (nq == 0) return;  // uniform: every thread read the same count after the barrier
    if (warp == 0) {  // lengths -> exclusive prefix, LQ_CAP / 32 entries a lane
        constexpr int PL = LQ_CAP / 32;
        int v[PL], run = 0;
#pragma unroll
        for (int k = 0; k < PL; k++) {
            const int i = lane * PL + k;
            v[k] = i < nq ? lq->pre[i] : 0;
            run += v[k];
        }
        int inc = run;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const int o = __shfl_up_sync(FULL, inc, d);
            if (lane >= d) inc += o;
        }
        int ex = inc - run;
#pragma unroll
        for (int k = 0; k < PL; k++) {
            lq->pre[lane * PL + k] = ex;
            ex += v[k];
        }
        if (lane == 31) lq->pre[LQ_CAP] = inc;
        if (lane == 0) lq->next = 0;
    }
    __syncthreads();
    const int total = lq->pre[LQ_CAP];
    while (true) {
        int q0 = 0;
        if (lane == 0) q0 = atomicAdd(&lq->next, 32 * SWU);
        q0 = __shfl_sync(FULL, q0, 0);
        if (q0 >= total) break;
        int pp[SWU], rr[SWU];
        typename Op::Entry ee[SWU];
#pragma unroll
        for (int u = 0; u < SWU; u++) {
            const int q = q0 + u * 32 + lane;
            pp[u] = -1;
            if (q < total) {
                int lo = 0, hi = nq;  // last segment with pre <= q
                while (hi - lo > 1) {
                    const int mid = (lo + hi) >> 1;
                    if (lq->pre[mid] <= q) lo = mid; else hi = mid;
                }
                pp[u] = lq->p0[lo] + (q - lq->pre[lo]);
                rr[u] = lq->r[lo];
                ee[u] = lq->e[lo];
            }
        }
        typename Op::Loaded ld[SWU];
        int cc[SWU];
#pragma unroll
        for (int u = 0; u < SWU; u++) op.fetch(pp[u], &cc[u], &ld[u]);
#pragma unroll
        for (int u = 0; u < SWU; u++)
            if (pp[u] >= 0) op.apply(rr[u], cc[u], ee[u], ld[u]);
    }
    (void)col;
}

// The walk's operations: entry(x) once per active nonzero (handed to the
// lanes sweeping its products through the owner table), fetch(p) per product with the round's other loads (the B
// entry's column, and its value for the numeric product; p < 0: none), and
// apply(r, c, entry, loaded).

// Symbolic product: OR the column's bit into C's row mask.
struct SymOp {
    struct Entry {};
    struct Loaded {};
    const uint2* bp;
    int wlo;
    uint32_t* masks32;
    const int* b_ci;
    __device__ __forceinline__ Entry entry(int) const { return Entry{}; }
    __device__ __forceinline__ void fetch(int p, int* c, Loaded*) const { *c = p >= 0 ? __ldg(&b_ci[p]) : 0; }
    __device__ __forceinline__ void apply(int r, int c, Entry, Loaded) const {
        const int idx = r * WS + wrank(bp, wlo, c >> 4);
        atomicOr(&masks32[idx >> 1], (0x8000u >> (c & 15)) << ((idx & 1) * 16));
    }
};

// Numeric product: a_ik * b_kc into C's value slot.  A window's C tiles are
// one uint2 each, {value offset of the tile, (first row word << 16) | mask of
// its non-empty rows}; each non-empty row is one word, (value offset of the
// row << 16) | row mask.
template <typename V, typename ACC>
struct NumOp {
    struct Entry { ACC va; };
    struct Loaded { ACC vb; };
    const uint2* bp;
    int wlo;
    const uint2* tinfo;
    const uint32_t* rows;
    ACC* acc;
    const V* a_val;
    const BEntry<V>* bcv;
    int e0;
    __device__ __forceinline__ Entry entry(int x) const { return Entry{(ACC)__ldg(&a_val[e0 + x])}; }
    __device__ __forceinline__ void fetch(int p, int* c, Loaded* l) const {
        if (p >= 0) {
            const BEntry<V> e = bcv[p];
            *c = e.c;
            l->vb = (ACC)e.v;
        } else {
            *c = 0;
            l->vb = ACC(0);
        }
    }
    __device__ __forceinline__ void apply(int r, int c, Entry e, Loaded l) const {
        const uint32_t ti = tinfo[wrank(bp, wlo, c >> 4)].y;
        const uint32_t w = rows[(ti >> 16) + __popc(ti & ((1u << r) - 1u))];
        atomicAdd(&acc[(int)(w >> 16) + __popc((w & 0xffffu) >> (16 - (c & 15)))], e.va * l.vb);
    }
};

// ---------------------------------------------------------------------------
// symbolic
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(RW_THREADS, 2)
rw_symbolic_kernel(int m, int nwords_b, const int64_t* __restrict__ item_prefix, int tilem, int64_t nitems,
                   const int* __restrict__ tile_ptrC, const int* __restrict__ colidxC,
                   const int* __restrict__ a_rp, const int* __restrict__ a_ci, const int* __restrict__ b_rp,
                   const int* __restrict__ b_ci, uint16_t* __restrict__ maskC, uint8_t* __restrict__ ptrRowC,
                   int64_t* __restrict__ tile_cnt, unsigned long long* ticket, int* __restrict__ cursor_g,
                   int max_na, const uint8_t* __restrict__ skip_rows) {
    extern __shared__ __align__(16) uint32_t smem[];
    uint32_t* masks32 = smem;                      // [16][WS] halfwords
    int* cur_s = reinterpret_cast<int*>(masks32 + WS * 8);  // 4 x MAXA_SMEM
    uint2* bp = reinterpret_cast<uint2*>(cur_s + 4 * MAXA_SMEM);  // nwords_b
    __shared__ ItemInfo s_it;
    __shared__ int s_rows[TS + 1];
    __shared__ int64_t s_sh[RW_WARPS + 1];
    __shared__ int s_fx;
    __shared__ Owner<SymOp::Entry> s_own[RW_THREADS];  // 32 entries per warp
    const int tid = threadIdx.x;

    while (next_item(ticket, item_prefix, tilem, 0, nitems, tile_ptrC, a_rp, m, &s_it, s_rows)) {
        const ItemInfo it = s_it;
        if (skip_rows && skip_rows[it.i]) continue;  // a tile-row the plain kernels take
        const Cursors cu = it.na <= MAXA_SMEM ? cursors_at(cur_s, MAXA_SMEM)
                                              : cursors_at(cursor_g + (int64_t)blockIdx.x * 4 * max_na, max_na);
        init_cursors(it, cu, colidxC, a_ci, b_rp, ColArray{b_ci});
        for (int w0 = it.rs; w0 < it.re; w0 += WS) {
            const int nt = min(WS, it.re - w0);
            const int jlo = colidxC[w0], jhi = colidxC[w0 + nt - 1];
            const int wlo = jlo >> 5, nwd = (jhi >> 5) - wlo + 1;
            const int limit = (jhi + 1) * TS;
            {  // clear the window's 16 rows of masks (nt halfwords each), one warp a row
                static_assert(RW_WARPS == TS, "one warp per tile row");
                const int nh = (nt + 1) >> 1;
                uint32_t* row = masks32 + (tid >> 5) * (WS / 2);
                for (int w = tid & 31; w < nh; w += 32) row[w] = 0u;
            }
            if (tid == 0) s_fx = 0;
            build_window_rank(colidxC, w0, nt, wlo, nwd, bp, s_sh);
            // (one atomicOr a product: long segments cost their warp little,
            // and a queue's two barriers cost more than it saved)
            walk_window(it, cu, s_rows, limit, ColArray{b_ci}, &s_fx, SymOp{bp, wlo, masks32, b_ci},
                        static_cast<LongQueue<SymOp::Entry>*>(nullptr), s_own + (tid & ~31));
            __syncthreads();
            // write-out: lane pair (2j, 2j+1) takes one tile, each lane 8 of its
            // rows, so a warp's stores cover 16 tiles' contiguous masks (512 B)
            // and row offsets (256 B); the low half's count reaches the high
            // half by shuffle
            for (int q0 = 0; q0 < 2 * nt; q0 += RW_THREADS) {
                const int q = q0 + tid;
                const bool act = q < 2 * nt;
                const int x = q >> 1, hh = q & 1;
                uint32_t mw[4] = {0u, 0u, 0u, 0u};
                uint32_t pw[2] = {0u, 0u};
                int tot = 0;
                if (act) {
#pragma unroll
                    for (int r8 = 0; r8 < 8; r8++) {
                        const int idx = (8 * hh + r8) * WS + x;
                        const uint32_t m16 = (masks32[idx >> 1] >> ((idx & 1) * 16)) & 0xffffu;
                        mw[r8 >> 1] |= m16 << (16 * (r8 & 1));
                        pw[r8 >> 2] |= (uint32_t)tot << (8 * (r8 & 3));
                        tot += __popc(m16);
                    }
                }
                const int low = __shfl_xor_sync(0xffffffffu, tot, 1);  // the pair's other half
                if (act) {
                    const int64_t t = (int64_t)w0 + x;
                    if (hh) {  // rows 8..15 start after rows 0..7 (every byte stays <= 240)
                        pw[0] += (uint32_t)low * 0x01010101u;
                        pw[1] += (uint32_t)low * 0x01010101u;
                        __stcs(reinterpret_cast<long long*>(tile_cnt) + t, (long long)(low + tot));
                    }
                    __stcs(reinterpret_cast<uint4*>(maskC) + 2 * t + hh, make_uint4(mw[0], mw[1], mw[2], mw[3]));
                    __stcs(reinterpret_cast<uint2*>(ptrRowC) + 2 * t + hh, make_uint2(pw[0], pw[1]));
                }
            }
            __syncthreads();
        }
    }
}

// ---------------------------------------------------------------------------
// numeric
// ---------------------------------------------------------------------------
template <typename ACC>
__device__ __forceinline__ void acc_add(ACC* a, ACC v) { atomicAdd(a, v); }

template <typename V, typename ACC>
__global__ void __launch_bounds__(RW_THREADS, sizeof(ACC) == 4 ? 2 : 1)
rw_numeric_kernel(int m, const int64_t* __restrict__ item_prefix, int tilem, int64_t item_lo,
                  int64_t item_hi,
                  const int* __restrict__ tile_ptrC, const int* __restrict__ colidxC,
                  const int64_t* __restrict__ tile_nnzC, const uint16_t* __restrict__ maskC,
                  const uint8_t* __restrict__ ptrRowC, const int* __restrict__ a_rp, const int* __restrict__ a_ci,
                  const V* __restrict__ a_val, const int* __restrict__ b_rp, const BEntry<V>* __restrict__ bcv,
                  V* __restrict__ valC, uint8_t* __restrict__ colC,
                  unsigned long long* ticket, int* __restrict__ cursor_g, int max_na, int nbands,
                  const int64_t* __restrict__ band_end, unsigned* __restrict__ band_cnt,
                  volatile int* band_flag, int band_rev, int arena, const uint8_t* __restrict__ skip_rows) {
    extern __shared__ __align__(16) uint32_t smem[];
    const int ARENA = arena;  // bytes, a multiple of 16
    uint2* tinfo = reinterpret_cast<uint2*>(smem);  // [ntw], then rows, acc and the rank bitmap
    int* cur_s = reinterpret_cast<int*>(reinterpret_cast<char*>(smem) + ARENA); // 4 x MAXA_SMEM
    __shared__ ItemInfo s_it;
    __shared__ int s_rows[TS + 1];
    __shared__ int64_t s_sh[RW_WARPS + 1];
    __shared__ int s_nt, s_fx, s_nrow;
    __shared__ LongQueue<typename NumOp<V, ACC>::Entry> s_lq;
    __shared__ Owner<typename NumOp<V, ACC>::Entry> s_own[RW_THREADS];  // 32 entries per warp
    const int tid = threadIdx.x;
    if (tid == 0) s_lq.n = 0;

    while (next_item(ticket, item_prefix, tilem, item_lo, item_hi, tile_ptrC, a_rp, m, &s_it, s_rows,
                     band_rev ? nbands : 0, band_end)) {
        const ItemInfo it = s_it;
        const Cursors cu = it.na <= MAXA_SMEM ? cursors_at(cur_s, MAXA_SMEM)
                                              : cursors_at(cursor_g + (int64_t)blockIdx.x * 4 * max_na, max_na);
        // a tile-row the plain kernels take: no work, but the item still
        // counts down its band below
        const bool skip = skip_rows && skip_rows[it.i];
        if (!skip) init_cursors(it, cu, colidxC, a_ci, b_rp, ColEntries<V>{bcv});
        int t0 = skip ? it.re : it.rs;
        while (t0 < it.re) {
            // window [t0, t1): the longest run of n tiles whose metadata (8 B
            // a tile, 5 B a non-empty row: at most min(values, 16 a tile)),
            // values, rank bitmap (8 B per 32 tile columns spanned) and 32 B
            // of alignment slack fit the arena (one tile always fits).
            // fits(n) is monotone (the tile-row's columns ascend): one sample
            // per thread, then the bracket after the last fitting sample.
            const int64_t v0 = tile_nnzC[t0];
            const int wlo0 = colidxC[t0] >> 5;
            const int cap_t = min(ARENA / 8, it.re - t0);
            auto fits = [&](int n) {
                const int64_t nvx = tile_nnzC[t0 + n] - v0;
                const int64_t rb = nvx < 16 * (int64_t)n ? nvx : 16 * (int64_t)n;
                const int64_t nwdx = (int64_t)((colidxC[t0 + n - 1] >> 5) - wlo0 + 1);
                return 8 * (int64_t)n + 5 * rb + (int64_t)sizeof(ACC) * nvx + 8 * nwdx + 32 <= ARENA;
            };
            const int step = (cap_t + RW_THREADS - 1) / RW_THREADS;
            if (tid == 0) { s_nt = 0; s_nrow = 0; }
            __syncthreads();
            {
                const int n = (tid + 1) * step;
                if (n <= cap_t && fits(n)) atomicMax(&s_nt, n);
            }
            __syncthreads();
            const int lo_n = s_nt;  // fits; lo_n + step does not (or passes cap_t)
            const int hi_n = min(cap_t, lo_n + step - 1);
            __syncthreads();
            if (tid < hi_n - lo_n && fits(lo_n + 1 + tid)) atomicMax(&s_nt, lo_n + 1 + tid);
            __syncthreads();
            const int ntw = max(1, s_nt);
            const int t1 = t0 + ntw;
            const int64_t v1 = tile_nnzC[t1];
            const int nv = (int)(v1 - v0);
            if (nv == 0) {
                t0 = t1;
                __syncthreads();
                continue;
            }
            const int jlo = colidxC[t0], jhi = colidxC[t1 - 1];
            const int wlo = jlo >> 5, nwd = (jhi >> 5) - wlo + 1;
            const int limit = (jhi + 1) * TS;
            uint32_t* rows = reinterpret_cast<uint32_t*>(tinfo + ntw);
            const int64_t rcap = nv < 16 * (int64_t)ntw ? nv : 16 * (int64_t)ntw;
            uint8_t* rowr = reinterpret_cast<uint8_t*>(rows + rcap);  // each row word's row in its tile
            const size_t aoff = ((size_t)(rowr + rcap - reinterpret_cast<uint8_t*>(smem)) + 15) & ~(size_t)15;
            ACC* acc = reinterpret_cast<ACC*>(reinterpret_cast<uint8_t*>(smem) + aoff);  // 16-byte aligned
            const size_t boff = (aoff + sizeof(ACC) * (size_t)nv + 7) & ~(size_t)7;
            uint2* bp = reinterpret_cast<uint2*>(reinterpret_cast<uint8_t*>(smem) + boff);  // nwd words
            // tile and row words, one thread per tile: 2 x 16 B of masks, 16 B
            // of row offsets and the tile's value offset, all loads in flight;
            // the tile's non-empty rows get a block of row words from a counter
            for (int lt = tid; lt < ntw; lt += RW_THREADS) {
                const int64_t t = (int64_t)t0 + lt;
                const uint4 m0 = __ldcs(reinterpret_cast<const uint4*>(maskC) + 2 * t);
                const uint4 m1 = __ldcs(reinterpret_cast<const uint4*>(maskC) + 2 * t + 1);
                const uint4 po = __ldcs(reinterpret_cast<const uint4*>(ptrRowC) + t);
                const uint32_t vb = (uint32_t)(tile_nnzC[t] - v0);
                const uint32_t mw[8] = {m0.x, m0.y, m0.z, m0.w, m1.x, m1.y, m1.z, m1.w};
                const uint32_t pw[4] = {po.x, po.y, po.z, po.w};
                uint32_t occ = 0;
#pragma unroll
                for (int r = 0; r < TS; r++)
                    if ((mw[r >> 1] >> (16 * (r & 1))) & 0xffffu) occ |= 1u << r;
                const int rs = occ ? atomicAdd(&s_nrow, __popc(occ)) : 0;
                tinfo[lt] = make_uint2(vb, ((uint32_t)rs << 16) | occ);
                int k = rs;
#pragma unroll
                for (int r = 0; r < TS; r++) {
                    const uint32_t m16 = (mw[r >> 1] >> (16 * (r & 1))) & 0xffffu;
                    if (m16) {
                        rowr[k] = (uint8_t)r;
                        rows[k++] = ((vb + ((pw[r >> 2] >> (8 * (r & 3))) & 0xffu)) << 16) | m16;
                    }
                }
            }
            for (int x = tid; x < nv; x += RW_THREADS) acc[x] = ACC(0);
            if (tid == 0) s_fx = 0;
            build_window_rank(colidxC, t0, ntw, wlo, nwd, bp, s_sh);
            const NumOp<V, ACC> nop{bp, wlo, tinfo, rows, acc, a_val, bcv, it.e0};
            walk_window(it, cu, s_rows, limit, ColEntries<V>{bcv}, &s_fx, nop, &s_lq, s_own + (tid & ~31));
            __syncthreads();
            drain_long(&s_lq, ColEntries<V>{bcv}, nop);
            __syncthreads();
            if (tid == 0) s_lq.n = 0;
            // column bytes: one thread per non-empty tile row writes its run;
            // values leave coalesced
            const int nrow = s_nrow;
            for (int k = tid; k < nrow; k += RW_THREADS) {
                const uint32_t w = rows[k];
                uint32_t m16 = w & 0xffffu;
                uint8_t* o = colC + v0 + (w >> 16);
                const uint8_t rb = (uint8_t)(rowr[k] << 4);
                while (m16) {
                    const int c = __clz(m16) - 16;
                    __stcs(o++, (uint8_t)(rb | (uint8_t)c));
                    m16 &= ~(0x8000u >> c);
                }
            }
            for (int x = tid; x < nv; x += RW_THREADS) __stcs(&valC[v0 + x], (V)acc[x]);
            __syncthreads();
            t0 = t1;
        }
        if (nbands > 0) {
            // band accounting: every thread's stores of this item are made
            // visible system-wide, then the item counts down its band; the
            // item that completes the band raises the band's host flag
            __threadfence_system();
            __syncthreads();
            if (tid == 0) {
                int lo = 0, hi = nbands - 1;  // first band whose item end is > id
                while (lo < hi) {
                    const int mid = (lo + hi) >> 1;
                    if (band_end[mid] > it.id) hi = mid; else lo = mid + 1;
                }
                const int64_t start = lo > 0 ? band_end[lo - 1] : 0;
                const unsigned done = atomicAdd(&band_cnt[lo], 1u) + 1u;
                if ((int64_t)done == band_end[lo] - start) {
                    __threadfence_system();
                    band_flag[lo] = 1;
                }
            }
        }
    }
}

// band_end[k] = first work item after band k (band k = tile-rows
// [rows[k], rows[k+1])); band counters cleared.
__global__ void band_plan_kernel(int nbands, const int* __restrict__ rows, const int64_t* __restrict__ item_prefix,
                                 int64_t* __restrict__ band_end, unsigned* __restrict__ band_cnt) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nbands; k += gridDim.x * blockDim.x) {
        band_end[k] = item_prefix[rows[k + 1]];
        band_cnt[k] = 0u;
    }
}

// Static shared memory of the kernels (owner tables, queue, item state) is
// kept below this reserve: the dynamic sizes are checked against the opt-in
// limit less it.
constexpr size_t RW_STATIC_RESERVE = 12288;

size_t sym_smem(int nwords_b) {
    return (size_t)WS * 8 * 4 + (size_t)MAXA_SMEM * 16 + (size_t)nwords_b * 8;
}

template <typename ACC>
size_t num_smem() {
    return (size_t)nw_arena<ACC>() + (size_t)MAXA_SMEM * 16;
}

}  // namespace

// Whether the row-wise kernels can run with B's width: the symbolic kernel
// keeps a rank bitmap as wide as B in shared memory.  AUTO then bins each
// tile-row (mlp.cu, bin_rows_kernel): row-wise windows for sparse tiles (few
// products per tile pair: the per-C-tile intersections and 16-wide register
// walks are mostly empty work), the plain per-C-tile register kernels for
// dense-ish tiles (stencils: their register accumulation beats shared-memory
// atomics).  Measured on GB300: R-MAT 2^18 (1.4 nnz/tile) row-wise 77 ms vs
// plain 982 ms; 27-point x 3 dof (50 nnz/tile) plain 19 ms vs row-wise 45 ms.
bool rowwise_fits(spg_handle_t h, const spg_tiles* B) {
    const int nwords_b = (B->tilen + 31) / 32;
    return sym_smem(nwords_b) + RW_STATIC_RESERVE <= h->smem_optin && rowwise_numeric_fits(h);
}

bool rowwise_numeric_fits(spg_handle_t h) { return num_smem<double>() + RW_STATIC_RESERVE <= h->smem_optin; }

static spg_status rw_prepare(spg_handle_t h, const spg_tiles* A, const spg_tiles* B, spg_ctiles* C,
                             RowwisePriv* rp) {
    if (rp->item_prefix) return SPG_OK;
    const int tilem = C->tilem;
    ScratchList sc(h);
    int64_t* nit = nullptr;
    int64_t* prod = nullptr;
    SPG_TRY(sc.alloc(&nit, (size_t)tilem + 1));
    SPG_TRY(sc.alloc(&prod, (size_t)tilem + 1));
    SPG_TRY(spg_alloc_t(h, &rp->item_prefix, (size_t)tilem + 1));
    SPG_TRY(spg_alloc_t(h, &rp->counters, 4));
    SPG_CUDA(h, cudaMemsetAsync(rp->counters, 0, 4 * sizeof(unsigned long long), h->stream));
    if (tilem > 0) {
        int g = (int)ceil_div((int64_t)tilem * 32, 256);
        if (g > h->num_sms * 8) g = h->num_sms * 8;
        rw_plan_kernel<<<g, 256, 0, h->stream>>>(tilem, A->m, C->tile_ptrC, A->row_ptr, A->col_idx, B->row_ptr, prod,
                                                 rp->counters + 2, rp->counters + 3);
        SPG_LAUNCHED(h);
        int g2 = (int)ceil_div(tilem, 256);
        if (g2 > h->num_sms * 8) g2 = h->num_sms * 8;
        rw_plan2_kernel<<<g2, 256, 0, h->stream>>>(tilem, h->num_sms, C->tile_ptrC, prod, rp->counters + 3, nit);
        SPG_LAUNCHED(h);
    }
    SPG_TRY(spg_scan_i64_to_i64(h, nit, rp->item_prefix, tilem));
    SPG_TRY(spg_read_i64(h, rp->item_prefix + tilem, &rp->nitems));
    int64_t mx = 0;
    SPG_TRY(spg_read_i64(h, (const int64_t*)(rp->counters + 2), &mx));
    rp->max_na = (int)mx;
    SPG_TRY(spg_read_i64(h, (const int64_t*)(rp->counters + 3), &h->stats.products));
    // cursor scratch for tile-rows with more A nonzeros than fit in shared
    // memory: one slice of 4 ints per nonzero per resident CTA (<= 4 CTAs of
    // 512 threads per SM)
    rp->grid = h->num_sms * 4;
    if (rp->max_na > MAXA_SMEM)
        SPG_TRY(spg_alloc_t(h, &rp->cursor_g, (size_t)rp->grid * rp->max_na * 4 + 4));
    return SPG_OK;
}

spg_status rowwise_symbolic(spg_handle_t h, const spg_tiles* A, const spg_tiles* B, spg_ctiles* C, RowwisePriv* rp,
                            int64_t* tile_cnt, const uint8_t* skip_rows) {
    if (C->numtileC == 0) return SPG_OK;
    SPG_TRY(rw_prepare(h, A, B, C, rp));
    h->stats.work_items = rp->nitems;
    const int nwords_b = (B->tilen + 31) / 32;
    const size_t smem = sym_smem(nwords_b);
    if (smem + RW_STATIC_RESERVE > h->smem_optin) return spg_fail(h, SPG_ERR_UNSUPPORTED, "row-wise symbolic: B too wide");
    SPG_CUDA(h, cudaFuncSetAttribute(rw_symbolic_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    SPG_CUDA(h, cudaMemsetAsync(rp->counters, 0, sizeof(unsigned long long), h->stream));
    int occ = 1;
    SPG_CUDA(h, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, rw_symbolic_kernel, RW_THREADS, smem));
    const int grid = h->num_sms * (occ < 1 ? 1 : (occ > 4 ? 4 : occ));
    rw_symbolic_kernel<<<grid, RW_THREADS, smem, h->stream>>>(
        A->m, nwords_b, rp->item_prefix, C->tilem, rp->nitems, C->tile_ptrC, C->tile_colidxC, A->row_ptr,
        A->col_idx, B->row_ptr, B->col_idx, C->maskC, C->ptrRowC, tile_cnt, rp->counters, rp->cursor_g, rp->max_na,
        skip_rows);
    SPG_LAUNCHED(h);
    return SPG_OK;
}

// Band reporting of one numeric launch (nbands == 0: none).
struct BandArgs {
    const uint8_t* skip_rows = nullptr;  // tile-rows left to the plain kernels
    int nbands = 0;
    const int64_t* band_end = nullptr;
    unsigned* band_cnt = nullptr;
    volatile int* band_flag = nullptr;
    int rev = 0;  // bands dispatched from the last to the first
};

template <typename V, typename ACC>
static spg_status launch_numeric(spg_handle_t h, const spg_tiles* A, const spg_tiles* B, spg_ctiles* C,
                                 RowwisePriv* rp, int64_t item_lo, int64_t item_hi, const BandArgs& ba) {
    size_t smem = num_smem<ACC>();
    if (smem + RW_STATIC_RESERVE > h->smem_optin)
        return spg_fail(h, SPG_ERR_UNSUPPORTED, "row-wise numeric: shared memory too small");
    // grow the arena into the shared memory left at the blocks per SM the
    // registers allow (two for FP32 accumulators, one for FP64); keep the
    // fixed size if the occupancy query disagrees
    int arena = nw_arena<ACC>();
    {
        const int target = sizeof(ACC) == 4 ? 2 : 1;
        cudaFuncAttributes fa{};
        SPG_CUDA(h, cudaFuncGetAttributes(&fa, rw_numeric_kernel<V, ACC>));
        const size_t fixed = smem - (size_t)arena + fa.sharedSizeBytes + 1024;  // + per-block reservation
        size_t per_block = h->smem_per_sm / target;
        if (per_block > h->smem_optin + 1024) per_block = h->smem_optin + 1024;
        if (per_block > fixed) {
            size_t cand = (per_block - fixed) & ~(size_t)15;
            if (cand > (size_t)NW_ARENA_MAX) cand = NW_ARENA_MAX;
            if (cand > (size_t)arena) {
                const size_t s2 = smem - (size_t)arena + cand;
                SPG_CUDA(h, cudaFuncSetAttribute(rw_numeric_kernel<V, ACC>,
                                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s2));
                int o2 = 0;
                SPG_CUDA(h, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o2, rw_numeric_kernel<V, ACC>,
                                                                          RW_THREADS, s2));
                if (o2 >= target) {
                    arena = (int)cand;
                    smem = s2;
                }
            }
        }
    }
    SPG_CUDA(h, cudaFuncSetAttribute(rw_numeric_kernel<V, ACC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)smem));
    SPG_CUDA(h, cudaMemsetAsync(rp->counters + 1, 0, sizeof(unsigned long long), h->stream));
    // B's {column, value} entries, refreshed on every launch (a numeric
    // re-run may come with new values on the same structure)
    ScratchList sc(h);
    BEntry<V>* bcv = nullptr;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    SPG_CUDA(h, cudaStreamIsCapturing(h->stream, &cap));
    if (cap == cudaStreamCaptureStatusNone)
        SPG_TRY(spg_workspace(h, SPG_WS_BENTRY, sizeof(BEntry<V>) * ((size_t)B->nnz + 1),
                              reinterpret_cast<void**>(&bcv)));
    else  // inside a graph: a block of the graph's own
        SPG_TRY(sc.alloc(&bcv, (size_t)B->nnz + 1));
    if (B->nnz > 0) {
        int g = (int)ceil_div(B->nnz, 256);
        if (g > h->num_sms * 16) g = h->num_sms * 16;
        bentry_fill_kernel<V><<<g, 256, 0, h->stream>>>(B->nnz, B->col_idx, (const V*)B->row_val, bcv);
        SPG_LAUNCHED(h);
    }
    int occ = 1;
    SPG_CUDA(h, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, rw_numeric_kernel<V, ACC>, RW_THREADS, smem));
    const int grid = h->num_sms * (occ < 1 ? 1 : (occ > 4 ? 4 : occ));
    rw_numeric_kernel<V, ACC><<<grid, RW_THREADS, smem, h->stream>>>(
        A->m, rp->item_prefix, C->tilem, item_lo, item_hi, C->tile_ptrC, C->tile_colidxC, C->tile_nnzC,
        C->maskC, C->ptrRowC, A->row_ptr, A->col_idx, (const V*)A->row_val, B->row_ptr, bcv, (V*)C->tile_valC,
        C->tile_colC, rp->counters + 1, rp->cursor_g, rp->max_na, ba.nbands, ba.band_end, ba.band_cnt,
        ba.band_flag, ba.rev, arena, ba.skip_rows);
    SPG_LAUNCHED(h);
    return SPG_OK;
}

spg_status rowwise_numeric(spg_handle_t h, const spg_tiles* A, const spg_tiles* B, spg_ctiles* C, RowwisePriv* rp,
                           spg_precision prec, int r0, int r1, const uint8_t* skip_rows) {
    if (C->numtileC == 0 || C->nnzC == 0) return SPG_OK;
    SPG_TRY(rw_prepare(h, A, B, C, rp));
    // the items of tile-rows [r0, r1); the whole range needs no device read
    // (the batch path captures this launch into CUDA graphs)
    int64_t lo = 0, hi = rp->nitems;
    if (r1 < 0) r1 = C->tilem;
    if (r0 > 0) SPG_TRY(spg_read_i64(h, rp->item_prefix + r0, &lo));
    if (r1 < C->tilem) SPG_TRY(spg_read_i64(h, rp->item_prefix + r1, &hi));
    if (hi <= lo) return SPG_OK;
    BandArgs none{};
    none.skip_rows = skip_rows;
    if (A->dtype == SPG_F64) return launch_numeric<double, double>(h, A, B, C, rp, lo, hi, none);
    if (prec == SPG_PREC_F64) return launch_numeric<float, double>(h, A, B, C, rp, lo, hi, none);
    return launch_numeric<float, float>(h, A, B, C, rp, lo, hi, none);
}

spg_status rowwise_numeric_bands_launch(spg_handle_t h, const spg_tiles* A, const spg_tiles* B, spg_ctiles* C,
                                        RowwisePriv* rp, spg_precision prec, int nbands, const int* d_rows,
                                        int64_t* d_band_end, unsigned* d_band_cnt, volatile int* band_flag_dev,
                                        int64_t* h_band_end, bool last_first, const uint8_t* skip_rows) {
    SPG_TRY(rw_prepare(h, A, B, C, rp));
    band_plan_kernel<<<(nbands + 255) / 256, 256, 0, h->stream>>>(nbands, d_rows, rp->item_prefix, d_band_end,
                                                                  d_band_cnt);
    SPG_LAUNCHED(h);
    SPG_CUDA(h, cudaMemcpyAsync(h_band_end, d_band_end, (size_t)nbands * sizeof(int64_t), cudaMemcpyDeviceToHost,
                                h->stream));
    SPG_CUDA(h, cudaStreamSynchronize(h->stream));
    if (C->numtileC == 0 || C->nnzC == 0 || rp->nitems == 0) return SPG_OK;
    BandArgs ba;
    ba.skip_rows = skip_rows;
    ba.nbands = nbands;
    ba.band_end = d_band_end;
    ba.band_cnt = d_band_cnt;
    ba.band_flag = band_flag_dev;
    ba.rev = last_first ? 1 : 0;
    if (A->dtype == SPG_F64) return launch_numeric<double, double>(h, A, B, C, rp, 0, rp->nitems, ba);
    if (prec == SPG_PREC_F64) return launch_numeric<float, double>(h, A, B, C, rp, 0, rp->nitems, ba);
    return launch_numeric<float, float>(h, A, B, C, rp, 0, rp->nitems, ba);
}

// Numeric launch only (no host synchronisation once the plan exists): the
// form captured into CUDA graphs by the batch path.
spg_status rowwise_numeric_launch(spg_handle_t h, const spg_tiles* A, const spg_tiles* B, spg_ctiles* C,
                                  RowwisePriv* rp, spg_precision prec) {
    return rowwise_numeric(h, A, B, C, rp, prec);
}

void rowwise_free_priv(spg_handle_t h, RowwisePriv* rp) {
    spg_free_async(h, rp->item_prefix);
    spg_free_async(h, rp->counters);
    spg_free_async(h, rp->cursor_g);
    *rp = RowwisePriv{};
}

void rowwise_free_bview(spg_handle_t, spg_tiles*) {}
