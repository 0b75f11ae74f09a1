// plain.cu -- the plain tiled SpGEMM kernels: the reference's three steps
// (src/spgemm_raw_kernels.cuh:23-215, src/spgemm_raw_kernels_v2.cuh:10-139)
// written from scratch for sm_103a.  One thread block per C tile-row for the
// structure, one half-warp per C tile for the symbolic phase, one warp per C
// tile with register accumulators for the numeric phase.  This is the baseline
// the row-wise binned path is measured against.
#include <cuda_fp16.h>

#include <cstdlib>

#include "spg_common.cuh"
#include "plain.cuh"

namespace {

constexpr int C1_THREADS = 256;
constexpr int C1_WARPS = C1_THREADS / 32;
constexpr int SPEC_MAX = SPEC_PAIRS_MAX;  // pairs cached per C tile (MAX_MATCHED)

// Union of B's tile columns over A's tiles (i,k) as a bitmap.  The bitmap
// covers only the tile-row's column span [jlo, jhi] (first / last tile column
// of the B tile-rows it reaches; B's tile-rows are sorted), so clearing and
// scanning cost O(span / 32) rather than O(tilenB / 32): a block-diagonal
// batch of many small products stays cheap.  Word w of the bitmap holds
// columns 32*(wlo + w) ... ; *s_span receives {wlo, nwd}.  Returns the
// tile-row's tile pairs (thread 0; 0 elsewhere).
// Saturation: with occ (B's occupied tile columns, exclusive prefix over
// tilenB + 1) a tile-row whose tile pairs are at least 4x the occupied B
// columns of its span stops probing once every one of them is set -- no
// further pair can add a column.  Each warp counts the bitmap after probing
// 32x as many pairs as it has words, at most four times a row (the counts
// cost a row that never fills a few percent of its probing at most).  An Erdos-Renyi tile-row (one nonzero
// a tile) pairs each A tile with all of B's tile-row and fills its span long
// before its last pair.
__device__ int64_t build_c_bitmap(int i, const int* __restrict__ a_tp, const int* __restrict__ a_tc,
                                  const int* __restrict__ b_tp, const int* __restrict__ b_tc, uint32_t* bm,
                                  int* s_span, const int* __restrict__ occ) {
    __shared__ unsigned long long s_pairs;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int as = a_tp[i], ae = a_tp[i + 1];
    if (threadIdx.x == 0) { s_span[0] = 0x7fffffff; s_span[1] = -1; s_pairs = 0ull; }
    __syncthreads();
    int lo = 0x7fffffff, hi = -1;
    unsigned long long pp = 0;
    for (int a = as + threadIdx.x; a < ae; a += C1_THREADS) {
        const int k = __ldg(&a_tc[a]);
        const int bs = __ldg(&b_tp[k]), be = __ldg(&b_tp[k + 1]);
        pp += (unsigned long long)(be - bs);
        if (be > bs) {
            lo = min(lo, __ldg(&b_tc[bs]));
            hi = max(hi, __ldg(&b_tc[be - 1]));
        }
    }
    if (hi >= 0) { atomicMin(&s_span[0], lo); atomicMax(&s_span[1], hi); }
    pp = warp_sum(pp);
    if (lane == 0 && pp) atomicAdd(&s_pairs, pp);
    __syncthreads();
    const int jlo = s_span[0], jhi = s_span[1];
    const int wlo = jhi >= 0 ? (jlo >> 5) : 0;
    const int nwd = jhi >= 0 ? (jhi >> 5) - wlo + 1 : 0;
    const unsigned long long pairs = s_pairs;
    const int target = (occ && jhi >= 0) ? __ldg(&occ[jhi + 1]) - __ldg(&occ[jlo]) : 0;
    const bool sat = target > 0 && pairs >= 4ull * (unsigned long long)target;  // block-uniform
    for (int w = threadIdx.x; w < nwd; w += C1_THREADS) bm[w] = 0u;
    __syncthreads();
    if (threadIdx.x == 0) { s_span[2] = wlo; s_span[3] = nwd; }
    int a = as + warp;
    if (sat) {
        int64_t since = 0;  // pairs this warp probed since its last count
        int counts = 4;     // a row still short of full after four counts (a power-law hub) stops counting
        for (; a < ae && counts > 0; a += C1_WARPS) {
            if (since >= 32 * (int64_t)nwd) {  // warp-uniform
                since = 0;
                counts--;
                int c = 0;
                for (int w = lane; w < nwd; w += 32) c += __popc(bm[w]);
                if (warp_sum(c) >= target) { a = ae; break; }  // bits are only ever added: a full count is final
            }
            const int k = __ldg(&a_tc[a]);
            const int bs = __ldg(&b_tp[k]), be = __ldg(&b_tp[k + 1]);
            since += be - bs;
            for (int b = bs + lane; b < be; b += 32) {
                const int j = __ldg(&b_tc[b]) - (wlo << 5);
                const uint32_t bit = 1u << (j & 31);
                if (!(bm[j >> 5] & bit)) atomicOr(&bm[j >> 5], bit);
            }
        }
    }
    for (; a < ae; a += C1_WARPS) {  // every pair (after the counts, for a row that did not fill)
        const int k = __ldg(&a_tc[a]);
        const int bs = __ldg(&b_tp[k]), be = __ldg(&b_tp[k + 1]);
        for (int b = bs + lane; b < be; b += 32) {
            const int j = __ldg(&b_tc[b]) - (wlo << 5);
            const uint32_t bit = 1u << (j & 31);
            if (!(bm[j >> 5] & bit)) atomicOr(&bm[j >> 5], bit);
        }
    }
    __syncthreads();
    return threadIdx.x == 0 ? (int64_t)pairs : 0;
}

__global__ void __launch_bounds__(C1_THREADS)
c1_count_kernel(int nwords, const int* __restrict__ a_tp, const int* __restrict__ a_tc,
                const int* __restrict__ b_tp, const int* __restrict__ b_tc, int* __restrict__ cnt,
                int64_t* __restrict__ row_pairs, unsigned long long* __restrict__ pairs_total,
                const int* __restrict__ occ) {
    extern __shared__ uint32_t bm[];
    __shared__ int s_c[C1_WARPS];
    __shared__ int64_t s_p[C1_WARPS];
    __shared__ int s_span[4];
    const int i = blockIdx.x;
    (void)nwords;
    if (a_tp[i] == a_tp[i + 1]) {
        if (threadIdx.x == 0) { cnt[i] = 0; row_pairs[i] = 0; }
        return;
    }
    int64_t pairs = build_c_bitmap(i, a_tp, a_tc, b_tp, b_tc, bm, s_span, occ);
    const int nwd = s_span[3];
    int c = 0;
    for (int w = threadIdx.x; w < nwd; w += C1_THREADS) c += __popc(bm[w]);
    c = warp_sum(c);
    pairs = warp_sum(pairs);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) { s_c[warp] = c; s_p[warp] = pairs; }
    __syncthreads();
    if (threadIdx.x == 0) {
        int t = 0;
        int64_t p = 0;
        for (int w = 0; w < C1_WARPS; w++) { t += s_c[w]; p += s_p[w]; }
        cnt[i] = t;
        row_pairs[i] = p;
        if (p) atomicAdd(pairs_total, (unsigned long long)p);
    }
}

__global__ void __launch_bounds__(C1_THREADS)
c1_fill_kernel(int nwords, const int* __restrict__ a_tp, const int* __restrict__ a_tc,
               const int* __restrict__ b_tp, const int* __restrict__ b_tc,
               const int* __restrict__ tile_ptrC, int* __restrict__ rowidxC, int* __restrict__ colidxC,
               const int* __restrict__ rows, const int* __restrict__ occ) {
    extern __shared__ uint32_t bm[];
    __shared__ int64_t s_sh[C1_WARPS + 1];
    __shared__ int s_span[4];
    const int i = rows ? rows[blockIdx.x] : (int)blockIdx.x;
    (void)nwords;
    if (tile_ptrC[i] == tile_ptrC[i + 1]) return;
    build_c_bitmap(i, a_tp, a_tc, b_tp, b_tc, bm, s_span, occ);
    const int wlo = s_span[2], nwd = s_span[3];
    const int wpt = (nwd + C1_THREADS - 1) / C1_THREADS;
    const int w0 = min(nwd, (int)threadIdx.x * wpt), w1 = min(nwd, w0 + wpt);
    int64_t local = 0;
    for (int w = w0; w < w1; w++) local += __popc(bm[w]);
    int64_t tot;
    int64_t run = block_excl_scan<int64_t>(local, s_sh, &tot);
    int64_t pos = (int64_t)tile_ptrC[i] + run;
    for (int w = w0; w < w1; w++) {
        uint32_t bits = bm[w];
        while (bits) {
            const int b = __ffs(bits) - 1;
            rowidxC[pos] = i;
            colidxC[pos] = (wlo + w) * 32 + b;
            pos++;
            bits &= bits - 1u;
        }
    }
}

// Step 1 with learned sizing: every tile-row i owns a slot of predicted size
// in a staging array (slot_off = exclusive scan of the predicted sizes).  One
// block per tile-row builds its bitmap once, records the exact count, and
// writes its tile columns into its slot when they fit.  No block waits on
// another.  Rows that outgrow their slot only keep their count and rebuild
// their bitmap in the exact fill afterwards (c1_fill_kernel on a row list).
__global__ void __launch_bounds__(C1_THREADS)
c1_slot_kernel(const int* __restrict__ a_tp, const int* __restrict__ a_tc, const int* __restrict__ b_tp,
               const int* __restrict__ b_tc, const int64_t* __restrict__ slot_off, int* __restrict__ slot_col,
               int* __restrict__ cnt, int64_t* __restrict__ row_pairs, unsigned long long* __restrict__ pairs_total,
               const int* __restrict__ occ) {
    extern __shared__ uint32_t bm[];
    __shared__ int s_span[4];
    __shared__ int64_t s_sh[C1_WARPS + 1];
    __shared__ int64_t s_p[C1_WARPS];
    const int i = blockIdx.x;
    if (a_tp[i] == a_tp[i + 1]) {
        if (threadIdx.x == 0) { cnt[i] = 0; row_pairs[i] = 0; }
        return;
    }
    int64_t pairs = build_c_bitmap(i, a_tp, a_tc, b_tp, b_tc, bm, s_span, occ);
    const int wlo = s_span[2], nwd = s_span[3];
    const int wpt = (nwd + C1_THREADS - 1) / C1_THREADS;
    const int w0 = min(nwd, (int)threadIdx.x * wpt), w1 = min(nwd, w0 + wpt);
    int64_t local = 0;
    for (int w = w0; w < w1; w++) local += __popc(bm[w]);
    int64_t tot;
    const int64_t run = block_excl_scan<int64_t>(local, s_sh, &tot);
    pairs = warp_sum(pairs);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) s_p[warp] = pairs;
    __syncthreads();
    if (threadIdx.x == 0) {
        int64_t p = 0;
        for (int w = 0; w < C1_WARPS; w++) p += s_p[w];
        cnt[i] = (int)tot;
        row_pairs[i] = p;
        if (p) atomicAdd(pairs_total, (unsigned long long)p);
    }
    if (tot > slot_off[i + 1] - slot_off[i]) return;  // outgrew its slot: exact fill later
    int64_t pos = slot_off[i] + run;
    for (int w = w0; w < w1; w++) {
        uint32_t bits = bm[w];
        while (bits) {
            const int b = __ffs(bits) - 1;
            __stcs(&slot_col[pos++], (wlo + w) * 32 + b);
            bits &= bits - 1u;
        }
    }
}

// Slots -> C's exact tile arrays, one warp per tile-row (coalesced copies);
// rows that outgrew their slot are listed for the exact fill.
__global__ void c1_compact_kernel(int tilem, const int* __restrict__ tile_ptrC, const int64_t* __restrict__ slot_off,
                                  const int* __restrict__ slot_col, int* __restrict__ rowidxC, int* __restrict__ colidxC,
                                  int* __restrict__ over_rows, unsigned* __restrict__ n_over) {
    const int lane = threadIdx.x & 31;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < tilem; i += nw) {
        const int t0 = tile_ptrC[i], n = tile_ptrC[i + 1] - t0;
        if (n == 0) continue;
        const int64_t s0 = slot_off[i];
        if (n > slot_off[i + 1] - s0) {
            if (lane == 0) over_rows[atomicAdd(n_over, 1u)] = i;
            continue;
        }
        for (int k = lane; k < n; k += 32) {
            __stcs(&colidxC[t0 + k], __ldcs(&slot_col[s0 + k]));
            __stcs(&rowidxC[t0 + k], i);
        }
    }
}

// occ[j] = 1 where B's tile column j holds a tile (scanned into the prefix
// build_c_bitmap's saturation exit reads).
__global__ void occupied_cols_kernel(int tilen, const int* __restrict__ csc_tile_ptr, int* __restrict__ occ) {
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < tilen; j += gridDim.x * blockDim.x)
        occ[j] = csc_tile_ptr[j + 1] > csc_tile_ptr[j] ? 1 : 0;
}

__device__ __forceinline__ int lower_bound_dev(const int* __restrict__ a, int lo, int hi, int key) {
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(&a[mid]) < key) lo = mid + 1; else hi = mid;
    }
    return lo;
}

// Step 2, one half-warp per C tile.  Matched pairs come from binary-searching
// the shorter tile list in the longer one (src/spgemm_raw_kernels.cuh:146-158);
// each pair ORs B's row masks selected by A's column bytes into C's 16 row
// masks (:173-184); up to SPEC_MAX pairs are cached for step 3 with the bound
// checked before any write (the reference writes past its buffer first).
template <bool CACHE, typename CNT = int, bool LIST = false>
__global__ void __launch_bounds__(128)
c2_symbolic_kernel(int64_t ntiles, const int* __restrict__ tlist, const int* __restrict__ rowidxC,
                   const int* __restrict__ colidxC,
                   const int* __restrict__ a_tp, const int* __restrict__ a_tc,
                   const int* __restrict__ a_tnnz, const uint8_t* __restrict__ a_col,
                   const uint8_t* __restrict__ a_ptr16, const int* __restrict__ b_cscp,
                   const int* __restrict__ b_cscr, const uint16_t* __restrict__ b_mask,
                   uint16_t* __restrict__ maskC, uint8_t* __restrict__ ptrRowC, CNT* __restrict__ tile_cnt,
                   int* __restrict__ spec_cnt, int* __restrict__ spec_off, int* __restrict__ spec_pa,
                   int* __restrict__ spec_pb, int64_t spec_cap, unsigned long long* __restrict__ alloc_ctr,
                   unsigned long long* __restrict__ pairs_total, unsigned* flags) {
    __shared__ int s_pa[8][SPEC_MAX];
    __shared__ int s_pb[8][SPEC_MAX];
    const int lane = threadIdx.x & 31, r = lane & 15, half = lane >> 4;
    const int hw = threadIdx.x >> 4;  // half-warp in block
    const unsigned hmask = 0xffffu << (16 * half);
    unsigned long long my_pairs = 0;
    const int64_t nhw = (int64_t)gridDim.x * 8;
    for (int64_t idx = (int64_t)blockIdx.x * 8 + hw; idx < ntiles; idx += nhw) {
        const int64_t t = LIST ? (int64_t)tlist[idx] : idx;  // the C tile (a listed one, or every one)
        const int bi = rowidxC[t], bj = colidxC[t];
        const int as = a_tp[bi], ae = a_tp[bi + 1];
        const int bs = b_cscp[bj], be = b_cscp[bj + 1];
        const bool a_short = (ae - as) <= (be - bs);
        const int ss = a_short ? as : bs, se = a_short ? ae : be;
        const int ls = a_short ? bs : as, le = a_short ? be : ae;
        const int* sl = a_short ? a_tc : b_cscr;
        const int* ll = a_short ? b_cscr : a_tc;
        uint32_t rm = 0;
        int nm = 0;
        for (int base = ss; base < se; base += 16) {
            const int idx = base + r;
            int pos = -1;
            if (idx < se) {
                const int key = __ldg(&sl[idx]);
                const int p = lower_bound_dev(ll, ls, le, key);
                if (p < le && __ldg(&ll[p]) == key) pos = p;
            }
            unsigned mm = (__ballot_sync(hmask, pos >= 0) >> (16 * half)) & 0xffffu;
            while (mm) {
                const int src = __ffs(mm) - 1;
                mm &= mm - 1u;
                const int sp = __shfl_sync(hmask, idx, src, 16);
                const int lp = __shfl_sync(hmask, pos, src, 16);
                const int pa = a_short ? sp : lp, pb = a_short ? lp : sp;
                if (CACHE && r == 0 && nm < SPEC_MAX) { s_pa[hw][nm] = pa; s_pb[hw][nm] = pb; }
                nm++;
                const int s = __ldg(&a_tnnz[pa]), na = __ldg(&a_tnnz[pa + 1]) - s;
                const int rs = __ldg(&a_ptr16[(int64_t)pa * TS + r]);
                const int re = (r == TS - 1) ? na : (int)__ldg(&a_ptr16[(int64_t)pa * TS + r + 1]);
                for (int e = rs; e < re; e++)
                    rm |= __ldg(&b_mask[(int64_t)pb * TS + (__ldg(&a_col[s + e]) & 15)]);
            }
        }
        my_pairs += (r == 0) ? (unsigned long long)nm : 0ull;
        if (CACHE) {
            __syncwarp(hmask);
            int off = -1, cached = -1;
            if (r == 0) {
                if (nm >= 1 && nm <= SPEC_MAX) {
                    unsigned long long o = atomicAdd(alloc_ctr, (unsigned long long)nm);
                    if ((int64_t)(o + nm) <= spec_cap) { off = (int)o; cached = nm; }
                    else atomicOr(flags, DERR_OVERFLOW);
                } else if (nm == 0) {
                    cached = 0;
                }
            }
            off = __shfl_sync(hmask, off, 0, 16);
            cached = __shfl_sync(hmask, cached, 0, 16);
            if (cached > 0)
                for (int q = r; q < cached; q += 16) { spec_pa[off + q] = s_pa[hw][q]; spec_pb[off + q] = s_pb[hw][q]; }
            if (r == 0) { spec_cnt[t] = cached; spec_off[t] = off; }
            __syncwarp(hmask);
        }
        maskC[t * TS + r] = (uint16_t)rm;
        int pc = __popc(rm);
        int inc = pc;
#pragma unroll
        for (int d = 1; d < 16; d <<= 1) {
            const int o = __shfl_up_sync(hmask, inc, d, 16);
            if (r >= d) inc += o;
        }
        ptrRowC[t * TS + r] = (uint8_t)(inc - pc);
        if (r == TS - 1) tile_cnt[t] = (CNT)inc;
    }
    my_pairs = warp_sum(my_pairs);
    if (lane == 0 && my_pairs) atomicAdd(pairs_total, my_pairs);
}

// Step 3, one warp per C tile: lane = (row r, half h); the two halves take
// alternate A entries of row r (src/spgemm_raw_kernels_v2.cuh:36-37,83) and
// keep 16 register accumulators; B's row is walked through its 16-bit mask
// with predicated FMAs instead of the reference's 16-way switch; a shuffle
// combines the halves and half 0 compacts the row by maskC.
template <typename V, bool CACHE, bool SKIP_DENSE = false, bool LIST = false>
__global__ void __launch_bounds__(256)
c3_numeric_kernel(int64_t ntiles, const int* __restrict__ tlist, const int* __restrict__ rowidxC,
                  const int* __restrict__ colidxC,
                  const int* __restrict__ a_tp, const int* __restrict__ a_tc, const int* __restrict__ a_tnnz,
                  const V* __restrict__ a_val, const uint8_t* __restrict__ a_col,
                  const uint8_t* __restrict__ a_ptr16, const int* __restrict__ b_cscp,
                  const int* __restrict__ b_cscr, const int* __restrict__ b_tnnz,
                  const V* __restrict__ b_val, const uint8_t* __restrict__ b_ptr16,
                  const uint16_t* __restrict__ b_mask, const int64_t* __restrict__ tile_nnzC,
                  const uint16_t* __restrict__ maskC, const uint8_t* __restrict__ ptrRowC,
                  V* __restrict__ valC, uint8_t* __restrict__ colC, const int* __restrict__ spec_cnt,
                  const int* __restrict__ spec_off, const int* __restrict__ spec_pa,
                  const int* __restrict__ spec_pb, int dense_thr = 0, int* __restrict__ dense_tiles = nullptr,
                  unsigned* __restrict__ n_dense_tiles = nullptr) {
    const int lane = threadIdx.x & 31, r = lane & 15, hsel = lane >> 4;
    const int64_t nwarps = (int64_t)gridDim.x * (blockDim.x >> 5);
    // FP64 accumulates in shared memory, one row of 16 per lane (padded rows:
    // the 16 rows of a half-warp fall in distinct banks), and each A entry
    // walks only its B row's set bits: GB300 issues FP64 at 1/64 of its FP32
    // rate, and the register walk's 16 masked FMAs per A entry cost as much
    // FP64 issue as a full B row.  FP32 keeps its registers.
    constexpr bool SACC = sizeof(V) == 8;
    __shared__ V s_acc[SACC ? 256 / 32 * 2 * TS * (TS + 1) : 1];
    V* srow = s_acc + (SACC ? ((threadIdx.x >> 5) * 2 * TS + hsel * TS + r) * (TS + 1) : 0);
    for (int64_t idx = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); idx < ntiles; idx += nwarps) {
        const int64_t t = LIST ? (int64_t)tlist[idx] : idx;  // the C tile (a listed one, or every one)
        const int64_t cbase = tile_nnzC[t];
        if (tile_nnzC[t + 1] == cbase) continue;
        V acc[TS];
#pragma unroll
        for (int c = 0; c < TS; c++) acc[c] = V(0);
        if (SACC) {
#pragma unroll
            for (int c = 0; c < TS; c++) srow[c] = V(0);
        }
        bool skipped = false;  // warp-uniform: a dense pair was left to the tensor kernel
        auto do_pair = [&](int pa, int pb) {
            const int sA = __ldg(&a_tnnz[pa]), na = __ldg(&a_tnnz[pa + 1]) - sA;
            if (SKIP_DENSE && na >= dense_thr && __ldg(&b_tnnz[pb + 1]) - __ldg(&b_tnnz[pb]) >= dense_thr) {
                skipped = true;
                return;
            }
            const int rs = __ldg(&a_ptr16[(int64_t)pa * TS + r]);
            const int re = (r == TS - 1) ? na : (int)__ldg(&a_ptr16[(int64_t)pa * TS + r + 1]);
            const int sB = __ldg(&b_tnnz[pb]);
            for (int e = rs + hsel; e < re; e += 2) {
                const int kk = __ldg(&a_col[sA + e]) & 15;
                const V va = __ldg(&a_val[sA + e]);
                const uint32_t mb = __ldg(&b_mask[(int64_t)pb * TS + kk]);
                int off = sB + __ldg(&b_ptr16[(int64_t)pb * TS + kk]);
                if (SACC) {
                    for (uint32_t m = mb; m; off++) {  // set bits only, MSB-first (bit 15: column 0)
                        const int c = __clz(m) - 16;
                        m &= ~(0x8000u >> c);
                        srow[c] = fma(va, __ldg(&b_val[off]), srow[c]);
                    }
                } else {
#pragma unroll
                    for (int c = 0; c < TS; c++) {
                        if (mb & (0x8000u >> c)) {
                            acc[c] = fma(va, __ldg(&b_val[off]), acc[c]);
                            off++;
                        }
                    }
                }
            }
        };
        int cnt = CACHE ? spec_cnt[t] : -1;
        if (cnt >= 0) {
            const int off = spec_off[t];
            for (int q = 0; q < cnt; q++) do_pair(spec_pa[off + q], spec_pb[off + q]);
        } else {
            const int bi = rowidxC[t], bj = colidxC[t];
            const int as = a_tp[bi], ae = a_tp[bi + 1];
            const int bs = b_cscp[bj], be = b_cscp[bj + 1];
            const bool a_short = (ae - as) <= (be - bs);
            const int ss = a_short ? as : bs, se = a_short ? ae : be;
            const int ls = a_short ? bs : as, le = a_short ? be : ae;
            const int* sl = a_short ? a_tc : b_cscr;
            const int* ll = a_short ? b_cscr : a_tc;
            for (int base = ss; base < se; base += 32) {
                const int idx = base + lane;
                int pos = -1;
                if (idx < se) {
                    const int key = __ldg(&sl[idx]);
                    const int p = lower_bound_dev(ll, ls, le, key);
                    if (p < le && __ldg(&ll[p]) == key) pos = p;
                }
                unsigned mm = __ballot_sync(0xffffffffu, pos >= 0);
                while (mm) {
                    const int src = __ffs(mm) - 1;
                    mm &= mm - 1u;
                    const int sp = __shfl_sync(0xffffffffu, idx, src);
                    const int lp = __shfl_sync(0xffffffffu, pos, src);
                    do_pair(a_short ? sp : lp, a_short ? lp : sp);
                }
            }
        }
        if (SACC) {
            __syncwarp();  // both halves' rows are complete
            if (hsel == 0) {
                const V* other = srow + TS * (TS + 1);  // the same row of half 1
                int64_t p = cbase + ptrRowC[t * TS + r];
                for (uint32_t m = maskC[t * TS + r]; m; p++) {
                    const int c = __clz(m) - 16;
                    m &= ~(0x8000u >> c);
                    valC[p] = srow[c] + other[c];
                    colC[p] = (uint8_t)((r << 4) | c);
                }
            }
            __syncwarp();  // half 1 clears its rows for the next tile only after the reads
        } else {
#pragma unroll
            for (int c = 0; c < TS; c++) acc[c] += __shfl_xor_sync(0xffffffffu, acc[c], 16);
            if (hsel == 0) {
                const uint32_t mc = maskC[t * TS + r];
                int64_t p = cbase + ptrRowC[t * TS + r];
#pragma unroll
                for (int c = 0; c < TS; c++) {
                    if (mc & (0x8000u >> c)) {
                        valC[p] = acc[c];
                        colC[p] = (uint8_t)((r << 4) | c);
                        p++;
                    }
                }
            }
        }
        if (SKIP_DENSE && skipped && lane == 0) dense_tiles[atomicAdd(n_dense_tiles, 1u)] = (int)t;
    }
}

// ---------------------------------------------------------------------------
// Mixed precision (SPG_PREC_MIXED, FP32 data): every matched tile pair whose
// A and B tiles both hold >= dense_thr nonzeros is computed as a real
// 16x16x16 contraction on the tensor cores: mma.sync m16n8k16, FP16 operands,
// FP32 accumulation, each FP32 value split x = hi + lo (hi = fp16(x), lo =
// fp16(x - hi)) and hi*hi + hi*lo + lo*hi accumulated (the dropped lo*lo term
// is ~2^-22 relative).  tcgen05.mma needs M >= 64; one 16x16 tile pair fills
// a single m16n8k16 pair exactly, and stacking tile pairs to M = 64/128 would
// multiply mostly zero padding on these tile rows.  Two kernels: the plain
// register kernel writes every C tile from its sparse pairs (dense pairs
// skipped, tiles that had one listed), then the tensor kernel adds the listed
// tiles' dense pairs from fragments built once per dense tile.  A |A|*|B|
// magnitude product (hi parts) flags C tiles whose entries cancelled to below
// cancel_eps of their magnitude; those tiles are recomputed in FP64 by
// c3_fp64_list_kernel.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void mma16816(float* d, const uint32_t* a, const uint32_t* b) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// element (r, c) of a compressed tile: value if present, else 0
__device__ __forceinline__ float tile_elem(const float* __restrict__ vals, int base, uint32_t mask_r, int ptr_r,
                                           int c) {
    if (!((mask_r >> (15 - c)) & 1u)) return 0.f;
    return __ldg(&vals[base + ptr_r + __popc(mask_r >> (16 - c))]);
}

__device__ __forceinline__ void split2(float x0, float x1, uint32_t& hi, uint32_t& lo, uint32_t& ab) {
    const __half h0 = __float2half_rn(x0), h1 = __float2half_rn(x1);
    const __half l0 = __float2half_rn(x0 - __half2float(h0)), l1 = __float2half_rn(x1 - __half2float(h1));
    const __half2 H = __halves2half2(h0, h1), Lo = __halves2half2(l0, l1);
    hi = *reinterpret_cast<const uint32_t*>(&H);
    lo = *reinterpret_cast<const uint32_t*>(&Lo);
    const __half2 A = __habs2(H);
    ab = *reinterpret_cast<const uint32_t*>(&A);
}

// Dense tiles (>= dense_thr nonzeros) in mma.sync fragment form, built once
// per product: per tile and lane 12 words, read back with three coalesced
// 16-byte loads per pair instead of rebuilding the fragment from the
// compressed tile for every pair.
//   A (row operand, m16 x k16): ah[4], al[4], |a|[4] for rows g, g+8 and
//     columns 2q, 2q+1, 2q+8, 2q+9 (g = lane/4, q = lane%4);
//   B (column operand, k16 x n16): for n halves h = 0, 1: bh[2], bl[2], |b|[2]
//     for rows 2q, 2q+1, 2q+8, 2q+9 and column g + 8h.
__global__ void dense_flag_kernel(int64_t numtile, const int* __restrict__ tnnz, int dense_thr, int* __restrict__ flag) {
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < numtile; t += (int64_t)gridDim.x * blockDim.x)
        flag[t] = (tnnz[t + 1] - tnnz[t] >= dense_thr) ? 1 : 0;
}

template <bool IS_B>
__global__ void __launch_bounds__(256)
dense_frag_kernel(int64_t numtile, const int* __restrict__ tnnz, const float* __restrict__ val,
                  const uint8_t* __restrict__ ptr16, const uint16_t* __restrict__ mask, int dense_thr,
                  const int* __restrict__ slot, uint4* __restrict__ frag) {
    const int lane = threadIdx.x & 31, g = lane >> 2, tq = lane & 3;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t t = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; t < numtile; t += nw) {
        const int s0 = tnnz[t];
        if (tnnz[t + 1] - s0 < dense_thr) continue;
        uint32_t w[12];
        if (!IS_B) {
            const uint32_t m0 = mask[t * TS + g], m1 = mask[t * TS + g + 8];
            const int p0 = ptr16[t * TS + g], p1 = ptr16[t * TS + g + 8];
            const int c0 = 2 * tq;
            split2(tile_elem(val, s0, m0, p0, c0), tile_elem(val, s0, m0, p0, c0 + 1), w[0], w[4], w[8]);
            split2(tile_elem(val, s0, m1, p1, c0), tile_elem(val, s0, m1, p1, c0 + 1), w[1], w[5], w[9]);
            split2(tile_elem(val, s0, m0, p0, c0 + 8), tile_elem(val, s0, m0, p0, c0 + 9), w[2], w[6], w[10]);
            split2(tile_elem(val, s0, m1, p1, c0 + 8), tile_elem(val, s0, m1, p1, c0 + 9), w[3], w[7], w[11]);
        } else {
            const int k0 = 2 * tq;
            const uint32_t bm0 = mask[t * TS + k0], bm1 = mask[t * TS + k0 + 1];
            const uint32_t bm2 = mask[t * TS + k0 + 8], bm3 = mask[t * TS + k0 + 9];
            const int bp0 = ptr16[t * TS + k0], bp1 = ptr16[t * TS + k0 + 1];
            const int bp2 = ptr16[t * TS + k0 + 8], bp3 = ptr16[t * TS + k0 + 9];
#pragma unroll
            for (int nh = 0; nh < 2; nh++) {
                const int n = g + 8 * nh;
                split2(tile_elem(val, s0, bm0, bp0, n), tile_elem(val, s0, bm1, bp1, n), w[6 * nh + 0], w[6 * nh + 2],
                       w[6 * nh + 4]);
                split2(tile_elem(val, s0, bm2, bp2, n), tile_elem(val, s0, bm3, bp3, n), w[6 * nh + 1], w[6 * nh + 3],
                       w[6 * nh + 5]);
            }
        }
        uint4* dst = frag + ((int64_t)slot[t] * 32 + lane) * 3;
        dst[0] = make_uint4(w[0], w[1], w[2], w[3]);
        dst[1] = make_uint4(w[4], w[5], w[6], w[7]);
        dst[2] = make_uint4(w[8], w[9], w[10], w[11]);
    }
}

// Tensor part of SPG_PREC_MIXED, run after the register kernel has written
// every C tile from its sparse pairs: one warp per listed C tile (those with a
// pair of dense tiles) accumulates the dense pairs with mma.sync from the
// precomputed fragments (hi*hi + hi*lo + lo*hi, and |a|*|b| for the
// cancellation test), adds them to the tile's values and lists the tile for
// FP64 recomputation if an entry cancelled below cancel_eps of its magnitude.
template <bool CACHE>
__global__ void __launch_bounds__(256)
c3_tensor_kernel(int ntiles, const int* __restrict__ tiles, const int* __restrict__ rowidxC,
                 const int* __restrict__ colidxC, const int* __restrict__ a_tp, const int* __restrict__ a_tc,
                 const int* __restrict__ a_tnnz, const int* __restrict__ b_cscp, const int* __restrict__ b_cscr,
                 const int* __restrict__ b_tnnz, const int64_t* __restrict__ tile_nnzC,
                 const uint16_t* __restrict__ maskC, const uint8_t* __restrict__ ptrRowC, float* __restrict__ valC,
                 const int* __restrict__ spec_cnt, const int* __restrict__ spec_off, const int* __restrict__ spec_pa,
                 const int* __restrict__ spec_pb, int dense_thr, float cancel_eps,
                 unsigned long long* __restrict__ tensor_pairs, int* __restrict__ flag_list,
                 unsigned* __restrict__ nflag, const uint4* __restrict__ fragA, const int* __restrict__ slotA,
                 const uint4* __restrict__ fragB, const int* __restrict__ slotB) {
    __shared__ float s_tile[8][TS][TS + 1];
    __shared__ float s_mag[8][TS][TS + 1];
    const int lane = threadIdx.x & 31, r = lane & 15, hsel = lane >> 4;
    const int g = lane >> 2, tq = lane & 3;
    const int wib = threadIdx.x >> 5;
    unsigned long long my_tensor = 0;
    const int nwarps = gridDim.x * (blockDim.x >> 5);
    for (int w = blockIdx.x * (blockDim.x >> 5) + wib; w < ntiles; w += nwarps) {
        const int64_t t = tiles[w];
        float d[8], mg[8];
#pragma unroll
        for (int q = 0; q < 8; q++) { d[q] = 0.f; mg[q] = 0.f; }
        auto do_pair = [&](int pa, int pb) {
            if (__ldg(&a_tnnz[pa + 1]) - __ldg(&a_tnnz[pa]) < dense_thr ||
                __ldg(&b_tnnz[pb + 1]) - __ldg(&b_tnnz[pb]) < dense_thr)
                return;
            __syncwarp();  // mma.sync.aligned: the whole warp converged
            if (lane == 0) my_tensor++;
            const uint4* fa = fragA + ((int64_t)__ldg(&slotA[pa]) * 32 + lane) * 3;
            const uint4* fb = fragB + ((int64_t)__ldg(&slotB[pb]) * 32 + lane) * 3;
            const uint4 a0 = __ldg(fa), a1 = __ldg(fa + 1), a2 = __ldg(fa + 2);
            const uint4 b0 = __ldg(fb), b1 = __ldg(fb + 1), b2 = __ldg(fb + 2);
            const uint32_t ah[4] = {a0.x, a0.y, a0.z, a0.w}, al[4] = {a1.x, a1.y, a1.z, a1.w};
            const uint32_t aa[4] = {a2.x, a2.y, a2.z, a2.w};
            const uint32_t bw[12] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w, b2.x, b2.y, b2.z, b2.w};
#pragma unroll
            for (int nh = 0; nh < 2; nh++) {
                const uint32_t* bb = bw + 6 * nh;  // bh[2], bl[2], |b|[2]
                mma16816(d + 4 * nh, ah, bb);
                mma16816(d + 4 * nh, ah, bb + 2);
                mma16816(d + 4 * nh, al, bb);
                mma16816(mg + 4 * nh, aa, bb + 4);
            }
        };
        int cnt = CACHE ? spec_cnt[t] : -1;
        if (cnt >= 0) {
            const int off = spec_off[t];
            for (int q = 0; q < cnt; q++) do_pair(spec_pa[off + q], spec_pb[off + q]);
        } else {
            const int bi = rowidxC[t], bj = colidxC[t];
            const int as = a_tp[bi], ae = a_tp[bi + 1];
            const int bs = b_cscp[bj], be = b_cscp[bj + 1];
            const bool a_short = (ae - as) <= (be - bs);
            const int ss = a_short ? as : bs, se = a_short ? ae : be;
            const int ls = a_short ? bs : as, le = a_short ? be : ae;
            const int* sl = a_short ? a_tc : b_cscr;
            const int* ll = a_short ? b_cscr : a_tc;
            for (int base = ss; base < se; base += 32) {
                const int idx = base + lane;
                int pos = -1;
                if (idx < se) {
                    const int key = __ldg(&sl[idx]);
                    const int p = lower_bound_dev(ll, ls, le, key);
                    if (p < le && __ldg(&ll[p]) == key) pos = p;
                }
                unsigned mm = __ballot_sync(0xffffffffu, pos >= 0);
                while (mm) {
                    const int src = __ffs(mm) - 1;
                    mm &= mm - 1u;
                    const int sp = __shfl_sync(0xffffffffu, idx, src);
                    const int lp = __shfl_sync(0xffffffffu, pos, src);
                    do_pair(a_short ? sp : lp, a_short ? lp : sp);
                }
            }
        }
#pragma unroll
        for (int nh = 0; nh < 2; nh++) {
            const int c = 2 * tq + 8 * nh;
            s_tile[wib][g][c] = d[4 * nh + 0];
            s_tile[wib][g][c + 1] = d[4 * nh + 1];
            s_tile[wib][g + 8][c] = d[4 * nh + 2];
            s_tile[wib][g + 8][c + 1] = d[4 * nh + 3];
            s_mag[wib][g][c] = mg[4 * nh + 0];
            s_mag[wib][g][c + 1] = mg[4 * nh + 1];
            s_mag[wib][g + 8][c] = mg[4 * nh + 2];
            s_mag[wib][g + 8][c + 1] = mg[4 * nh + 3];
        }
        __syncwarp();
        int flagged = 0;
        if (hsel == 0) {
            const uint32_t mc = maskC[t * TS + r];
            int64_t p = tile_nnzC[t] + ptrRowC[t * TS + r];
#pragma unroll
            for (int c = 0; c < TS; c++) {
                if (mc & (0x8000u >> c)) {
                    const float v = valC[p] + s_tile[wib][r][c];
                    const float mag = s_mag[wib][r][c];
                    if (mag > 0.f && fabsf(v) < cancel_eps * mag) flagged = 1;
                    valC[p] = v;
                    p++;
                }
            }
        }
        if (__any_sync(0xffffffffu, flagged) && lane == 0) flag_list[atomicAdd(nflag, 1u)] = (int)t;
        __syncwarp();
    }
    my_tensor = warp_sum(my_tensor);
    if (lane == 0 && my_tensor) atomicAdd(tensor_pairs, my_tensor);
}

// FP64 recomputation of the flagged C tiles (warp per tile, FP32 data).
__global__ void __launch_bounds__(256)
c3_fp64_list_kernel(int nlist, const int* __restrict__ list, const int* __restrict__ rowidxC,
                    const int* __restrict__ colidxC, const int* __restrict__ a_tp, const int* __restrict__ a_tc,
                    const int* __restrict__ a_tnnz, const float* __restrict__ a_val, const uint8_t* __restrict__ a_col,
                    const uint8_t* __restrict__ a_ptr16, const int* __restrict__ b_cscp, const int* __restrict__ b_cscr,
                    const int* __restrict__ b_tnnz, const float* __restrict__ b_val,
                    const uint8_t* __restrict__ b_ptr16, const uint16_t* __restrict__ b_mask,
                    const int64_t* __restrict__ tile_nnzC, const uint16_t* __restrict__ maskC,
                    const uint8_t* __restrict__ ptrRowC, float* __restrict__ valC) {
    const int lane = threadIdx.x & 31, r = lane & 15, hsel = lane >> 4;
    const int nw = gridDim.x * (blockDim.x >> 5);
    for (int w = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); w < nlist; w += nw) {
        const int64_t t = list[w];
        double acc[TS];
#pragma unroll
        for (int c = 0; c < TS; c++) acc[c] = 0.0;
        const int bi = rowidxC[t], bj = colidxC[t];
        int a = a_tp[bi];
        const int ae = a_tp[bi + 1];
        int b = b_cscp[bj];
        const int be = b_cscp[bj + 1];
        while (a < ae && b < be) {  // merge of the two sorted tile lists, warp-uniform
            const int ka = __ldg(&a_tc[a]), kb = __ldg(&b_cscr[b]);
            if (ka < kb) { a++; continue; }
            if (kb < ka) { b++; continue; }
            const int sA = __ldg(&a_tnnz[a]), na = __ldg(&a_tnnz[a + 1]) - sA;
            const int rs = __ldg(&a_ptr16[(int64_t)a * TS + r]);
            const int re = (r == TS - 1) ? na : (int)__ldg(&a_ptr16[(int64_t)a * TS + r + 1]);
            const int sB = __ldg(&b_tnnz[b]);
            for (int e = rs + hsel; e < re; e += 2) {
                const int kk = __ldg(&a_col[sA + e]) & 15;
                const double va = __ldg(&a_val[sA + e]);
                const uint32_t mb = __ldg(&b_mask[(int64_t)b * TS + kk]);
                int off = sB + __ldg(&b_ptr16[(int64_t)b * TS + kk]);
#pragma unroll
                for (int c = 0; c < TS; c++) {
                    if (mb & (0x8000u >> c)) {
                        acc[c] = fma(va, (double)__ldg(&b_val[off]), acc[c]);
                        off++;
                    }
                }
            }
            a++;
            b++;
        }
#pragma unroll
        for (int c = 0; c < TS; c++) acc[c] += __shfl_xor_sync(0xffffffffu, acc[c], 16);
        if (hsel == 0) {
            const uint32_t mc = maskC[t * TS + r];
            int64_t p = tile_nnzC[t] + ptrRowC[t * TS + r];
#pragma unroll
            for (int c = 0; c < TS; c++)
                if (mc & (0x8000u >> c)) valC[p++] = (float)acc[c];
        }
    }
}

__global__ void i64_to_i32_kernel(const int64_t* __restrict__ in, int* __restrict__ out, int64_t n) {
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x)
        out[t] = (int)in[t];
}

int grid_cap(spg_handle_t h, int64_t units, int per_block, int per_sm) {
    int64_t g = ceil_div(units, per_block);
    const int64_t cap = (int64_t)h->num_sms * per_sm;
    if (g > cap) g = cap;
    return (int)(g < 1 ? 1 : g);
}

// B's occupied tile columns as an exclusive prefix (tilen + 1 entries), for
// step 1's saturation exit; built for products of at least 65,536 A tiles
// (two launches are noise there), null below.
spg_status occupied_prefix(spg_handle_t h, const spg_tiles* A, const spg_tiles* B, ScratchList& sc, int** occ) {
    *occ = nullptr;
    if (A->numtile < 65536 || B->tilen <= 0 || !B->csc_tile_ptr) return SPG_OK;
    SPG_TRY(sc.alloc(occ, (size_t)B->tilen + 1));
    occupied_cols_kernel<<<grid_cap(h, B->tilen, 256, 8), 256, 0, h->stream>>>(B->tilen, B->csc_tile_ptr, *occ);
    SPG_LAUNCHED(h);
    return spg_scan_i32_to_i32(h, *occ, *occ, B->tilen);
}

// C's tile count and step 1's tile pairs (C->pairs) in one round trip,
// with step 1's device errors.
spg_status read_tiles_and_pairs(spg_handle_t h, const int64_t* d_numtile, const unsigned long long* pairs_total,
                                spg_ctiles* C, int64_t* numtileC) {
    const int64_t* src[2] = {d_numtile, reinterpret_cast<const int64_t*>(pairs_total)};
    int64_t v[2] = {0, 0};
    SPG_TRY(spg_read_i64s_checked(h, 2, src, v, "symbolic step 1"));
    if (v[0] > 0x7fffffffLL) return spg_fail(h, SPG_ERR_INVALID, "C has more than 2^31-1 tiles");
    *numtileC = v[0];
    C->numtileC = v[0];
    C->pairs = v[1];
    return SPG_OK;
}



}  // namespace

spg_status plain_step1(spg_handle_t h, const spg_tiles* A, const spg_tiles* B, spg_ctiles* C,
                       int64_t* row_pairs, unsigned long long* pairs_total) {
    const int tilem = A->tilem;
    const int nwords = (B->tilen + 31) / 32;
    const size_t smem = sizeof(uint32_t) * (size_t)nwords;
    if (smem > h->smem_optin)
        return spg_fail(h, SPG_ERR_UNSUPPORTED, "step 1: B has too many tile columns for one bitmap");
    SPG_CUDA(h, cudaFuncSetAttribute(c1_count_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    SPG_CUDA(h, cudaFuncSetAttribute(c1_fill_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    ScratchList sc(h);
    int* cnt = nullptr;
    int64_t* ptr64 = nullptr;
    int* occ = nullptr;
    SPG_TRY(sc.alloc(&cnt, (size_t)tilem + 1));
    SPG_TRY(sc.alloc(&ptr64, (size_t)tilem + 1));
    SPG_TRY(occupied_prefix(h, A, B, sc, &occ));
    if (tilem > 0) {
        c1_count_kernel<<<tilem, C1_THREADS, smem, h->stream>>>(nwords, A->tile_ptr, A->tile_columnidx,
                                                               B->tile_ptr, B->tile_columnidx, cnt, row_pairs,
                                                               pairs_total, occ);
        SPG_LAUNCHED(h);
    }
    SPG_TRY(spg_scan_i32_to_i64(h, cnt, ptr64, tilem));
    int64_t numtileC = 0;
    SPG_TRY(read_tiles_and_pairs(h, ptr64 + tilem, pairs_total, C, &numtileC));
    SPG_TRY(spg_alloc_t(h, &C->tile_ptrC, (size_t)tilem + 1));
    i64_to_i32_kernel<<<grid_cap(h, tilem + 1, 256, 8), 256, 0, h->stream>>>(ptr64, C->tile_ptrC, tilem + 1);
    SPG_LAUNCHED(h);
    SPG_TRY(spg_alloc_t(h, &C->tile_rowidxC, (size_t)numtileC + 1));
    SPG_TRY(spg_alloc_t(h, &C->tile_colidxC, (size_t)numtileC + 1));
    if (tilem > 0 && numtileC > 0) {
        c1_fill_kernel<<<tilem, C1_THREADS, smem, h->stream>>>(nwords, A->tile_ptr, A->tile_columnidx, B->tile_ptr,
                                                              B->tile_columnidx, C->tile_ptrC, C->tile_rowidxC,
                                                              C->tile_colidxC, nullptr, occ);
        SPG_LAUNCHED(h);
    }
    return SPG_OK;
}

// Step 1 with learned sizing: slot_sz[i] is the predicted tile count of
// tile-row i (with margin).  Slots are laid out by a scan, filled in one
// bitmap pass, then compacted into C's exact arrays; rows whose prediction
// was too small re-run the exact fill.  The structure is exact whatever the
// prediction.
spg_status plain_step1_sized(spg_handle_t h, const spg_tiles* A, const spg_tiles* B, spg_ctiles* C,
                             int64_t* row_pairs, unsigned long long* pairs_total, const int* slot_sz) {
    const int tilem = A->tilem;
    const int nwords = (B->tilen + 31) / 32;
    const size_t smem = sizeof(uint32_t) * (size_t)nwords;
    if (smem > h->smem_optin)
        return spg_fail(h, SPG_ERR_UNSUPPORTED, "step 1: B has too many tile columns for one bitmap");
    SPG_CUDA(h, cudaFuncSetAttribute(c1_slot_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    SPG_CUDA(h, cudaFuncSetAttribute(c1_fill_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    ScratchList sc(h);
    int64_t* slot_off = nullptr;
    SPG_TRY(sc.alloc(&slot_off, (size_t)tilem + 1));
    SPG_TRY(spg_scan_i32_to_i64(h, slot_sz, slot_off, tilem));
    int64_t cap = 0;
    SPG_TRY(spg_read_i64(h, slot_off + tilem, &cap));
    h->stats.predicted_tiles = cap;
    {   // an optional cap on the staging (SPG_SLOT_BUDGET_BYTES); without one
        // the staging takes what the pool gives, and an allocation that fails
        // sends the caller to the exact two passes, which need no staging
        if (const char* e = getenv("SPG_SLOT_BUDGET_BYTES"))
            if ((unsigned long long)cap * sizeof(int) > strtoull(e, nullptr, 10))
                return spg_fail(h, SPG_ERR_OOM, "step 1: predicted slots exceed the staging budget");
    }
    int* slot_col = nullptr;
    int* cnt = nullptr;
    int64_t* ptr64 = nullptr;
    int* occ = nullptr;
    SPG_TRY(spg_workspace(h, SPG_WS_SLOTS, sizeof(int) * ((size_t)cap + 1), reinterpret_cast<void**>(&slot_col)));
    SPG_TRY(sc.alloc(&cnt, (size_t)tilem + 1));
    SPG_TRY(sc.alloc(&ptr64, (size_t)tilem + 1));
    SPG_TRY(occupied_prefix(h, A, B, sc, &occ));
    if (tilem > 0) {
        c1_slot_kernel<<<tilem, C1_THREADS, smem, h->stream>>>(A->tile_ptr, A->tile_columnidx, B->tile_ptr,
                                                              B->tile_columnidx, slot_off, slot_col, cnt, row_pairs,
                                                              pairs_total, occ);
        SPG_LAUNCHED(h);
    }
    SPG_TRY(spg_scan_i32_to_i64(h, cnt, ptr64, tilem));
    int64_t numtileC = 0;
    SPG_TRY(read_tiles_and_pairs(h, ptr64 + tilem, pairs_total, C, &numtileC));
    SPG_TRY(spg_alloc_t(h, &C->tile_ptrC, (size_t)tilem + 1));
    i64_to_i32_kernel<<<grid_cap(h, tilem + 1, 256, 8), 256, 0, h->stream>>>(ptr64, C->tile_ptrC, tilem + 1);
    SPG_LAUNCHED(h);
    SPG_TRY(spg_alloc_t(h, &C->tile_rowidxC, (size_t)numtileC + 1));
    SPG_TRY(spg_alloc_t(h, &C->tile_colidxC, (size_t)numtileC + 1));
    int* over_rows = cnt;  // reused: counts are no longer needed
    unsigned* n_over = reinterpret_cast<unsigned*>(ptr64);
    SPG_CUDA(h, cudaMemsetAsync(n_over, 0, sizeof(unsigned), h->stream));
    if (tilem > 0 && numtileC > 0) {
        c1_compact_kernel<<<grid_cap(h, (int64_t)tilem * 32, 256, 16), 256, 0, h->stream>>>(
            tilem, C->tile_ptrC, slot_off, slot_col, C->tile_rowidxC, C->tile_colidxC, over_rows, n_over);
        SPG_LAUNCHED(h);
        int nov = 0;
        SPG_TRY(spg_read_i32(h, reinterpret_cast<const int*>(n_over), &nov));
        if (nov > 0) {  // prediction too small for these rows: exact fill of just them
            h->stats.overflow_reruns += nov;
            c1_fill_kernel<<<nov, C1_THREADS, smem, h->stream>>>(nwords, A->tile_ptr, A->tile_columnidx, B->tile_ptr,
                                                                B->tile_columnidx, C->tile_ptrC, C->tile_rowidxC,
                                                                C->tile_colidxC, over_rows, occ);
            SPG_LAUNCHED(h);
        }
    }
    return SPG_OK;
}

// Step 2 over C's tiles, or over the listed ones (tlist: nlist ascending tile
// indices); each tile's nonzero count goes to cnt32[t] or, when cnt32 is
// null, to cnt64[t].
template <typename CNT, bool LIST>
static void launch_c2(spg_handle_t h, const spg_tiles* A, const spg_tiles* B, spg_ctiles* C, PlainPriv* pp,
                      int64_t nt, const int* tlist, CNT* cnt, int grid) {
    unsigned long long* ctr = pp->counters;
    if (pp->spec_cap > 0)
        c2_symbolic_kernel<true, CNT, LIST><<<grid, 128, 0, h->stream>>>(
            nt, tlist, C->tile_rowidxC, C->tile_colidxC, A->tile_ptr, A->tile_columnidx, A->tile_nnz,
            A->tile_csr_Col, A->tile_csr_Ptr, B->csc_tile_ptr, B->csc_tile_rowidx, B->mask, C->maskC, C->ptrRowC, cnt,
            pp->spec_cnt, pp->spec_off, pp->spec_pa, pp->spec_pb, pp->spec_cap, ctr, ctr + 1, h->d_flags);
    else
        c2_symbolic_kernel<false, CNT, LIST><<<grid, 128, 0, h->stream>>>(
            nt, tlist, C->tile_rowidxC, C->tile_colidxC, A->tile_ptr, A->tile_columnidx, A->tile_nnz,
            A->tile_csr_Col, A->tile_csr_Ptr, B->csc_tile_ptr, B->csc_tile_rowidx, B->mask, C->maskC, C->ptrRowC, cnt,
            nullptr, nullptr, nullptr, nullptr, 0, ctr, ctr + 1, h->d_flags);
}

spg_status plain_step2(spg_handle_t h, const spg_tiles* A, const spg_tiles* B, spg_ctiles* C, PlainPriv* pp,
                       int* cnt32, int64_t* cnt64, const int* tlist, int64_t nlist) {
    const int64_t nt = tlist ? nlist : C->numtileC;
    unsigned long long* ctr = pp->counters;  // [0] alloc, [1] pairs
    SPG_CUDA(h, cudaMemsetAsync(ctr, 0, 2 * sizeof(unsigned long long), h->stream));
    if (nt == 0) return SPG_OK;
    const int grid = grid_cap(h, nt, 8, 64);
    for (int attempt = 0; attempt < 2; attempt++) {
        if (cnt32 && !tlist)
            launch_c2<int, false>(h, A, B, C, pp, nt, nullptr, cnt32, grid);
        else if (cnt32)
            launch_c2<int, true>(h, A, B, C, pp, nt, tlist, cnt32, grid);
        else if (!tlist)
            launch_c2<int64_t, false>(h, A, B, C, pp, nt, nullptr, cnt64, grid);
        else
            launch_c2<int64_t, true>(h, A, B, C, pp, nt, tlist, cnt64, grid);
        SPG_LAUNCHED(h);
        if (pp->spec_cap == 0) break;
        // overflow re-run (src/spgemm_raw_v2.cu:191-200, with the bound honoured in-kernel)
        int64_t used = 0;
        const int64_t* src[1] = {(const int64_t*)ctr};
        const spg_status rs = spg_read_i64s_checked(h, 1, src, &used, "symbolic step 2");
        if (rs == SPG_OK) break;                      // no overflow
        if (rs != SPG_ERR_OVERFLOW_RERUN) return rs;  // another device error
        used = h->h_pinned[8];
        h->stats.overflow_reruns++;
        spg_free_async(h, pp->spec_pa);
        spg_free_async(h, pp->spec_pb);
        pp->spec_pa = pp->spec_pb = nullptr;
        size_t fr = 0, tot = 0;
        if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) fr = 0;
        if (attempt == 0 && (size_t)used * 8 < fr / 2) {
            pp->spec_cap = used;
            SPG_TRY(spg_alloc_t(h, &pp->spec_pa, (size_t)used + 1));
            SPG_TRY(spg_alloc_t(h, &pp->spec_pb, (size_t)used + 1));
            SPG_CUDA(h, cudaMemsetAsync(ctr, 0, 2 * sizeof(unsigned long long), h->stream));
        } else {
            pp->spec_cap = 0;  // numeric recomputes the intersections
            SPG_CUDA(h, cudaMemsetAsync(ctr, 0, 2 * sizeof(unsigned long long), h->stream));
        }
    }
    return SPG_OK;
}

// The per-C-tile arrays seen from tile t0 on: the kernels index them by the
// tile's position in [t0, t1) and reach values and column bytes through the
// absolute nonzero prefix, so a tile range needs no other change.
struct CTileView {
    const int* rowidx;
    const int* colidx;
    const int64_t* nnz;
    const uint16_t* mask;
    const uint8_t* ptr16;
    const int* spec_cnt;
    const int* spec_off;
};

static CTileView ctile_view(const spg_ctiles* C, const PlainPriv* pp, int64_t t0) {
    const bool cache = pp && pp->spec_cap > 0;
    return CTileView{C->tile_rowidxC + t0, C->tile_colidxC + t0, C->tile_nnzC + t0, C->maskC + t0 * TS,
                     C->ptrRowC + t0 * TS, cache ? pp->spec_cnt + t0 : nullptr,
                     cache ? pp->spec_off + t0 : nullptr};
}

template <typename V>
static spg_status plain_step3_t(spg_handle_t h, const spg_tiles* A, const spg_tiles* B, spg_ctiles* C,
                                PlainPriv* pp, int64_t t0, int64_t t1, const int* tlist) {
    const int64_t nt = t1 - t0;
    if (nt <= 0 || C->nnzC == 0) return SPG_OK;
    // a tile range is a view of C's arrays from t0; listed tiles index C whole
    const CTileView cv = ctile_view(C, pp, tlist ? 0 : t0);
    const int* lst = tlist ? tlist + t0 : nullptr;
    const int grid = grid_cap(h, nt, 8, 32);
    const bool cache = pp && pp->spec_cap > 0;
#define C3_ARGS(SPEC)                                                                                              \
    nt, lst, cv.rowidx, cv.colidx, A->tile_ptr, A->tile_columnidx, A->tile_nnz, (const V*)A->tile_csr_Val,          \
        A->tile_csr_Col, A->tile_csr_Ptr, B->csc_tile_ptr, B->csc_tile_rowidx, B->tile_nnz,                          \
        (const V*)B->tile_csr_Val, B->tile_csr_Ptr, B->mask, cv.nnz, cv.mask, cv.ptr16, (V*)C->tile_valC,            \
        C->tile_colC, SPEC
#define C3_SPEC cv.spec_cnt, cv.spec_off, pp->spec_pa, pp->spec_pb
#define C3_NOSPEC nullptr, nullptr, nullptr, nullptr
    // the list is a template flag: the whole-range kernel keeps its registers
    if (cache && lst)
        c3_numeric_kernel<V, true, false, true><<<grid, 256, 0, h->stream>>>(C3_ARGS(C3_SPEC));
    else if (cache)
        c3_numeric_kernel<V, true, false, false><<<grid, 256, 0, h->stream>>>(C3_ARGS(C3_SPEC));
    else if (lst)
        c3_numeric_kernel<V, false, false, true><<<grid, 256, 0, h->stream>>>(C3_ARGS(C3_NOSPEC));
    else
        c3_numeric_kernel<V, false, false, false><<<grid, 256, 0, h->stream>>>(C3_ARGS(C3_NOSPEC));
#undef C3_ARGS
#undef C3_SPEC
#undef C3_NOSPEC
    SPG_LAUNCHED(h);
    return SPG_OK;
}

spg_status plain_step3(spg_handle_t h, const spg_tiles* A, const spg_tiles* B, spg_ctiles* C, PlainPriv* pp,
                       int64_t t0, int64_t t1, const int* tlist) {
    if (t1 < 0) t1 = C->numtileC;
    if (A->dtype == SPG_F64) return plain_step3_t<double>(h, A, B, C, pp, t0, t1, tlist);
    return plain_step3_t<float>(h, A, B, C, pp, t0, t1, tlist);
}

// Mixed-precision numeric (FP32 data): dense tile pairs on tensor cores, the
// rest on FP32 registers, cancellation-flagged C tiles recomputed in FP64.
spg_status plain_step3_mixed(spg_handle_t h, const spg_tiles* A, const spg_tiles* B, spg_ctiles* C, PlainPriv* pp,
                             int dense_thr, float cancel_eps, int64_t t0, int64_t t1) {
    if (t1 < 0) t1 = C->numtileC;
    const int64_t nt = t1 - t0;
    if (nt <= 0 || C->nnzC == 0) return SPG_OK;
    const CTileView cv = ctile_view(C, pp, t0);
    if (A->dtype != SPG_F32) return spg_fail(h, SPG_ERR_INVALID, "mixed precision needs FP32 data");
    unsigned long long* ctr = nullptr;
    int* list = nullptr;
    SPG_TRY(spg_alloc_t(h, &ctr, 2));  // [0] tensor pairs, [1] low word: flagged tiles, high word: dense tiles
    SPG_TRY(spg_alloc_t(h, &list, (size_t)nt + 1));
    SPG_CUDA(h, cudaMemsetAsync(ctr, 0, 16, h->stream));
    // dense tiles of A (row order) and B (CSC order) into fragment form
    int *slotA = nullptr, *slotB = nullptr;
    uint4 *fragA = nullptr, *fragB = nullptr;
    auto build = [&](const spg_tiles* T, bool is_b, int** slot, uint4** frag) -> spg_status {
        const int64_t n = T->numtile;
        SPG_TRY(spg_alloc_t(h, slot, (size_t)n + 1));
        if (n > 0) {
            dense_flag_kernel<<<grid_cap(h, n, 256, 8), 256, 0, h->stream>>>(n, T->tile_nnz, dense_thr, *slot);
            SPG_LAUNCHED(h);
        }
        SPG_TRY(spg_scan_i32_to_i32(h, *slot, *slot, n));
        int nd = 0;
        SPG_TRY(spg_read_i32(h, *slot + n, &nd));
        SPG_TRY(spg_alloc_t(h, frag, (size_t)nd * 32 * 3 + 1));
        if (nd > 0) {
            if (is_b)
                dense_frag_kernel<true><<<grid_cap(h, n * 32, 256, 16), 256, 0, h->stream>>>(
                    n, T->tile_nnz, (const float*)T->tile_csr_Val, T->tile_csr_Ptr, T->mask, dense_thr, *slot, *frag);
            else
                dense_frag_kernel<false><<<grid_cap(h, n * 32, 256, 16), 256, 0, h->stream>>>(
                    n, T->tile_nnz, (const float*)T->tile_csr_Val, T->tile_csr_Ptr, T->mask, dense_thr, *slot, *frag);
            SPG_LAUNCHED(h);
        }
        return SPG_OK;
    };
    SPG_TRY(build(A, false, &slotA, &fragA));
    SPG_TRY(build(B, true, &slotB, &fragB));
    const int grid = grid_cap(h, nt, 8, 32);
    const bool cache = pp && pp->spec_cap > 0;
    // 1. every C tile from its sparse pairs on FP32 registers (the plain
    //    kernel, dense pairs skipped); tiles with a dense pair are listed
    int* dense_tiles = nullptr;
    unsigned* n_dense = reinterpret_cast<unsigned*>(ctr) + 3;  // high word of ctr[1]
    SPG_TRY(spg_alloc_t(h, &dense_tiles, (size_t)nt + 1));
#define REG_ARGS                                                                                                    \
    nt, nullptr, cv.rowidx, cv.colidx, A->tile_ptr, A->tile_columnidx, A->tile_nnz, (const float*)A->tile_csr_Val,          \
        A->tile_csr_Col, A->tile_csr_Ptr, B->csc_tile_ptr, B->csc_tile_rowidx, B->tile_nnz,                        \
        (const float*)B->tile_csr_Val, B->tile_csr_Ptr, B->mask, cv.nnz, cv.mask, cv.ptr16,                        \
        (float*)C->tile_valC, C->tile_colC
    if (cache)
        c3_numeric_kernel<float, true, true><<<grid, 256, 0, h->stream>>>(
            REG_ARGS, cv.spec_cnt, cv.spec_off, pp->spec_pa, pp->spec_pb, dense_thr, dense_tiles, n_dense);
    else
        c3_numeric_kernel<float, false, true><<<grid, 256, 0, h->stream>>>(REG_ARGS, nullptr, nullptr, nullptr, nullptr,
                                                                           dense_thr, dense_tiles, n_dense);
#undef REG_ARGS
    SPG_LAUNCHED(h);
    int nd_tiles = 0;
    SPG_TRY(spg_read_i32(h, reinterpret_cast<const int*>(n_dense), &nd_tiles));
    // 2. the listed tiles' dense pairs on tensor cores, added to their values
    if (nd_tiles > 0) {
        const int g2 = grid_cap(h, nd_tiles, 8, 32);
#define TENSOR_ARGS                                                                                                \
    nd_tiles, dense_tiles, cv.rowidx, cv.colidx, A->tile_ptr, A->tile_columnidx, A->tile_nnz,                        \
        B->csc_tile_ptr, B->csc_tile_rowidx, B->tile_nnz, cv.nnz, cv.mask, cv.ptr16, (float*)C->tile_valC
        if (cache)
            c3_tensor_kernel<true><<<g2, 256, 0, h->stream>>>(TENSOR_ARGS, cv.spec_cnt, cv.spec_off, pp->spec_pa,
                                                               pp->spec_pb, dense_thr, cancel_eps, ctr, list,
                                                               reinterpret_cast<unsigned*>(ctr + 1), fragA, slotA,
                                                               fragB, slotB);
        else
            c3_tensor_kernel<false><<<g2, 256, 0, h->stream>>>(TENSOR_ARGS, nullptr, nullptr, nullptr, nullptr,
                                                                dense_thr, cancel_eps, ctr, list,
                                                                reinterpret_cast<unsigned*>(ctr + 1), fragA, slotA,
                                                                fragB, slotB);
#undef TENSOR_ARGS
    }
    spg_free_async(h, dense_tiles);
    SPG_LAUNCHED(h);
    int64_t v[2] = {0, 0};
    SPG_CUDA(h, cudaMemcpyAsync(h->h_pinned + 20, ctr, 16, cudaMemcpyDeviceToHost, h->stream));
    SPG_CUDA(h, cudaStreamSynchronize(h->stream));
    v[0] = h->h_pinned[20];
    v[1] = (int64_t)(uint32_t)h->h_pinned[21];
    h->stats.tensor_pairs = v[0];
    h->stats.fp64_tiles = v[1];
    if (v[1] > 0) {
        const int g2 = grid_cap(h, v[1], 8, 32);
        c3_fp64_list_kernel<<<g2, 256, 0, h->stream>>>(
            (int)v[1], list, cv.rowidx, cv.colidx, A->tile_ptr, A->tile_columnidx, A->tile_nnz,
            (const float*)A->tile_csr_Val, A->tile_csr_Col, A->tile_csr_Ptr, B->csc_tile_ptr, B->csc_tile_rowidx,
            B->tile_nnz, (const float*)B->tile_csr_Val, B->tile_csr_Ptr, B->mask, cv.nnz, cv.mask,
            cv.ptr16, (float*)C->tile_valC);
        SPG_LAUNCHED(h);
    }
    spg_free_async(h, ctr);
    spg_free_async(h, list);
    spg_free_async(h, slotA);
    spg_free_async(h, slotB);
    spg_free_async(h, fragA);
    spg_free_async(h, fragB);
    return SPG_OK;
}
