// tiler.cu -- device CSR -> 16x16 tile conversion.
//
// Produces exactly the arrays of csr2tile (src/tile_format.h:93-222) for the
// row-major layout and of csr2tile + build_csc_tiles (src/tile_format.h:424-585)
// for B's CSC tile order.  The reference does this on one host thread with
// std::sort per tile-row; here every tile-row is a thread block:
//
//   tiler_class   tile-rows classed: empty, narrow (one warp each), wide (one
//                 thread block each)
//   tiler_count   shared-memory bitmap over tile columns -> #tiles
//   (scan)        tile_ptr
//   tiler_fill    rebuild bitmap, word-prefix ranks -> sorted tile_columnidx;
//                 per nonzero: tile index by rank, position inside its
//                 (row, tile) segment; segment heads write the row count and
//                 the 16-bit row mask
//   tile_rowscan  one thread per tile: 128-bit load of the 16 row counts,
//                 exclusive scan in registers -> tile_csr_Ptr, tile nnz
//   (scan)        tile_nnz
//   [B only]      stable radix sort of tiles by tile column -> CSC tile order
//   tiler_scatter one thread per nonzero: value and column byte to their slot
//
// Inputs must be canonical CSR (columns strictly ascending inside each row);
// violations raise DERR_NONCANONICAL and the call fails with SPG_ERR_INVALID.
#include "spg_common.cuh"

namespace {

constexpr int TL_THREADS = 256;
constexpr int TL_WARPS = TL_THREADS / 32;
constexpr int TL_MAX_WORDS = 16384;  // tilen <= 524288 (n <= 8,388,608)

__device__ __forceinline__ uint16_t colbit(int c) { return (uint16_t)(0x8000u >> (c & 15)); }

// Tile-rows are classed once per tiling: an empty one gets its count of 0
// here; a narrow one (at most TL_NARROW_NNZ nonzeros over at most
// TL_NARROW_WORDS bitmap words of tile columns -- stencils, aggregation
// operators) is tiled by one warp; the rest (power-law rows spanning the
// matrix) by one thread block each.  The lists are unordered: counts and
// positions come from the tile-row index.
constexpr int TL_NARROW_WORDS = 128;
constexpr int TL_NARROW_NNZ = 4096;

__global__ void tiler_class_kernel(int tilem, int m, const int* __restrict__ rp, const int* __restrict__ ci,
                                   int* __restrict__ tile_cnt, int* __restrict__ narrow, int* __restrict__ wide,
                                   int* __restrict__ n_lists) {
    const int lane = threadIdx.x & 31;
    for (int i0 = blockIdx.x * blockDim.x; i0 < tilem; i0 += gridDim.x * blockDim.x) {
        const int i = i0 + (int)threadIdx.x;
        int cls = -1;  // -1 none, 0 narrow, 1 wide
        if (i < tilem) {
            const int r0 = i * TS, r1 = min(r0 + TS, m);
            if (rp[r0] == rp[r1]) {
                tile_cnt[i] = 0;
            } else {
                int lo = 0x7fffffff, hi = -1;
                for (int r = r0; r < r1; r++) {
                    const int s = rp[r], e = rp[r + 1];
                    if (e > s) { lo = min(lo, ci[s]); hi = max(hi, ci[e - 1]); }
                }
                // columns outside [0, n) or out of order are caught by the count passes
                const int nwd = (max(hi, 0) >> 9) - (max(lo, 0) >> 9) + 1;
                cls = (rp[r1] - rp[r0] <= TL_NARROW_NNZ && nwd <= TL_NARROW_WORDS && lo >= 0) ? 0 : 1;
            }
        }
#pragma unroll
        for (int c = 0; c < 2; c++) {
            const unsigned b = __ballot_sync(0xffffffffu, cls == c);
            int base = 0;
            if (lane == 0 && b) base = atomicAdd(&n_lists[c], __popc(b));
            base = __shfl_sync(0xffffffffu, base, 0);
            if (cls == c) (c ? wide : narrow)[base + __popc(b & lanemask_lt())] = i;
        }
    }
}

// Start word (tile column / 32) of a narrow tile-row: the smallest first
// column of its rows, reduced across the warp (lanes < 16 hold a row each).
__device__ __forceinline__ int narrow_wlo(int r0, int r1, const int* __restrict__ rp, const int* __restrict__ ci) {
    const int lane = threadIdx.x & 31;
    int lo = 0x7fffffff;
    if (lane < r1 - r0) {
        const int s = rp[r0 + lane], e = rp[r0 + lane + 1];
        if (e > s) lo = ci[s];
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, d));
    return max(lo, 0) >> 9;
}

// A narrow tile-row's nonzeros are one contiguous CSR range: its warp takes
// them 32 at a time, each lane finding its nonzero's row among the tile-row's
// row pointers (srp, rows + 1 entries in shared memory): the last q with
// srp[q] <= j (an empty row shares its pointer with the next one, and the
// search lands past it).  Walking the 16 rows one after another left most
// lanes idle on short rows (a 7-point stencil row has 7 nonzeros).
__device__ __forceinline__ int narrow_row(const int* srp, int nrows, int j) {
    int q = 0;
#pragma unroll
    for (int b = 8; b > 0; b >>= 1)
        if (q + b < nrows && srp[q + b] <= j) q += b;
    return q;
}

// One warp per narrow tile-row: its tile columns in a per-warp bitmap of
// TL_NARROW_WORDS words (validating canonical CSR on the way), the count.
__global__ void __launch_bounds__(TL_THREADS)
tiler_count_narrow_kernel(int m, int n, const int* __restrict__ rp, const int* __restrict__ ci,
                          const int* __restrict__ rows, const int* __restrict__ n_rows, int* __restrict__ tile_cnt,
                          unsigned* flags) {
    __shared__ uint32_t s_bm[TL_WARPS][TL_NARROW_WORDS];
    __shared__ int s_rp[TL_WARPS][TS + 1];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t* bm = s_bm[warp];
    int* srp = s_rp[warp];
    const int nr = *n_rows;
    for (int idx = blockIdx.x * TL_WARPS + warp; idx < nr; idx += gridDim.x * TL_WARPS) {
        const int i = rows[idx];
        const int r0 = i * TS, r1 = min(r0 + TS, m), nrows = r1 - r0;
        const int wlo = narrow_wlo(r0, r1, rp, ci);
        if (lane <= nrows) srp[lane] = rp[r0 + lane];
        for (int w = lane; w < TL_NARROW_WORDS; w += 32) bm[w] = 0u;
        __syncwarp();
        for (int j = srp[0] + lane; j < srp[nrows]; j += 32) {
            const int s = srp[narrow_row(srp, nrows, j)];
            const int c = ci[j];
            const int prev = (j > s) ? ci[j - 1] : -1;
            if (c < 0 || c >= n || (j > s && prev >= c)) {
                atomicOr(flags, DERR_NONCANONICAL);
                continue;
            }
            const int tc = c >> 4;
            if (j > s && (prev >> 4) == tc) continue;  // segment already marked
            const int w = (tc >> 5) - wlo;
            if (w < 0 || w >= TL_NARROW_WORDS) { atomicOr(flags, DERR_NONCANONICAL); continue; }
            atomicOr(&bm[w], 1u << (tc & 31));
        }
        __syncwarp();
        int cnt = 0;
        for (int w = lane; w < TL_NARROW_WORDS; w += 32) cnt += __popc(bm[w]);
        cnt = warp_sum(cnt);
        if (lane == 0) tile_cnt[i] = cnt;
        __syncwarp();
    }
}

// One warp per narrow tile-row: sorted tile columns, and per nonzero its
// tile and its position in its (row, tile) segment; segment heads write the
// row count and row mask (tiler_fill_kernel's work for one tile-row).
__global__ void __launch_bounds__(TL_THREADS)
tiler_fill_narrow_kernel(int m, const int* __restrict__ rp, const int* __restrict__ ci,
                         const int* __restrict__ rows, const int* __restrict__ n_rows,
                         const int* __restrict__ tile_ptr, int* __restrict__ tile_columnidx,
                         int* __restrict__ tile_rowof, uint8_t* __restrict__ row_cnt, uint16_t* __restrict__ mask,
                         int* __restrict__ tmp_t, uint8_t* __restrict__ tmp_rp) {
    __shared__ uint32_t s_bm[TL_WARPS][TL_NARROW_WORDS];
    __shared__ uint32_t s_pre[TL_WARPS][TL_NARROW_WORDS];
    __shared__ int s_rp[TL_WARPS][TS + 1];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t* bm = s_bm[warp];
    uint32_t* pre = s_pre[warp];
    int* srp = s_rp[warp];
    constexpr int WPL = TL_NARROW_WORDS / 32;  // words per lane, contiguous
    const int nr = *n_rows;
    for (int idx = blockIdx.x * TL_WARPS + warp; idx < nr; idx += gridDim.x * TL_WARPS) {
        const int i = rows[idx];
        const int r0 = i * TS, r1 = min(r0 + TS, m), nrows = r1 - r0;
        const int wlo = narrow_wlo(r0, r1, rp, ci);
        if (lane <= nrows) srp[lane] = rp[r0 + lane];
        for (int w = lane; w < TL_NARROW_WORDS; w += 32) bm[w] = 0u;
        __syncwarp();
        for (int j = srp[0] + lane; j < srp[nrows]; j += 32) {
            const int s = srp[narrow_row(srp, nrows, j)];
            const int tc = ci[j] >> 4;
            if (j > s && (ci[j - 1] >> 4) == tc) continue;
            atomicOr(&bm[(tc >> 5) - wlo], 1u << (tc & 31));
        }
        __syncwarp();
        // exclusive popcount prefix of the words, WPL contiguous words a lane
        uint32_t local = 0;
#pragma unroll
        for (int q = 0; q < WPL; q++) local += __popc(bm[lane * WPL + q]);
        const uint32_t inc = warp_incl_scan(local, (unsigned)lane);
        uint32_t run = inc - local;
        const int tbase = tile_ptr[i];
#pragma unroll
        for (int q = 0; q < WPL; q++) {
            const int w = lane * WPL + q;
            uint32_t bits = bm[w];
            pre[w] = run;
            int pos = tbase + (int)run;
            run += __popc(bits);
            while (bits) {
                const int b = __ffs(bits) - 1;
                tile_columnidx[pos] = (wlo + w) * 32 + b;
                if (tile_rowof) tile_rowof[pos] = i;
                pos++;
                bits &= bits - 1u;
            }
        }
        __syncwarp();
        for (int j = srp[0] + lane; j < srp[nrows]; j += 32) {
            const int rl = narrow_row(srp, nrows, j);
            const int s = srp[rl], e = srp[rl + 1];
            const int c = ci[j], tc = c >> 4;
            const int w = (tc >> 5) - wlo;
            const int t = tbase + (int)pre[w] + __popc(bm[w] & ((1u << (tc & 31)) - 1u));
            int p = 0;
            for (int q = j - 1; q >= s && (ci[q] >> 4) == tc; q--) p++;
            tmp_t[j] = t;
            tmp_rp[j] = (uint8_t)((rl << 4) | p);
            if (p == 0) {
                int len = 1;
                uint16_t mk = colbit(c);
                for (int q = j + 1; q < e && (ci[q] >> 4) == tc; q++) {
                    len++;
                    mk |= colbit(ci[q]);
                }
                row_cnt[(int64_t)t * TS + rl] = (uint8_t)len;
                mask[(int64_t)t * TS + rl] = mk;
            }
        }
        __syncwarp();
    }
}

// One thread block per wide tile-row (persistent over the list of them).
__global__ void __launch_bounds__(TL_THREADS)
tiler_count_kernel(int m, int n, int nwords, const int* __restrict__ rp, const int* __restrict__ ci,
                   const int* __restrict__ rows, const int* __restrict__ n_rows, int* __restrict__ tile_cnt,
                   unsigned* flags) {
    extern __shared__ uint32_t bm[];
    __shared__ int s_red[TL_WARPS];
    __shared__ int s_span[2];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nr = *n_rows;
    for (int idx = blockIdx.x; idx < nr; idx += gridDim.x) {
    const int i = rows[idx];
    const int r0 = i * TS, r1 = min(r0 + TS, m);
    if (threadIdx.x == 0) { s_span[0] = 0x7fffffff; s_span[1] = -1; }
    __syncthreads();
    if (threadIdx.x < (unsigned)(r1 - r0)) {
        const int s = rp[r0 + threadIdx.x], e = rp[r0 + threadIdx.x + 1];
        if (e > s) {
            atomicMin(&s_span[0], min(max(ci[s], 0), n - 1) >> 4);
            atomicMax(&s_span[1], min(max(ci[e - 1], 0), n - 1) >> 4);
        }
    }
    __syncthreads();
    const int wlo = s_span[1] >= 0 ? (s_span[0] >> 5) : 0;
    // non-canonical rows can put columns outside [first, last]; those set the
    // error flag and are skipped, so a span from the row ends is safe
    const int nwd_span = s_span[1] >= 0 ? (s_span[1] >> 5) - wlo + 1 : 0;
    for (int w = threadIdx.x; w < nwd_span; w += TL_THREADS) bm[w] = 0u;
    __syncthreads();
    for (int r = r0 + warp; r < r1; r += TL_WARPS) {
        const int s = rp[r], e = rp[r + 1];
        for (int j = s + lane; j < e; j += 32) {
            const int c = ci[j];
            const int prev = (j > s) ? ci[j - 1] : -1;
            if (c < 0 || c >= n || (j > s && prev >= c)) {
                atomicOr(flags, DERR_NONCANONICAL);
                continue;
            }
            const int tc = c >> 4;
            if (j > s && (prev >> 4) == tc) continue;  // segment already marked
            const int w = (tc >> 5) - wlo;
            if (w < 0 || w >= nwd_span) { atomicOr(flags, DERR_NONCANONICAL); continue; }
            atomicOr(&bm[w], 1u << (tc & 31));
        }
    }
    __syncthreads();
    int cnt = 0;
    for (int w = threadIdx.x; w < nwd_span; w += TL_THREADS) cnt += __popc(bm[w]);
    cnt = warp_sum(cnt);
    if (lane == 0) s_red[warp] = cnt;
    __syncthreads();
    if (threadIdx.x == 0) {
        int t = 0;
        for (int w = 0; w < TL_WARPS; w++) t += s_red[w];
        tile_cnt[i] = t;
    }
    __syncthreads();
    }
}

// Builds the tile-column bitmap of tile-row i over its column span (first /
// last column of its rows; the CSR was validated canonical by the count pass)
// and the per-word exclusive popcount prefix: bm[0..nwd), pre[0..nwd) hold
// words wlo .. wlo+nwd-1.  Returns {wlo, nwd} in s_span.
__device__ void build_rank_table(int i, int m, const int* __restrict__ rp, const int* __restrict__ ci,
                                 uint32_t* bm, uint32_t* pre, int64_t* s_sh, int* s_span) {
    const int r0 = i * TS, r1 = min(r0 + TS, m);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) { s_span[0] = 0x7fffffff; s_span[1] = -1; }
    __syncthreads();
    if (threadIdx.x < (unsigned)(r1 - r0)) {
        const int s = rp[r0 + threadIdx.x], e = rp[r0 + threadIdx.x + 1];
        if (e > s) { atomicMin(&s_span[0], ci[s] >> 4); atomicMax(&s_span[1], ci[e - 1] >> 4); }
    }
    __syncthreads();
    const int wlo = s_span[1] >= 0 ? (s_span[0] >> 5) : 0;
    const int nwd = s_span[1] >= 0 ? (s_span[1] >> 5) - wlo + 1 : 0;
    for (int w = threadIdx.x; w < nwd; w += TL_THREADS) bm[w] = 0u;
    __syncthreads();
    for (int r = r0 + warp; r < r1; r += TL_WARPS) {
        const int s = rp[r], e = rp[r + 1];
        for (int j = s + lane; j < e; j += 32) {
            const int tc = ci[j] >> 4;
            if (j > s && (ci[j - 1] >> 4) == tc) continue;
            atomicOr(&bm[(tc >> 5) - wlo], 1u << (tc & 31));
        }
    }
    __syncthreads();
    // blocked word ranges per thread
    const int wpt = (nwd + TL_THREADS - 1) / TL_THREADS;
    const int w0 = min(nwd, (int)threadIdx.x * wpt), w1 = min(nwd, w0 + wpt);
    int64_t local = 0;
    for (int w = w0; w < w1; w++) local += __popc(bm[w]);
    int64_t tot;
    int64_t run = block_excl_scan<int64_t>(local, s_sh, &tot);
    for (int w = w0; w < w1; w++) {
        pre[w] = (uint32_t)run;
        run += __popc(bm[w]);
    }
    if (threadIdx.x == 0) { s_span[2] = wlo; s_span[3] = nwd; }
    __syncthreads();
}

__device__ __forceinline__ int rank_of(const uint32_t* bm, const uint32_t* pre, int wlo, int tc) {
    const int w = (tc >> 5) - wlo;
    return (int)pre[w] + __popc(bm[w] & ((1u << (tc & 31)) - 1u));
}

__global__ void __launch_bounds__(TL_THREADS)
tiler_fill_kernel(int m, int nwords, const int* __restrict__ rp, const int* __restrict__ ci,
                  const int* __restrict__ rows, const int* __restrict__ n_rows,
                  const int* __restrict__ tile_ptr, int* __restrict__ tile_columnidx,
                  int* __restrict__ tile_rowof, uint8_t* __restrict__ row_cnt,
                  uint16_t* __restrict__ mask, int* __restrict__ tmp_t, uint8_t* __restrict__ tmp_rp) {
    extern __shared__ uint32_t sm[];
    uint32_t* bm = sm;
    uint32_t* pre = sm + nwords;
    __shared__ int64_t s_sh[TL_WARPS + 1];
    __shared__ int s_span[4];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nr = *n_rows;
    for (int idx = blockIdx.x; idx < nr; idx += gridDim.x) {
    const int i = rows[idx];
    const int r0 = i * TS, r1 = min(r0 + TS, m);
    build_rank_table(i, m, rp, ci, bm, pre, s_sh, s_span);
    const int wlo = s_span[2], nwd = s_span[3];
    const int tbase = tile_ptr[i];
    // sorted tile columns of this tile-row
    {
        const int wpt = (nwd + TL_THREADS - 1) / TL_THREADS;
        const int w0 = min(nwd, (int)threadIdx.x * wpt), w1 = min(nwd, w0 + wpt);
        for (int w = w0; w < w1; w++) {
            uint32_t bits = bm[w];
            int pos = tbase + (int)pre[w];
            while (bits) {
                const int b = __ffs(bits) - 1;
                tile_columnidx[pos] = (wlo + w) * 32 + b;
                if (tile_rowof) tile_rowof[pos] = i;
                pos++;
                bits &= bits - 1u;
            }
        }
    }
    // per nonzero: tile index, position in its (row, tile) segment
    for (int r = r0 + warp; r < r1; r += TL_WARPS) {
        const int s = rp[r], e = rp[r + 1], rl = r - r0;
        for (int j = s + lane; j < e; j += 32) {
            const int c = ci[j], tc = c >> 4;
            const int t = tbase + rank_of(bm, pre, wlo, tc);
            int p = 0;
            for (int q = j - 1; q >= s && (ci[q] >> 4) == tc; q--) p++;
            tmp_t[j] = t;
            tmp_rp[j] = (uint8_t)((rl << 4) | p);
            if (p == 0) {
                int len = 1;
                uint16_t mk = colbit(c);
                for (int q = j + 1; q < e && (ci[q] >> 4) == tc; q++) {
                    len++;
                    mk |= colbit(ci[q]);
                }
                row_cnt[(int64_t)t * TS + rl] = (uint8_t)len;
                mask[(int64_t)t * TS + rl] = mk;
            }
        }
    }
    __syncthreads();
    }
}

// One thread per tile: 16 row counts -> exclusive row offsets (uint8 as the
// reference stores them), tile nnz.
__global__ void tile_rowscan_kernel(int64_t numtile, uint8_t* __restrict__ row_ptr16,
                                    int* __restrict__ tile_cnt) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= numtile) return;
    uint4 v = reinterpret_cast<uint4*>(row_ptr16)[t];
    uint32_t w[4] = {v.x, v.y, v.z, v.w};
    uint32_t s = 0;
#pragma unroll
    for (int q = 0; q < 4; q++) {
        uint32_t o = 0;
#pragma unroll
        for (int b = 0; b < 4; b++) {
            const uint32_t c = (w[q] >> (8 * b)) & 0xffu;
            o |= (s & 0xffu) << (8 * b);
            s += c;
        }
        w[q] = o;
    }
    reinterpret_cast<uint4*>(row_ptr16)[t] = make_uint4(w[0], w[1], w[2], w[3]);
    tile_cnt[t] = (int)s;
}

__global__ void iota_kernel(uint32_t* v, int64_t n) {
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n;
         t += (int64_t)gridDim.x * blockDim.x)
        v[t] = (uint32_t)t;
}

__global__ void hist_kernel(const int* __restrict__ keys, int64_t n, int* __restrict__ hist) {
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n;
         t += (int64_t)gridDim.x * blockDim.x)
        atomicAdd(&hist[keys[t]], 1);
}

// CSC tile p <- row-major tile csc_to_row[p]: tile row index, row offsets,
// masks and nnz count.
__global__ void csc_gather_kernel(int64_t numtile, const uint32_t* __restrict__ csc_to_row,
                                  const int* __restrict__ tile_rowof, const int* __restrict__ cnt_row,
                                  const uint8_t* __restrict__ ptr_row, const uint16_t* __restrict__ mask_row,
                                  int* __restrict__ csc_rowidx, int* __restrict__ csc_to_row_out,
                                  int* __restrict__ row_to_csc, int* __restrict__ cnt_csc,
                                  uint8_t* __restrict__ ptr_csc, uint16_t* __restrict__ mask_csc) {
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < numtile;
         p += (int64_t)gridDim.x * blockDim.x) {
        const int t = (int)csc_to_row[p];
        csc_rowidx[p] = tile_rowof[t];
        csc_to_row_out[p] = t;
        row_to_csc[t] = (int)p;
        cnt_csc[p] = cnt_row[t];
        reinterpret_cast<uint4*>(ptr_csc)[p] = reinterpret_cast<const uint4*>(ptr_row)[t];
        reinterpret_cast<uint4*>(mask_csc)[2 * p] = reinterpret_cast<const uint4*>(mask_row)[2 * t];
        reinterpret_cast<uint4*>(mask_csc)[2 * p + 1] = reinterpret_cast<const uint4*>(mask_row)[2 * t + 1];
    }
}

template <typename V>
__global__ void tiler_scatter_kernel(int64_t nnz, const int* __restrict__ ci, const V* __restrict__ val,
                                     const int* __restrict__ tmp_t, const uint8_t* __restrict__ tmp_rp,
                                     const int* __restrict__ row_to_csc, const int* __restrict__ tile_nnz,
                                     const uint8_t* __restrict__ ptr16, V* __restrict__ out_val,
                                     uint8_t* __restrict__ out_col, int packed) {
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < nnz;
         j += (int64_t)gridDim.x * blockDim.x) {
        int t = tmp_t[j];
        if (row_to_csc) t = row_to_csc[t];
        const int rp_ = tmp_rp[j], r = rp_ >> 4, p = rp_ & 15;
        const int64_t dst = (int64_t)tile_nnz[t] + ptr16[(int64_t)t * TS + r] + p;
        const int c = ci[j] & 15;
        out_val[dst] = val[j];
        out_col[dst] = (uint8_t)(packed ? ((r << 4) | c) : c);
    }
}

// In-tile CSC of a B tile (src/tile_format.h:547-584): per-column offsets and
// the entries regrouped column by column, rows ascending.
template <typename V>
__global__ void tile_csc_kernel(int64_t numtile, const int* __restrict__ tile_nnz,
                                const uint8_t* __restrict__ ptr16, const uint16_t* __restrict__ mask,
                                const V* __restrict__ val, uint8_t* __restrict__ csc_ptr,
                                uint8_t* __restrict__ csc_row, V* __restrict__ csc_val) {
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < numtile;
         t += (int64_t)gridDim.x * blockDim.x) {
        uint16_t mk[TS];
        int cnt[TS];
#pragma unroll
        for (int c = 0; c < TS; c++) cnt[c] = 0;
#pragma unroll
        for (int r = 0; r < TS; r++) {
            mk[r] = mask[t * TS + r];
#pragma unroll
            for (int c = 0; c < TS; c++) cnt[c] += (mk[r] >> (15 - c)) & 1;
        }
        int cur[TS];
        int s = 0;
#pragma unroll
        for (int c = 0; c < TS; c++) {
            csc_ptr[t * TS + c] = (uint8_t)s;
            cur[c] = s;
            s += cnt[c];
        }
        const int base = tile_nnz[t];
        for (int r = 0; r < TS; r++) {
            int e = base + ptr16[t * TS + r];
            uint32_t bits = mk[r];
            for (int c = 0; c < TS; c++) {
                if ((bits >> (15 - c)) & 1u) {
                    int dst = 0;
#pragma unroll
                    for (int q = 0; q < TS; q++)
                        if (q == c) { dst = cur[q]; cur[q]++; }
                    csc_row[base + dst] = (uint8_t)r;
                    csc_val[base + dst] = val[e];
                    e++;
                }
            }
        }
    }
}

int grid_for(spg_handle_t h, int64_t n, int threads) {
    int64_t g = ceil_div(n, threads);
    int64_t cap = (int64_t)h->num_sms * 16;
    if (g > cap) g = cap;
    if (g < 1) g = 1;
    return (int)g;
}

}  // namespace

// Internal: build the tile matrix.  On success the caller owns *out.
spg_status spg_build_tiles(spg_handle_t h, int m, int n, int64_t nnz, const int* d_rp,
                           const int* d_ci, const void* d_val, spg_dtype dtype, spg_layout layout,
                           int flags, spg_tiles* out) {
    const int tilem = (m + TS - 1) / TS, tilen = (n + TS - 1) / TS;
    const int nwords = (tilen + 31) / 32;
    if (nwords > TL_MAX_WORDS)
        return spg_fail(h, SPG_ERR_UNSUPPORTED, "tiling: more than 524288 tile columns");
    const size_t vs = val_size(dtype);
    *out = spg_tiles{};
    out->m = m; out->n = n; out->nnz = nnz; out->tilem = tilem; out->tilen = tilen;
    out->dtype = dtype; out->layout = layout;

    // row view (device copy of the CSR)
    SPG_TRY(spg_alloc_t(h, &out->row_ptr, (size_t)m + 1));
    SPG_TRY(spg_alloc_t(h, &out->col_idx, (size_t)nnz + 1));
    SPG_TRY(spg_alloc(h, &out->row_val, vs * ((size_t)nnz + 1)));
    SPG_CUDA(h, cudaMemcpyAsync(out->row_ptr, d_rp, sizeof(int) * ((size_t)m + 1), cudaMemcpyDeviceToDevice, h->stream));
    if (nnz > 0) {
        SPG_CUDA(h, cudaMemcpyAsync(out->col_idx, d_ci, sizeof(int) * (size_t)nnz, cudaMemcpyDeviceToDevice, h->stream));
        SPG_CUDA(h, cudaMemcpyAsync(out->row_val, d_val, vs * (size_t)nnz, cudaMemcpyDeviceToDevice, h->stream));
    }
    const int* rp = out->row_ptr;
    const int* ci = out->col_idx;

    // pass 1: tiles per tile-row (narrow tile-rows one warp each, wide ones
    // one thread block each)
    ScratchList sc(h);
    int* tile_cnt_rows = nullptr;
    int *narrow = nullptr, *wide = nullptr, *n_lists = nullptr;
    SPG_TRY(sc.alloc(&tile_cnt_rows, (size_t)tilem + 1));
    SPG_TRY(sc.alloc(&narrow, (size_t)tilem + 1));
    SPG_TRY(sc.alloc(&wide, (size_t)tilem + 1));
    SPG_TRY(sc.alloc(&n_lists, 2));
    SPG_TRY(spg_alloc_t(h, &out->tile_ptr, (size_t)tilem + 1));
    const size_t smem1 = sizeof(uint32_t) * nwords;
    const size_t smem2 = 2 * sizeof(uint32_t) * nwords;
    SPG_CUDA(h, cudaFuncSetAttribute(tiler_count_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem1));
    SPG_CUDA(h, cudaFuncSetAttribute(tiler_fill_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem2));
    SPG_CUDA(h, cudaMemsetAsync(n_lists, 0, 2 * sizeof(int), h->stream));
    const int grid_rows = grid_for(h, (int64_t)tilem * 32, TL_THREADS);  // a warp per tile-row, capped
    const int grid_wide = h->num_sms * 8;  // persistent blocks over the wide tile-rows
    if (tilem > 0) {
        tiler_class_kernel<<<grid_for(h, tilem, 256), 256, 0, h->stream>>>(tilem, m, rp, ci, tile_cnt_rows, narrow,
                                                                          wide, n_lists);
        SPG_LAUNCHED(h);
        tiler_count_narrow_kernel<<<grid_rows, TL_THREADS, 0, h->stream>>>(m, n, rp, ci, narrow, n_lists,
                                                                           tile_cnt_rows, h->d_flags);
        SPG_LAUNCHED(h);
        tiler_count_kernel<<<grid_wide, TL_THREADS, smem1, h->stream>>>(m, n, nwords, rp, ci, wide, n_lists + 1,
                                                                        tile_cnt_rows, h->d_flags);
        SPG_LAUNCHED(h);
    }
    SPG_TRY(spg_scan_i32_to_i32(h, tile_cnt_rows, out->tile_ptr, tilem));
    int numtile = 0;
    SPG_TRY(spg_read_i32(h, out->tile_ptr + tilem, &numtile));
    SPG_TRY(spg_check_flags(h, "tiling"));
    out->numtile = numtile;

    // pass 2: tile columns, segment counts and masks
    int* tile_rowof = nullptr;
    int* tmp_t = nullptr;
    uint8_t* tmp_rp = nullptr;
    uint8_t* ptr_row = nullptr;
    uint16_t* mask_row = nullptr;
    int* cnt_row = nullptr;
    SPG_TRY(spg_alloc_t(h, &out->tile_columnidx, (size_t)numtile + 1));
    SPG_TRY(sc.alloc(&tile_rowof, (size_t)numtile + 1));
    SPG_TRY(sc.alloc(&tmp_t, (size_t)nnz + 1));
    SPG_TRY(sc.alloc(&tmp_rp, (size_t)nnz + 1));
    SPG_TRY(sc.alloc(&ptr_row, (size_t)numtile * TS + 16));
    SPG_TRY(sc.alloc(&mask_row, (size_t)numtile * TS + 16));
    SPG_TRY(sc.alloc(&cnt_row, (size_t)numtile + 1));
    SPG_CUDA(h, cudaMemsetAsync(ptr_row, 0, (size_t)numtile * TS, h->stream));
    SPG_CUDA(h, cudaMemsetAsync(mask_row, 0, sizeof(uint16_t) * (size_t)numtile * TS, h->stream));
    if (tilem > 0) {
        tiler_fill_narrow_kernel<<<grid_rows, TL_THREADS, 0, h->stream>>>(m, rp, ci, narrow, n_lists, out->tile_ptr,
                                                                          out->tile_columnidx, tile_rowof, ptr_row,
                                                                          mask_row, tmp_t, tmp_rp);
        SPG_LAUNCHED(h);
        tiler_fill_kernel<<<grid_wide, TL_THREADS, smem2, h->stream>>>(m, nwords, rp, ci, wide, n_lists + 1,
                                                                       out->tile_ptr, out->tile_columnidx, tile_rowof,
                                                                       ptr_row, mask_row, tmp_t, tmp_rp);
        SPG_LAUNCHED(h);
    }
    if (numtile > 0) {
        tile_rowscan_kernel<<<(unsigned)ceil_div(numtile, 256), 256, 0, h->stream>>>(numtile, ptr_row, cnt_row);
        SPG_LAUNCHED(h);
    }
    SPG_TRY(spg_alloc_t(h, &out->tile_nnz, (size_t)numtile + 1));
    SPG_TRY(spg_alloc(h, &out->tile_csr_Val, vs * ((size_t)nnz + 1)));
    SPG_TRY(spg_alloc_t(h, &out->tile_csr_Col, (size_t)nnz + 1));

    if (layout == SPG_LAYOUT_ROW) {
        SPG_TRY(spg_scan_i32_to_i32(h, cnt_row, out->tile_nnz, numtile));
        out->tile_csr_Ptr = ptr_row;  // the row-major per-tile arrays are the result
        out->mask = mask_row;
        sc.keep(ptr_row);
        sc.keep(mask_row);
        if (nnz > 0) {
            if (dtype == SPG_F64)
                tiler_scatter_kernel<double><<<grid_for(h, nnz, 256), 256, 0, h->stream>>>(
                    nnz, ci, (const double*)out->row_val, tmp_t, tmp_rp, nullptr, out->tile_nnz,
                    out->tile_csr_Ptr, (double*)out->tile_csr_Val, out->tile_csr_Col, 1);
            else
                tiler_scatter_kernel<float><<<grid_for(h, nnz, 256), 256, 0, h->stream>>>(
                    nnz, ci, (const float*)out->row_val, tmp_t, tmp_rp, nullptr, out->tile_nnz,
                    out->tile_csr_Ptr, (float*)out->tile_csr_Val, out->tile_csr_Col, 1);
            SPG_LAUNCHED(h);
        }
    } else {
        // CSC tile order = stable sort of row-major tiles by tile column
        uint32_t *keys = nullptr, *perm = nullptr;
        int* row_to_csc = nullptr;
        int* cnt_csc = nullptr;
        SPG_TRY(sc.alloc(&keys, (size_t)numtile + 1));
        SPG_TRY(sc.alloc(&perm, (size_t)numtile + 1));
        SPG_TRY(sc.alloc(&row_to_csc, (size_t)numtile + 1));
        SPG_TRY(sc.alloc(&cnt_csc, (size_t)numtile + 1));
        SPG_TRY(spg_alloc_t(h, &out->csc_tile_ptr, (size_t)tilen + 1));
        SPG_TRY(spg_alloc_t(h, &out->csc_tile_rowidx, (size_t)numtile + 1));
        SPG_TRY(spg_alloc_t(h, &out->csc_to_row, (size_t)numtile + 1));
        SPG_TRY(spg_alloc_t(h, &out->tile_csr_Ptr, (size_t)numtile * TS + 16));
        SPG_TRY(spg_alloc_t(h, &out->mask, (size_t)numtile * TS + 16));
        if (numtile > 0) {
            SPG_CUDA(h, cudaMemcpyAsync(keys, out->tile_columnidx, sizeof(int) * (size_t)numtile,
                                        cudaMemcpyDeviceToDevice, h->stream));
            iota_kernel<<<grid_for(h, numtile, 256), 256, 0, h->stream>>>(perm, numtile);
            SPG_LAUNCHED(h);
            int bits = 1;
            while (bits < 31 && (1LL << bits) < tilen) bits++;
            SPG_TRY(spg_radix_sort_pairs(h, keys, perm, numtile, bits));
        }
        int* hist = nullptr;
        SPG_TRY(sc.alloc(&hist, (size_t)tilen + 1));
        SPG_CUDA(h, cudaMemsetAsync(hist, 0, sizeof(int) * ((size_t)tilen + 1), h->stream));
        if (numtile > 0) {
            hist_kernel<<<grid_for(h, numtile, 256), 256, 0, h->stream>>>(out->tile_columnidx, numtile, hist);
            SPG_LAUNCHED(h);
        }
        SPG_TRY(spg_scan_i32_to_i32(h, hist, out->csc_tile_ptr, tilen));
        if (numtile > 0) {
            csc_gather_kernel<<<grid_for(h, numtile, 256), 256, 0, h->stream>>>(
                numtile, perm, tile_rowof, cnt_row, ptr_row, mask_row, out->csc_tile_rowidx, out->csc_to_row,
                row_to_csc, cnt_csc, out->tile_csr_Ptr, out->mask);
            SPG_LAUNCHED(h);
        }
        SPG_TRY(spg_scan_i32_to_i32(h, cnt_csc, out->tile_nnz, numtile));
        if (nnz > 0) {
            if (dtype == SPG_F64)
                tiler_scatter_kernel<double><<<grid_for(h, nnz, 256), 256, 0, h->stream>>>(
                    nnz, ci, (const double*)out->row_val, tmp_t, tmp_rp, row_to_csc, out->tile_nnz,
                    out->tile_csr_Ptr, (double*)out->tile_csr_Val, out->tile_csr_Col, 0);
            else
                tiler_scatter_kernel<float><<<grid_for(h, nnz, 256), 256, 0, h->stream>>>(
                    nnz, ci, (const float*)out->row_val, tmp_t, tmp_rp, row_to_csc, out->tile_nnz,
                    out->tile_csr_Ptr, (float*)out->tile_csr_Val, out->tile_csr_Col, 0);
            SPG_LAUNCHED(h);
        }
        if (flags & SPG_TILE_WITH_TILE_CSC) {
            SPG_TRY(spg_alloc_t(h, &out->tile_csc_Ptr, (size_t)numtile * TS + 16));
            SPG_TRY(spg_alloc_t(h, &out->tile_csc_Row, (size_t)nnz + 1));
            SPG_TRY(spg_alloc(h, &out->tile_csc_Val, vs * ((size_t)nnz + 1)));
        }
        if ((flags & SPG_TILE_WITH_TILE_CSC) && numtile > 0) {
            if (dtype == SPG_F64)
                tile_csc_kernel<double><<<grid_for(h, numtile, 128), 128, 0, h->stream>>>(
                    numtile, out->tile_nnz, out->tile_csr_Ptr, out->mask, (const double*)out->tile_csr_Val,
                    out->tile_csc_Ptr, out->tile_csc_Row, (double*)out->tile_csc_Val);
            else
                tile_csc_kernel<float><<<grid_for(h, numtile, 128), 128, 0, h->stream>>>(
                    numtile, out->tile_nnz, out->tile_csr_Ptr, out->mask, (const float*)out->tile_csr_Val,
                    out->tile_csc_Ptr, out->tile_csc_Row, (float*)out->tile_csc_Val);
            SPG_LAUNCHED(h);
        }
    }
    return spg_check_flags(h, "tiling");
}
