// spg_abi.cu -- C ABI of libspgemm_gb300.so (declared in include/spgemm_gb300.h).
//
// Drives the steps the reference's main() drives (src/spgemm_raw_v2.cu:101-243):
// tiling, C tile structure, bitmask symbolic, scans, numeric.  Differences from
// the reference's host program: all work is ordered on one caller-chosen stream, device
// memory comes from the stream-ordered pool allocator (the reference's
// cudaMalloc/cudaFree pairs around each CUB scan disappear), every CUDA call is
// checked, C's nnz prefix is int64, and device-side error bits are turned into
// status codes.
#include <cstdio>
#include <cstdlib>
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstring>
#include <new>
#include <thread>
#include <vector>

#include "plain.cuh"
#include "rowwise.cuh"
#include "spg_common.cuh"

struct CPriv {
    PlainPriv plain;
    int64_t* row_pairs = nullptr;  // tilem: tile pairs per C tile-row (step 1)
    spg_algo algo = SPG_ALGO_PLAIN;
    RowwisePriv rw;
    bool vals_joint = false;       // tile_colC lives inside tile_valC's allocation
    // SPG_ALGO_BINNED: the tile-rows the plain kernels take
    uint8_t* rowbin = nullptr;     // tilem: 1 = plain kernels, 0 = row-wise windows
    int64_t* plain_off = nullptr;  // tilem+1: prefix of the plain tile-rows' C tiles
    int* plain_list = nullptr;     // those C tiles, ascending
    int64_t nplain = 0;
    int64_t plain_pairs = 0;       // tile pairs of the plain tile-rows (step 1's count)
};

RowwisePriv* ctiles_rowwise_priv(spg_ctiles* C) {
    return C && C->priv ? &static_cast<CPriv*>(C->priv)->rw : nullptr;
}

// ---------------------------------------------------------------------------
// handle and helpers
// ---------------------------------------------------------------------------
spg_status spg_fail(spg_handle_t h, spg_status s, const std::string& msg) {
    if (h) h->err = msg;
    return s;
}

spg_status spg_cuda_fail(spg_handle_t h, cudaError_t e, const char* what) {
    std::string m = std::string(what) + ": " + cudaGetErrorString(e);
    if (e == cudaErrorMemoryAllocation) return spg_fail(h, SPG_ERR_OOM, m);
    return spg_fail(h, SPG_ERR_CUDA, m);
}

spg_status spg_alloc(spg_handle_t h, void** p, size_t bytes) {
    if (bytes == 0) bytes = 16;
    cudaError_t e = cudaMallocAsync(p, bytes, h->stream);
    if (e != cudaSuccess) {
        cudaGetLastError();
        *p = nullptr;
        char buf[128];
        snprintf(buf, sizeof(buf), "device allocation of %zu bytes failed: %s", bytes, cudaGetErrorString(e));
        return spg_fail(h, SPG_ERR_OOM, buf);
    }
    return SPG_OK;
}

void spg_free_async(spg_handle_t h, void* p) {
    if (p) cudaFreeAsync(p, h->stream);
}

spg_status spg_workspace(spg_handle_t h, int kind, size_t bytes, void** out) {
    if (kind < 0 || kind >= (int)(sizeof(h->ws) / sizeof(h->ws[0])))
        return spg_fail(h, SPG_ERR_INVALID, "internal: bad workspace kind");
    if (bytes > h->ws_bytes[kind]) {
        spg_free_async(h, h->ws[kind]);
        h->ws[kind] = nullptr;
        h->ws_bytes[kind] = 0;
        const size_t grow = bytes + bytes / 8;  // some headroom for the next, slightly larger, call
        SPG_TRY(spg_alloc(h, &h->ws[kind], grow));
        h->ws_bytes[kind] = grow;
    }
    *out = h->ws[kind];
    return SPG_OK;
}

spg_status spg_read_i64(spg_handle_t h, const int64_t* d, int64_t* out) {
    SPG_CUDA(h, cudaMemcpyAsync(h->h_pinned, d, sizeof(int64_t), cudaMemcpyDeviceToHost, h->stream));
    SPG_CUDA(h, cudaStreamSynchronize(h->stream));
    *out = h->h_pinned[0];
    return SPG_OK;
}

spg_status spg_read_i32(spg_handle_t h, const int* d, int* out) {
    SPG_CUDA(h, cudaMemcpyAsync(h->h_pinned, d, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    SPG_CUDA(h, cudaStreamSynchronize(h->stream));
    *out = reinterpret_cast<int*>(h->h_pinned)[0];
    return SPG_OK;
}

// Turns device error bits read back into h_pinned[1] into a status.
static spg_status flags_status(spg_handle_t h, const char* where) {
    const unsigned f = *reinterpret_cast<unsigned*>(h->h_pinned + 1);
    if (f == 0) return SPG_OK;
    SPG_CUDA(h, cudaMemsetAsync(h->d_flags, 0, sizeof(unsigned), h->stream));
    std::string w(where);
    if (f & DERR_NONCANONICAL)
        return spg_fail(h, SPG_ERR_INVALID, w + ": CSR columns must be strictly ascending and within [0, n)");
    if (f & DERR_TIMEOUT) return spg_fail(h, SPG_ERR_TIMEOUT, w + ": a bounded device wait gave up");
    if (f & DERR_TOO_BIG) return spg_fail(h, SPG_ERR_INVALID, w + ": a count overflowed its index type");
    if (f & DERR_OVERFLOW) return spg_fail(h, SPG_ERR_OVERFLOW_RERUN, w + ": a pre-sized buffer overflowed");
    return spg_fail(h, SPG_ERR_CUDA, w + ": unknown device error");
}

spg_status spg_check_flags(spg_handle_t h, const char* where) {
    SPG_CUDA(h, cudaMemcpyAsync(h->h_pinned + 1, h->d_flags, sizeof(unsigned), cudaMemcpyDeviceToHost, h->stream));
    SPG_CUDA(h, cudaStreamSynchronize(h->stream));
    return flags_status(h, where);
}

// n (<= 8) device int64 scalars and the device error bits in one round trip:
// the stream's work so far is complete when this returns.
spg_status spg_read_i64s_checked(spg_handle_t h, int n, const int64_t* const* src, int64_t* out, const char* where) {
    SPG_CUDA(h, cudaMemcpyAsync(h->h_pinned + 1, h->d_flags, sizeof(unsigned), cudaMemcpyDeviceToHost, h->stream));
    for (int k = 0; k < n; k++)
        SPG_CUDA(h, cudaMemcpyAsync(h->h_pinned + 8 + k, src[k], sizeof(int64_t), cudaMemcpyDeviceToHost,
                                    h->stream));
    SPG_CUDA(h, cudaStreamSynchronize(h->stream));
    SPG_TRY(flags_status(h, where));
    for (int k = 0; k < n; k++) out[k] = h->h_pinned[8 + k];
    return SPG_OK;
}

extern "C" spg_status spg_create(spg_handle_t* out, int device, void* stream) {
    if (!out) return SPG_ERR_INVALID;
    *out = nullptr;
    spg_handle_t h = new (std::nothrow) spg_handle_s();
    if (!h) return SPG_ERR_OOM;
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) { delete h; return SPG_ERR_CUDA; }
    h->device = device;
    h->stream = (cudaStream_t)stream;
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) { delete h; return SPG_ERR_CUDA; }
    h->num_sms = prop.multiProcessorCount;
    h->smem_optin = prop.sharedMemPerBlockOptin;
    h->smem_per_sm = prop.sharedMemPerMultiprocessor;
    if (cudaMalloc(&h->d_flags, 256) != cudaSuccess) { delete h; return SPG_ERR_OOM; }
    cudaMemset(h->d_flags, 0, 256);
    if (cudaMallocHost(&h->h_pinned, 64 * sizeof(int64_t)) != cudaSuccess) {
        cudaFree(h->d_flags);
        delete h;
        return SPG_ERR_OOM;
    }
    for (auto& ev : h->ev) cudaEventCreate(&ev);
    // keep freed pool memory cached for the next call instead of returning it
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
        uint64_t thr = ~0ull;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
    }
    *out = h;
    return SPG_OK;
}

extern "C" spg_status spg_destroy(spg_handle_t h) {
    if (!h) return SPG_ERR_INVALID;
    for (void* p : h->ws) spg_free_async(h, p);
    cudaStreamSynchronize(h->stream);
    for (auto& ev : h->ev) cudaEventDestroy(ev);
    cudaFree(h->d_flags);
    cudaFreeHost(h->h_pinned);
    if (h->h_band) cudaFreeHost(h->h_band);
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, h->device) == cudaSuccess) cudaMemPoolTrimTo(pool, 0);
    delete h;
    return SPG_OK;
}

extern "C" spg_status spg_set_stream(spg_handle_t h, void* stream) {
    if (!h) return SPG_ERR_INVALID;
    h->stream = (cudaStream_t)stream;
    return SPG_OK;
}

extern "C" const char* spg_last_error(spg_handle_t h) { return h ? h->err.c_str() : "null handle"; }

extern "C" spg_status spg_get_stats(spg_handle_t h, spg_stats* out) {
    if (!h || !out) return SPG_ERR_INVALID;
    *out = h->stats;
    return SPG_OK;
}

extern "C" spg_status spg_kernel_launches(spg_handle_t h, int64_t* out) {
    if (!h || !out) return SPG_ERR_INVALID;
    *out = h->launches;
    return SPG_OK;
}

// ---------------------------------------------------------------------------
// tiling
// ---------------------------------------------------------------------------
static spg_status validate_csr_args(spg_handle_t h, int m, int n, int64_t nnz, const void* rp,
                                    const void* ci, const void* v, spg_dtype dtype, spg_layout layout,
                                    spg_tiles* out) {
    if (!h) return SPG_ERR_INVALID;
    if (!out) return spg_fail(h, SPG_ERR_INVALID, "tiling: null output");
    if (m < 0 || n < 0 || nnz < 0) return spg_fail(h, SPG_ERR_INVALID, "tiling: negative size");
    if (nnz >= 0x7fffffffLL) return spg_fail(h, SPG_ERR_INVALID, "tiling: nnz must fit int32");
    if (m >= 0x7ffffff0 || n >= 0x7ffffff0) return spg_fail(h, SPG_ERR_INVALID, "tiling: dimension too large");
    if (!rp || (nnz > 0 && (!ci || !v))) return spg_fail(h, SPG_ERR_INVALID, "tiling: null CSR array");
    if (dtype != SPG_F32 && dtype != SPG_F64) return spg_fail(h, SPG_ERR_INVALID, "tiling: bad dtype");
    if (layout != SPG_LAYOUT_ROW && layout != SPG_LAYOUT_B_CSC)
        return spg_fail(h, SPG_ERR_INVALID, "tiling: bad layout");
    return SPG_OK;
}

extern "C" spg_status spg_tile_from_csr(spg_handle_t h, int m, int n, int64_t nnz, const int* d_row_ptr,
                                        const int* d_col_idx, const void* d_val, spg_dtype dtype,
                                        spg_layout layout, int flags, spg_tiles* out) {
    SPG_TRY(validate_csr_args(h, m, n, nnz, d_row_ptr, d_col_idx, d_val, dtype, layout, out));
    spg_status s = spg_build_tiles(h, m, n, nnz, d_row_ptr, d_col_idx, d_val, dtype, layout, flags, out);
    if (s != SPG_OK) { std::string e = h->err; spg_tiles_free(h, out); h->err = e; }
    return s;
}

extern "C" spg_status spg_tile_from_csr_host(spg_handle_t h, int m, int n, int64_t nnz, const int* row_ptr,
                                             const int* col_idx, const void* val, spg_dtype dtype,
                                             spg_layout layout, int flags, spg_tiles* out) {
    SPG_TRY(validate_csr_args(h, m, n, nnz, row_ptr, col_idx, val, dtype, layout, out));
    const size_t vs = val_size(dtype);
    int *drp = nullptr, *dci = nullptr;
    void* dv = nullptr;
    SPG_TRY(spg_alloc_t(h, &drp, (size_t)m + 1));
    SPG_TRY(spg_alloc_t(h, &dci, (size_t)nnz + 1));
    SPG_TRY(spg_alloc(h, &dv, vs * ((size_t)nnz + 1)));
    SPG_CUDA(h, cudaMemcpyAsync(drp, row_ptr, sizeof(int) * ((size_t)m + 1), cudaMemcpyHostToDevice, h->stream));
    if (nnz > 0) {
        SPG_CUDA(h, cudaMemcpyAsync(dci, col_idx, sizeof(int) * (size_t)nnz, cudaMemcpyHostToDevice, h->stream));
        SPG_CUDA(h, cudaMemcpyAsync(dv, val, vs * (size_t)nnz, cudaMemcpyHostToDevice, h->stream));
    }
    spg_status s = spg_build_tiles(h, m, n, nnz, drp, dci, dv, dtype, layout, flags, out);
    spg_free_async(h, drp);
    spg_free_async(h, dci);
    spg_free_async(h, dv);
    if (s != SPG_OK) { std::string e = h->err; spg_tiles_free(h, out); h->err = e; }
    return s;
}

extern "C" spg_status spg_tiles_free(spg_handle_t h, spg_tiles* t) {
    if (!h || !t) return SPG_ERR_INVALID;
    void* ptrs[] = {t->tile_ptr, t->tile_columnidx, t->tile_nnz, t->tile_csr_Ptr, t->mask, t->tile_csr_Val,
                    t->tile_csr_Col, t->csc_tile_ptr, t->csc_tile_rowidx, t->csc_to_row, t->tile_csc_Ptr,
                    t->tile_csc_Row, t->tile_csc_Val, t->row_ptr, t->col_idx, t->row_val};
    for (void* p : ptrs) spg_free_async(h, p);
    rowwise_free_bview(h, t);
    *t = spg_tiles{};
    return SPG_OK;
}

// ---------------------------------------------------------------------------
// SpGEMM
// ---------------------------------------------------------------------------
static spg_status validate_pair(spg_handle_t h, const spg_tiles* A, const spg_tiles* B, const spg_ctiles* C) {
    if (!h) return SPG_ERR_INVALID;
    if (!A || !B || !C) return spg_fail(h, SPG_ERR_INVALID, "null argument");
    if (A->layout != SPG_LAYOUT_ROW) return spg_fail(h, SPG_ERR_INVALID, "A must be tiled with SPG_LAYOUT_ROW");
    if (B->layout != SPG_LAYOUT_B_CSC) return spg_fail(h, SPG_ERR_INVALID, "B must be tiled with SPG_LAYOUT_B_CSC");
    if (A->n != B->m) return spg_fail(h, SPG_ERR_INVALID, "inner dimensions differ (A.n != B.m)");
    if (A->dtype != B->dtype) return spg_fail(h, SPG_ERR_INVALID, "A and B value types differ");
    return SPG_OK;
}

// Whether a pair cache of `bytes` leaves enough device memory: small caches
// always do (no query); larger ones may take a quarter of the free memory.
static bool cache_fits(spg_handle_t h, size_t bytes) {
    (void)h;
    if (bytes <= ((size_t)1 << 30)) return true;
    size_t fr = 0, tot = 0;
    if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) return false;
    return bytes < fr / 4;
}

// Pair-cache capacity for step 2 over nt C tiles holding `pairs` tile pairs
// (step 1's count): the cache holds at most SPEC_PAIRS_MAX pairs a tile and,
// in all, no more than those pairs, so with that capacity it never
// overflows.  Where that does not fit beside C, the reference's 8 a tile
// (src/spgemm_raw_v2.cu:170) with its overflow re-run; 0 when neither fits
// (no cache: step 3 intersects the tile lists again).
static int64_t spec_capacity(spg_handle_t h, const spg_ctiles* C, int64_t nt, int64_t pairs) {
    int64_t cap = std::min<int64_t>(pairs, (int64_t)SPEC_PAIRS_MAX * nt);
    if (const char* d = getenv("SPG_SPEC_CAP_DIV")) {  // test knob: force the overflow re-run
        const long div = atol(d);
        if (div > 1) return std::max<int64_t>(1, std::min<int64_t>(cap, 8 * nt) / div);
    }
    if (cap > 0 && cache_fits(h, (size_t)cap * 8 + (size_t)C->numtileC * 8)) return cap;
    cap = 8 * nt;
    return cap > 0 && cache_fits(h, (size_t)cap * 8 + (size_t)C->numtileC * 8) ? cap : 0;
}

static float elapsed(spg_handle_t h, int a, int b) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, h->ev[a], h->ev[b]);
    return ms;
}

extern "C" spg_status spg_ctiles_free(spg_handle_t h, spg_ctiles* C) {
    if (!h || !C) return SPG_ERR_INVALID;
    const bool joint = C->priv && static_cast<CPriv*>(C->priv)->vals_joint;
    void* ptrs[] = {C->tile_ptrC, C->tile_rowidxC, C->tile_colidxC, C->maskC, C->tile_nnzC, C->ptrRowC,
                    C->tile_valC, joint ? nullptr : C->tile_colC};
    for (void* p : ptrs) spg_free_async(h, p);
    if (C->priv) {
        CPriv* cp = static_cast<CPriv*>(C->priv);
        void* pp[] = {cp->plain.spec_cnt, cp->plain.spec_off, cp->plain.spec_pa, cp->plain.spec_pb,
                      cp->plain.counters, cp->row_pairs, cp->rowbin, cp->plain_off, cp->plain_list};
        for (void* p : pp) spg_free_async(h, p);
        rowwise_free_priv(h, &cp->rw);
        delete cp;
    }
    *C = spg_ctiles{};
    return SPG_OK;
}

// ---------------------------------------------------------------------------
// SPG_ALGO_BINNED: the C tiles of the tile-rows binned to the plain kernels
// ---------------------------------------------------------------------------
// Per tile-row: its C tiles if it is binned plain (else 0); the plain
// tile-rows' tile pairs summed into *plain_pairs (the pair cache's bound).
__global__ void plain_count_kernel(int tilem, const uint8_t* __restrict__ rowbin, const int* __restrict__ tile_ptrC,
                                   const int64_t* __restrict__ row_pairs, int* __restrict__ cnt,
                                   unsigned long long* __restrict__ plain_pairs) {
    unsigned long long p = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < tilem; i += gridDim.x * blockDim.x) {
        cnt[i] = rowbin[i] ? tile_ptrC[i + 1] - tile_ptrC[i] : 0;
        if (rowbin[i]) p += (unsigned long long)row_pairs[i];
    }
    p = warp_sum(p);
    if ((threadIdx.x & 31) == 0 && p) atomicAdd(plain_pairs, p);
}

__global__ void plain_list_kernel(int tilem, const uint8_t* __restrict__ rowbin, const int* __restrict__ tile_ptrC,
                                  const int64_t* __restrict__ off, int* __restrict__ list) {
    const int lane = threadIdx.x & 31;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < tilem; i += nw) {
        if (!rowbin[i]) continue;
        const int t0 = tile_ptrC[i], n = tile_ptrC[i + 1] - t0;
        for (int k = lane; k < n; k += 32) list[off[i] + k] = t0 + k;
    }
}

static int small_grid(spg_handle_t h, int64_t units, int per_block) {
    int64_t g = ceil_div(units, per_block);
    if (g > (int64_t)h->num_sms * 8) g = (int64_t)h->num_sms * 8;
    return (int)(g < 1 ? 1 : g);
}

// After step 1 of a binned product: the plain tile-rows' C tiles as a list.
// A product whose tile-rows all went one way runs that algorithm alone.
static spg_status bin_tiles(spg_handle_t h, spg_ctiles* C, CPriv* cp, spg_algo* algo) {
    const int tilem = C->tilem;
    ScratchList sc(h);
    int* cnt = nullptr;
    SPG_TRY(sc.alloc(&cnt, (size_t)tilem + 1));
    SPG_TRY(spg_alloc_t(h, &cp->plain_off, (size_t)tilem + 1));
    unsigned long long* plain_pairs = cp->plain.counters + 3;
    SPG_CUDA(h, cudaMemsetAsync(plain_pairs, 0, sizeof(unsigned long long), h->stream));
    if (tilem > 0) {
        plain_count_kernel<<<small_grid(h, tilem, 256), 256, 0, h->stream>>>(tilem, cp->rowbin, C->tile_ptrC,
                                                                             cp->row_pairs, cnt, plain_pairs);
        SPG_LAUNCHED(h);
    }
    SPG_TRY(spg_scan_i32_to_i64(h, cnt, cp->plain_off, tilem));
    {
        const int64_t* src[2] = {cp->plain_off + tilem, reinterpret_cast<const int64_t*>(plain_pairs)};
        int64_t v[2] = {0, 0};
        SPG_TRY(spg_read_i64s_checked(h, 2, src, v, "binning"));
        cp->nplain = v[0];
        cp->plain_pairs = v[1];
    }
    if (cp->nplain == 0 || cp->nplain == C->numtileC) {
        *algo = cp->nplain == 0 ? SPG_ALGO_ROWWISE : SPG_ALGO_PLAIN;
        spg_free_async(h, cp->rowbin);
        spg_free_async(h, cp->plain_off);
        cp->rowbin = nullptr;
        cp->plain_off = nullptr;
        cp->nplain = 0;
        return SPG_OK;
    }
    SPG_TRY(spg_alloc_t(h, &cp->plain_list, (size_t)cp->nplain + 1));
    plain_list_kernel<<<small_grid(h, (int64_t)tilem * 32, 256), 256, 0, h->stream>>>(tilem, cp->rowbin,
                                                                                        C->tile_ptrC, cp->plain_off,
                                                                                        cp->plain_list);
    SPG_LAUNCHED(h);
    return SPG_OK;
}

// Step 1: C's tile structure (tile_ptrC, tile_rowidxC, tile_colidxC).
// final: step 1 alone (spg_symbolic_tiles) -- wait for it and check its
// device errors here; otherwise step 2's read-back does both.
static spg_status tiles_impl(spg_handle_t h, const spg_tiles* A, const spg_tiles* B, spg_algo algo,
                             spg_ctiles* C, bool final) {
    *C = spg_ctiles{};
    C->m = A->m; C->n = B->n; C->tilem = A->tilem; C->tilen = B->tilen; C->dtype = A->dtype;
    CPriv* cp = new (std::nothrow) CPriv();
    if (!cp) return spg_fail(h, SPG_ERR_OOM, "host allocation failed");
    C->priv = cp;
    // AUTO: each tile-row to the plain or the row-wise kernels (below).  On a
    // small A (under 65,536 tiles) one choice for the whole product, by A's
    // nonzeros per tile: binning costs a features pass and a read-back that
    // such a product cannot win back.  The row-wise kernels need B narrow
    // enough for their shared memory.
    if (algo == SPG_ALGO_AUTO) {
        if (!rowwise_fits(h, B))
            algo = SPG_ALGO_PLAIN;
        else if (A->numtile >= 65536)
            algo = SPG_ALGO_BINNED;
        else
            algo = A->numtile > 0 && (double)A->nnz / (double)A->numtile < 6.0 ? SPG_ALGO_ROWWISE : SPG_ALGO_PLAIN;
    } else if (algo == SPG_ALGO_BINNED && !rowwise_fits(h, B)) {
        algo = SPG_ALGO_PLAIN;
    }
    const bool binned = algo == SPG_ALGO_BINNED;
    SPG_TRY(spg_alloc_t(h, &cp->plain.counters, 4));
    SPG_CUDA(h, cudaMemsetAsync(cp->plain.counters, 0, 4 * sizeof(unsigned long long), h->stream));
    SPG_TRY(spg_alloc_t(h, &cp->row_pairs, (size_t)A->tilem + 1));
    if (binned) SPG_TRY(spg_alloc_t(h, &cp->rowbin, (size_t)A->tilem + 16));
    SPG_CUDA(h, cudaEventRecord(h->ev[0], h->stream));
    // ---- step 1: C tile structure
    if (h->sizing) {
        spg_status st;
        {
            ScratchList sc(h);
            int* slot = nullptr;
            st = sc.alloc(&slot, (size_t)A->tilem + 1);
            if (st == SPG_OK) st = mlp_predict_rows(h, A, B, slot, cp->rowbin);
            if (st == SPG_OK) st = plain_step1_sized(h, A, B, C, cp->row_pairs, cp->plain.counters + 2, slot);
        }
        if (st == SPG_ERR_OOM) {
            // The predicted slots (or C's arrays beside them) did not fit:
            // drop what the sized pass allocated and run the exact two-pass
            // step 1, which needs no staging.  The structure is the same.
            spg_free_async(h, C->tile_ptrC);
            spg_free_async(h, C->tile_rowidxC);
            spg_free_async(h, C->tile_colidxC);
            C->tile_ptrC = C->tile_rowidxC = C->tile_colidxC = nullptr;
            C->numtileC = 0;
            h->stats.overflow_reruns = 0;
            h->stats.sizing_fallbacks++;
            SPG_CUDA(h, cudaMemsetAsync(cp->plain.counters + 2, 0, sizeof(unsigned long long), h->stream));
            SPG_TRY(plain_step1(h, A, B, C, cp->row_pairs, cp->plain.counters + 2));
        } else {
            SPG_TRY(st);
        }
    } else {
        if (binned) SPG_TRY(mlp_predict_rows(h, A, B, nullptr, cp->rowbin));
        SPG_TRY(plain_step1(h, A, B, C, cp->row_pairs, cp->plain.counters + 2));
    }
    if (binned) SPG_TRY(bin_tiles(h, C, cp, &algo));
    cp->algo = algo;
    h->stats.algo_used = (int32_t)algo;
    SPG_CUDA(h, cudaEventRecord(h->ev[1], h->stream));
    if (!final) return SPG_OK;  // step 2 follows: its read-back checks both steps
    SPG_TRY(spg_check_flags(h, "symbolic step 1"));
    h->stats.ms_step1 = elapsed(h, 0, 1);
    return SPG_OK;
}

// Step 2 on C's tile structure from tiles_impl: masks, row offsets, tile
// nonzero prefix, value arrays.
static spg_status masks_impl(spg_handle_t h, const spg_tiles* A, const spg_tiles* B, spg_ctiles* C) {
    CPriv* cp = static_cast<CPriv*>(C->priv);
    const spg_algo algo = cp->algo;
    SPG_CUDA(h, cudaEventRecord(h->ev[7], h->stream));
    const int64_t nt = C->numtileC;
    // ---- step 2: bitmask symbolic
    int* tile_cnt = nullptr;
    SPG_TRY(spg_alloc_t(h, &C->maskC, (size_t)nt * TS + 16));
    SPG_TRY(spg_alloc_t(h, &C->ptrRowC, (size_t)nt * TS + 16));
    SPG_TRY(spg_alloc_t(h, &C->tile_nnzC, (size_t)nt + 1));
    if (algo == SPG_ALGO_ROWWISE) {
        // tile counts land in tile_nnzC itself and are scanned in place
        SPG_TRY(rowwise_symbolic(h, A, B, C, &cp->rw, C->tile_nnzC));
        SPG_TRY(spg_scan_i64_to_i64(h, C->tile_nnzC, C->tile_nnzC, nt));
    } else if (algo == SPG_ALGO_BINNED) {
        // the row-wise tile-rows, then the plain kernels over the listed
        // tiles; both leave tile counts in tile_nnzC, scanned in place.  The
        // pair cache covers the listed tiles; every other tile reads "not
        // cached" (-1) and intersects its lists if a plain kernel meets it.
        SPG_TRY(rowwise_symbolic(h, A, B, C, &cp->rw, C->tile_nnzC, cp->rowbin));
        const int64_t cap = spec_capacity(h, C, cp->nplain, cp->plain_pairs);
        if (cap > 0) {
            cp->plain.spec_cap = cap;
            SPG_TRY(spg_alloc_t(h, &cp->plain.spec_cnt, (size_t)nt + 1));
            SPG_TRY(spg_alloc_t(h, &cp->plain.spec_off, (size_t)nt + 1));
            SPG_TRY(spg_alloc_t(h, &cp->plain.spec_pa, (size_t)cap + 1));
            SPG_TRY(spg_alloc_t(h, &cp->plain.spec_pb, (size_t)cap + 1));
            SPG_CUDA(h, cudaMemsetAsync(cp->plain.spec_cnt, 0xff, sizeof(int) * ((size_t)nt + 1), h->stream));
        }
        SPG_TRY(plain_step2(h, A, B, C, &cp->plain, nullptr, C->tile_nnzC, cp->plain_list, cp->nplain));
        SPG_TRY(spg_scan_i64_to_i64(h, C->tile_nnzC, C->tile_nnzC, nt));
    } else {
        SPG_TRY(spg_alloc_t(h, &tile_cnt, (size_t)nt + 1));
        const int64_t cap = spec_capacity(h, C, nt, C->pairs);
        if (cap > 0) {
            cp->plain.spec_cap = cap;
            SPG_TRY(spg_alloc_t(h, &cp->plain.spec_cnt, (size_t)nt + 1));
            SPG_TRY(spg_alloc_t(h, &cp->plain.spec_off, (size_t)nt + 1));
            SPG_TRY(spg_alloc_t(h, &cp->plain.spec_pa, (size_t)cap + 1));
            SPG_TRY(spg_alloc_t(h, &cp->plain.spec_pb, (size_t)cap + 1));
        }
        SPG_TRY(plain_step2(h, A, B, C, &cp->plain, tile_cnt));
        SPG_TRY(spg_scan_i32_to_i64(h, tile_cnt, C->tile_nnzC, nt));
        spg_free_async(h, tile_cnt);
    }
    SPG_CUDA(h, cudaEventRecord(h->ev[2], h->stream));
    {   // nnzC, the tile pairs and both steps' device errors in one round trip
        const int64_t* src[2] = {C->tile_nnzC + nt, (const int64_t*)(cp->plain.counters + 2)};
        int64_t v[2] = {0, 0};
        SPG_TRY(spg_read_i64s_checked(h, 2, src, v, "symbolic"));
        C->nnzC = v[0];
        C->pairs = v[1];
    }
    if (!h->stats.ms_step1) h->stats.ms_step1 = elapsed(h, 0, 1);
    h->stats.ms_step2 = elapsed(h, 7, 2);
    const size_t vs = val_size(C->dtype);
    {   // values and column bytes in one allocation: a repeated product of the
        // same size then reuses one pooled block instead of splitting others
        const size_t vbytes = (vs * ((size_t)C->nnzC + 1) + 255) & ~(size_t)255;
        SPG_TRY(spg_alloc(h, &C->tile_valC, vbytes + (size_t)C->nnzC + 16));
        C->tile_colC = static_cast<uint8_t*>(C->tile_valC) + vbytes;
        cp->vals_joint = true;
    }
    return SPG_OK;
}

static spg_status symbolic_impl(spg_handle_t h, const spg_tiles* A, const spg_tiles* B, spg_algo algo,
                                spg_ctiles* C) {
    SPG_TRY(tiles_impl(h, A, B, algo, C, false));
    return masks_impl(h, A, B, C);
}

extern "C" spg_status spg_symbolic(spg_handle_t h, const spg_tiles* A, const spg_tiles* B, spg_algo algo,
                                   spg_ctiles* C) {
    SPG_TRY(validate_pair(h, A, B, C));
    h->stats = spg_stats{};
    spg_status s = symbolic_impl(h, A, B, algo, C);
    if (s != SPG_OK) { std::string e = h->err; spg_ctiles_free(h, C); h->err = e; }
    return s;
}

extern "C" spg_status spg_set_mixed_params(spg_handle_t h, int dense_thr, float cancel_eps) {
    if (!h) return SPG_ERR_INVALID;
    if (dense_thr < 1 || dense_thr > 256 || !(cancel_eps >= 0.f) || cancel_eps >= 1.f)
        return spg_fail(h, SPG_ERR_INVALID, "mixed params: dense_thr in [1, 256], cancel_eps in [0, 1)");
    h->dense_thr = dense_thr;
    h->cancel_eps = cancel_eps;
    return SPG_OK;
}

extern "C" spg_status spg_set_bin_params(spg_handle_t h, float pp_thr, float fill_thr) {
    if (!h) return SPG_ERR_INVALID;
    if (!(pp_thr >= 0.f) || !(fill_thr >= 0.f) || pp_thr > 1e9f || fill_thr > 256.f)
        return spg_fail(h, SPG_ERR_INVALID, "bin params: pp_thr in [0, 1e9], fill_thr in [0, 256]");
    h->bin_pp_thr = pp_thr;
    h->bin_fill_thr = fill_thr;
    return SPG_OK;
}

extern "C" spg_status spg_symbolic_tiles(spg_handle_t h, const spg_tiles* A, const spg_tiles* B, spg_algo algo,
                                         spg_ctiles* C) {
    SPG_TRY(validate_pair(h, A, B, C));
    h->stats = spg_stats{};
    spg_status s = tiles_impl(h, A, B, algo, C, true);
    if (s != SPG_OK) { std::string e = h->err; spg_ctiles_free(h, C); h->err = e; }
    return s;
}

extern "C" spg_status spg_symbolic_masks(spg_handle_t h, const spg_tiles* A, const spg_tiles* B, spg_ctiles* C) {
    SPG_TRY(validate_pair(h, A, B, C));
    if (!C->priv || (!C->tile_colidxC && C->numtileC > 0) || C->maskC)
        return spg_fail(h, SPG_ERR_INVALID, "symbolic masks: C must come from spg_symbolic_tiles");
    spg_status s = masks_impl(h, A, B, C);
    if (s != SPG_OK) { std::string e = h->err; spg_ctiles_free(h, C); h->err = e; }
    return s;
}

// Step 3 on C tile-rows [r0, r1).
// The kernels step 3 runs on: row-wise windows, plain per-C-tile registers,
// or plain with dense pairs on the tensor cores.
enum class NumPath { ROWWISE, PLAIN, MIXED, BINNED };

// Checks that C is ready for step 3 (symbolic structure and masks) and picks
// its path: MIXED for SPG_PREC_MIXED on FP32 data; ROWWISE when C's structure
// came from the row-wise symbolic phase, when it is asked for, or when FP64
// accumulation of FP32 data is; BINNED for a binned C; PLAIN otherwise.  The
// row-wise kernels build their plan (work items per tile-row) on first use
// when the symbolic phase did not.
static spg_status numeric_path(spg_handle_t h, const spg_tiles* A, const spg_tiles* B, spg_algo algo,
                               spg_precision prec, const spg_ctiles* C, NumPath* path) {
    SPG_TRY(validate_pair(h, A, B, C));
    if (!C->priv) return spg_fail(h, SPG_ERR_INVALID, "numeric: C has no symbolic structure");
    if (C->numtileC > 0 && (!C->maskC || !C->tile_nnzC || !C->tile_valC))
        return spg_fail(h, SPG_ERR_INVALID, "numeric: C has no symbolic masks yet (spg_symbolic_masks)");
    const CPriv* cp = static_cast<const CPriv*>(C->priv);
    const bool rw_ok = rowwise_numeric_fits(h);
    if (algo == SPG_ALGO_AUTO) algo = cp->algo;
    if (algo == SPG_ALGO_BINNED && cp->algo != SPG_ALGO_BINNED) algo = cp->algo;  // the bins come from step 1
    if (algo == SPG_ALGO_ROWWISE && !rw_ok) algo = SPG_ALGO_PLAIN;
    if (prec == SPG_PREC_MIXED && A->dtype == SPG_F32)
        *path = NumPath::MIXED;
    else if (algo == SPG_ALGO_ROWWISE || (prec == SPG_PREC_F64 && A->dtype == SPG_F32 && rw_ok))
        *path = NumPath::ROWWISE;  // FP64 accumulation of FP32 data: the row-wise kernels, every tile-row
    else if (prec == SPG_PREC_F64 && A->dtype == SPG_F32)
        return spg_fail(h, SPG_ERR_UNSUPPORTED,
                        "numeric: FP64 accumulation of FP32 data needs the row-wise kernels' shared memory");
    else if (algo == SPG_ALGO_BINNED)
        *path = NumPath::BINNED;
    else
        *path = NumPath::PLAIN;
    return SPG_OK;
}

static int32_t path_algo(NumPath p) {
    return p == NumPath::ROWWISE ? SPG_ALGO_ROWWISE : p == NumPath::BINNED ? SPG_ALGO_BINNED : SPG_ALGO_PLAIN;
}

static spg_status numeric_impl(spg_handle_t h, const spg_tiles* A, const spg_tiles* B, spg_algo algo,
                               spg_precision prec, spg_ctiles* C, int r0, int r1) {
    NumPath path;
    SPG_TRY(numeric_path(h, A, B, algo, prec, C, &path));
    if (r0 < 0 || r1 < r0 || r1 > C->tilem) return spg_fail(h, SPG_ERR_INVALID, "numeric: bad tile-row range");
    CPriv* cp = static_cast<CPriv*>(C->priv);
    const bool whole = r0 == 0 && r1 == C->tilem;
    h->stats.numeric_algo = path_algo(path);
    SPG_CUDA(h, cudaEventRecord(h->ev[3], h->stream));
    const bool mixed = path == NumPath::MIXED;
    if (path == NumPath::ROWWISE) {
        SPG_TRY(rowwise_numeric(h, A, B, C, &cp->rw, prec, r0, r1));
    } else if (path == NumPath::BINNED) {
        int64_t l0 = 0, l1 = cp->nplain;  // the listed tiles of tile-rows [r0, r1)
        if (!whole) {
            SPG_TRY(spg_read_i64(h, cp->plain_off + r0, &l0));
            SPG_TRY(spg_read_i64(h, cp->plain_off + r1, &l1));
        }
        SPG_TRY(plain_step3(h, A, B, C, &cp->plain, l0, l1, cp->plain_list));
        SPG_TRY(rowwise_numeric(h, A, B, C, &cp->rw, prec, r0, r1, cp->rowbin));
    } else {
        int64_t t0 = 0, t1 = C->numtileC;  // C tiles of the tile-rows
        if (!whole) {
            int x0 = 0, x1 = 0;
            SPG_TRY(spg_read_i32(h, C->tile_ptrC + r0, &x0));
            SPG_TRY(spg_read_i32(h, C->tile_ptrC + r1, &x1));
            t0 = x0;
            t1 = x1;
        }
        if (mixed)  // dense tile pairs on tensor cores (plain per-C-tile structure)
            SPG_TRY(plain_step3_mixed(h, A, B, C, &cp->plain, h->dense_thr, h->cancel_eps, t0, t1));
        else
            SPG_TRY(plain_step3(h, A, B, C, &cp->plain, t0, t1));
    }
    SPG_CUDA(h, cudaEventRecord(h->ev[4], h->stream));
    SPG_TRY(spg_check_flags(h, "numeric"));  // waits for the stream, so ev[4] is done
    h->stats.ms_step3 = elapsed(h, 3, 4);
    return SPG_OK;
}

extern "C" spg_status spg_numeric(spg_handle_t h, const spg_tiles* A, const spg_tiles* B, spg_algo algo,
                                  spg_precision prec, spg_ctiles* C) {
    if (!h || !C) return SPG_ERR_INVALID;
    return numeric_impl(h, A, B, algo, prec, C, 0, C->tilem);
}

// spg_numeric that reports bands of tile-rows as they complete.  Row-wise:
// one launch; its work items count down per band and the item completing a
// band sets the band's flag in mapped host memory, which this thread polls
// (sleeping between polls, bounded by the stream finishing or a time limit).
// Plain and mixed: one launch per band, reported in order.
extern "C" spg_status spg_numeric_bands(spg_handle_t h, const spg_tiles* A, const spg_tiles* B, spg_algo algo,
                                        spg_precision prec, spg_ctiles* C, int nbands, const int* band_rows,
                                        int order, spg_band_fn fn, void* user) {
    if (!h || !C) return SPG_ERR_INVALID;
    SPG_TRY(validate_pair(h, A, B, C));
    if (nbands < 1 || nbands > (1 << 16) || !band_rows || !fn ||
        (order != SPG_BANDS_FIRST_TO_LAST && order != SPG_BANDS_LAST_TO_FIRST))
        return spg_fail(h, SPG_ERR_INVALID, "numeric bands: 1..65536 bands, row bounds, an order and a callback");
    const bool last_first = order == SPG_BANDS_LAST_TO_FIRST;
    if (band_rows[0] != 0 || band_rows[nbands] != C->tilem)
        return spg_fail(h, SPG_ERR_INVALID, "numeric bands: bounds must run from 0 to tilem");
    for (int k = 0; k < nbands; k++)
        if (band_rows[k + 1] < band_rows[k]) return spg_fail(h, SPG_ERR_INVALID, "numeric bands: bounds descend");
    NumPath path;
    SPG_TRY(numeric_path(h, A, B, algo, prec, C, &path));
    CPriv* cp = static_cast<CPriv*>(C->priv);
    h->stats.numeric_algo = path_algo(path);
    if (path != NumPath::ROWWISE && path != NumPath::BINNED) {
        float ms = 0.f;
        for (int j = 0; j < nbands; j++) {
            const int k = last_first ? nbands - 1 - j : j;
            SPG_TRY(numeric_impl(h, A, B, algo, prec, C, band_rows[k], band_rows[k + 1]));
            ms += h->stats.ms_step3;
            fn(user, k, band_rows[k], band_rows[k + 1]);
        }
        h->stats.ms_step3 = ms;
        return SPG_OK;
    }
    if (h->band_cap < nbands) {
        if (h->h_band) cudaFreeHost(h->h_band);
        h->h_band = nullptr;
        h->d_band = nullptr;
        h->band_cap = 0;
        SPG_CUDA(h, cudaHostAlloc(reinterpret_cast<void**>(&h->h_band), (size_t)nbands * sizeof(int),
                                  cudaHostAllocMapped));
        SPG_CUDA(h, cudaHostGetDevicePointer(reinterpret_cast<void**>(&h->d_band), h->h_band, 0));
        h->band_cap = nbands;
    }
    volatile int* flag = h->h_band;
    for (int k = 0; k < nbands; k++) flag[k] = 0;
    int* d_rows = nullptr;
    int64_t* d_end = nullptr;
    unsigned* d_cnt = nullptr;
    struct Scratch {  // released on every return, stream-ordered after the launch
        spg_handle_t h;
        int** a;
        int64_t** b;
        unsigned** c;
        ~Scratch() {
            spg_free_async(h, *a);
            spg_free_async(h, *b);
            spg_free_async(h, *c);
        }
    } scratch{h, &d_rows, &d_end, &d_cnt};
    SPG_TRY(spg_alloc_t(h, &d_rows, (size_t)nbands + 1));
    SPG_TRY(spg_alloc_t(h, &d_end, (size_t)nbands));
    SPG_TRY(spg_alloc_t(h, &d_cnt, (size_t)nbands));
    SPG_CUDA(h, cudaMemcpyAsync(d_rows, band_rows, ((size_t)nbands + 1) * sizeof(int), cudaMemcpyHostToDevice,
                                h->stream));
    std::vector<int64_t> end((size_t)nbands);
    SPG_CUDA(h, cudaEventRecord(h->ev[3], h->stream));
    // binned: the plain kernels' tiles first (one launch), so a band is
    // complete once the row-wise items of its tile-rows are
    if (path == NumPath::BINNED) SPG_TRY(plain_step3(h, A, B, C, &cp->plain, 0, cp->nplain, cp->plain_list));
    const spg_status ls = rowwise_numeric_bands_launch(h, A, B, C, &cp->rw, prec, nbands, d_rows, d_end, d_cnt,
                                                       h->d_band, end.data(), last_first,
                                                       path == NumPath::BINNED ? cp->rowbin : nullptr);
    if (ls != SPG_OK) return ls;
    SPG_CUDA(h, cudaEventRecord(h->ev[4], h->stream));
    std::vector<char> told((size_t)nbands, 0);
    int left = nbands;
    for (int k = 0; k < nbands; k++)  // bands without work items are complete now
        if (end[k] == (k ? end[k - 1] : 0) || C->nnzC == 0) {
            told[k] = 1;
            left--;
            fn(user, k, band_rows[k], band_rows[k + 1]);
        }
    const auto t_start = std::chrono::steady_clock::now();
    bool finished = false;
    while (left > 0) {
        bool any = false;
        for (int k = 0; k < nbands; k++)
            if (!told[k] && flag[k]) {
                std::atomic_thread_fence(std::memory_order_acquire);
                told[k] = 1;
                left--;
                any = true;
                fn(user, k, band_rows[k], band_rows[k + 1]);
            }
        if (left == 0 || any) continue;
        if (finished) return spg_fail(h, SPG_ERR_CUDA, "numeric bands: launch ended with bands unreported");
        const cudaError_t q = cudaEventQuery(h->ev[4]);
        if (q == cudaSuccess) {
            finished = true;  // every flag store is visible now: one more scan
            continue;
        }
        if (q != cudaErrorNotReady) return spg_cuda_fail(h, q, "numeric bands");
        if (std::chrono::steady_clock::now() - t_start > std::chrono::seconds(600))
            return spg_fail(h, SPG_ERR_TIMEOUT, "numeric bands: no completion within 600 s");
        std::this_thread::sleep_for(std::chrono::microseconds(20));
    }
    SPG_CUDA(h, cudaEventSynchronize(h->ev[4]));
    h->stats.ms_step3 = elapsed(h, 3, 4);
    return spg_check_flags(h, "numeric bands");
}

extern "C" spg_status spg_numeric_rows(spg_handle_t h, const spg_tiles* A, const spg_tiles* B, spg_algo algo,
                                       spg_precision prec, spg_ctiles* C, int row_begin, int row_end) {
    if (!h || !C) return SPG_ERR_INVALID;
    return numeric_impl(h, A, B, algo, prec, C, row_begin, row_end);
}

extern "C" spg_status spg_spgemm(spg_handle_t h, const spg_tiles* A, const spg_tiles* B, spg_algo algo,
                                 spg_precision prec, spg_ctiles* C) {
    SPG_TRY(spg_symbolic(h, A, B, algo, C));
    spg_stats keep = h->stats;
    // an explicit PLAIN keeps the numeric phase on the plain kernels too
    spg_status s = spg_numeric(h, A, B, algo == SPG_ALGO_PLAIN ? SPG_ALGO_PLAIN : SPG_ALGO_AUTO, prec, C);
    keep.ms_step3 = h->stats.ms_step3;
    keep.numeric_algo = h->stats.numeric_algo;
    keep.tensor_pairs = h->stats.tensor_pairs;
    keep.fp64_tiles = h->stats.fp64_tiles;
    keep.work_items += h->stats.work_items;
    keep.products = keep.products ? keep.products : h->stats.products;
    h->stats = keep;
    return s;
}

// ---------------------------------------------------------------------------
// copies
// ---------------------------------------------------------------------------
template <typename T>
static spg_status d2h(spg_handle_t h, T* dst, const T* src, size_t count) {
    if (!dst || !src || count == 0) return SPG_OK;
    SPG_CUDA(h, cudaMemcpyAsync(dst, src, count * sizeof(T), cudaMemcpyDeviceToHost, h->stream));
    return SPG_OK;
}

extern "C" spg_status spg_ctiles_to_host(spg_handle_t h, const spg_ctiles* C, int* tile_ptrC, int* tile_rowidxC,
                                         int* tile_colidxC, uint16_t* maskC, int64_t* tile_nnzC,
                                         uint8_t* ptrRowC, void* tile_valC, uint8_t* tile_colC) {
    if (!h || !C) return SPG_ERR_INVALID;
    const size_t nt = (size_t)C->numtileC, nz = (size_t)C->nnzC;
    SPG_TRY(d2h(h, tile_ptrC, C->tile_ptrC, (size_t)C->tilem + 1));
    SPG_TRY(d2h(h, tile_rowidxC, C->tile_rowidxC, nt));
    SPG_TRY(d2h(h, tile_colidxC, C->tile_colidxC, nt));
    SPG_TRY(d2h(h, maskC, C->maskC, nt * TS));
    SPG_TRY(d2h(h, tile_nnzC, C->tile_nnzC, nt + 1));
    SPG_TRY(d2h(h, ptrRowC, C->ptrRowC, nt * TS));
    SPG_TRY(d2h(h, (uint8_t*)tile_valC, (const uint8_t*)C->tile_valC, nz * val_size(C->dtype)));
    SPG_TRY(d2h(h, tile_colC, C->tile_colC, nz));
    SPG_CUDA(h, cudaStreamSynchronize(h->stream));
    return SPG_OK;
}

extern "C" spg_status spg_ctiles_to_host_range(spg_handle_t h, const spg_ctiles* C, int64_t tb, int64_t te,
                                               int* tile_rowidxC, int* tile_colidxC, uint16_t* maskC,
                                               int64_t* tile_nnzC, uint8_t* ptrRowC, void* tile_valC,
                                               uint8_t* tile_colC, int64_t val_capacity, int64_t* n_values) {
    if (!h || !C) return SPG_ERR_INVALID;
    if (tb < 0 || te < tb || te > C->numtileC) return spg_fail(h, SPG_ERR_INVALID, "range: bad tile range");
    int64_t v0 = 0, v1 = 0;
    const bool need_nnz = tile_valC || tile_colC || tile_nnzC || n_values;
    if (need_nnz && C->numtileC > 0) {
        if (!C->tile_nnzC) return spg_fail(h, SPG_ERR_INVALID, "range: C has no symbolic masks yet");
        SPG_TRY(spg_read_i64(h, C->tile_nnzC + tb, &v0));
        SPG_TRY(spg_read_i64(h, C->tile_nnzC + te, &v1));
    }
    if (n_values) *n_values = v1 - v0;
    if ((tile_valC || tile_colC) && v1 - v0 > val_capacity)
        return spg_fail(h, SPG_ERR_INVALID, "range: value buffers too small");
    const size_t nt = (size_t)(te - tb), nz = (size_t)(v1 - v0);
    SPG_TRY(d2h(h, tile_rowidxC, C->tile_rowidxC + tb, nt));
    SPG_TRY(d2h(h, tile_colidxC, C->tile_colidxC + tb, nt));
    SPG_TRY(d2h(h, maskC, C->maskC + tb * TS, nt * TS));
    SPG_TRY(d2h(h, tile_nnzC, C->tile_nnzC + tb, nt + 1));
    SPG_TRY(d2h(h, ptrRowC, C->ptrRowC + tb * TS, nt * TS));
    SPG_TRY(d2h(h, (uint8_t*)tile_valC, (const uint8_t*)C->tile_valC + v0 * val_size(C->dtype),
                nz * val_size(C->dtype)));
    SPG_TRY(d2h(h, tile_colC, C->tile_colC + v0, nz));
    SPG_CUDA(h, cudaStreamSynchronize(h->stream));
    return SPG_OK;
}

extern "C" spg_status spg_tiles_to_host(spg_handle_t h, const spg_tiles* T, int* tile_ptr, int* tile_columnidx,
                                        int* tile_nnz, uint8_t* tile_csr_Ptr, uint16_t* mask, void* tile_csr_Val,
                                        uint8_t* tile_csr_Col, int* csc_tile_ptr, int* csc_tile_rowidx,
                                        uint8_t* tile_csc_Ptr, uint8_t* tile_csc_Row, void* tile_csc_Val) {
    if (!h || !T) return SPG_ERR_INVALID;
    const size_t nt = (size_t)T->numtile, nz = (size_t)T->nnz, vs = val_size(T->dtype);
    SPG_TRY(d2h(h, tile_ptr, T->tile_ptr, (size_t)T->tilem + 1));
    SPG_TRY(d2h(h, tile_columnidx, T->tile_columnidx, nt));
    SPG_TRY(d2h(h, tile_nnz, T->tile_nnz, nt + 1));
    SPG_TRY(d2h(h, tile_csr_Ptr, T->tile_csr_Ptr, nt * TS));
    SPG_TRY(d2h(h, mask, T->mask, nt * TS));
    SPG_TRY(d2h(h, (uint8_t*)tile_csr_Val, (const uint8_t*)T->tile_csr_Val, nz * vs));
    SPG_TRY(d2h(h, tile_csr_Col, T->tile_csr_Col, nz));
    SPG_TRY(d2h(h, csc_tile_ptr, T->csc_tile_ptr, (size_t)T->tilen + 1));
    SPG_TRY(d2h(h, csc_tile_rowidx, T->csc_tile_rowidx, nt));
    SPG_TRY(d2h(h, tile_csc_Ptr, T->tile_csc_Ptr, nt * TS));
    SPG_TRY(d2h(h, tile_csc_Row, T->tile_csc_Row, nz));
    SPG_TRY(d2h(h, (uint8_t*)tile_csc_Val, (const uint8_t*)T->tile_csc_Val, nz * vs));
    SPG_CUDA(h, cudaStreamSynchronize(h->stream));
    return SPG_OK;
}

// ---------------------------------------------------------------------------
// products (src/spgemm_raw_v2.cu:95-99)
// ---------------------------------------------------------------------------
__global__ void products_kernel(int64_t nnz, const int* __restrict__ a_ci, const int* __restrict__ b_rp,
                                unsigned long long* out) {
    unsigned long long s = 0;
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < nnz; j += (int64_t)gridDim.x * blockDim.x) {
        const int k = a_ci[j];
        s += (unsigned long long)(b_rp[k + 1] - b_rp[k]);
    }
    s = warp_sum(s);
    if ((threadIdx.x & 31) == 0 && s) atomicAdd(out, s);
}

extern "C" spg_status spg_products(spg_handle_t h, const spg_tiles* A, const spg_tiles* B, int64_t* out) {
    if (!h || !A || !B || !out) return SPG_ERR_INVALID;
    if (A->n != B->m) return spg_fail(h, SPG_ERR_INVALID, "inner dimensions differ");
    unsigned long long* d = nullptr;
    SPG_TRY(spg_alloc_t(h, &d, 1));
    SPG_CUDA(h, cudaMemsetAsync(d, 0, sizeof(unsigned long long), h->stream));
    if (A->nnz > 0) {
        int64_t g = ceil_div(A->nnz, 256);
        if (g > h->num_sms * 8) g = h->num_sms * 8;
        products_kernel<<<(int)g, 256, 0, h->stream>>>(A->nnz, A->col_idx, B->row_ptr, d);
        SPG_LAUNCHED(h);
    }
    SPG_TRY(spg_read_i64(h, (const int64_t*)d, out));
    spg_free_async(h, d);
    return SPG_OK;
}
