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

spg_status spg_check_flags(spg_handle_t h, const char* where) {
    SPG_CUDA(h, cudaMemcpyAsync(h->h_pinned + 1, h->d_flags, sizeof(unsigned), cudaMemcpyDeviceToHost, h->stream));
    SPG_CUDA(h, cudaStreamSynchronize(h->stream));
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
                      cp->plain.counters, cp->row_pairs};
        for (void* p : pp) spg_free_async(h, p);
        rowwise_free_priv(h, &cp->rw);
        delete cp;
    }
    *C = spg_ctiles{};
    return SPG_OK;
}

// Step 1: C's tile structure (tile_ptrC, tile_rowidxC, tile_colidxC).
static spg_status tiles_impl(spg_handle_t h, const spg_tiles* A, const spg_tiles* B, spg_algo algo,
                             spg_ctiles* C) {
    *C = spg_ctiles{};
    C->m = A->m; C->n = B->n; C->tilem = A->tilem; C->tilen = B->tilen; C->dtype = A->dtype;
    CPriv* cp = new (std::nothrow) CPriv();
    if (!cp) return spg_fail(h, SPG_ERR_OOM, "host allocation failed");
    C->priv = cp;
    if (algo == SPG_ALGO_AUTO) algo = rowwise_choose(h, A, B);
    cp->algo = algo;
    h->stats.algo_used = (int32_t)algo;
    SPG_TRY(spg_alloc_t(h, &cp->plain.counters, 4));
    SPG_CUDA(h, cudaMemsetAsync(cp->plain.counters, 0, 4 * sizeof(unsigned long long), h->stream));
    SPG_TRY(spg_alloc_t(h, &cp->row_pairs, (size_t)A->tilem + 1));
    SPG_CUDA(h, cudaEventRecord(h->ev[0], h->stream));
    // ---- step 1: C tile structure
    if (h->sizing) {
        spg_status st;
        {
            ScratchList sc(h);
            int* slot = nullptr;
            st = sc.alloc(&slot, (size_t)A->tilem + 1);
            if (st == SPG_OK) st = mlp_predict_rows(h, A, B, slot);
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
        SPG_TRY(plain_step1(h, A, B, C, cp->row_pairs, cp->plain.counters + 2));
    }
    SPG_CUDA(h, cudaEventRecord(h->ev[1], h->stream));
    SPG_CUDA(h, cudaEventSynchronize(h->ev[1]));
    h->stats.ms_step1 = elapsed(h, 0, 1);
    return spg_check_flags(h, "symbolic step 1");
}

// Step 2 on C's tile structure from tiles_impl: masks, row offsets, tile
// nonzero prefix, value arrays.
static spg_status masks_impl(spg_handle_t h, const spg_tiles* A, const spg_tiles* B, spg_ctiles* C) {
    CPriv* cp = static_cast<CPriv*>(C->priv);
    const spg_algo algo = cp->algo;
    SPG_CUDA(h, cudaEventRecord(h->ev[1], h->stream));
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
    } else {
        SPG_TRY(spg_alloc_t(h, &tile_cnt, (size_t)nt + 1));
        size_t fr = 0, tot = 0;
        cudaMemGetInfo(&fr, &tot);
        int64_t cap = 8 * nt;  // src/spgemm_raw_v2.cu:170
        if (const char* d = getenv("SPG_SPEC_CAP_DIV")) {  // test knob: force the overflow re-run
            const long div = atol(d);
            if (div > 1) cap = cap / div > 0 ? cap / div : 1;
        }
        if (cap > 0 && (size_t)cap * 8 + (size_t)nt * 8 < fr / 4) {
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
    SPG_TRY(spg_read_i64(h, C->tile_nnzC + nt, &C->nnzC));
    {
        int64_t pairs = 0;
        SPG_TRY(spg_read_i64(h, (const int64_t*)(cp->plain.counters + 2), &pairs));
        C->pairs = pairs;
    }
    const size_t vs = val_size(C->dtype);
    {   // values and column bytes in one allocation: a repeated product of the
        // same size then reuses one pooled block instead of splitting others
        const size_t vbytes = (vs * ((size_t)C->nnzC + 1) + 255) & ~(size_t)255;
        SPG_TRY(spg_alloc(h, &C->tile_valC, vbytes + (size_t)C->nnzC + 16));
        C->tile_colC = static_cast<uint8_t*>(C->tile_valC) + vbytes;
        cp->vals_joint = true;
    }
    SPG_CUDA(h, cudaEventRecord(h->ev[2], h->stream));
    SPG_CUDA(h, cudaEventSynchronize(h->ev[2]));
    h->stats.ms_step2 = elapsed(h, 1, 2);
    return spg_check_flags(h, "symbolic");
}

static spg_status symbolic_impl(spg_handle_t h, const spg_tiles* A, const spg_tiles* B, spg_algo algo,
                                spg_ctiles* C) {
    SPG_TRY(tiles_impl(h, A, B, algo, C));
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

extern "C" spg_status spg_symbolic_tiles(spg_handle_t h, const spg_tiles* A, const spg_tiles* B, spg_algo algo,
                                         spg_ctiles* C) {
    SPG_TRY(validate_pair(h, A, B, C));
    h->stats = spg_stats{};
    spg_status s = tiles_impl(h, A, B, algo, C);
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
enum class NumPath { ROWWISE, PLAIN, MIXED };

// Checks that C is ready for step 3 (symbolic structure and masks) and picks
// its path: MIXED for SPG_PREC_MIXED on FP32 data; ROWWISE when C's structure
// came from the row-wise symbolic phase (or FP64 accumulation of FP32 data is
// asked for); PLAIN otherwise.
static spg_status numeric_path(spg_handle_t h, const spg_tiles* A, const spg_tiles* B, spg_algo algo,
                               spg_precision prec, const spg_ctiles* C, NumPath* path) {
    SPG_TRY(validate_pair(h, A, B, C));
    if (!C->priv) return spg_fail(h, SPG_ERR_INVALID, "numeric: C has no symbolic structure");
    if (C->numtileC > 0 && (!C->maskC || !C->tile_nnzC || !C->tile_valC))
        return spg_fail(h, SPG_ERR_INVALID, "numeric: C has no symbolic masks yet (spg_symbolic_masks)");
    const CPriv* cp = static_cast<const CPriv*>(C->priv);
    if (algo == SPG_ALGO_AUTO) algo = cp->algo;
    if (algo == SPG_ALGO_ROWWISE && cp->algo != SPG_ALGO_ROWWISE) algo = SPG_ALGO_PLAIN;
    if (prec == SPG_PREC_MIXED && A->dtype == SPG_F32)
        *path = NumPath::MIXED;
    else if (algo == SPG_ALGO_ROWWISE || (prec == SPG_PREC_F64 && A->dtype == SPG_F32))
        *path = NumPath::ROWWISE;
    else
        *path = NumPath::PLAIN;
    return SPG_OK;
}

static spg_status numeric_impl(spg_handle_t h, const spg_tiles* A, const spg_tiles* B, spg_algo algo,
                               spg_precision prec, spg_ctiles* C, int r0, int r1) {
    NumPath path;
    SPG_TRY(numeric_path(h, A, B, algo, prec, C, &path));
    if (r0 < 0 || r1 < r0 || r1 > C->tilem) return spg_fail(h, SPG_ERR_INVALID, "numeric: bad tile-row range");
    CPriv* cp = static_cast<CPriv*>(C->priv);
    const bool whole = r0 == 0 && r1 == C->tilem;
    SPG_CUDA(h, cudaEventRecord(h->ev[3], h->stream));
    const bool mixed = path == NumPath::MIXED;
    if (path == NumPath::ROWWISE) {
        SPG_TRY(rowwise_numeric(h, A, B, C, &cp->rw, prec, r0, r1));
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
    SPG_CUDA(h, cudaEventSynchronize(h->ev[4]));
    h->stats.ms_step3 = elapsed(h, 3, 4);
    return spg_check_flags(h, "numeric");
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
    if (path != NumPath::ROWWISE) {
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
    const spg_status ls = rowwise_numeric_bands_launch(h, A, B, C, &cp->rw, prec, nbands, d_rows, d_end, d_cnt,
                                                       h->d_band, end.data(), last_first);
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
    spg_status s = spg_numeric(h, A, B, SPG_ALGO_AUTO, prec, C);
    keep.ms_step3 = h->stats.ms_step3;
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
