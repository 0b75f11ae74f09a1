// convert.cu -- device format conversions around the SpGEMM steps:
//
//   spg_csr_transpose   element CSR -> CSR of the transpose (stable: rows stay
//                       ascending inside each column), the device form of the
//                       reference's --aat transpose (src/spgemm_raw_v2.cu:79-90)
//   spg_ctiles_to_csr   C's tiles -> CSR, the device form of the reference's
//                       expansion of C for its CPU check (src/spgemm_raw_v2.cu:268-284);
//                       used to chain SpGEMMs (Galerkin P^T (A P))
#include "plain.cuh"
#include "spg_common.cuh"

namespace {

__global__ void row_ids_kernel(int m, const int* __restrict__ rp, uint32_t* __restrict__ rows) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int r = warp; r < m; r += nw)
        for (int j = rp[r] + lane; j < rp[r + 1]; j += 32) rows[j] = (uint32_t)r;
}

__global__ void copy_u32_kernel(const int* __restrict__ src, uint32_t* __restrict__ dst, int64_t n) {
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x)
        dst[t] = (uint32_t)src[t];
}

__global__ void col_hist_kernel(const int* __restrict__ ci, int64_t nnz, int* __restrict__ hist) {
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < nnz; t += (int64_t)gridDim.x * blockDim.x)
        atomicAdd(&hist[ci[t]], 1);
}

template <typename V>
__global__ void transpose_gather_kernel(int64_t nnz, const uint32_t* __restrict__ perm,
                                        const uint32_t* __restrict__ rows, const V* __restrict__ val,
                                        int* __restrict__ out_ci, V* __restrict__ out_val) {
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < nnz; p += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t j = perm[p];
        out_ci[p] = (int)rows[j];
        out_val[p] = val[j];
    }
}

// Row counts of C's CSR: thread per (C tile, row) adds popc(mask) to row_cnt.
__global__ void ctile_rowcount_kernel(int64_t numtileC, int m, const int* __restrict__ rowidxC,
                                      const uint16_t* __restrict__ maskC, int* __restrict__ row_cnt) {
    for (int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; x < numtileC * TS;
         x += (int64_t)gridDim.x * blockDim.x) {
        const int64_t t = x >> 4;
        const int r = (int)(x & 15);
        const int R = rowidxC[t] * TS + r;
        const int c = __popc((uint32_t)maskC[x]);
        if (c && R < m) atomicAdd(&row_cnt[R], c);
    }
}

// CSR fill: one warp per C tile-row, lanes over its tiles in chunks of 32;
// each of the 16 rows keeps a running offset so columns come out ascending.
template <typename V>
__global__ void ctile_fill_kernel(int tilem, int m, const int* __restrict__ tile_ptrC,
                                  const int* __restrict__ colidxC, const uint16_t* __restrict__ maskC,
                                  const int64_t* __restrict__ tile_nnzC, const uint8_t* __restrict__ ptrRowC,
                                  const V* __restrict__ valC, const int64_t* __restrict__ rp,
                                  int* __restrict__ out_ci, V* __restrict__ out_val) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int i = warp; i < tilem; i += nw) {
        const int ts = tile_ptrC[i], te = tile_ptrC[i + 1];
        for (int r = 0; r < TS; r++) {
            const int R = i * TS + r;
            if (R >= m) break;
            int64_t run = rp[R];
            for (int b = ts; b < te; b += 32) {
                const int t = b + lane;
                uint32_t mk = 0;
                if (t < te) mk = maskC[(int64_t)t * TS + r];
                const int c = __popc(mk);
                int inc = c;
#pragma unroll
                for (int d = 1; d < 32; d <<= 1) {
                    const int o = __shfl_up_sync(0xffffffffu, inc, d);
                    if (lane >= d) inc += o;
                }
                if (c) {
                    int64_t dst = run + inc - c;
                    const int64_t src = tile_nnzC[t] + ptrRowC[(int64_t)t * TS + r];
                    const int j = colidxC[t];
                    int q = 0;
                    while (mk) {
                        const int cl = __clz(mk) - 16;
                        out_ci[dst] = j * TS + cl;
                        out_val[dst] = valC[src + q];
                        dst++;
                        q++;
                        mk &= ~(0x8000u >> cl);
                    }
                }
                run += __shfl_sync(0xffffffffu, inc, 31);
            }
        }
    }
}

__global__ void i64_to_i32_rp_kernel(const int64_t* __restrict__ in, int* __restrict__ out, int64_t n) {
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x)
        out[t] = (int)in[t];
}

int cgrid(spg_handle_t h, int64_t n, int threads) {
    int64_t g = ceil_div(n, threads);
    const int64_t cap = (int64_t)h->num_sms * 16;
    if (g > cap) g = cap;
    return (int)(g < 1 ? 1 : g);
}

}  // namespace

extern "C" spg_status spg_csr_transpose(spg_handle_t h, int m, int n, int64_t nnz, const int* d_rp, const int* d_ci,
                                        const void* d_val, spg_dtype dtype, int* out_rp, int* out_ci,
                                        void* out_val) {
    if (!h) return SPG_ERR_INVALID;
    if (m < 0 || n < 0 || nnz < 0 || nnz >= 0x7fffffffLL) return spg_fail(h, SPG_ERR_INVALID, "transpose: bad size");
    if (!d_rp || !out_rp || (nnz > 0 && (!d_ci || !d_val || !out_ci || !out_val)))
        return spg_fail(h, SPG_ERR_INVALID, "transpose: null array");
    ScratchList sc(h);
    int* hist = nullptr;
    SPG_TRY(sc.alloc(&hist, (size_t)n + 1));
    SPG_CUDA(h, cudaMemsetAsync(hist, 0, sizeof(int) * ((size_t)n + 1), h->stream));
    if (nnz > 0) {
        col_hist_kernel<<<cgrid(h, nnz, 256), 256, 0, h->stream>>>(d_ci, nnz, hist);
        SPG_LAUNCHED(h);
    }
    SPG_TRY(spg_scan_i32_to_i32(h, hist, out_rp, n));
    if (nnz == 0) return SPG_OK;
    uint32_t *keys = nullptr, *perm = nullptr, *rows = nullptr;
    SPG_TRY(sc.alloc(&keys, (size_t)nnz));
    SPG_TRY(sc.alloc(&perm, (size_t)nnz));
    SPG_TRY(sc.alloc(&rows, (size_t)nnz));
    copy_u32_kernel<<<cgrid(h, nnz, 256), 256, 0, h->stream>>>(d_ci, keys, nnz);
    SPG_LAUNCHED(h);
    row_ids_kernel<<<cgrid(h, (int64_t)m * 32, 256), 256, 0, h->stream>>>(m, d_rp, rows);
    SPG_LAUNCHED(h);
    // the original position of each entry: its index (entries are in row order)
    SPG_TRY(spg_iota_u32(h, perm, nnz));
    int bits = 1;
    while (bits < 31 && (1LL << bits) < n) bits++;
    SPG_TRY(spg_radix_sort_pairs(h, keys, perm, nnz, bits));
    if (dtype == SPG_F64)
        transpose_gather_kernel<double><<<cgrid(h, nnz, 256), 256, 0, h->stream>>>(
            nnz, perm, rows, (const double*)d_val, out_ci, (double*)out_val);
    else
        transpose_gather_kernel<float><<<cgrid(h, nnz, 256), 256, 0, h->stream>>>(
            nnz, perm, rows, (const float*)d_val, out_ci, (float*)out_val);
    SPG_LAUNCHED(h);
    return SPG_OK;
}

spg_status ctiles_to_csr_impl(spg_handle_t h, const spg_ctiles* C, int* out_rp, int* out_ci, void* out_val,
                              int64_t* nnz_out) {
    const int m = C->m;
    ScratchList sc(h);
    int* cnt = nullptr;
    int64_t* rp64 = nullptr;
    SPG_TRY(sc.alloc(&cnt, (size_t)m + 1));
    SPG_TRY(sc.alloc(&rp64, (size_t)m + 1));
    SPG_CUDA(h, cudaMemsetAsync(cnt, 0, sizeof(int) * ((size_t)m + 1), h->stream));
    if (C->numtileC > 0) {
        ctile_rowcount_kernel<<<cgrid(h, C->numtileC * TS, 256), 256, 0, h->stream>>>(C->numtileC, m, C->tile_rowidxC,
                                                                                      C->maskC, cnt);
        SPG_LAUNCHED(h);
    }
    SPG_TRY(spg_scan_i32_to_i64(h, cnt, rp64, m));
    int64_t nnz = 0;
    SPG_TRY(spg_read_i64(h, rp64 + m, &nnz));
    if (nnz_out) *nnz_out = nnz;
    if (!out_rp) return SPG_OK;
    if (nnz >= 0x7fffffffLL) return spg_fail(h, SPG_ERR_INVALID, "to_csr: nnz does not fit int32 CSR");
    i64_to_i32_rp_kernel<<<cgrid(h, m + 1, 256), 256, 0, h->stream>>>(rp64, out_rp, m + 1);
    SPG_LAUNCHED(h);
    if (nnz > 0 && C->tilem > 0) {
        if (C->dtype == SPG_F64)
            ctile_fill_kernel<double><<<cgrid(h, (int64_t)C->tilem * 32, 256), 256, 0, h->stream>>>(
                C->tilem, m, C->tile_ptrC, C->tile_colidxC, C->maskC, C->tile_nnzC, C->ptrRowC,
                (const double*)C->tile_valC, rp64, out_ci, (double*)out_val);
        else
            ctile_fill_kernel<float><<<cgrid(h, (int64_t)C->tilem * 32, 256), 256, 0, h->stream>>>(
                C->tilem, m, C->tile_ptrC, C->tile_colidxC, C->maskC, C->tile_nnzC, C->ptrRowC,
                (const float*)C->tile_valC, rp64, out_ci, (float*)out_val);
        SPG_LAUNCHED(h);
    }
    return SPG_OK;
}

extern "C" spg_status spg_ctiles_to_csr(spg_handle_t h, const spg_ctiles* C, int* out_rp, int* out_ci,
                                        void* out_val, int64_t* nnz) {
    if (!h || !C) return SPG_ERR_INVALID;
    SPG_TRY(ctiles_to_csr_impl(h, C, out_rp, out_ci, out_val, nnz));
    return spg_check_flags(h, "to_csr");
}

// ---------------------------------------------------------------------------
// Galerkin triple product P^T (A P): two chained SpGEMMs on the device.
// ---------------------------------------------------------------------------
extern "C" spg_status spg_galerkin(spg_handle_t h, int m, int nc, int64_t nnzA, const int* A_rp, const int* A_ci,
                                   const void* A_val, int64_t nnzP, const int* P_rp, const int* P_ci,
                                   const void* P_val, spg_dtype dtype, spg_algo algo, spg_precision prec,
                                   spg_ctiles* RAP, int64_t* products_out) {
    if (!h || !RAP) return SPG_ERR_INVALID;
    const size_t vs = val_size(dtype);
    spg_tiles tA{}, tP{}, tAP{}, tPT{};
    spg_ctiles AP{};
    int *ap_rp = nullptr, *ap_ci = nullptr, *pt_rp = nullptr, *pt_ci = nullptr;
    void *ap_val = nullptr, *pt_val = nullptr;
    int64_t prod1 = 0, prod2 = 0, nnzAP = 0;
    spg_status s = SPG_OK;
    auto cleanup = [&]() {
        std::string e = h->err;
        spg_tiles_free(h, &tA); spg_tiles_free(h, &tP); spg_tiles_free(h, &tAP); spg_tiles_free(h, &tPT);
        spg_ctiles_free(h, &AP);
        spg_free_async(h, ap_rp); spg_free_async(h, ap_ci); spg_free_async(h, ap_val);
        spg_free_async(h, pt_rp); spg_free_async(h, pt_ci); spg_free_async(h, pt_val);
        h->err = e;
    };
#define GTRY(call) do { s = (call); if (s != SPG_OK) { cleanup(); return s; } } while (0)
    GTRY(spg_tile_from_csr(h, m, m, nnzA, A_rp, A_ci, A_val, dtype, SPG_LAYOUT_ROW, 0, &tA));
    GTRY(spg_tile_from_csr(h, m, nc, nnzP, P_rp, P_ci, P_val, dtype, SPG_LAYOUT_B_CSC, 0, &tP));
    GTRY(spg_products(h, &tA, &tP, &prod1));
    GTRY(spg_spgemm(h, &tA, &tP, algo, prec, &AP));
    const spg_stats first = h->stats;
    nnzAP = AP.nnzC;  // known from the symbolic phase: one export pass, no counting pass
    if (nnzAP >= 0x7fffffffLL) { s = spg_fail(h, SPG_ERR_INVALID, "galerkin: A*P does not fit an int32 CSR"); cleanup(); return s; }
    GTRY(spg_alloc_t(h, &ap_rp, (size_t)m + 1));
    GTRY(spg_alloc_t(h, &ap_ci, (size_t)nnzAP + 1));
    GTRY(spg_alloc(h, &ap_val, vs * ((size_t)nnzAP + 1)));
    GTRY(ctiles_to_csr_impl(h, &AP, ap_rp, ap_ci, ap_val, &nnzAP));
    spg_ctiles_free(h, &AP);
    GTRY(spg_tile_from_csr(h, m, nc, nnzAP, ap_rp, ap_ci, ap_val, dtype, SPG_LAYOUT_B_CSC, 0, &tAP));
    GTRY(spg_alloc_t(h, &pt_rp, (size_t)nc + 1));
    GTRY(spg_alloc_t(h, &pt_ci, (size_t)nnzP + 1));
    GTRY(spg_alloc(h, &pt_val, vs * ((size_t)nnzP + 1)));
    GTRY(spg_csr_transpose(h, m, nc, nnzP, P_rp, P_ci, P_val, dtype, pt_rp, pt_ci, pt_val));
    GTRY(spg_tile_from_csr(h, nc, m, nnzP, pt_rp, pt_ci, pt_val, dtype, SPG_LAYOUT_ROW, 0, &tPT));
    GTRY(spg_products(h, &tPT, &tAP, &prod2));
    GTRY(spg_spgemm(h, &tPT, &tAP, algo, prec, RAP));
#undef GTRY
    // the call's statistics cover both products
    spg_stats& st = h->stats;
    st.ms_step1 += first.ms_step1;
    st.ms_step2 += first.ms_step2;
    st.ms_step3 += first.ms_step3;
    st.products += first.products;
    st.overflow_reruns += first.overflow_reruns;
    st.work_items += first.work_items;
    st.tensor_pairs += first.tensor_pairs;
    st.fp64_tiles += first.fp64_tiles;
    st.sizing_fallbacks += first.sizing_fallbacks;
    st.predicted_tiles += first.predicted_tiles;
    if (products_out) *products_out = prod1 + prod2;
    cleanup();
    return SPG_OK;
}
