// batch.cu -- many independent SpGEMMs C_p = A_p * B_p in one launch per phase.
//
// The reference multiplies one matrix per process run (src/spgemm_raw_v2.cu:61).
// For a batch of uneven products (n from 1,024 to 65,536) one launch per
// product leaves most of the GPU idle and pays ~10 launches and 3 host
// round trips per product.  Here a batch -- or each bin of it -- is assembled
// on the device as ONE block-diagonal product
//     diag(A_0, A_1, ...) * diag(B_0, B_1, ...) = diag(A_0 B_0, A_1 B_1, ...)
// with every block at a 16-aligned offset, so no tile straddles two problems,
// the tile format of the big product is the union of the per-problem tile
// formats (shifted), and each problem's C is a contiguous range of C tiles.
// The persistent, work-balanced kernels then schedule all problems together.
//
// The numeric phase of a bin can be re-run for new values of the same
// structure without any host synchronisation, so it is captured once into a
// CUDA graph (values host->device, numeric kernel, C values device->host) and
// replayed.  An autotuner picks the bin thresholds and, per bin, the algorithm
// (plain per-C-tile or row-wise) by timing them on the batch itself.
#include <algorithm>
#include <cstring>
#include <new>
#include <vector>

#include "plain.cuh"
#include "rowwise.cuh"
#include "spg_common.cuh"

namespace {

__global__ void bd_rowptr_kernel(int64_t M, int nprob, const int64_t* __restrict__ roff,
                                 const int* __restrict__ mrows, const int64_t* __restrict__ nzoff,
                                 const int64_t* __restrict__ rpslot, const int* __restrict__ rp_local,
                                 const int64_t* __restrict__ nnz, int* __restrict__ rp_big) {
    for (int64_t R = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; R <= M; R += (int64_t)gridDim.x * blockDim.x) {
        if (R == M) {
            rp_big[R] = (int)(nzoff[nprob - 1] + nnz[nprob - 1]);
            continue;
        }
        int lo = 0, hi = nprob;  // last p with roff[p] <= R
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (roff[mid] <= R) lo = mid; else hi = mid;
        }
        const int64_t r = R - roff[lo];
        rp_big[R] = (int)(nzoff[lo] + (r < mrows[lo] ? rp_local[rpslot[lo] + r] : nnz[lo]));
    }
}

__global__ void bd_colshift_kernel(int64_t NZ, int nprob, const int64_t* __restrict__ nzoff,
                                   const int64_t* __restrict__ coff, int* __restrict__ ci) {
    for (int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; j < NZ; j += (int64_t)gridDim.x * blockDim.x) {
        int lo = 0, hi = nprob;  // last p with nzoff[p] <= j
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (nzoff[mid] <= j) lo = mid; else hi = mid;
        }
        ci[j] += (int)coff[lo];
    }
}

inline int64_t pad16(int64_t x) { return (x + 15) & ~int64_t(15); }

}  // namespace

// One bin: a subset of the problems assembled block-diagonally.
struct BatchBin {
    std::vector<int> probs;                        // problem ids in this bin
    std::vector<int64_t> roff, koff, noff, aoff, boff;  // per member
    int64_t M = 0, K = 0, N = 0, NA = 0, NB = 0;
    spg_tiles A{}, B{};
    spg_ctiles C{};
    bool has_c = false;
    spg_algo algo = SPG_ALGO_ROWWISE;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
};

struct spg_batch_s {
    int nprob = 0;
    spg_dtype dtype = SPG_F32;
    std::vector<int> m, k, n;
    std::vector<int64_t> nnzA, nnzB;
    std::vector<const int*> a_rp, a_ci, b_rp, b_ci;
    std::vector<const void*> a_val, b_val;
    std::vector<BatchBin> bins;
    std::vector<int> bin_of, slot_of;  // problem -> (bin, position in bin)
    std::vector<int> thresholds;       // bin upper bounds on n (ascending)
    int64_t products = 0;
};

static void free_bin(spg_handle_t h, BatchBin& b) {
    if (b.exec) cudaGraphExecDestroy(b.exec);
    if (b.graph) cudaGraphDestroy(b.graph);
    b.exec = nullptr;
    b.graph = nullptr;
    spg_tiles_free(h, &b.A);
    spg_tiles_free(h, &b.B);
    if (b.has_c) spg_ctiles_free(h, &b.C);
    b.has_c = false;
}

// Assemble one block-diagonal operand on the device from host CSR blocks.
static spg_status assemble(spg_handle_t h, spg_batch_t bt, const std::vector<int>& probs, bool left,
                           const std::vector<int64_t>& roff, const std::vector<int64_t>& coff,
                           const std::vector<int64_t>& nzoff, int64_t rows, int64_t cols, int64_t NZ,
                           spg_tiles* out) {
    const int np = (int)probs.size();
    const size_t vs = val_size(bt->dtype);
    std::vector<int> mrows(np);
    std::vector<int64_t> rpslot(np), nnz(np);
    int64_t slots = 0;
    for (int q = 0; q < np; q++) {
        const int p = probs[q];
        mrows[q] = left ? bt->m[p] : bt->k[p];
        nnz[q] = left ? bt->nnzA[p] : bt->nnzB[p];
        rpslot[q] = slots;
        slots += mrows[q] + 1;
    }
    int *rp_big = nullptr, *ci_big = nullptr, *rp_local = nullptr, *d_mrows = nullptr;
    int64_t *d_roff = nullptr, *d_coff = nullptr, *d_nzoff = nullptr, *d_slot = nullptr, *d_nnz = nullptr;
    void* val_big = nullptr;
    SPG_TRY(spg_alloc_t(h, &rp_big, (size_t)rows + 1));
    SPG_TRY(spg_alloc_t(h, &ci_big, (size_t)NZ + 1));
    SPG_TRY(spg_alloc(h, &val_big, vs * ((size_t)NZ + 1)));
    SPG_TRY(spg_alloc_t(h, &rp_local, (size_t)slots + 1));
    SPG_TRY(spg_alloc_t(h, &d_mrows, (size_t)np));
    SPG_TRY(spg_alloc_t(h, &d_roff, (size_t)np));
    SPG_TRY(spg_alloc_t(h, &d_coff, (size_t)np));
    SPG_TRY(spg_alloc_t(h, &d_nzoff, (size_t)np));
    SPG_TRY(spg_alloc_t(h, &d_slot, (size_t)np));
    SPG_TRY(spg_alloc_t(h, &d_nnz, (size_t)np));
    for (int q = 0; q < np; q++) {
        const int p = probs[q];
        const int* rp = left ? bt->a_rp[p] : bt->b_rp[p];
        const int* ci = left ? bt->a_ci[p] : bt->b_ci[p];
        const void* v = left ? bt->a_val[p] : bt->b_val[p];
        SPG_CUDA(h, cudaMemcpyAsync(rp_local + rpslot[q], rp, sizeof(int) * (mrows[q] + 1), cudaMemcpyHostToDevice,
                                    h->stream));
        if (nnz[q] > 0) {
            SPG_CUDA(h, cudaMemcpyAsync(ci_big + nzoff[q], ci, sizeof(int) * nnz[q], cudaMemcpyHostToDevice, h->stream));
            SPG_CUDA(h, cudaMemcpyAsync((char*)val_big + vs * nzoff[q], v, vs * nnz[q], cudaMemcpyHostToDevice,
                                        h->stream));
        }
    }
    SPG_CUDA(h, cudaMemcpyAsync(d_mrows, mrows.data(), sizeof(int) * np, cudaMemcpyHostToDevice, h->stream));
    SPG_CUDA(h, cudaMemcpyAsync(d_roff, roff.data(), sizeof(int64_t) * np, cudaMemcpyHostToDevice, h->stream));
    SPG_CUDA(h, cudaMemcpyAsync(d_coff, coff.data(), sizeof(int64_t) * np, cudaMemcpyHostToDevice, h->stream));
    SPG_CUDA(h, cudaMemcpyAsync(d_nzoff, nzoff.data(), sizeof(int64_t) * np, cudaMemcpyHostToDevice, h->stream));
    SPG_CUDA(h, cudaMemcpyAsync(d_slot, rpslot.data(), sizeof(int64_t) * np, cudaMemcpyHostToDevice, h->stream));
    SPG_CUDA(h, cudaMemcpyAsync(d_nnz, nnz.data(), sizeof(int64_t) * np, cudaMemcpyHostToDevice, h->stream));
    {
        int64_t g = ceil_div(rows + 1, 256);
        if (g > h->num_sms * 16) g = h->num_sms * 16;
        bd_rowptr_kernel<<<(int)g, 256, 0, h->stream>>>(rows, np, d_roff, d_mrows, d_nzoff, d_slot, rp_local, d_nnz,
                                                        rp_big);
        SPG_LAUNCHED(h);
        if (NZ > 0) {
            int64_t g2 = ceil_div(NZ, 256);
            if (g2 > h->num_sms * 16) g2 = h->num_sms * 16;
            bd_colshift_kernel<<<(int)g2, 256, 0, h->stream>>>(NZ, np, d_nzoff, d_coff, ci_big);
            SPG_LAUNCHED(h);
        }
    }
    spg_status s = spg_tile_from_csr(h, (int)rows, (int)cols, NZ, rp_big, ci_big, val_big, bt->dtype,
                                     left ? SPG_LAYOUT_ROW : SPG_LAYOUT_B_CSC, 0, out);
    void* tmp[] = {rp_big, ci_big, val_big, rp_local, d_mrows, d_roff, d_coff, d_nzoff, d_slot, d_nnz};
    for (void* p : tmp) spg_free_async(h, p);
    return s;
}

static spg_status build_bins(spg_handle_t h, spg_batch_t bt, const std::vector<int>& thresholds) {
    for (auto& b : bt->bins) free_bin(h, b);
    bt->bins.clear();
    bt->thresholds = thresholds;
    const int nb = (int)thresholds.size() + 1;
    bt->bins.resize(nb);
    bt->bin_of.assign(bt->nprob, 0);
    bt->slot_of.assign(bt->nprob, 0);
    for (int p = 0; p < bt->nprob; p++) {
        int b = 0;
        while (b < (int)thresholds.size() && bt->n[p] > thresholds[b]) b++;
        bt->bin_of[p] = b;
        bt->slot_of[p] = (int)bt->bins[b].probs.size();
        bt->bins[b].probs.push_back(p);
    }
    for (auto& b : bt->bins) {
        int64_t R = 0, K = 0, N = 0, NA = 0, NB = 0;
        for (int p : b.probs) {
            b.roff.push_back(R); b.koff.push_back(K); b.noff.push_back(N);
            b.aoff.push_back(NA); b.boff.push_back(NB);
            R += pad16(bt->m[p]); K += pad16(bt->k[p]); N += pad16(bt->n[p]);
            NA += bt->nnzA[p]; NB += bt->nnzB[p];
        }
        b.M = R; b.K = K; b.N = N; b.NA = NA; b.NB = NB;
        if (b.probs.empty()) continue;
        if (R >= 0x7ffffff0 || K >= 0x7ffffff0 || N >= 0x7ffffff0 || NA >= 0x7fffffff || NB >= 0x7fffffff)
            return spg_fail(h, SPG_ERR_INVALID, "batch: a bin exceeds int32 indexing");
        SPG_TRY(assemble(h, bt, b.probs, true, b.roff, b.koff, b.aoff, R, K, NA, &b.A));
        SPG_TRY(assemble(h, bt, b.probs, false, b.koff, b.noff, b.boff, K, N, NB, &b.B));
    }
    return SPG_OK;
}

extern "C" spg_status spg_batch_create_host(spg_handle_t h, int nprob, const int* m, const int* k, const int* n,
                                            const int64_t* nnzA, const int* const* A_rp, const int* const* A_ci,
                                            const void* const* A_val, const int64_t* nnzB, const int* const* B_rp,
                                            const int* const* B_ci, const void* const* B_val, spg_dtype dtype,
                                            spg_batch_t* out) {
    if (!h || !out || nprob <= 0) return spg_fail(h, SPG_ERR_INVALID, "batch: bad arguments");
    spg_batch_t bt = new (std::nothrow) spg_batch_s();
    if (!bt) return spg_fail(h, SPG_ERR_OOM, "batch: host allocation failed");
    bt->nprob = nprob;
    bt->dtype = dtype;
    for (int p = 0; p < nprob; p++) {
        if (m[p] < 0 || k[p] < 0 || n[p] < 0 || nnzA[p] < 0 || nnzB[p] < 0) {
            delete bt;
            return spg_fail(h, SPG_ERR_INVALID, "batch: negative size");
        }
        bt->m.push_back(m[p]); bt->k.push_back(k[p]); bt->n.push_back(n[p]);
        bt->nnzA.push_back(nnzA[p]); bt->nnzB.push_back(nnzB[p]);
        bt->a_rp.push_back(A_rp[p]); bt->a_ci.push_back(A_ci[p]); bt->a_val.push_back(A_val[p]);
        bt->b_rp.push_back(B_rp[p]); bt->b_ci.push_back(B_ci[p]); bt->b_val.push_back(B_val[p]);
    }
    spg_status s = build_bins(h, bt, {});
    if (s != SPG_OK) {
        std::string e = h->err;
        spg_batch_free(h, bt);
        h->err = e;
        return s;
    }
    *out = bt;
    return SPG_OK;
}

extern "C" spg_status spg_batch_free(spg_handle_t h, spg_batch_t bt) {
    if (!h || !bt) return SPG_ERR_INVALID;
    for (auto& b : bt->bins) free_bin(h, b);
    delete bt;
    return SPG_OK;
}

static spg_status run_bin(spg_handle_t h, BatchBin& b, spg_algo algo, spg_precision prec) {
    if (b.probs.empty()) return SPG_OK;
    if (b.exec) { cudaGraphExecDestroy(b.exec); b.exec = nullptr; }
    if (b.graph) { cudaGraphDestroy(b.graph); b.graph = nullptr; }
    if (b.has_c) spg_ctiles_free(h, &b.C);
    b.has_c = false;
    SPG_TRY(spg_spgemm(h, &b.A, &b.B, algo, prec, &b.C));
    b.has_c = true;
    return SPG_OK;
}

extern "C" spg_status spg_batch_spgemm(spg_handle_t h, spg_batch_t bt, spg_algo algo, spg_precision prec) {
    if (!h || !bt) return SPG_ERR_INVALID;
    bt->products = 0;
    float ms = 0.f;
    SPG_CUDA(h, cudaEventRecord(h->ev[5], h->stream));
    for (auto& b : bt->bins) {
        if (b.probs.empty()) continue;
        SPG_TRY(run_bin(h, b, algo == SPG_ALGO_AUTO ? b.algo : algo, prec));
        int64_t pr = 0;
        SPG_TRY(spg_products(h, &b.A, &b.B, &pr));
        bt->products += pr;
    }
    SPG_CUDA(h, cudaEventRecord(h->ev[6], h->stream));
    SPG_CUDA(h, cudaEventSynchronize(h->ev[6]));
    cudaEventElapsedTime(&ms, h->ev[5], h->ev[6]);
    h->stats.ms_step1 = ms;  // whole batch
    h->stats.ms_step2 = 0.f;
    h->stats.ms_step3 = 0.f;
    h->stats.products = bt->products;
    return SPG_OK;
}

extern "C" spg_status spg_batch_info(spg_handle_t h, spg_batch_t bt, int p, int64_t* numtileC, int64_t* nnzC,
                                     int64_t* products) {
    if (!h || !bt) return SPG_ERR_INVALID;
    if (products) *products = bt->products;
    if (p < 0) return SPG_OK;
    if (p >= bt->nprob) return spg_fail(h, SPG_ERR_INVALID, "batch: bad problem index");
    BatchBin& b = bt->bins[bt->bin_of[p]];
    if (!b.has_c) return spg_fail(h, SPG_ERR_INVALID, "batch: not multiplied yet");
    const int q = bt->slot_of[p];
    const int64_t tr0 = b.roff[q] / TS, tr1 = tr0 + pad16(bt->m[p]) / TS;
    int* tp = reinterpret_cast<int*>(h->h_pinned + 8);
    SPG_CUDA(h, cudaMemcpyAsync(tp, b.C.tile_ptrC + tr0, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    SPG_CUDA(h, cudaMemcpyAsync(tp + 1, b.C.tile_ptrC + tr1, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    SPG_CUDA(h, cudaStreamSynchronize(h->stream));
    const int64_t t0 = tp[0], t1 = tp[1];
    int64_t v0 = 0, v1 = 0;
    SPG_TRY(spg_read_i64(h, b.C.tile_nnzC + t0, &v0));
    SPG_TRY(spg_read_i64(h, b.C.tile_nnzC + t1, &v1));
    if (numtileC) *numtileC = t1 - t0;
    if (nnzC) *nnzC = v1 - v0;
    return SPG_OK;
}

extern "C" spg_status spg_batch_to_host(spg_handle_t h, spg_batch_t bt, int p, int* tile_ptrC, int* tile_rowidxC,
                                        int* tile_colidxC, uint16_t* maskC, int64_t* tile_nnzC, uint8_t* ptrRowC,
                                        void* tile_valC, uint8_t* tile_colC) {
    if (!h || !bt || p < 0 || p >= bt->nprob) return spg_fail(h, SPG_ERR_INVALID, "batch: bad problem index");
    BatchBin& b = bt->bins[bt->bin_of[p]];
    if (!b.has_c) return spg_fail(h, SPG_ERR_INVALID, "batch: not multiplied yet");
    const int q = bt->slot_of[p];
    const int64_t tr0 = b.roff[q] / TS;
    const int tilem = (bt->m[p] + TS - 1) / TS;
    std::vector<int> tp(tilem + 1);
    SPG_CUDA(h, cudaMemcpyAsync(tp.data(), b.C.tile_ptrC + tr0, sizeof(int) * (tilem + 1), cudaMemcpyDeviceToHost,
                                h->stream));
    SPG_CUDA(h, cudaStreamSynchronize(h->stream));
    const int64_t t0 = tp[0], t1 = tp[tilem];
    std::vector<int64_t> nz(t1 - t0 + 1);
    SPG_CUDA(h, cudaMemcpyAsync(nz.data(), b.C.tile_nnzC + t0, sizeof(int64_t) * (t1 - t0 + 1),
                                cudaMemcpyDeviceToHost, h->stream));
    SPG_CUDA(h, cudaStreamSynchronize(h->stream));
    const int64_t v0 = nz[0], v1 = nz[t1 - t0], nt = t1 - t0, nv = v1 - v0;
    const size_t vs = val_size(bt->dtype);
    if (tile_ptrC)
        for (int i = 0; i <= tilem; i++) tile_ptrC[i] = (int)(tp[i] - t0);
    if (tile_nnzC)
        for (int64_t t = 0; t <= nt; t++) tile_nnzC[t] = nz[t] - v0;
    if (tile_rowidxC && nt)
        SPG_CUDA(h, cudaMemcpyAsync(tile_rowidxC, b.C.tile_rowidxC + t0, sizeof(int) * nt, cudaMemcpyDeviceToHost,
                                    h->stream));
    if (tile_colidxC && nt)
        SPG_CUDA(h, cudaMemcpyAsync(tile_colidxC, b.C.tile_colidxC + t0, sizeof(int) * nt, cudaMemcpyDeviceToHost,
                                    h->stream));
    if (maskC && nt)
        SPG_CUDA(h, cudaMemcpyAsync(maskC, b.C.maskC + t0 * TS, sizeof(uint16_t) * nt * TS, cudaMemcpyDeviceToHost,
                                    h->stream));
    if (ptrRowC && nt)
        SPG_CUDA(h, cudaMemcpyAsync(ptrRowC, b.C.ptrRowC + t0 * TS, nt * TS, cudaMemcpyDeviceToHost, h->stream));
    if (tile_valC && nv)
        SPG_CUDA(h, cudaMemcpyAsync(tile_valC, (const char*)b.C.tile_valC + vs * v0, vs * nv,
                                    cudaMemcpyDeviceToHost, h->stream));
    if (tile_colC && nv)
        SPG_CUDA(h, cudaMemcpyAsync(tile_colC, b.C.tile_colC + v0, nv, cudaMemcpyDeviceToHost, h->stream));
    SPG_CUDA(h, cudaStreamSynchronize(h->stream));
    const int64_t rbase = b.roff[q] / TS, cbase = b.noff[q] / TS;
    if (tile_rowidxC)
        for (int64_t t = 0; t < nt; t++) tile_rowidxC[t] -= (int)rbase;
    if (tile_colidxC)
        for (int64_t t = 0; t < nt; t++) tile_colidxC[t] -= (int)cbase;
    return SPG_OK;
}

// ---------------------------------------------------------------------------
// values of the same structure: update, numeric only, CUDA graph
// ---------------------------------------------------------------------------
extern "C" spg_status spg_batch_set_values_host(spg_handle_t h, spg_batch_t bt, const void* const* A_val,
                                                const void* const* B_val) {
    if (!h || !bt) return SPG_ERR_INVALID;
    const size_t vs = val_size(bt->dtype);
    for (auto& b : bt->bins) {
        for (size_t q = 0; q < b.probs.size(); q++) {
            const int p = b.probs[q];
            if (A_val && A_val[p] && bt->nnzA[p])
                SPG_CUDA(h, cudaMemcpyAsync((char*)b.A.row_val + vs * b.aoff[q], A_val[p], vs * bt->nnzA[p],
                                            cudaMemcpyHostToDevice, h->stream));
            if (B_val && B_val[p] && bt->nnzB[p])
                SPG_CUDA(h, cudaMemcpyAsync((char*)b.B.row_val + vs * b.boff[q], B_val[p], vs * bt->nnzB[p],
                                            cudaMemcpyHostToDevice, h->stream));
        }
    }
    return SPG_OK;
}

spg_status rowwise_numeric_launch(spg_handle_t h, const spg_tiles* A, const spg_tiles* B, spg_ctiles* C,
                                  RowwisePriv* rp, spg_precision prec);
RowwisePriv* ctiles_rowwise_priv(spg_ctiles* C);

extern "C" spg_status spg_batch_numeric(spg_handle_t h, spg_batch_t bt, spg_precision prec) {
    if (!h || !bt) return SPG_ERR_INVALID;
    for (auto& b : bt->bins) {
        if (b.probs.empty()) continue;
        if (!b.has_c) return spg_fail(h, SPG_ERR_INVALID, "batch: run spg_batch_spgemm first");
        RowwisePriv* rp = ctiles_rowwise_priv(&b.C);
        SPG_TRY(rowwise_numeric_launch(h, &b.A, &b.B, &b.C, rp, prec));
    }
    return SPG_OK;
}

// Capture (values H2D for every problem -> row-wise numeric -> C values D2H)
// of every bin into one CUDA graph per bin; replays with spg_batch_graph_launch.
// host_vals_out[bin] receives C's values of the bin in block order.
extern "C" spg_status spg_batch_graph_capture(spg_handle_t h, spg_batch_t bt, const void* const* A_val,
                                              const void* const* B_val, void* const* host_vals_out,
                                              spg_precision prec) {
    if (!h || !bt) return SPG_ERR_INVALID;
    if (!h->stream) return spg_fail(h, SPG_ERR_INVALID, "batch graph: the handle needs a non-default stream");
    SPG_TRY(spg_batch_numeric(h, bt, prec));  // sets kernel attributes before capture
    SPG_CUDA(h, cudaStreamSynchronize(h->stream));
    int bi = 0;
    for (auto& b : bt->bins) {
        if (b.probs.empty()) { bi++; continue; }
        if (b.exec) { cudaGraphExecDestroy(b.exec); b.exec = nullptr; }
        if (b.graph) { cudaGraphDestroy(b.graph); b.graph = nullptr; }
        SPG_CUDA(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
        const size_t vs = val_size(bt->dtype);
        spg_status s = SPG_OK;
        for (size_t q = 0; q < b.probs.size() && s == SPG_OK; q++) {
            const int p = b.probs[q];
            if (A_val && A_val[p] && bt->nnzA[p] &&
                cudaMemcpyAsync((char*)b.A.row_val + vs * b.aoff[q], A_val[p], vs * bt->nnzA[p],
                                cudaMemcpyHostToDevice, h->stream) != cudaSuccess)
                s = SPG_ERR_CUDA;
            if (B_val && B_val[p] && bt->nnzB[p] &&
                cudaMemcpyAsync((char*)b.B.row_val + vs * b.boff[q], B_val[p], vs * bt->nnzB[p],
                                cudaMemcpyHostToDevice, h->stream) != cudaSuccess)
                s = SPG_ERR_CUDA;
        }
        if (s == SPG_OK) s = rowwise_numeric_launch(h, &b.A, &b.B, &b.C, ctiles_rowwise_priv(&b.C), prec);
        if (s == SPG_OK && host_vals_out && host_vals_out[bi] && b.C.nnzC > 0 &&
            cudaMemcpyAsync(host_vals_out[bi], b.C.tile_valC, vs * b.C.nnzC, cudaMemcpyDeviceToHost, h->stream) !=
                cudaSuccess)
            s = SPG_ERR_CUDA;
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamEndCapture(h->stream, &g);
        if (s != SPG_OK || e != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            cudaGetLastError();
            return spg_fail(h, SPG_ERR_CUDA, "batch graph: capture failed");
        }
        b.graph = g;
        SPG_CUDA(h, cudaGraphInstantiate(&b.exec, g, 0));
        bi++;
    }
    return SPG_OK;
}

extern "C" spg_status spg_batch_graph_launch(spg_handle_t h, spg_batch_t bt) {
    if (!h || !bt) return SPG_ERR_INVALID;
    for (auto& b : bt->bins) {
        if (b.probs.empty()) continue;
        if (!b.exec) return spg_fail(h, SPG_ERR_INVALID, "batch graph: not captured");
        SPG_CUDA(h, cudaGraphLaunch(b.exec, h->stream));
    }
    return SPG_OK;
}

extern "C" spg_status spg_batch_bin_count(spg_handle_t h, spg_batch_t bt, int* nbins, int64_t* nnz_per_bin) {
    if (!h || !bt || !nbins) return SPG_ERR_INVALID;
    *nbins = (int)bt->bins.size();
    if (nnz_per_bin)
        for (size_t b = 0; b < bt->bins.size(); b++) nnz_per_bin[b] = bt->bins[b].has_c ? bt->bins[b].C.nnzC : 0;
    return SPG_OK;
}

// ---------------------------------------------------------------------------
// autotuner: bin thresholds x per-bin algorithm, timed on the batch itself
// ---------------------------------------------------------------------------
extern "C" spg_status spg_batch_tune(spg_handle_t h, spg_batch_t bt, spg_precision prec, int* n_thresholds,
                                     int* thresholds_out, int* algos_out) {
    if (!h || !bt) return SPG_ERR_INVALID;
    std::vector<int> ns(bt->n.begin(), bt->n.end());
    std::sort(ns.begin(), ns.end());
    auto q = [&](double f) { return ns[std::min<size_t>(ns.size() - 1, (size_t)(f * ns.size()))]; };
    std::vector<std::vector<int>> cands = {{}, {q(0.5)}, {q(0.33), q(0.67)}};
    const spg_algo algos[2] = {SPG_ALGO_PLAIN, SPG_ALGO_ROWWISE};
    double best = 1e30;
    std::vector<int> best_thr;
    std::vector<spg_algo> best_alg;
    for (auto& thr : cands) {
        SPG_TRY(build_bins(h, bt, thr));
        double total = 0;
        std::vector<spg_algo> chosen;
        for (auto& b : bt->bins) {
            if (b.probs.empty()) { chosen.push_back(SPG_ALGO_ROWWISE); continue; }
            double bt_best = 1e30;
            spg_algo ab = SPG_ALGO_ROWWISE;
            for (spg_algo a : algos) {
                SPG_TRY(run_bin(h, b, a, prec));  // warm
                float ms = 0.f;
                SPG_CUDA(h, cudaEventRecord(h->ev[5], h->stream));
                SPG_TRY(run_bin(h, b, a, prec));
                SPG_CUDA(h, cudaEventRecord(h->ev[6], h->stream));
                SPG_CUDA(h, cudaEventSynchronize(h->ev[6]));
                cudaEventElapsedTime(&ms, h->ev[5], h->ev[6]);
                if (ms < bt_best) { bt_best = ms; ab = a; }
            }
            b.algo = ab;
            chosen.push_back(ab);
            total += bt_best;
        }
        if (total < best) { best = total; best_thr = thr; best_alg = chosen; }
    }
    SPG_TRY(build_bins(h, bt, best_thr));
    for (size_t b = 0; b < bt->bins.size(); b++) bt->bins[b].algo = best_alg[b];
    if (n_thresholds) *n_thresholds = (int)best_thr.size();
    for (size_t i = 0; i < best_thr.size() && thresholds_out; i++) thresholds_out[i] = best_thr[i];
    for (size_t b = 0; b < best_alg.size() && algos_out; b++) algos_out[b] = (int)best_alg[b];
    return SPG_OK;
}

extern "C" spg_status spg_batch_set_bins(spg_handle_t h, spg_batch_t bt, int n_thresholds, const int* thresholds,
                                         const int* algos) {
    if (!h || !bt || n_thresholds < 0) return SPG_ERR_INVALID;
    std::vector<int> thr(thresholds, thresholds + n_thresholds);
    SPG_TRY(build_bins(h, bt, thr));
    if (algos)
        for (size_t b = 0; b < bt->bins.size(); b++) bt->bins[b].algo = (spg_algo)algos[b];
    return SPG_OK;
}
