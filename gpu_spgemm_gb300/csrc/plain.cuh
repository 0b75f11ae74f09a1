// plain.cuh -- interface of the plain per-C-tile kernels (plain.cu).
#pragma once
#include "spg_common.cuh"

// Per-C private state of the plain path: the matched-pair cache of step 2
// (spec_* in src/spgemm_raw_v2.cu:161-172) and two device counters.
// Pairs the step-2 cache holds per C tile (the reference's MAX_MATCHED);
// a tile with more intersects its lists again in step 3.
constexpr int SPEC_PAIRS_MAX = 32;

struct PlainPriv {
    int* spec_cnt = nullptr;   // numtileC: cached pair count, -1 = not cached
    int* spec_off = nullptr;   // numtileC
    int* spec_pa = nullptr;    // spec_cap
    int* spec_pb = nullptr;    // spec_cap
    int64_t spec_cap = 0;
    unsigned long long* counters = nullptr;  // [0] cache allocation, [1] matched pairs (step 2), [2] tile pairs (step 1),
                                             // [3] tile pairs of the plain tile-rows of a binned product
};

spg_status plain_step1(spg_handle_t h, const spg_tiles* A, const spg_tiles* B, spg_ctiles* C,
                       int64_t* row_pairs, unsigned long long* pairs_total);
spg_status plain_step1_sized(spg_handle_t h, const spg_tiles* A, const spg_tiles* B, spg_ctiles* C,
                             int64_t* row_pairs, unsigned long long* pairs_total, const int* slot_sz);
// Per tile-row slot sizes (predicted C tiles with margin) from the sizing MLP
// (slot_sz, when a model is attached) and kernel variants (rowbin: 1 plain,
// 0 row-wise; from the exact features, refined by the model's predictions
// when one is attached).  Either output may be null.
spg_status mlp_predict_rows(spg_handle_t h, const spg_tiles* A, const spg_tiles* B, int* slot_sz,
                            uint8_t* rowbin = nullptr);
// Step 2 over every C tile, or over the nlist tiles of tlist (ascending C
// tile indices); tile nonzero counts into cnt32[t] (int) or, with cnt32
// null, into cnt64[t].
spg_status plain_step2(spg_handle_t h, const spg_tiles* A, const spg_tiles* B, spg_ctiles* C,
                       PlainPriv* pp, int* cnt32, int64_t* cnt64 = nullptr, const int* tlist = nullptr,
                       int64_t nlist = 0);
// Step 3 on C tiles [t0, t1) (t1 < 0: every tile), or with tlist on the
// listed tiles tlist[t0] .. tlist[t1 - 1].
spg_status plain_step3(spg_handle_t h, const spg_tiles* A, const spg_tiles* B, spg_ctiles* C,
                       PlainPriv* pp, int64_t t0 = 0, int64_t t1 = -1, const int* tlist = nullptr);
spg_status plain_step3_mixed(spg_handle_t h, const spg_tiles* A, const spg_tiles* B, spg_ctiles* C, PlainPriv* pp,
                             int dense_thr, float cancel_eps, int64_t t0 = 0, int64_t t1 = -1);

spg_status spg_build_tiles(spg_handle_t h, int m, int n, int64_t nnz, const int* d_rp, const int* d_ci,
                           const void* d_val, spg_dtype dtype, spg_layout layout, int flags, spg_tiles* out);

spg_status ctiles_to_csr_impl(spg_handle_t h, const spg_ctiles* C, int* out_rp, int* out_ci, void* out_val,
                              int64_t* nnz_out);
