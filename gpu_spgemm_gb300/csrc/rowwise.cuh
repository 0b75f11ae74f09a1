// rowwise.cuh -- interface of the row-wise binned kernels (rowwise.cu).
#pragma once
#include "spg_common.cuh"

// Per-C private state of the row-wise path.
struct RowwisePriv {
    int64_t* item_prefix = nullptr;  // tilem+1: prefix of work items (regions) per C tile-row
    int64_t nitems = 0;
    int max_na = 0;                  // largest number of A nonzeros in one tile-row
    unsigned long long* counters = nullptr;  // [0] symbolic ticket, [1] numeric ticket, [2] max nA
    int* cursor_g = nullptr;         // per-CTA cursor scratch (4 ints per A nonzero) for tile-rows with many A nonzeros
    int grid = 0;
};

spg_algo rowwise_choose(spg_handle_t h, const spg_tiles* A, const spg_tiles* B);
spg_status rowwise_symbolic(spg_handle_t h, const spg_tiles* A, const spg_tiles* B, spg_ctiles* C,
                            RowwisePriv* rp, int64_t* tile_cnt);
spg_status rowwise_numeric(spg_handle_t h, const spg_tiles* A, const spg_tiles* B, spg_ctiles* C,
                           RowwisePriv* rp, spg_precision prec);
void rowwise_free_priv(spg_handle_t h, RowwisePriv* rp);
void rowwise_free_bview(spg_handle_t h, spg_tiles* t);
