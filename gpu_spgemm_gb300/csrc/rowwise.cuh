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

// Whether the row-wise kernels can run this product (shared memory for the
// symbolic windows over B's tile columns, and for the numeric arena).
bool rowwise_fits(spg_handle_t h, const spg_tiles* B);
// Whether the row-wise numeric kernel can run (any B: its windows carry
// their own rank bitmaps).
bool rowwise_numeric_fits(spg_handle_t h);
// skip_rows (optional, tilem flags): tile-rows whose work items are skipped
// (the binned algorithm leaves them to the plain kernels).
spg_status rowwise_symbolic(spg_handle_t h, const spg_tiles* A, const spg_tiles* B, spg_ctiles* C,
                            RowwisePriv* rp, int64_t* tile_cnt, const uint8_t* skip_rows = nullptr);
// Numeric phase on C tile-rows [r0, r1) (r1 < 0: every tile-row).
spg_status rowwise_numeric(spg_handle_t h, const spg_tiles* A, const spg_tiles* B, spg_ctiles* C,
                           RowwisePriv* rp, spg_precision prec, int r0 = 0, int r1 = -1,
                           const uint8_t* skip_rows = nullptr);
// One numeric launch over every tile-row that reports bands of tile-rows as
// they complete: band k = tile-rows [rows[k], rows[k+1]) (d_rows on the
// device, nbands + 1 entries).  Fills h_band_end[k] (first work item after
// band k; host memory) before the launch; the kernel sets band_flag[k] (a
// device pointer to mapped host memory, cleared by the caller) when every
// item of band k is written.  last_first: work items are taken from the
// last band to the first.  Returns after the launch without waiting.
spg_status rowwise_numeric_bands_launch(spg_handle_t h, const spg_tiles* A, const spg_tiles* B, spg_ctiles* C,
                                        RowwisePriv* rp, spg_precision prec, int nbands, const int* d_rows,
                                        int64_t* d_band_end, unsigned* d_band_cnt, volatile int* band_flag_dev,
                                        int64_t* h_band_end, bool last_first, const uint8_t* skip_rows = nullptr);
void rowwise_free_priv(spg_handle_t h, RowwisePriv* rp);
void rowwise_free_bview(spg_handle_t h, spg_tiles* t);
