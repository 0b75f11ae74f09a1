/*
 * spgemm_gb300.h -- C ABI of the GB300 tiled SpGEMM library (libspgemm_gb300.so).
 *
 * The library computes C = A * B for sparse matrices stored in the 16x16 tile
 * format of jianjianh1/GPU_SPGEMM (src/tile_format.h:15-42): per tile-row a tile
 * pointer, per tile its column, an nnz prefix, 16 per-row uint8 offsets and 16
 * per-row uint16 occupancy masks (bit 15-c set <=> column c occupied, 256 bits
 * per tile), per nonzero a value and a column byte.  A is tiled row-major
 * (column byte = (row<<4)|col); B is tiled in CSC tile order (column byte = col),
 * exactly as csr2tile / build_csc_tiles lay them out.
 *
 * The reference has no library API: its "interface" is the host functions of
 * tile_format.h, the kernel signatures and the host call sequence of
 * src/spgemm_raw_v2.cu:101-243.  Each entry point below names the reference code
 * it replaces.
 *
 * Conventions
 *   - Every call returns an spg_status; spg_last_error() gives a message.
 *   - Work is ordered on the handle's CUDA stream (given at spg_create).
 *   - Device buffers inside spg_tiles / spg_ctiles are allocated by the
 *     library and released by spg_tiles_free / spg_ctiles_free.
 *   - A handle is not thread safe; use one handle per host thread.
 *   - Offsets that can exceed 2^31 (C's nnz prefix) are int64; everything the
 *     reference stores as int stays int32 and the library rejects inputs whose
 *     counts would overflow it (SPG_ERR_INVALID).
 */
#ifndef SPGEMM_GB300_H
#define SPGEMM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SPG_TILE 16

typedef enum {
    SPG_OK = 0,
    SPG_ERR_INVALID = 1,          /* bad argument or non-canonical CSR           */
    SPG_ERR_OOM = 2,              /* device allocation failed                    */
    SPG_ERR_OVERFLOW_RERUN = 3,   /* a pre-sized buffer overflowed; re-run done  */
    SPG_ERR_TIMEOUT = 4,          /* a bounded device wait gave up               */
    SPG_ERR_CUDA = 5,             /* CUDA runtime error                          */
    SPG_ERR_UNSUPPORTED = 6
} spg_status;

typedef enum { SPG_F32 = 0, SPG_F64 = 1 } spg_dtype;

/* Tiling layouts: ROW = csr2tile (src/tile_format.h:93-222);
   B_CSC = csr2tile + build_csc_tiles (src/tile_format.h:424-585). */
typedef enum { SPG_LAYOUT_ROW = 0, SPG_LAYOUT_B_CSC = 1 } spg_layout;

/* spg_tile_from_csr flags */
#define SPG_TILE_WITH_TILE_CSC 0x1   /* also build tile_csc_Ptr/Row/Val (B only) */

/* Algorithms of steps 2 and 3.  PLAIN: one warp per C tile, matched tile
   pairs by list intersection, register accumulators (the reference's
   structure).  ROWWISE: tile-row work items in shared-memory windows.
   BINNED: each C tile-row to one of the two, by its products per tile pair
   and, with a sizing model attached (spg_set_sizing_model), by the model's
   predicted C nonzeros per C tile (spg_set_bin_params); a product whose
   tile-rows all bin one way runs that algorithm alone.  AUTO is BINNED
   for an A of at least 65,536 tiles; for a smaller A it picks one of the two
   for the whole product by A's nonzeros per tile (ROWWISE below 6); PLAIN
   where B is too wide for the row-wise kernels' shared memory. */
typedef enum { SPG_ALGO_AUTO = 0, SPG_ALGO_PLAIN = 1, SPG_ALGO_ROWWISE = 2, SPG_ALGO_BINNED = 3 } spg_algo;

/* Precision of the numeric phase for FP32 inputs.  F32: FP32 register path.
   MIXED: FP32 bulk, tiles above the fill threshold on BF16/FP16 tensor cores
   with split hi+lo products, FP64 for cancellation-flagged tiles.  FP64
   inputs always compute in FP64. */
typedef enum { SPG_PREC_F32 = 0, SPG_PREC_MIXED = 1, SPG_PREC_F64 = 2 } spg_precision;

typedef struct spg_handle_s* spg_handle_t;

/* Device-resident tile matrix: the reference's TileMatrix (src/tile_format.h:15-42)
   plus the row view used by the row-wise kernels.  All pointers are device
   pointers owned by the library. */
typedef struct {
    int m, n;
    int64_t nnz;
    int tilem, tilen;
    int64_t numtile;
    spg_dtype dtype;
    spg_layout layout;
    /* tile level (row-major tiling, always present) */
    int* tile_ptr;              /* tilem+1                                     */
    int* tile_columnidx;        /* numtile                                     */
    /* per tile, in this layout's tile order (row-major for ROW, CSC for B_CSC) */
    int* tile_nnz;              /* numtile+1, exclusive prefix                 */
    uint8_t* tile_csr_Ptr;      /* numtile*16, per-row offset inside the tile  */
    uint16_t* mask;             /* numtile*16, bit 15-c <=> column c           */
    void* tile_csr_Val;         /* nnz, float or double                        */
    uint8_t* tile_csr_Col;      /* nnz, (r<<4)|c for ROW, c for B_CSC          */
    /* B_CSC only */
    int* csc_tile_ptr;          /* tilen+1                                     */
    int* csc_tile_rowidx;       /* numtile                                     */
    int* csc_to_row;            /* numtile: CSC tile index -> row-major index  */
    uint8_t* tile_csc_Ptr;      /* numtile*16 (optional)                       */
    uint8_t* tile_csc_Row;      /* nnz (optional)                              */
    void* tile_csc_Val;         /* nnz (optional)                              */
    /* scalar row view (CSR) of the same matrix */
    int* row_ptr;               /* m+1                                         */
    int* col_idx;               /* nnz                                         */
    void* row_val;              /* nnz                                         */
    void* priv;                 /* library private                             */
} spg_tiles;

/* Device-resident tile matrix C as steps 1-3 of src/spgemm_raw_v2.cu:111-243
   produce it.  tile_nnzC is an int64 exclusive prefix (the reference's int
   overflows beyond 2^31 nonzeros). */
typedef struct {
    int m, n;
    int tilem, tilen;
    int64_t numtileC;
    int64_t nnzC;
    spg_dtype dtype;
    int* tile_ptrC;             /* tilem+1                                     */
    int* tile_rowidxC;          /* numtileC                                    */
    int* tile_colidxC;          /* numtileC                                    */
    uint16_t* maskC;            /* numtileC*16                                 */
    int64_t* tile_nnzC;         /* numtileC+1                                  */
    uint8_t* ptrRowC;           /* numtileC*16                                 */
    void* tile_valC;            /* nnzC                                        */
    uint8_t* tile_colC;         /* nnzC, (r<<4)|c                              */
    int64_t pairs;              /* matched tile pairs (filled by symbolic)     */
    void* priv;
} spg_ctiles;

/* Per-call statistics of the last spg_symbolic / spg_numeric / spg_spgemm. */
typedef struct {
    float ms_step1;             /* C tile structure (count + scan + fill)      */
    float ms_step2;             /* bitmask symbolic + scan + ptrRowC           */
    float ms_step3;             /* numeric                                     */
    int64_t products;           /* sum over A nonzeros of nnz(B row)           */
    int64_t overflow_reruns;    /* re-runs: pair cache, or tile-rows that outgrew their predicted slot */
    int64_t work_items;         /* row-wise work items: (C tile-row, region) pairs */
    int64_t tensor_pairs;       /* tile pairs computed on tensor cores         */
    int64_t fp64_tiles;         /* C tiles recomputed in FP64                  */
    int32_t algo_used;          /* spg_algo the symbolic phase ran             */
    int32_t sizing_fallbacks;   /* step 1 ran exact because the learned slots did not fit */
    int64_t predicted_tiles;    /* C tile capacity from the sizing model (0: none) */
    int32_t numeric_algo;       /* spg_algo the numeric phase ran (PLAIN for mixed precision) */
    int32_t reserved;
} spg_stats;

/* ---- handle ---------------------------------------------------------------
 * Replaces: the implicit global state of main() (default stream, device
 * selection) in src/spgemm_raw_v2.cu:61-71.  `stream` is a cudaStream_t (NULL =
 * legacy default stream). */
spg_status spg_create(spg_handle_t* h, int device, void* stream);
spg_status spg_destroy(spg_handle_t h);
spg_status spg_set_stream(spg_handle_t h, void* stream);
const char* spg_last_error(spg_handle_t h);
spg_status spg_get_stats(spg_handle_t h, spg_stats* out);
/* Kernels this handle has launched since spg_create (a running count, so the
   difference of two reads counts the launches of the calls between them).
   No reference counterpart. */
spg_status spg_kernel_launches(spg_handle_t h, int64_t* out);

/* ---- tiling ----------------------------------------------------------------
 * Replaces csr2tile (src/tile_format.h:93-222), build_csc_tiles
 * (src/tile_format.h:424-585) and upload_tiles (src/spgemm_raw_v2.cu:25-48).
 * Input is a canonical CSR (columns strictly ascending within each row) in
 * DEVICE memory; values are float (SPG_F32) or double (SPG_F64).  The result
 * keeps a device copy of the CSR as its row view. */
spg_status spg_tile_from_csr(spg_handle_t h, int m, int n, int64_t nnz, const int* d_row_ptr,
                             const int* d_col_idx, const void* d_val, spg_dtype dtype,
                             spg_layout layout, int flags, spg_tiles* out);

/* Same, with the CSR in HOST memory (copied on the handle's stream). */
spg_status spg_tile_from_csr_host(spg_handle_t h, int m, int n, int64_t nnz, const int* row_ptr,
                                  const int* col_idx, const void* val, spg_dtype dtype,
                                  spg_layout layout, int flags, spg_tiles* out);

/* Replaces free_dev / free_tile_matrix (src/spgemm_raw_v2.cu:50-59,
   src/tile_format.h:647-659). */
spg_status spg_tiles_free(spg_handle_t h, spg_tiles* t);

/* ---- SpGEMM steps ----------------------------------------------------------
 * spg_symbolic replaces steps 1 and 2 of src/spgemm_raw_v2.cu:111-221
 * (step1_count_kernel, ExclusiveSum, step1_fill_kernel, step2_symbolic_kernel,
 * ExclusiveSum, step2_build_ptrRowC_kernel; src/spgemm_raw_kernels.cuh:23-215):
 * fills tile_ptrC, tile_rowidxC, tile_colidxC, maskC, tile_nnzC, ptrRowC,
 * numtileC and nnzC of *C and allocates tile_valC / tile_colC.
 * A must be SPG_LAYOUT_ROW, B SPG_LAYOUT_B_CSC, A.n == B.m, same dtype. */
spg_status spg_symbolic(spg_handle_t h, const spg_tiles* A, const spg_tiles* B, spg_algo algo,
                        spg_ctiles* C);

/* SPG_ALGO_BINNED thresholds: a tile-row runs the plain kernels when its
 * products per matched tile pair reach pp_thr (default 12) and, with a sizing
 * model attached, its predicted C nonzeros per predicted C tile reach
 * fill_thr (default 16).  No reference counterpart (the reference runs one
 * kernel configuration for every tile-row, src/spgemm_raw_kernels.cuh:9-14). */
spg_status spg_set_bin_params(spg_handle_t h, float pp_thr, float fill_thr);

/* SPG_PREC_MIXED parameters: tile pairs whose A and B tiles both hold >=
 * dense_thr nonzeros run on the tensor cores (default 32); C tiles with an
 * entry below cancel_eps times its magnitude sum are recomputed in FP64
 * (default 2^-20).  No reference counterpart (the reference is FP64 only). */
spg_status spg_set_mixed_params(spg_handle_t h, int dense_thr, float cancel_eps);

/* spg_symbolic in its two steps.  spg_symbolic_tiles is step 1: C's tile
 * structure (tile_ptrC, tile_rowidxC, tile_colidxC, numtileC;
 * src/spgemm_raw_v2.cu:111-158).  spg_symbolic_masks on that C is step 2:
 * maskC, ptrRowC, tile_nnzC, nnzC and the value arrays (:160-221).  Called
 * separately, a caller can start copying C's tile indices while step 2 runs,
 * e.g. with spg_ctiles_to_host_range on another handle. */
spg_status spg_symbolic_tiles(spg_handle_t h, const spg_tiles* A, const spg_tiles* B, spg_algo algo,
                              spg_ctiles* C);
spg_status spg_symbolic_masks(spg_handle_t h, const spg_tiles* A, const spg_tiles* B, spg_ctiles* C);

/* Replaces step 3 (step3_numeric_kernel_v2, src/spgemm_raw_kernels_v2.cuh:10-139,
 * launched at src/spgemm_raw_v2.cu:228-238): fills tile_valC and tile_colC.
 * algo AUTO follows C's symbolic phase; SPG_ALGO_ROWWISE runs the row-wise
 * kernels on any C (their plan is built here when the symbolic phase did not
 * build it), as does SPG_PREC_F64 on FP32 data.  stats.numeric_algo reports
 * the choice. */
spg_status spg_numeric(spg_handle_t h, const spg_tiles* A, const spg_tiles* B, spg_algo algo,
                       spg_precision prec, spg_ctiles* C);

/* spg_numeric on the C tile-rows [row_begin, row_end) only (0 <= row_begin <=
 * row_end <= C->tilem): the values and column bytes of tiles tile_ptrC[row_begin]
 * .. tile_ptrC[row_end] - 1.  Calls over bands that cover every tile-row once
 * give what one spg_numeric gives, so a caller can copy a finished band to the
 * host while the next band computes.  Same step of the reference as
 * spg_numeric. */
spg_status spg_numeric_rows(spg_handle_t h, const spg_tiles* A, const spg_tiles* B, spg_algo algo,
                            spg_precision prec, spg_ctiles* C, int row_begin, int row_end);

/* spg_numeric that reports its progress in bands of C tile-rows: band k is
 * tile-rows [band_rows[k], band_rows[k+1]) (band_rows: nbands + 1 ascending
 * bounds from 0 to C->tilem, 1 <= nbands <= 65536).  order says which bands
 * are worked on first: SPG_BANDS_FIRST_TO_LAST, or SPG_BANDS_LAST_TO_FIRST
 * (when the first tile-rows hold most of the work, as the hub rows of a
 * power-law matrix do, the other bands' results are then ready early and can
 * be copied while the heavy band computes).  fn(user, k, row_begin,
 * row_end) is called on the calling thread once per band, as soon as the
 * values and column bytes of that band's tiles are final in device memory
 * (bands may complete out of order; a band without work is reported at
 * once).  The call returns when the whole phase has finished.  fn may
 * enqueue copies of the finished band on other streams or handles; it must
 * not call into this handle.  The row-wise path runs one launch whose work
 * items count down per band; the plain and mixed paths run one launch per
 * band.  Same step of the reference as spg_numeric. */
typedef void (*spg_band_fn)(void* user, int band, int row_begin, int row_end);
enum { SPG_BANDS_FIRST_TO_LAST = 0, SPG_BANDS_LAST_TO_FIRST = 1 };
spg_status spg_numeric_bands(spg_handle_t h, const spg_tiles* A, const spg_tiles* B, spg_algo algo,
                             spg_precision prec, spg_ctiles* C, int nbands, const int* band_rows, int order,
                             spg_band_fn fn, void* user);

/* Steps 1-3 in one call (the timed region of src/spgemm_raw_v2.cu:115-240). */
spg_status spg_spgemm(spg_handle_t h, const spg_tiles* A, const spg_tiles* B, spg_algo algo,
                      spg_precision prec, spg_ctiles* C);

/* Copy C's arrays to host buffers sized from C->numtileC / C->nnzC (any
   pointer may be NULL to skip that array).  tile_ptrC needs tilem+1 ints. */
spg_status spg_ctiles_to_host(spg_handle_t h, const spg_ctiles* C, int* tile_ptrC, int* tile_rowidxC,
                              int* tile_colidxC, uint16_t* maskC, int64_t* tile_nnzC,
                              uint8_t* ptrRowC, void* tile_valC, uint8_t* tile_colC);

/* Copy C tiles [tile_begin, tile_end) to host buffers indexed from 0: their
   tile_rowidxC, tile_colidxC, maskC (16 per tile), ptrRowC (16 per tile), the
   tile_end-tile_begin+1 entries of tile_nnzC starting at tile_begin (absolute
   offsets), and the values / column bytes tile_nnzC[tile_begin] ..
   tile_nnzC[tile_end]-1.  `val_capacity` is the number of values the value
   and column buffers hold; SPG_ERR_INVALID (nothing copied) if the range holds
   more.  *n_values receives the range's value count.  Lets a caller stream a C
   larger than host memory (the reference reads C back whole,
   src/spgemm_raw_v2.cu:257-266). */
spg_status spg_ctiles_to_host_range(spg_handle_t h, const spg_ctiles* C, int64_t tile_begin, int64_t tile_end,
                                    int* tile_rowidxC, int* tile_colidxC, uint16_t* maskC, int64_t* tile_nnzC,
                                    uint8_t* ptrRowC, void* tile_valC, uint8_t* tile_colC, int64_t val_capacity,
                                    int64_t* n_values);

/* Copy a tile matrix's arrays to host buffers (NULL skips an array). */
spg_status spg_tiles_to_host(spg_handle_t h, const spg_tiles* T, int* tile_ptr, int* tile_columnidx,
                             int* tile_nnz, uint8_t* tile_csr_Ptr, uint16_t* mask, void* tile_csr_Val,
                             uint8_t* tile_csr_Col, int* csc_tile_ptr, int* csc_tile_rowidx,
                             uint8_t* tile_csc_Ptr, uint8_t* tile_csc_Row, void* tile_csc_Val);

/* Replaces the free calls at src/spgemm_raw_v2.cu:361-367. */
spg_status spg_ctiles_free(spg_handle_t h, spg_ctiles* C);

/* ---- format conversions and chained products ------------------------------
 * Device CSR transpose (m x n -> n x m), stable: rows stay ascending inside
 * each column.  Replaces the host transpose of the --aat path
 * (src/spgemm_raw_v2.cu:79-90).  Output arrays are caller-allocated device
 * memory: out_rp n+1, out_ci / out_val nnz. */
spg_status spg_csr_transpose(spg_handle_t h, int m, int n, int64_t nnz, const int* d_rp, const int* d_ci,
                             const void* d_val, spg_dtype dtype, int* out_rp, int* out_ci, void* out_val);

/* C's tiles -> device CSR (rows ascending, columns ascending), the device form
   of the expansion at src/spgemm_raw_v2.cu:268-284.  Call with out_rp == NULL
   to get *nnz only; then with caller-allocated device arrays (m+1, nnz, nnz). */
spg_status spg_ctiles_to_csr(spg_handle_t h, const spg_ctiles* C, int* out_rp, int* out_ci, void* out_val,
                             int64_t* nnz);

/* C's tiles -> device CSR like spg_ctiles_to_csr, but the library allocates
   no device memory at all.  No counterpart in the reference (which owns all
   its buffers).  For callers that cannot let a library allocate: a serving
   process or host framework that owns every byte of HBM through its own pool,
   code where an allocation could block or fail at an unpredictable time, a
   plugin handed only a stream and buffers.  The caller passes the outputs
   (out_rp: m+1 ints, out_ci / out_val: C->nnzC entries); the working memory
   is a fixed area inside the library (a static device array of about 4 MiB,
   held on every GPU that loads the library until the process exits), so C may
   have at most 1,048,576 rows; more returns SPG_ERR_INVALID.  The first call
   on a device looks up that area's address, so make it before any stream
   capture.  All calls share the area: calls whose work overlaps on the GPU
   race on it, so order them on one stream. *nnz receives C->nnzC. */
spg_status spg_ctiles_to_csr_noalloc(spg_handle_t h, const spg_ctiles* C, int* out_rp, int* out_ci,
                                     void* out_val, int64_t* nnz);

/* Galerkin triple product RAP = P^T (A P) on the device (no reference
   counterpart; it chains two of the reference's SpGEMMs): A (m x m) and P
   (m x nc) are device CSR; A*P is formed, converted to CSR and re-tiled as the
   B operand, P^T comes from spg_csr_transpose.  *products_out receives the
   intermediate products of both SpGEMMs; spg_get_stats afterwards sums the
   two products' statistics (step times, counts). */
spg_status spg_galerkin(spg_handle_t h, int m, int nc, int64_t nnzA, const int* A_rp, const int* A_ci,
                        const void* A_val, int64_t nnzP, const int* P_rp, const int* P_ci, const void* P_val,
                        spg_dtype dtype, spg_algo algo, spg_precision prec, spg_ctiles* RAP,
                        int64_t* products_out);

/* ---- batches of independent products -----------------------------------
 * No reference counterpart: the reference multiplies one matrix per run
 * (src/spgemm_raw_v2.cu:61).  A batch C_p = A_p * B_p (p < nprob, A_p m_p x
 * k_p, B_p k_p x n_p, host CSR) is assembled on the device as block-diagonal
 * products (one per bin of problems, blocks at 16-aligned offsets) and each
 * phase runs as one launch for the whole bin. */
typedef struct spg_batch_s* spg_batch_t;

spg_status spg_batch_create_host(spg_handle_t h, int nprob, const int* m, const int* k, const int* n,
                                 const int64_t* nnzA, const int* const* A_rp, const int* const* A_ci,
                                 const void* const* A_val, const int64_t* nnzB, const int* const* B_rp,
                                 const int* const* B_ci, const void* const* B_val, spg_dtype dtype,
                                 spg_batch_t* out);
spg_status spg_batch_free(spg_handle_t h, spg_batch_t b);
/* Steps 1-3 for every problem (AUTO: each bin's tuned algorithm). */
spg_status spg_batch_spgemm(spg_handle_t h, spg_batch_t b, spg_algo algo, spg_precision prec);
/* Problem p's C sizes (p < 0: only *products, the batch's total). */
spg_status spg_batch_info(spg_handle_t h, spg_batch_t b, int p, int64_t* numtileC, int64_t* nnzC,
                          int64_t* products);
/* Problem p's C arrays with problem-local indices (layout of spg_ctiles). */
spg_status spg_batch_to_host(spg_handle_t h, spg_batch_t b, int p, int* tile_ptrC, int* tile_rowidxC,
                             int* tile_colidxC, uint16_t* maskC, int64_t* tile_nnzC, uint8_t* ptrRowC,
                             void* tile_valC, uint8_t* tile_colC);
/* New values (same structure) from host arrays; NULL entries are kept. */
spg_status spg_batch_set_values_host(spg_handle_t h, spg_batch_t b, const void* const* A_val,
                                     const void* const* B_val);
/* Numeric phase only, one launch per bin, no host synchronisation. */
spg_status spg_batch_numeric(spg_handle_t h, spg_batch_t b, spg_precision prec);
/* Capture, per bin, [values host->device, numeric, C values -> host_vals_out[bin]]
   into a CUDA graph (the handle must use a non-default stream); replay with
   spg_batch_graph_launch.  Host buffers should be pinned. */
spg_status spg_batch_graph_capture(spg_handle_t h, spg_batch_t b, const void* const* A_val,
                                   const void* const* B_val, void* const* host_vals_out, spg_precision prec);
spg_status spg_batch_graph_launch(spg_handle_t h, spg_batch_t b);
/* Number of bins and each bin's C nonzeros (for sizing host_vals_out). */
spg_status spg_batch_bin_count(spg_handle_t h, spg_batch_t b, int* nbins, int64_t* nnz_per_bin);
/* Autotuner: tries bin thresholds on n (none, median, terciles) and, per bin,
   the plain and row-wise algorithms, timing each on the batch; keeps the
   fastest.  thresholds_out gets <= 2 values, algos_out <= 3. */
spg_status spg_batch_tune(spg_handle_t h, spg_batch_t b, spg_precision prec, int* n_thresholds,
                          int* thresholds_out, int* algos_out);
/* Set bins explicitly: n_thresholds ascending upper bounds on n, algos per bin. */
spg_status spg_batch_set_bins(spg_handle_t h, spg_batch_t b, int n_thresholds, const int* thresholds,
                              const int* algos);

/* ---- learned sizing --------------------------------------------------------
 * No reference counterpart: the reference sizes C by a full counting pass and
 * a host read-back before filling (src/spgemm_raw_v2.cu:119-156).  An MLP
 * (8 per-tile-row features -> 32 -> 32 -> 2) predicts each C tile-row's tile
 * count and nonzeros; with a model attached (spg_set_sizing_model) step 1
 * gives every C tile-row a slot of its predicted size, builds each row's
 * bitmap once (exact count, tiles written into the slot) and compacts the
 * slots into C's exact arrays; a row whose slot was too small re-runs the
 * exact fill (stats.overflow_reruns counts those rows).  The structure is
 * exact whatever the prediction.  The model is trained on the GPU by
 * spg_mlp_train (forward, backward and Adam kernels of this library). */
typedef struct spg_mlp_s* spg_mlp_t;
int spg_mlp_num_params(void);
int spg_mlp_num_features(void);
/* host_params (spg_mlp_num_params floats) / host_norm (20 floats: feature
   mean[8], feature inv-std[8], target mean[2], target std[2]) may be NULL. */
spg_status spg_mlp_create(spg_handle_t h, const float* host_params, const float* host_norm, spg_mlp_t* out);
spg_status spg_mlp_free(spg_handle_t h, spg_mlp_t m);
spg_status spg_mlp_get_params(spg_handle_t h, spg_mlp_t m, float* host_params, float* host_norm);
spg_status spg_mlp_set_norm(spg_handle_t h, spg_mlp_t m, const float* host_norm);
/* Features of C = A*B per tile-row of A into d_feat (A->tilem x 8 floats). */
spg_status spg_mlp_features(spg_handle_t h, const spg_tiles* A, const spg_tiles* B, float* d_feat);
/* Predictions (log1p of C tiles and C nonzeros per tile-row), n x 2 floats. */
spg_status spg_mlp_forward(spg_handle_t h, spg_mlp_t m, const float* d_feat, int64_t n, float* d_out);
/* Gradient of the mean squared error (standardised targets) without update. */
spg_status spg_mlp_gradient(spg_handle_t h, spg_mlp_t m, const float* d_feat, const float* d_target, int64_t n,
                            float* d_grad_out, float* loss_out);
/* Adam, `epochs` passes, mini-batches of `batch`; d_perm: epochs*n sample
   indices (NULL = in order). */
spg_status spg_mlp_train(spg_handle_t h, spg_mlp_t m, const float* d_feat, const float* d_target, int64_t n,
                         const int* d_perm, int epochs, int batch, float lr, float* last_epoch_loss);
/* Attach (m) or detach (NULL) the sizing model; slot of a tile-row = prediction * (1+margin) + 2
   tiles (1.0 is a good margin: slots cost 4 bytes a tile, re-filled rows a bitmap pass). */
spg_status spg_set_sizing_model(spg_handle_t h, spg_mlp_t m, float margin);

/* Intermediate products sum_{(i,k) in A} nnz(B(k,:)) (src/spgemm_raw_v2.cu:95-99),
   computed on the device from the row views. */
spg_status spg_products(spg_handle_t h, const spg_tiles* A, const spg_tiles* B, int64_t* out);

#ifdef __cplusplus
}
#endif

#endif /* SPGEMM_GB300_H */
