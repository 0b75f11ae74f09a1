// ref_shim.cpp -- TEST INFRASTRUCTURE.  Exposes the reference project's own
// host tiler (src/tile_format.h: csr2tile at :93, build_csc_tiles at :424) to
// Python through a C ABI so its outputs can pin the oracle and the CUDA tiler.
// The header is compiled from the reference checkout where it lies (see
// oracle/build_ref.sh); nothing of it is copied here.
#include <cstring>
#include "tile_format.h"

static TileMatrix g_T;
static bool g_has = false;
static bool g_csc = false;

extern "C" int ref_build(int m, int n, int nnz, const int* rp, const int* ci, const double* val, int csc) {
    if (g_has) free_tile_matrix(g_T);
    HostCSR h;
    h.m = m; h.n = n; h.nnz = nnz;
    h.row_ptr.assign(rp, rp + m + 1);
    h.col_idx.assign(ci, ci + nnz);
    h.val.assign(val, val + nnz);
    g_T = csr2tile(h);
    if (csc) build_csc_tiles(g_T, h);
    g_has = true;
    g_csc = csc != 0;
    return g_T.numtile;
}

extern "C" void ref_get(int* tile_ptr, int* tile_columnidx, int* tile_nnz, unsigned char* ptr16,
                        unsigned short* mask, double* val, unsigned char* col, int* csc_ptr, int* csc_row,
                        unsigned char* tcsc_ptr, unsigned char* tcsc_row, double* tcsc_val) {
    const TileMatrix& T = g_T;
    const int nt = g_csc ? T.numtileB_csc : T.numtile;
    const int nz = T.tile_nnz[nt];
    memcpy(tile_ptr, T.tile_ptr, sizeof(int) * (T.tilem + 1));
    memcpy(tile_columnidx, T.tile_columnidx, sizeof(int) * T.numtile);
    memcpy(tile_nnz, T.tile_nnz, sizeof(int) * (nt + 1));
    memcpy(ptr16, T.tile_csr_Ptr, (size_t)nt * TILE_SIZE);
    memcpy(mask, T.mask, sizeof(unsigned short) * (size_t)nt * TILE_SIZE);
    memcpy(val, T.tile_csr_Val, sizeof(double) * nz);
    memcpy(col, T.tile_csr_Col, nz);
    if (g_csc) {
        memcpy(csc_ptr, T.csc_tile_ptr, sizeof(int) * (T.tilen + 1));
        memcpy(csc_row, T.csc_tile_rowidx, sizeof(int) * nt);
        memcpy(tcsc_ptr, T.tile_csc_Ptr, (size_t)nt * TILE_SIZE);
        memcpy(tcsc_row, T.tile_csc_Row, nz);
        memcpy(tcsc_val, T.tile_csc_Val, sizeof(double) * nz);
    }
}

// The reference's own Matrix Market reader (src/tile_format.h:51-90): loads
// `path` and gives m, n and the entry count; ref_mtx_get copies the
// CSR it built (duplicates kept, as the reference keeps them).
static HostCSR g_mtx;

extern "C" int ref_mtx_load(const char* path, int* m, int* n, int* nnz) {
    g_mtx = load_mtx(path);
    *m = g_mtx.m;
    *n = g_mtx.n;
    *nnz = g_mtx.nnz;
    return 0;
}

extern "C" void ref_mtx_get(int* rp, int* ci, double* val) {
    memcpy(rp, g_mtx.row_ptr.data(), sizeof(int) * (g_mtx.m + 1));
    memcpy(ci, g_mtx.col_idx.data(), sizeof(int) * g_mtx.nnz);
    for (int i = 0; i < g_mtx.nnz; i++) val[i] = (double)g_mtx.val[i];
}
