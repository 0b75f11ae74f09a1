// A C++ caller of libspgemm_gb300 written the way the reference's main()
// (src/spgemm_raw_v2.cu:61-243) would call it after switching to the library:
// read a CSR, tile A row-major and B in CSC tile order on the device
// (csr2tile / build_csc_tiles / upload_tiles), run steps 1-3 in one call,
// print the per-step times and GFLOP/s the reference prints (:245-250), read C
// back (:257-266) and release everything (:361-368).
//
// It includes only the library's C header.  The reference's HostCSR /
// load_mtx (src/tile_format.h:44-90) are replaced by a small binary reader so
// the program builds where the reference's sources are absent.
//
// Usage: dropin_main IN.bin OUT.bin [algo]
//   IN.bin : int32 m, n; int64 nnz; int32 dtype (0 float, 1 double);
//            int32 row_ptr[m+1]; int32 col_idx[nnz]; values[nnz]
//   OUT.bin: int64 numtileC, nnzC, tilem; then tile_ptrC, tile_rowidxC,
//            tile_colidxC, maskC, tile_nnzC, ptrRowC, tile_colC, tile_valC
// Exit status 0 on success; the library's message on stderr otherwise.
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "spgemm_gb300.h"

namespace {

struct HostCSR {
    int m = 0, n = 0;
    int64_t nnz = 0;
    int dtype = SPG_F64;
    std::vector<int> row_ptr, col_idx;
    std::vector<unsigned char> val;  // nnz values of the dtype
};

bool read_csr(const char* path, HostCSR* a) {
    FILE* f = std::fopen(path, "rb");
    if (!f) return false;
    bool ok = std::fread(&a->m, 4, 1, f) == 1 && std::fread(&a->n, 4, 1, f) == 1 &&
              std::fread(&a->nnz, 8, 1, f) == 1 && std::fread(&a->dtype, 4, 1, f) == 1;
    if (ok) {
        const size_t vs = a->dtype == SPG_F64 ? 8 : 4;
        a->row_ptr.resize((size_t)a->m + 1);
        a->col_idx.resize((size_t)a->nnz + 1);
        a->val.resize(vs * ((size_t)a->nnz + 1));
        ok = std::fread(a->row_ptr.data(), 4, a->row_ptr.size(), f) == a->row_ptr.size() &&
             std::fread(a->col_idx.data(), 4, (size_t)a->nnz, f) == (size_t)a->nnz &&
             std::fread(a->val.data(), vs, (size_t)a->nnz, f) == (size_t)a->nnz;
    }
    std::fclose(f);
    return ok;
}

template <typename T>
void put(FILE* f, const std::vector<T>& v) {
    if (!v.empty()) std::fwrite(v.data(), sizeof(T), v.size(), f);
}

int fail(spg_handle_t h, const char* what) {
    std::fprintf(stderr, "%s: %s\n", what, h ? spg_last_error(h) : "no handle");
    return 1;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 3) {
        std::fprintf(stderr, "usage: %s IN.bin OUT.bin [auto|plain|rowwise]\n", argv[0]);
        return 2;
    }
    HostCSR hA;
    if (!read_csr(argv[1], &hA)) {
        std::fprintf(stderr, "cannot read %s\n", argv[1]);
        return 2;
    }
    spg_algo algo = SPG_ALGO_AUTO;
    if (argc > 3 && argv[3][0] == 'p') algo = SPG_ALGO_PLAIN;
    if (argc > 3 && argv[3][0] == 'r') algo = SPG_ALGO_ROWWISE;
    const HostCSR& hB = hA;  // C = A * A, as the reference runs without --aat
    const spg_dtype dt = hA.dtype == SPG_F64 ? SPG_F64 : SPG_F32;

    spg_handle_t h = nullptr;
    if (spg_create(&h, 0, nullptr) != SPG_OK) return fail(h, "spg_create");
    spg_tiles A{}, B{};
    if (spg_tile_from_csr_host(h, hA.m, hA.n, hA.nnz, hA.row_ptr.data(), hA.col_idx.data(), hA.val.data(), dt,
                               SPG_LAYOUT_ROW, 0, &A) != SPG_OK)
        return fail(h, "tiling A");
    if (spg_tile_from_csr_host(h, hB.m, hB.n, hB.nnz, hB.row_ptr.data(), hB.col_idx.data(), hB.val.data(), dt,
                               SPG_LAYOUT_B_CSC, SPG_TILE_WITH_TILE_CSC, &B) != SPG_OK)
        return fail(h, "tiling B");
    int64_t products = 0;
    if (spg_products(h, &A, &B, &products) != SPG_OK) return fail(h, "products");
    spg_ctiles C{};
    if (spg_spgemm(h, &A, &B, algo, dt == SPG_F64 ? SPG_PREC_F64 : SPG_PREC_F32, &C) != SPG_OK)
        return fail(h, "spgemm");
    spg_stats st{};
    spg_get_stats(h, &st);
    const double ms = st.ms_step1 + st.ms_step2 + st.ms_step3;
    std::printf("step1 %.3f ms, step2 %.3f ms, step3 %.3f ms\n", st.ms_step1, st.ms_step2, st.ms_step3);
    std::printf("GPU time = %.3f ms, GFlops = %.3f, numtileC = %lld, nnzC = %lld\n", ms,
                ms > 0 ? 2.0 * (double)products / (ms * 1e6) : 0.0, (long long)C.numtileC, (long long)C.nnzC);

    const size_t nt = (size_t)C.numtileC, nz = (size_t)C.nnzC, vs = dt == SPG_F64 ? 8 : 4;
    std::vector<int> tile_ptrC((size_t)C.tilem + 1), rowidx(nt), colidx(nt);
    std::vector<uint16_t> maskC(nt * SPG_TILE);
    std::vector<int64_t> tile_nnzC(nt + 1);
    std::vector<uint8_t> ptrRowC(nt * SPG_TILE), colC(nz);
    std::vector<unsigned char> valC(nz * vs);
    if (spg_ctiles_to_host(h, &C, tile_ptrC.data(), rowidx.data(), colidx.data(), maskC.data(), tile_nnzC.data(),
                           ptrRowC.data(), valC.data(), colC.data()) != SPG_OK)
        return fail(h, "read-back");
    FILE* f = std::fopen(argv[2], "wb");
    if (!f) return 2;
    const int64_t head[3] = {C.numtileC, C.nnzC, (int64_t)C.tilem};
    std::fwrite(head, 8, 3, f);
    put(f, tile_ptrC); put(f, rowidx); put(f, colidx); put(f, maskC); put(f, tile_nnzC); put(f, ptrRowC);
    put(f, colC); put(f, valC);
    std::fclose(f);

    spg_ctiles_free(h, &C);
    spg_tiles_free(h, &A);
    spg_tiles_free(h, &B);
    spg_destroy(h);
    return 0;
}
