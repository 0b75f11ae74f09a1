// noalloc.cu -- C's tiles -> CSR without any device allocation.
//
// Some callers cannot let a library allocate device memory: code that owns
// every byte of the GPU through its own fixed pool (a serving process that
// reserved HBM at start-up, a host framework whose allocator must see every
// allocation), code running where an allocation could block or fail at an
// unpredictable moment (a real-time loop, a stream that another thread is
// capturing), or a plugin that is handed a stream and buffers and nothing
// else.  spg_ctiles_to_csr_noalloc gives them the tile -> CSR export with the
// caller's output buffers and a fixed working area that lives inside this
// library: the file-scope array below.  It makes no cudaMalloc / cudaFree /
// cudaMallocAsync call and calls no allocating library routine.
//
// The working area (g_noalloc_scratch) holds the per-row counts of C
// (SPG_NOALLOC_MAX_ROWS ints) and the per-block sums of their scan.  Every
// GPU that loads the library keeps it until the process exits.  Every call
// shares it and it keeps the previous call's contents, so each call clears the
// counts before using them, and two calls whose work overlaps on the GPU (on
// different streams, or different handles on one device) race on it: order
// such calls on one stream.
#include <mutex>

#include "plain.cuh"
#include "spg_common.cuh"

#define SPG_NOALLOC_MAX_ROWS (1 << 20)
#define NA_SCAN_ITEMS 1024  // rows per scan block
#define NA_MAX_BLOCKS (SPG_NOALLOC_MAX_ROWS / NA_SCAN_ITEMS + 1)

namespace {

struct NoallocScratch {
    int counts[SPG_NOALLOC_MAX_ROWS + 1];
    long long block_sums[NA_MAX_BLOCKS + 1];
};

static __device__ __align__(256) NoallocScratch g_noalloc_scratch;

// device address of g_noalloc_scratch, looked up once per device
constexpr int NA_MAX_DEVICES = 64;
NoallocScratch* g_scratch_ptr[NA_MAX_DEVICES] = {};
std::mutex g_scratch_mu;

__global__ void na_rowcount_kernel(int64_t numtileC, int m, const int* __restrict__ rowidxC,
                                   const uint16_t* __restrict__ maskC, int* __restrict__ counts) {
    for (int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; x < numtileC * TS;
         x += (int64_t)gridDim.x * blockDim.x) {
        const int R = rowidxC[x >> 4] * TS + (int)(x & 15);
        const int c = __popc((uint32_t)maskC[x]);
        if (c && R < m) atomicAdd(&counts[R], c);
    }
}

// per-block sums of NA_SCAN_ITEMS counts
__global__ void na_block_sum_kernel(int m, const int* __restrict__ counts, long long* __restrict__ bsum) {
    __shared__ long long s[256];
    long long v = 0;
    const int base = blockIdx.x * NA_SCAN_ITEMS;
    for (int i = threadIdx.x; i < NA_SCAN_ITEMS; i += blockDim.x)
        if (base + i < m) v += counts[base + i];
    s[threadIdx.x] = v;
    __syncthreads();
    for (int d = blockDim.x / 2; d > 0; d >>= 1) {
        if ((int)threadIdx.x < d) s[threadIdx.x] += s[threadIdx.x + d];
        __syncthreads();
    }
    if (threadIdx.x == 0) bsum[blockIdx.x] = s[0];
}

// exclusive scan of the block sums in one block (<= NA_MAX_BLOCKS entries);
// bsum[nb] receives the total
__global__ void na_block_scan_kernel(int nb, long long* __restrict__ bsum) {
    __shared__ long long s_sh[33];
    __shared__ long long s_carry;
    if (threadIdx.x == 0) s_carry = 0;
    __syncthreads();
    for (int b0 = 0; b0 < nb; b0 += blockDim.x) {
        const int b = b0 + threadIdx.x;
        const long long v = b < nb ? bsum[b] : 0;
        long long tot;
        const long long ex = block_excl_scan<long long>(v, s_sh, &tot);
        if (b < nb) bsum[b] = s_carry + ex;
        __syncthreads();
        if (threadIdx.x == 0) s_carry += tot;
        __syncthreads();
    }
    if (threadIdx.x == 0) bsum[nb] = s_carry;
}

// row pointers: block scan of its counts plus its block offset
__global__ void na_rowptr_kernel(int m, const int* __restrict__ counts, const long long* __restrict__ bsum,
                                 int nb, int* __restrict__ out_rp) {
    __shared__ long long s_sh[33];
    const int base = blockIdx.x * NA_SCAN_ITEMS;
    const int per = NA_SCAN_ITEMS / blockDim.x;
    long long local = 0;
    for (int q = 0; q < per; q++) {
        const int i = base + threadIdx.x * per + q;
        if (i < m) local += counts[i];
    }
    long long tot;
    long long run = bsum[blockIdx.x] + block_excl_scan<long long>(local, s_sh, &tot);
    for (int q = 0; q < per; q++) {
        const int i = base + threadIdx.x * per + q;
        if (i < m) {
            out_rp[i] = (int)run;
            run += counts[i];
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) out_rp[m] = (int)bsum[nb];
}

// one warp per C tile-row: its tiles' row masks expand to ascending columns
template <typename V>
__global__ void na_fill_kernel(int tilem, int m, const int* __restrict__ tile_ptrC, const int* __restrict__ colidxC,
                               const uint16_t* __restrict__ maskC, const int64_t* __restrict__ tile_nnzC,
                               const uint8_t* __restrict__ ptrRowC, const V* __restrict__ valC,
                               const int* __restrict__ rp, int* __restrict__ out_ci, V* __restrict__ out_val) {
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
                uint32_t mk = t < te ? (uint32_t)maskC[(int64_t)t * TS + r] : 0u;
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

// Device address of the working area on the handle's device (looked up on
// the first call on that device; that call should therefore come before any
// stream capture).
spg_status scratch_for_device(spg_handle_t h, NoallocScratch** out) {
    if (h->device < 0 || h->device >= NA_MAX_DEVICES)
        return spg_fail(h, SPG_ERR_UNSUPPORTED, "no-alloc export: device index out of range");
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch_ptr[h->device]) {
        int prev = 0;
        SPG_CUDA(h, cudaGetDevice(&prev));
        if (prev != h->device) SPG_CUDA(h, cudaSetDevice(h->device));
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (prev != h->device) cudaSetDevice(prev);
        if (e != cudaSuccess || !p) return spg_cuda_fail(h, e, "cudaGetSymbolAddress(g_noalloc_scratch)");
        g_scratch_ptr[h->device] = static_cast<NoallocScratch*>(p);
    }
    *out = g_scratch_ptr[h->device];
    return SPG_OK;
}

int na_grid(spg_handle_t h, int64_t n, int threads) {
    int64_t g = ceil_div(n, threads);
    if (g > (int64_t)h->num_sms * 16) g = (int64_t)h->num_sms * 16;
    return (int)(g < 1 ? 1 : g);
}

}  // namespace

extern "C" spg_status spg_ctiles_to_csr_noalloc(spg_handle_t h, const spg_ctiles* C, int* out_rp, int* out_ci,
                                               void* out_val, int64_t* nnz) {
    if (!h) return SPG_ERR_INVALID;
    if (!C || !out_rp) return spg_fail(h, SPG_ERR_INVALID, "no-alloc export: null argument");
    if (C->m < 0 || C->m > SPG_NOALLOC_MAX_ROWS)
        return spg_fail(h, SPG_ERR_INVALID, "no-alloc export: C has more than 1,048,576 rows (SPG_NOALLOC_MAX_ROWS)");
    if (C->nnzC >= 0x7fffffffLL) return spg_fail(h, SPG_ERR_INVALID, "no-alloc export: nnz does not fit int32 CSR");
    if (C->nnzC > 0 && (!out_ci || !out_val)) return spg_fail(h, SPG_ERR_INVALID, "no-alloc export: null output");
    NoallocScratch* sc = nullptr;
    SPG_TRY(scratch_for_device(h, &sc));
    const int m = C->m;
    const int nb = (m + NA_SCAN_ITEMS - 1) / NA_SCAN_ITEMS;
    // the working area keeps the previous call's counts: clear them first
    SPG_CUDA(h, cudaMemsetAsync(sc->counts, 0, sizeof(int) * ((size_t)m + 1), h->stream));
    if (C->numtileC > 0) {
        na_rowcount_kernel<<<na_grid(h, C->numtileC * TS, 256), 256, 0, h->stream>>>(C->numtileC, m, C->tile_rowidxC,
                                                                                    C->maskC, sc->counts);
        SPG_LAUNCHED(h);
    }
    if (nb > 0) {
        na_block_sum_kernel<<<nb, 256, 0, h->stream>>>(m, sc->counts, sc->block_sums);
        SPG_LAUNCHED(h);
    }
    na_block_scan_kernel<<<1, 1024, 0, h->stream>>>(nb, sc->block_sums);
    SPG_LAUNCHED(h);
    if (nb > 0) {
        na_rowptr_kernel<<<nb, 256, 0, h->stream>>>(m, sc->counts, sc->block_sums, nb, out_rp);
        SPG_LAUNCHED(h);
    } else {
        SPG_CUDA(h, cudaMemsetAsync(out_rp, 0, sizeof(int), h->stream));
    }
    if (C->nnzC > 0 && C->tilem > 0) {
        if (C->dtype == SPG_F64)
            na_fill_kernel<double><<<na_grid(h, (int64_t)C->tilem * 32, 256), 256, 0, h->stream>>>(
                C->tilem, m, C->tile_ptrC, C->tile_colidxC, C->maskC, C->tile_nnzC, C->ptrRowC,
                (const double*)C->tile_valC, out_rp, out_ci, (double*)out_val);
        else
            na_fill_kernel<float><<<na_grid(h, (int64_t)C->tilem * 32, 256), 256, 0, h->stream>>>(
                C->tilem, m, C->tile_ptrC, C->tile_colidxC, C->maskC, C->tile_nnzC, C->ptrRowC,
                (const float*)C->tile_valC, out_rp, out_ci, (float*)out_val);
        SPG_LAUNCHED(h);
    }
    if (nnz) *nnz = C->nnzC;
    return SPG_OK;
}
