// spg_common.cuh -- shared definitions for the GB300 tiled SpGEMM kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <string>

#include "../../include/spgemm_gb300.h"

#define TS 16

// Device error bits, written to a per-handle flag word by kernels and read
// back by the host after the call's synchronisation point.
enum : unsigned {
    DERR_NONCANONICAL = 1u << 0,  // CSR columns not strictly ascending / out of range
    DERR_TIMEOUT = 1u << 1,       // a bounded spin-wait gave up
    DERR_OVERFLOW = 1u << 2,      // a pre-sized buffer was too small (writes skipped)
    DERR_TOO_BIG = 1u << 3,       // a count overflowed its index type
};

// Upper bound on spin iterations of any device-side wait (decoupled look-back).
// Forward progress is guaranteed by ticket ordering; the bound is a safety net
// that turns a would-be hang into DERR_TIMEOUT.
#define SPG_SPIN_LIMIT (1 << 22)

__device__ __forceinline__ unsigned lanemask_lt() {
    unsigned m;
    asm volatile("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

template <typename T>
__device__ __forceinline__ T warp_incl_scan(T v, unsigned lane) {
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        T o = __shfl_up_sync(0xffffffffu, v, d);
        if (lane >= (unsigned)d) v += o;
    }
    return v;
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) v += __shfl_xor_sync(0xffffffffu, v, d);
    return v;
}

// Block-wide exclusive scan of one value per thread; `sh` needs blockDim/32 + 1
// entries.  Returns the exclusive prefix, writes the block total to *total.
template <typename T>
__device__ __forceinline__ T block_excl_scan(T v, T* sh, T* total) {
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    T inc = warp_incl_scan(v, lane);
    if (lane == 31) sh[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        T w = lane < nw ? sh[lane] : T(0);
        T wi = warp_incl_scan(w, lane);
        if (lane < nw) sh[lane] = wi - w;
        if (lane == nw - 1) sh[nw] = wi;
    }
    __syncthreads();
    T res = sh[warp] + inc - v;
    *total = sh[nw];
    __syncthreads();
    return res;
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
struct spg_handle_s {
    int device = 0;
    struct spg_mlp_s* sizing = nullptr;  // learned sizing model (optional)
    float sizing_margin = 1.0f;
    int dense_thr = 32;        // tile nnz above which a tile pair goes to tensor cores (MIXED)
    float cancel_eps = 9.5367431640625e-07f;  // 2^-20: |c| < eps * sum|a||b| flags a C tile for FP64
    cudaStream_t stream = nullptr;
    std::string err;
    spg_stats stats{};
    unsigned* d_flags = nullptr;      // device error bits
    int64_t* h_pinned = nullptr;      // 64 pinned words for read-backs
    int* h_band = nullptr;            // mapped pinned band flags (spg_numeric_bands), band_cap entries
    int* d_band = nullptr;            // the same flags' device address
    int band_cap = 0;
    cudaEvent_t ev[8]{};
    int num_sms = 0;
    size_t smem_optin = 0;
    size_t smem_per_sm = 0;
    int64_t launches = 0;             // kernels launched through this handle
    void* ws[4] = {};                 // grow-only workspaces of the large per-call temporaries
    size_t ws_bytes[4] = {};
    float bin_pp_thr = 12.0f;          // binned algorithm: products per tile pair for the plain kernels
    float bin_fill_thr = 16.0f;       // ... and predicted C nonzeros per C tile (with a sizing model)
};

spg_status spg_fail(spg_handle_t h, spg_status s, const std::string& msg);
spg_status spg_cuda_fail(spg_handle_t h, cudaError_t e, const char* what);

#define SPG_CUDA(h, call)                                              \
    do {                                                               \
        cudaError_t _e = (call);                                       \
        if (_e != cudaSuccess) return spg_cuda_fail((h), _e, #call);   \
    } while (0)

// After a kernel launch: counts the launch on the handle (spg_kernel_launches)
// and turns a launch error into a status.
#define SPG_LAUNCHED(h)                                                \
    do {                                                               \
        (h)->launches++;                                               \
        SPG_CUDA((h), cudaGetLastError());                             \
    } while (0)

#define SPG_TRY(call)                          \
    do {                                       \
        spg_status _s = (call);                \
        if (_s != SPG_OK) return _s;           \
    } while (0)

// Stream-ordered device allocation on the handle's stream.
spg_status spg_alloc(spg_handle_t h, void** p, size_t bytes);
void spg_free_async(spg_handle_t h, void* p);
template <typename T>
inline spg_status spg_alloc_t(spg_handle_t h, T** p, size_t count) {
    return spg_alloc(h, reinterpret_cast<void**>(p), count * sizeof(T));
}

// Device scratch of one call: every buffer taken through it is released
// (stream-ordered, after the work queued so far) when the scope ends, on
// every return path, so an error return leaks nothing.
class ScratchList {
  public:
    explicit ScratchList(spg_handle_t h) : h_(h) {}
    ScratchList(const ScratchList&) = delete;
    ScratchList& operator=(const ScratchList&) = delete;
    ~ScratchList() {
        for (int i = 0; i < n_; i++) spg_free_async(h_, p_[i]);
    }
    template <typename T>
    spg_status alloc(T** out, size_t count) {
        *out = nullptr;
        if (n_ == kMax) return spg_fail(h_, SPG_ERR_INVALID, "internal: too many scratch buffers in one call");
        SPG_TRY(spg_alloc_t(h_, out, count));
        p_[n_++] = *out;
        return SPG_OK;
    }
    // Hands a buffer over to a longer-lived owner: it is no longer released.
    void keep(const void* p) {
        for (int i = 0; i < n_; i++)
            if (p_[i] == p) p_[i] = nullptr;
    }

  private:
    static constexpr int kMax = 16;
    spg_handle_t h_;
    void* p_[kMax] = {};
    int n_ = 0;
};

// A large temporary that every call of a kind needs (the learned slots of
// step 1, B's interleaved entries of the numeric phase) lives in a grow-only
// buffer of the handle instead of a fresh pool block per call: a repeated
// product then allocates only C's own arrays, the same blocks each time.
// Uses are ordered on the handle's stream, so one call's use ends before the
// next begins; spg_destroy releases the buffers.  Not for work captured into
// a CUDA graph (a later growth would move the buffer under the graph).
enum { SPG_WS_SLOTS = 0, SPG_WS_BENTRY = 1 };
spg_status spg_workspace(spg_handle_t h, int kind, size_t bytes, void** out);

// Read device error bits (synchronises the stream) and clear them.
spg_status spg_check_flags(spg_handle_t h, const char* where);
// n (<= 8) device int64 scalars and the error bits in one round trip.
spg_status spg_read_i64s_checked(spg_handle_t h, int n, const int64_t* const* src, int64_t* out, const char* where);

// Exclusive scans: out[0..n] (n+1 entries, out[n] = total).  `in` may alias
// `out` when the types match.  Temporary storage comes from spg_alloc.
spg_status spg_scan_i32_to_i32(spg_handle_t h, const int* in, int* out, int64_t n);
spg_status spg_scan_i32_to_i64(spg_handle_t h, const int* in, int64_t* out, int64_t n);
spg_status spg_scan_i64_to_i64(spg_handle_t h, const int64_t* in, int64_t* out, int64_t n);

// Stable LSD radix sort of (key, value) pairs by the low `key_bits` of key.
spg_status spg_radix_sort_pairs(spg_handle_t h, uint32_t* keys, uint32_t* vals, int64_t n,
                                int key_bits);

// v[i] = i for i < n.
spg_status spg_iota_u32(spg_handle_t h, uint32_t* v, int64_t n);

// Read a device scalar (synchronises the stream).
spg_status spg_read_i64(spg_handle_t h, const int64_t* d, int64_t* out);
spg_status spg_read_i32(spg_handle_t h, const int* d, int* out);

inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }
inline size_t val_size(spg_dtype t) { return t == SPG_F64 ? 8 : 4; }
