// scan.cu -- single-pass exclusive scan (decoupled look-back) and stable LSD
// radix sort.  These replace the cub::DeviceScan::ExclusiveSum calls of
// src/spgemm_raw_v2.cu:132-138,202-208 (which also cudaMalloc'd their temp
// storage inside the timed region) with in-library primitives.
#include "spg_common.cuh"

namespace {

constexpr int SCAN_THREADS = 256;
constexpr int SCAN_ITEMS = 16;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;  // 4096 items per block

constexpr unsigned long long FLAG_AGG = 1ull << 62;
constexpr unsigned long long FLAG_PRE = 2ull << 62;
constexpr unsigned long long VAL_MASK = (1ull << 62) - 1;

__device__ __forceinline__ unsigned long long ld_volatile_u64(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.volatile.global.u64 %0, [%1];" : "=l"(v) : "l"(p));
    return v;
}

// Scans n+1 items (item n is taken as 0) so that out[n] holds the total.
// Blocks take tiles in ticket order, so a block only waits for tiles that are
// already running or done; every wait is bounded by SPG_SPIN_LIMIT.
template <typename Tin, typename Tout>
__global__ void __launch_bounds__(SCAN_THREADS)
scan_lookback_kernel(const Tin* in, Tout* out, int64_t n, unsigned long long* state,
                     unsigned* ticket, unsigned* flags) {
    __shared__ int64_t s_items[SCAN_TILE];
    __shared__ int64_t s_sh[SCAN_THREADS / 32 + 1];
    __shared__ unsigned s_bid;
    __shared__ int64_t s_prefix;
    if (threadIdx.x == 0) s_bid = atomicAdd(ticket, 1u);
    __syncthreads();
    const int64_t bid = s_bid;
    const int64_t base = bid * SCAN_TILE;
    const int64_t total_items = n + 1;
    // striped coalesced load
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) {
        int64_t idx = base + (int64_t)k * SCAN_THREADS + threadIdx.x;
        s_items[k * SCAN_THREADS + threadIdx.x] = (idx < n) ? (int64_t)in[idx] : 0;
    }
    __syncthreads();
    // blocked per-thread reduce
    int64_t local = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) local += s_items[threadIdx.x * SCAN_ITEMS + k];
    int64_t agg;
    int64_t excl = block_excl_scan<int64_t>(local, s_sh, &agg);
    if (threadIdx.x == 0) {
        int64_t prefix = 0;
        if (bid == 0) {
            atomicExch(&state[0], FLAG_PRE | ((unsigned long long)agg & VAL_MASK));
        } else {
            atomicExch(&state[bid], FLAG_AGG | ((unsigned long long)agg & VAL_MASK));
            int64_t j = bid - 1;
            int spins = 0;
            while (j >= 0) {
                unsigned long long s = ld_volatile_u64(&state[j]);
                unsigned long long f = s & ~VAL_MASK;
                if (f == 0) {
                    if (++spins > SPG_SPIN_LIMIT) { atomicOr(flags, DERR_TIMEOUT); break; }
                    continue;
                }
                prefix += (int64_t)(s & VAL_MASK);
                if (f == FLAG_PRE) break;
                j--;
            }
            __threadfence();
            atomicExch(&state[bid], FLAG_PRE | ((unsigned long long)(prefix + agg) & VAL_MASK));
        }
        s_prefix = prefix;
    }
    __syncthreads();
    int64_t run = s_prefix + excl;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) {
        int64_t v = s_items[threadIdx.x * SCAN_ITEMS + k];
        s_items[threadIdx.x * SCAN_ITEMS + k] = run;
        run += v;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) {
        int64_t idx = base + (int64_t)k * SCAN_THREADS + threadIdx.x;
        if (idx < total_items) out[idx] = (Tout)s_items[k * SCAN_THREADS + threadIdx.x];
    }
}

// Long scans (C's 1.8e9 tile counts on a power-law product) run as two
// streaming passes instead: per-warp sums of 1024-item slices, a (short)
// look-back scan of those sums, then every warp rescans its slice with
// shuffles from its offset.  No block waits on another, all accesses are
// coalesced, and the traffic is two reads and one write of the array.
constexpr int WS_THREADS = 256;
constexpr int WS_SLICE = 1024;  // items per warp
constexpr int64_t WS_MIN_N = 1 << 22;

template <typename Tin>
__global__ void __launch_bounds__(WS_THREADS)
slice_sum_kernel(const Tin* __restrict__ in, int64_t n, int64_t nslices, int64_t* __restrict__ sums) {
    const int lane = threadIdx.x & 31;
    const int64_t sl = (int64_t)blockIdx.x * (WS_THREADS / 32) + (threadIdx.x >> 5);
    if (sl >= nslices) return;
    const int64_t b = sl * WS_SLICE;
    int64_t v = 0;
#pragma unroll 8
    for (int k = 0; k < WS_SLICE / 32; k++) {
        const int64_t idx = b + k * 32 + lane;
        if (idx < n) v += (int64_t)in[idx];
    }
    v = warp_sum(v);
    if (lane == 0) sums[sl] = v;
}

template <typename Tin, typename Tout>
__global__ void __launch_bounds__(WS_THREADS)
slice_scan_kernel(const Tin* in, Tout* out, int64_t n, int64_t nslices, const int64_t* __restrict__ offs) {
    const int lane = threadIdx.x & 31;
    const int64_t sl = (int64_t)blockIdx.x * (WS_THREADS / 32) + (threadIdx.x >> 5);
    if (sl >= nslices) return;
    const int64_t b = sl * WS_SLICE;
    int64_t carry = offs[sl];
#pragma unroll 4
    for (int k = 0; k < WS_SLICE / 32; k++) {
        const int64_t idx = b + k * 32 + lane;
        const int64_t v = idx < n ? (int64_t)in[idx] : 0;
        int64_t inc = v;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const int64_t o = __shfl_up_sync(0xffffffffu, inc, d);
            if (lane >= d) inc += o;
        }
        if (idx <= n) out[idx] = (Tout)(carry + inc - v);
        carry += __shfl_sync(0xffffffffu, inc, 31);
    }
}

template <typename Tin, typename Tout>
spg_status scan_impl(spg_handle_t h, const Tin* in, Tout* out, int64_t n);

template <typename Tin, typename Tout>
spg_status scan_long(spg_handle_t h, const Tin* in, Tout* out, int64_t n) {
    const int64_t nslices = ceil_div(n + 1, WS_SLICE);
    const int64_t nblocks = ceil_div(nslices, WS_THREADS / 32);
    if (nblocks > 0x7fffffffLL) return spg_fail(h, SPG_ERR_INVALID, "scan: too long");
    ScratchList sc(h);
    int64_t* sums = nullptr;
    SPG_TRY(sc.alloc(&sums, (size_t)nslices + 1));
    slice_sum_kernel<Tin><<<(unsigned)nblocks, WS_THREADS, 0, h->stream>>>(in, n, nslices, sums);
    SPG_LAUNCHED(h);
    SPG_TRY((scan_impl<int64_t, int64_t>(h, sums, sums, nslices)));
    slice_scan_kernel<Tin, Tout><<<(unsigned)nblocks, WS_THREADS, 0, h->stream>>>(in, out, n, nslices, sums);
    SPG_LAUNCHED(h);
    return SPG_OK;
}

template <typename Tin, typename Tout>
spg_status scan_impl(spg_handle_t h, const Tin* in, Tout* out, int64_t n) {
    if (n < 0) return spg_fail(h, SPG_ERR_INVALID, "scan: negative length");
    if (n >= WS_MIN_N) return scan_long<Tin, Tout>(h, in, out, n);
    const int64_t nblocks = ceil_div(n + 1, SCAN_TILE);
    if (nblocks > 0x7fffffffLL) return spg_fail(h, SPG_ERR_INVALID, "scan: too long");
    ScratchList sc(h);
    unsigned long long* state = nullptr;
    SPG_TRY(sc.alloc(&state, (size_t)nblocks + 2));
    unsigned* ticket = reinterpret_cast<unsigned*>(state + nblocks);
    SPG_CUDA(h, cudaMemsetAsync(state, 0, sizeof(unsigned long long) * nblocks + 16, h->stream));
    scan_lookback_kernel<Tin, Tout><<<(unsigned)nblocks, SCAN_THREADS, 0, h->stream>>>(
        in, out, n, state, ticket, h->d_flags);
    SPG_LAUNCHED(h);
    return SPG_OK;
}

// ---------------------------------------------------------------------------
// Stable LSD radix sort, 8-bit digits.
// ---------------------------------------------------------------------------
constexpr int RS_THREADS = 256;
constexpr int RS_ROUNDS = 8;
constexpr int RS_CHUNK = RS_THREADS * RS_ROUNDS;  // 2048 items per block
constexpr int RS_WARPS = RS_THREADS / 32;

__global__ void __launch_bounds__(RS_THREADS)
radix_hist_kernel(const uint32_t* keys, int64_t n, int shift, int nblk, int* hist) {
    __shared__ int cnt[256];
    cnt[threadIdx.x] = 0;
    __syncthreads();
    const int64_t base = (int64_t)blockIdx.x * RS_CHUNK;
    for (int r = 0; r < RS_ROUNDS; r++) {
        int64_t idx = base + (int64_t)r * RS_THREADS + threadIdx.x;
        if (idx < n) atomicAdd(&cnt[(keys[idx] >> shift) & 255u], 1);
    }
    __syncthreads();
    hist[(int64_t)threadIdx.x * nblk + blockIdx.x] = cnt[threadIdx.x];
}

__global__ void __launch_bounds__(RS_THREADS)
radix_scatter_kernel(const uint32_t* kin, const uint32_t* vin, uint32_t* kout, uint32_t* vout,
                     int64_t n, int shift, int nblk, const int* hist_scan) {
    __shared__ int base[256];
    __shared__ int run[256];
    __shared__ int wcnt[RS_WARPS][256];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    base[tid] = hist_scan[(int64_t)tid * nblk + blockIdx.x];
    run[tid] = 0;
#pragma unroll
    for (int w = 0; w < RS_WARPS; w++) wcnt[w][tid] = 0;
    __syncthreads();
    const int64_t cbase = (int64_t)blockIdx.x * RS_CHUNK;
    for (int r = 0; r < RS_ROUNDS; r++) {
        int64_t idx = cbase + (int64_t)r * RS_THREADS + tid;
        bool valid = idx < n;
        uint32_t k = valid ? kin[idx] : 0u, v = valid ? vin[idx] : 0u;
        int d = valid ? (int)((k >> shift) & 255u) : 256;
        unsigned peers = __match_any_sync(0xffffffffu, d);
        int rank = __popc(peers & lanemask_lt());
        int leader = __ffs(peers) - 1;
        if (valid && lane == leader) wcnt[warp][d] = __popc(peers);
        __syncthreads();
        int sum = 0;
#pragma unroll
        for (int w = 0; w < RS_WARPS; w++) {
            int c = wcnt[w][tid];
            wcnt[w][tid] = sum;
            sum += c;
        }
        __syncthreads();
        if (valid) {
            int pos = base[d] + run[d] + wcnt[warp][d] + rank;
            kout[pos] = k;
            vout[pos] = v;
        }
        __syncthreads();
        run[tid] += sum;
#pragma unroll
        for (int w = 0; w < RS_WARPS; w++) wcnt[w][tid] = 0;
        __syncthreads();
    }
}

__global__ void iota_u32_kernel(uint32_t* v, int64_t n) {
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x)
        v[t] = (uint32_t)t;
}

}  // namespace

spg_status spg_iota_u32(spg_handle_t h, uint32_t* v, int64_t n) {
    if (n <= 0) return SPG_OK;
    int64_t g = ceil_div(n, 256);
    if (g > (int64_t)h->num_sms * 16) g = (int64_t)h->num_sms * 16;
    iota_u32_kernel<<<(int)g, 256, 0, h->stream>>>(v, n);
    SPG_LAUNCHED(h);
    return SPG_OK;
}

spg_status spg_scan_i32_to_i32(spg_handle_t h, const int* in, int* out, int64_t n) {
    return scan_impl<int, int>(h, in, out, n);
}
spg_status spg_scan_i32_to_i64(spg_handle_t h, const int* in, int64_t* out, int64_t n) {
    return scan_impl<int, int64_t>(h, in, out, n);
}
spg_status spg_scan_i64_to_i64(spg_handle_t h, const int64_t* in, int64_t* out, int64_t n) {
    return scan_impl<int64_t, int64_t>(h, in, out, n);
}

spg_status spg_radix_sort_pairs(spg_handle_t h, uint32_t* keys, uint32_t* vals, int64_t n,
                                int key_bits) {
    if (n <= 1) return SPG_OK;
    if (n >= 0x7fffffffLL) return spg_fail(h, SPG_ERR_INVALID, "radix sort: too many items");
    const int passes = key_bits <= 0 ? 1 : (key_bits + 7) / 8;
    const int nblk = (int)ceil_div(n, RS_CHUNK);
    uint32_t *k2 = nullptr, *v2 = nullptr;
    int* hist = nullptr;
    ScratchList sc(h);
    SPG_TRY(sc.alloc(&k2, n));
    SPG_TRY(sc.alloc(&v2, n));
    SPG_TRY(sc.alloc(&hist, (int64_t)256 * nblk + 1));
    uint32_t *ka = keys, *va = vals, *kb = k2, *vb = v2;
    for (int p = 0; p < passes; p++) {
        radix_hist_kernel<<<nblk, RS_THREADS, 0, h->stream>>>(ka, n, 8 * p, nblk, hist);
        SPG_LAUNCHED(h);
        SPG_TRY(spg_scan_i32_to_i32(h, hist, hist, (int64_t)256 * nblk));
        radix_scatter_kernel<<<nblk, RS_THREADS, 0, h->stream>>>(ka, va, kb, vb, n, 8 * p, nblk, hist);
        SPG_LAUNCHED(h);
        uint32_t* t = ka; ka = kb; kb = t;
        t = va; va = vb; vb = t;
    }
    if (ka != keys) {
        SPG_CUDA(h, cudaMemcpyAsync(keys, ka, n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, h->stream));
        SPG_CUDA(h, cudaMemcpyAsync(vals, va, n * sizeof(uint32_t), cudaMemcpyDeviceToDevice, h->stream));
    }
    return SPG_OK;
}
