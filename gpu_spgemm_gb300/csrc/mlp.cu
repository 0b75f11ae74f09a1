// mlp.cu -- learned sizing for the tiled SpGEMM.
//
// The reference sizes C by an exact upper-bound pass: step 1 counts the C
// tiles of every tile-row (a full bitmap pass), scans, reads the total back to
// the host and only then fills the tile indices in a second bitmap pass
// (src/spgemm_raw_v2.cu:119-156).  Here a small MLP reads cheap per-tile-row
// features of A and B and predicts each tile-row's C tile count and C
// nonzeros.  Each tile-row then gets a slot of its predicted size (times a
// margin), and step 1 builds every tile-row's bitmap ONCE: it counts exactly,
// writes the tile columns into the slot when they fit, and a compaction copies
// the slots into C's exact arrays (plain.cu, c1_slot_kernel and
// c1_compact_kernel).  The exact bitmap count has the last word: a tile-row that
// outgrew its slot re-runs the exact fill.  The structure is never
// approximated.
//
// Network: 8 -> 32 -> 32 -> 2, ReLU, linear output, MSE on standardised
// log1p targets.  Trained on the GPU by the kernels below (forward, backward
// with shared-memory gradient accumulation, Adam), gradients checked against a
// numpy restatement in the tests.
#include <cmath>
#include <new>
#include <vector>

#include "plain.cuh"
#include "spg_common.cuh"

#define NF 8
#define NH 32
#define NO 2
// parameter layout: W1[NH][NF] b1[NH] W2[NH][NH] b2[NH] W3[NO][NH] b3[NO]
#define OFF_W1 0
#define OFF_B1 (OFF_W1 + NH * NF)
#define OFF_W2 (OFF_B1 + NH)
#define OFF_B2 (OFF_W2 + NH * NH)
#define OFF_W3 (OFF_B2 + NH)
#define OFF_B3 (OFF_W3 + NO * NH)
#define NPARAM (OFF_B3 + NO)
// normalisation (not trained): feature mean / inv-std, target mean / std
#define NNORM (2 * NF + 2 * NO)

struct spg_mlp_s {
    float* d_param = nullptr;  // NPARAM
    float* d_norm = nullptr;   // NNORM
    float* d_grad = nullptr;   // NPARAM
    float* d_m = nullptr;      // Adam moments
    float* d_v = nullptr;
    float* d_loss = nullptr;
    int64_t step = 0;
};

namespace {

// ---------------------------------------------------------------------------
// features: one warp per tile-row of A
// ---------------------------------------------------------------------------
__global__ void mlp_features_kernel(int tilem, int m, int tilenB, const int* __restrict__ a_tp,
                                    const int* __restrict__ a_tc, const int* __restrict__ a_rp,
                                    const int* __restrict__ a_ci, const int* __restrict__ b_tp,
                                    const int* __restrict__ b_tc, const int* __restrict__ b_rp,
                                    float* __restrict__ feat) {
    const int lane = threadIdx.x & 31;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < tilem; i += nw) {
        const int as = a_tp[i], ae = a_tp[i + 1];
        unsigned long long pairs = 0, mxb = 0;
        int lo = 0x7fffffff, hi = -1;
        for (int a = as + lane; a < ae; a += 32) {
            const int k = __ldg(&a_tc[a]);
            const int bs = __ldg(&b_tp[k]), be = __ldg(&b_tp[k + 1]);
            pairs += (unsigned long long)(be - bs);
            if ((unsigned long long)(be - bs) > mxb) mxb = (unsigned long long)(be - bs);
            if (be > bs) { lo = min(lo, __ldg(&b_tc[bs])); hi = max(hi, __ldg(&b_tc[be - 1])); }
        }
        const int e0 = a_rp[i * TS], e1 = a_rp[min(i * TS + TS, m)];
        unsigned long long prod = 0;
        for (int e = e0 + lane; e < e1; e += 32) {
            const int k = __ldg(&a_ci[e]);
            prod += (unsigned long long)(__ldg(&b_rp[k + 1]) - __ldg(&b_rp[k]));
        }
        int occ = 0;
        if (lane < TS && i * TS + lane < m) occ = (a_rp[i * TS + lane + 1] > a_rp[i * TS + lane]) ? 1 : 0;
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) {
            pairs += __shfl_xor_sync(0xffffffffu, pairs, d);
            prod += __shfl_xor_sync(0xffffffffu, prod, d);
            const unsigned long long om = __shfl_xor_sync(0xffffffffu, mxb, d);
            mxb = om > mxb ? om : mxb;
            lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, d));
            hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, d));
            occ += __shfl_xor_sync(0xffffffffu, occ, d);
        }
        if (lane == 0) {
            float* f = feat + (int64_t)i * NF;
            f[0] = log1pf((float)(ae - as));
            f[1] = log1pf((float)(e1 - e0));
            f[2] = log1pf((float)pairs);
            f[3] = log1pf((float)prod);
            f[4] = log1pf((float)mxb);
            f[5] = log1pf((float)(hi >= lo ? hi - lo + 1 : 0));
            f[6] = (float)occ / 16.0f;
            f[7] = log1pf((float)tilenB);
        }
    }
}

// ---------------------------------------------------------------------------
// forward (inference): one thread per sample, parameters in shared memory
// ---------------------------------------------------------------------------
__device__ __forceinline__ void mlp_forward_one(const float* P, const float* nrm, const float* x_raw, float* h1,
                                                float* h2, float* out, float* xin) {
#pragma unroll
    for (int f = 0; f < NF; f++) xin[f] = (x_raw[f] - nrm[f]) * nrm[NF + f];
#pragma unroll 4
    for (int j = 0; j < NH; j++) {
        float s = P[OFF_B1 + j];
#pragma unroll
        for (int f = 0; f < NF; f++) s += P[OFF_W1 + j * NF + f] * xin[f];
        h1[j] = s > 0.f ? s : 0.f;
    }
#pragma unroll 4
    for (int j = 0; j < NH; j++) {
        float s = P[OFF_B2 + j];
        for (int q = 0; q < NH; q++) s += P[OFF_W2 + j * NH + q] * h1[q];
        h2[j] = s > 0.f ? s : 0.f;
    }
#pragma unroll
    for (int o = 0; o < NO; o++) {
        float s = P[OFF_B3 + o];
        for (int q = 0; q < NH; q++) s += P[OFF_W3 + o * NH + q] * h2[q];
        out[o] = s;
    }
}

__global__ void mlp_forward_kernel(int64_t n, const float* __restrict__ param, const float* __restrict__ norm,
                                   const float* __restrict__ feat, float* __restrict__ out) {
    __shared__ float P[NPARAM];
    __shared__ float N[NNORM];
    for (int t = threadIdx.x; t < NPARAM; t += blockDim.x) P[t] = param[t];
    for (int t = threadIdx.x; t < NNORM; t += blockDim.x) N[t] = norm[t];
    __syncthreads();
    for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < n; s += (int64_t)gridDim.x * blockDim.x) {
        float xin[NF], h1[NH], h2[NH], o[NO];
        mlp_forward_one(P, N, feat + s * NF, h1, h2, o, xin);
#pragma unroll
        for (int k = 0; k < NO; k++) out[s * NO + k] = o[k] * N[2 * NF + NO + k] + N[2 * NF + k];  // de-standardise
    }
}

// ---------------------------------------------------------------------------
// training: gradient of the mean squared error over a batch of samples
// (indices idx[0..nb)), accumulated in shared memory then into grad
// ---------------------------------------------------------------------------
__global__ void mlp_grad_kernel(int64_t nb, const int* __restrict__ idx, const float* __restrict__ param,
                                const float* __restrict__ norm, const float* __restrict__ feat,
                                const float* __restrict__ target, float* __restrict__ grad, float* __restrict__ loss) {
    __shared__ float P[NPARAM];
    __shared__ float G[NPARAM];
    __shared__ float N[NNORM];
    __shared__ float s_loss;
    for (int t = threadIdx.x; t < NPARAM; t += blockDim.x) { P[t] = param[t]; G[t] = 0.f; }
    for (int t = threadIdx.x; t < NNORM; t += blockDim.x) N[t] = norm[t];
    if (threadIdx.x == 0) s_loss = 0.f;
    __syncthreads();
    const float scale = 2.0f / (float)(nb * NO);
    for (int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; b < nb; b += (int64_t)gridDim.x * blockDim.x) {
        const int64_t s = idx ? idx[b] : b;
        float xin[NF], h1[NH], h2[NH], o[NO];
        mlp_forward_one(P, N, feat + s * NF, h1, h2, o, xin);
        float dout[NO];
        float l = 0.f;
#pragma unroll
        for (int k = 0; k < NO; k++) {
            const float y = (target[s * NO + k] - N[2 * NF + k]) / N[2 * NF + NO + k];
            const float d = o[k] - y;
            l += d * d;
            dout[k] = scale * d;
        }
        atomicAdd(&s_loss, l);
        float dh2[NH];
        for (int q = 0; q < NH; q++) {
            float g = 0.f;
#pragma unroll
            for (int k = 0; k < NO; k++) {
                atomicAdd(&G[OFF_W3 + k * NH + q], dout[k] * h2[q]);
                g += P[OFF_W3 + k * NH + q] * dout[k];
            }
            dh2[q] = h2[q] > 0.f ? g : 0.f;
        }
#pragma unroll
        for (int k = 0; k < NO; k++) atomicAdd(&G[OFF_B3 + k], dout[k]);
        float dh1[NH];
        for (int q = 0; q < NH; q++) dh1[q] = 0.f;
        for (int j = 0; j < NH; j++) {
            const float d = dh2[j];
            if (d == 0.f) continue;
            atomicAdd(&G[OFF_B2 + j], d);
            for (int q = 0; q < NH; q++) {
                atomicAdd(&G[OFF_W2 + j * NH + q], d * h1[q]);
                dh1[q] += P[OFF_W2 + j * NH + q] * d;
            }
        }
        for (int j = 0; j < NH; j++) {
            const float d = h1[j] > 0.f ? dh1[j] : 0.f;
            if (d == 0.f) continue;
            atomicAdd(&G[OFF_B1 + j], d);
#pragma unroll
            for (int f = 0; f < NF; f++) atomicAdd(&G[OFF_W1 + j * NF + f], d * xin[f]);
        }
    }
    __syncthreads();
    for (int t = threadIdx.x; t < NPARAM; t += blockDim.x)
        if (G[t] != 0.f) atomicAdd(&grad[t], G[t]);
    if (threadIdx.x == 0 && loss) atomicAdd(loss, s_loss / (float)(nb * NO));
}

__global__ void mlp_adam_kernel(float* __restrict__ p, float* __restrict__ g, float* __restrict__ m,
                                float* __restrict__ v, float lr, float b1, float b2, float c1, float c2) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= NPARAM) return;
    const float gr = g[t];
    const float mm = b1 * m[t] + (1.f - b1) * gr;
    const float vv = b2 * v[t] + (1.f - b2) * gr * gr;
    m[t] = mm;
    v[t] = vv;
    p[t] -= lr * (mm / c1) / (sqrtf(vv / c2) + 1e-8f);
    g[t] = 0.f;
}

// Slot size of each tile-row: the predicted C tile count (the network's
// target is log1p of it) grown by the margin, plus 2, and never more than the
// row can have: no more than B's tile columns, than the tile pairs the row
// reaches (feature 2) or than the span of tile columns they cover (feature 5).
// Those bounds come back from log1p-encoded floats, so they get 1e-4 of
// relative slack and 2 tiles on top (a bound read low only sends the row to
// the exact re-fill).  A wild prediction therefore never asks for more
// staging than an exact upper-bound pass would.
__global__ void mlp_slot_kernel(int tilem, int tilenB, const float* __restrict__ feat,
                                const float* __restrict__ pred, float margin, int* __restrict__ slot) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < tilem; i += gridDim.x * blockDim.x) {
        const float t = fmaxf(expm1f(fmaxf(pred[(int64_t)i * NO + 0], 0.f)), 0.f);
        const float* f = feat + (int64_t)i * NF;
        const float bound = fminf(fminf(expm1f(f[2]), expm1f(f[5])) * 1.0001f + 2.f, (float)tilenB);
        slot[i] = (int)fminf(ceilf(t * (1.f + margin) + 2.f), fmaxf(ceilf(bound), 0.f));
    }
}

// Kernel variant of each C tile-row (1: the plain per-C-tile kernels, 0: the
// row-wise windows).  The plain kernels spend one warp pass of 16x16 register
// accumulators per matched tile pair and write every C tile whole, so they
// pay off where a tile pair carries many products and C's tiles come out
// full; the row-wise windows spend their time per product.  A tile-row goes
// to the plain kernels when its products per tile pair (features 3 and 2,
// exact) reach pp_thr and, with a sizing model, its predicted C nonzeros per
// predicted C tile (the network's two outputs) reach fill_thr.
__global__ void bin_rows_kernel(int tilem, const float* __restrict__ feat, const float* __restrict__ pred,
                                float pp_thr, float fill_thr, uint8_t* __restrict__ bin) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < tilem; i += gridDim.x * blockDim.x) {
        const float* f = feat + (int64_t)i * NF;
        const float pairs = expm1f(f[2]), prod = expm1f(f[3]);
        bool plain = pairs > 0.5f && prod >= pp_thr * pairs;
        if (plain && pred) {
            const float tiles = expm1f(fmaxf(pred[(int64_t)i * NO + 0], 0.f));
            const float nnz = expm1f(fmaxf(pred[(int64_t)i * NO + 1], 0.f));
            plain = nnz >= fill_thr * fmaxf(tiles, 1.f);
        }
        bin[i] = plain ? 1 : 0;
    }
}

int mgrid(spg_handle_t h, int64_t n, int threads) {
    int64_t g = ceil_div(n, threads);
    if (g > (int64_t)h->num_sms * 8) g = (int64_t)h->num_sms * 8;
    return (int)(g < 1 ? 1 : g);
}

}  // namespace

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" int spg_mlp_num_params(void) { return NPARAM; }
extern "C" int spg_mlp_num_features(void) { return NF; }

extern "C" spg_status spg_mlp_create(spg_handle_t h, const float* host_params, const float* host_norm,
                                     spg_mlp_t* out) {
    if (!h || !out) return SPG_ERR_INVALID;
    spg_mlp_t mm = new (std::nothrow) spg_mlp_s();
    if (!mm) return spg_fail(h, SPG_ERR_OOM, "mlp: host allocation failed");
    if (cudaMalloc(&mm->d_param, 4 * NPARAM) != cudaSuccess || cudaMalloc(&mm->d_norm, 4 * NNORM) != cudaSuccess ||
        cudaMalloc(&mm->d_grad, 4 * NPARAM) != cudaSuccess || cudaMalloc(&mm->d_m, 4 * NPARAM) != cudaSuccess ||
        cudaMalloc(&mm->d_v, 4 * NPARAM) != cudaSuccess || cudaMalloc(&mm->d_loss, 16) != cudaSuccess) {
        spg_mlp_free(h, mm);
        return spg_fail(h, SPG_ERR_OOM, "mlp: device allocation failed");
    }
    std::vector<float> p(NPARAM), nrm(NNORM);
    if (host_params) {
        for (int i = 0; i < NPARAM; i++) p[i] = host_params[i];
    } else {  // He-style init from a fixed LCG (deterministic)
        uint64_t s = 0x9E3779B97F4A7C15ull;
        auto u = [&]() { s = s * 6364136223846793005ull + 1442695040888963407ull; return ((s >> 11) * (1.0 / 9007199254740992.0)) * 2.0 - 1.0; };
        for (int i = 0; i < NH * NF; i++) p[OFF_W1 + i] = (float)(u() * std::sqrt(6.0 / NF));
        for (int i = 0; i < NH * NH; i++) p[OFF_W2 + i] = (float)(u() * std::sqrt(6.0 / NH));
        for (int i = 0; i < NO * NH; i++) p[OFF_W3 + i] = (float)(u() * std::sqrt(3.0 / NH));
        for (int i = 0; i < NH; i++) { p[OFF_B1 + i] = 0.01f; p[OFF_B2 + i] = 0.01f; }
        for (int i = 0; i < NO; i++) p[OFF_B3 + i] = 0.f;
    }
    if (host_norm) {
        for (int i = 0; i < NNORM; i++) nrm[i] = host_norm[i];
    } else {
        for (int i = 0; i < NF; i++) { nrm[i] = 0.f; nrm[NF + i] = 1.f; }
        for (int i = 0; i < NO; i++) { nrm[2 * NF + i] = 0.f; nrm[2 * NF + NO + i] = 1.f; }
    }
    cudaMemcpy(mm->d_param, p.data(), 4 * NPARAM, cudaMemcpyHostToDevice);
    cudaMemcpy(mm->d_norm, nrm.data(), 4 * NNORM, cudaMemcpyHostToDevice);
    cudaMemset(mm->d_grad, 0, 4 * NPARAM);
    cudaMemset(mm->d_m, 0, 4 * NPARAM);
    cudaMemset(mm->d_v, 0, 4 * NPARAM);
    *out = mm;
    return SPG_OK;
}

extern "C" spg_status spg_mlp_free(spg_handle_t h, spg_mlp_t mm) {
    if (!mm) return SPG_ERR_INVALID;
    if (h && h->sizing == mm) h->sizing = nullptr;
    cudaFree(mm->d_param); cudaFree(mm->d_norm); cudaFree(mm->d_grad); cudaFree(mm->d_m); cudaFree(mm->d_v);
    cudaFree(mm->d_loss);
    delete mm;
    return SPG_OK;
}

extern "C" spg_status spg_mlp_get_params(spg_handle_t h, spg_mlp_t mm, float* host_params, float* host_norm) {
    if (!h || !mm) return SPG_ERR_INVALID;
    SPG_CUDA(h, cudaStreamSynchronize(h->stream));
    if (host_params) SPG_CUDA(h, cudaMemcpy(host_params, mm->d_param, 4 * NPARAM, cudaMemcpyDeviceToHost));
    if (host_norm) SPG_CUDA(h, cudaMemcpy(host_norm, mm->d_norm, 4 * NNORM, cudaMemcpyDeviceToHost));
    return SPG_OK;
}

extern "C" spg_status spg_mlp_set_norm(spg_handle_t h, spg_mlp_t mm, const float* host_norm) {
    if (!h || !mm || !host_norm) return SPG_ERR_INVALID;
    SPG_CUDA(h, cudaMemcpy(mm->d_norm, host_norm, 4 * NNORM, cudaMemcpyHostToDevice));
    return SPG_OK;
}

extern "C" spg_status spg_mlp_features(spg_handle_t h, const spg_tiles* A, const spg_tiles* B, float* d_feat) {
    if (!h || !A || !B || !d_feat) return SPG_ERR_INVALID;
    if (A->n != B->m) return spg_fail(h, SPG_ERR_INVALID, "mlp features: inner dimensions differ");
    if (A->tilem == 0) return SPG_OK;
    mlp_features_kernel<<<mgrid(h, (int64_t)A->tilem * 32, 256), 256, 0, h->stream>>>(
        A->tilem, A->m, B->tilen, A->tile_ptr, A->tile_columnidx, A->row_ptr, A->col_idx, B->tile_ptr,
        B->tile_columnidx, B->row_ptr, d_feat);
    SPG_LAUNCHED(h);
    return SPG_OK;
}

extern "C" spg_status spg_mlp_forward(spg_handle_t h, spg_mlp_t mm, const float* d_feat, int64_t n, float* d_out) {
    if (!h || !mm) return SPG_ERR_INVALID;
    if (n <= 0) return SPG_OK;
    mlp_forward_kernel<<<mgrid(h, n, 128), 128, 0, h->stream>>>(n, mm->d_param, mm->d_norm, d_feat, d_out);
    SPG_LAUNCHED(h);
    return SPG_OK;
}

// Gradient (sum over the batch, mean-squared-error scaling) into d_grad_out
// without updating: the form the tests compare with the CPU restatement.
extern "C" spg_status spg_mlp_gradient(spg_handle_t h, spg_mlp_t mm, const float* d_feat, const float* d_target,
                                       int64_t n, float* d_grad_out, float* loss_out) {
    if (!h || !mm || n <= 0) return SPG_ERR_INVALID;
    SPG_CUDA(h, cudaMemsetAsync(d_grad_out, 0, 4 * NPARAM, h->stream));
    SPG_CUDA(h, cudaMemsetAsync(mm->d_loss, 0, 4, h->stream));
    mlp_grad_kernel<<<mgrid(h, n, 128), 128, 0, h->stream>>>(n, nullptr, mm->d_param, mm->d_norm, d_feat, d_target,
                                                            d_grad_out, mm->d_loss);
    SPG_LAUNCHED(h);
    if (loss_out) {
        SPG_CUDA(h, cudaMemcpyAsync(loss_out, mm->d_loss, 4, cudaMemcpyDeviceToHost, h->stream));
        SPG_CUDA(h, cudaStreamSynchronize(h->stream));
    }
    return SPG_OK;
}

// Adam over mini-batches: `epochs` passes over the n samples in the order of
// d_perm (a permutation per epoch, epochs * n ints; NULL = in order).
extern "C" spg_status spg_mlp_train(spg_handle_t h, spg_mlp_t mm, const float* d_feat, const float* d_target,
                                    int64_t n, const int* d_perm, int epochs, int batch, float lr,
                                    float* last_epoch_loss) {
    if (!h || !mm || n <= 0 || epochs <= 0 || batch <= 0) return SPG_ERR_INVALID;
    const float b1 = 0.9f, b2 = 0.999f;
    for (int ep = 0; ep < epochs; ep++) {
        SPG_CUDA(h, cudaMemsetAsync(mm->d_loss, 0, 4, h->stream));
        const int* perm = d_perm ? d_perm + (int64_t)ep * n : nullptr;
        int nbatch = 0;
        for (int64_t s0 = 0; s0 < n; s0 += batch) {
            const int64_t nb = (s0 + batch <= n) ? batch : n - s0;
            mlp_grad_kernel<<<mgrid(h, nb, 128), 128, 0, h->stream>>>(nb, perm ? perm + s0 : nullptr, mm->d_param,
                                                                     mm->d_norm,
                                                                     perm ? d_feat : d_feat + s0 * NF,
                                                                     perm ? d_target : d_target + s0 * NO,
                                                                     mm->d_grad, mm->d_loss);
            SPG_LAUNCHED(h);
            mm->step++;
            const float c1 = 1.f - std::pow(b1, (float)mm->step), c2 = 1.f - std::pow(b2, (float)mm->step);
            mlp_adam_kernel<<<(NPARAM + 255) / 256, 256, 0, h->stream>>>(mm->d_param, mm->d_grad, mm->d_m, mm->d_v,
                                                                          lr, b1, b2, c1, c2);
            SPG_LAUNCHED(h);
            nbatch++;
        }
        if (last_epoch_loss && ep == epochs - 1) {
            float l = 0.f;
            SPG_CUDA(h, cudaMemcpyAsync(&l, mm->d_loss, 4, cudaMemcpyDeviceToHost, h->stream));
            SPG_CUDA(h, cudaStreamSynchronize(h->stream));
            *last_epoch_loss = l / (float)nbatch;
        }
    }
    return SPG_OK;
}

extern "C" spg_status spg_set_sizing_model(spg_handle_t h, spg_mlp_t mm, float margin) {
    if (!h) return SPG_ERR_INVALID;
    h->sizing = mm;
    h->sizing_margin = margin;
    return SPG_OK;
}

// Predicted capacities for C of A*B (tiles, nonzeros) from the sizing model.
spg_status mlp_predict_rows(spg_handle_t h, const spg_tiles* A, const spg_tiles* B, int* slot_sz, uint8_t* rowbin) {
    spg_mlp_t mm = h->sizing;
    const int tilem = A->tilem;
    ScratchList sc(h);
    float *feat = nullptr, *pred = nullptr;
    SPG_TRY(sc.alloc(&feat, (size_t)tilem * NF + 1));
    SPG_TRY(spg_mlp_features(h, A, B, feat));
    if (mm) {
        SPG_TRY(sc.alloc(&pred, (size_t)tilem * NO + 1));
        SPG_TRY(spg_mlp_forward(h, mm, feat, tilem, pred));
    }
    if (tilem > 0 && slot_sz && mm) {
        mlp_slot_kernel<<<mgrid(h, tilem, 256), 256, 0, h->stream>>>(tilem, B->tilen, feat, pred, h->sizing_margin,
                                                                   slot_sz);
        SPG_LAUNCHED(h);
    }
    if (tilem > 0 && rowbin) {
        bin_rows_kernel<<<mgrid(h, tilem, 256), 256, 0, h->stream>>>(tilem, feat, pred, h->bin_pp_thr,
                                                                   h->bin_fill_thr, rowbin);
        SPG_LAUNCHED(h);
    }
    return SPG_OK;
}
