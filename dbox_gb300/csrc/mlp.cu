// Training and batch inference of the learned warm-start MLP (see mlp.cuh), and its C ABI.
//
// One warp owns a 16-sample tile: the forward pass keeps the tile's pre-activations and
// activations in shared memory (bf16), the backward pass reuses them, and the weight
// gradients of the tile are added into one FP32 gradient vector with atomics.  Adam then
// updates the FP32 master parameters and refreshes the BF16 copies the tensor cores read.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>
#include <stdio.h>
#include <math.h>
#include <vector>
#include <algorithm>
#include "mlp.cuh"
#include "../../include/dbox_gpu.h"

static_assert(dg::kNParams == DBOX_MLP_PARAMS && dg::kSampleFloats == DBOX_MLP_SAMPLE, "header sizes");

extern "C" int dbox_set_error(int code, const char* msg);

namespace dg {

constexpr int kTrainWarps = 4;
// per warp: X 16x32, pre1/h1/pre2/h2/d2/d1 16x128 each, dY 16x16 (bf16)
constexpr int kTileX = 16 * kFeat, kTileH = 16 * kHid, kTileY = 16 * 16;
constexpr int kWarpTrainElems = kTileX + 6 * kTileH + kTileY;

__device__ __forceinline__ float bf(const __nv_bfloat16* s, int i) { return __bfloat162float(s[i]); }

// A fragment of the transpose of a row-major [K rows x M cols] tile: A[m][k] = s[k][m]
__device__ __forceinline__ void load_a_trans(uint32_t a[4], const __nv_bfloat16* s, int ld, int m0, int k0, int lane) {
    const int g = lane >> 2, t = lane & 3;
    auto e = [&](int m, int k) { return s[(k0 + k) * ld + m0 + m]; };
    a[0] = pack_raw(e(g, 2 * t), e(g, 2 * t + 1));
    a[1] = pack_raw(e(g + 8, 2 * t), e(g + 8, 2 * t + 1));
    a[2] = pack_raw(e(g, 2 * t + 8), e(g, 2 * t + 9));
    a[3] = pack_raw(e(g + 8, 2 * t + 8), e(g + 8, 2 * t + 9));
}
// B fragment of a row-major [K x N] tile: B[k][n] = s[k][n]
__device__ __forceinline__ void load_b_rowmajor(uint32_t b[2], const __nv_bfloat16* s, int ld, int k0, int n0, int lane) {
    const int g = lane >> 2, t = lane & 3;
    b[0] = pack_raw(s[(k0 + 2 * t) * ld + n0 + g], s[(k0 + 2 * t + 1) * ld + n0 + g]);
    b[1] = pack_raw(s[(k0 + 2 * t + 8) * ld + n0 + g], s[(k0 + 2 * t + 9) * ld + n0 + g]);
}

// column sums of a C fragment over its 16 rows, added into g[col0 + 2t .. +1] by the lanes of row group 0
__device__ __forceinline__ void add_colsum(float* g, int col0, const float c[4], int lane) {
    float s0 = c[0] + c[2], s1 = c[1] + c[3];
#pragma unroll
    for (int o = 4; o < 32; o <<= 1) {
        s0 += __shfl_xor_sync(0xffffffffu, s0, o);
        s1 += __shfl_xor_sync(0xffffffffu, s1, o);
    }
    if ((lane >> 2) == 0) {
        atomicAdd(g + col0 + 2 * (lane & 3), s0);
        atomicAdd(g + col0 + 2 * (lane & 3) + 1, s1);
    }
}

// Forward + backward of MSE(MLP(x), t) / (n * 4) over the samples idx[0 .. n) of `rows`
// (kSampleFloats per sample: features, then targets), normalised with the model's
// statistics; gradients added into grad (kNParams), the sum of squared errors into *loss.
__global__ void __launch_bounds__(kTrainWarps * 32) k_mlp_train(MlpDev m, float* grad, const float* rows,
                                                                const int* idx, int n, float* loss) {
    extern __shared__ __nv_bfloat16 sm_mlp[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int tile = blockIdx.x * kTrainWarps + wib;
    const int r0 = tile * 16;
    if (r0 >= n) return;
    __nv_bfloat16* X = sm_mlp + wib * kWarpTrainElems;
    __nv_bfloat16* P1 = X + kTileX;
    __nv_bfloat16* H1 = P1 + kTileH;
    __nv_bfloat16* P2 = H1 + kTileH;
    __nv_bfloat16* H2 = P2 + kTileH;
    __nv_bfloat16* D2 = H2 + kTileH;
    __nv_bfloat16* D1 = D2 + kTileH;
    __nv_bfloat16* DY = D1 + kTileH;
    const int g = lane >> 2, t = lane & 3;
    const float* b1 = m.p + kW1 + kW2 + kW3;
    const float* b2 = b1 + kHid;
    const float* b3 = b2 + kHid;
    float* gw1 = grad;
    float* gw2 = gw1 + kW1;
    float* gw3 = gw2 + kW2;
    float* gb1 = gw3 + kW3;
    float* gb2 = gb1 + kHid;
    float* gb3 = gb2 + kHid;
    const float inv = 1.0f / (4.0f * (float)n);
    // inputs
    for (int e = lane; e < 16 * kFeat; e += 32) {
        int r = e / kFeat, f = e % kFeat;
        float v = 0.0f;
        if (r0 + r < n) v = (rows[(size_t)idx[r0 + r] * kSampleFloats + f] - m.fmean[f]) / m.fstd[f];
        X[e] = __float2bfloat16_rn(v);
    }
    __syncwarp();
    uint32_t a[4], b[2];
    // layer 1
    for (int nb = 0; nb < kHid / 8; ++nb) {
        float c[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        for (int kb = 0; kb < kFeat / 16; ++kb) {
            load_a_rowmajor(a, X, kFeat, kb * 16, lane);
            load_b_trans(b, m.wt1, kFeat, kb * 16, nb * 8, lane);
            mma_bf16(c, a, b);
        }
        int col = nb * 8 + 2 * t;
        float p00 = c[0] + b1[col], p01 = c[1] + b1[col + 1], p10 = c[2] + b1[col], p11 = c[3] + b1[col + 1];
        *reinterpret_cast<uint32_t*>(P1 + g * kHid + col) = pack_bf16x2(p00, p01);
        *reinterpret_cast<uint32_t*>(P1 + (g + 8) * kHid + col) = pack_bf16x2(p10, p11);
        *reinterpret_cast<uint32_t*>(H1 + g * kHid + col) = pack_bf16x2(gelu_f(p00), gelu_f(p01));
        *reinterpret_cast<uint32_t*>(H1 + (g + 8) * kHid + col) = pack_bf16x2(gelu_f(p10), gelu_f(p11));
    }
    __syncwarp();
    // layer 2
    for (int nb = 0; nb < kHid / 8; ++nb) {
        float c[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        for (int kb = 0; kb < kHid / 16; ++kb) {
            load_a_rowmajor(a, H1, kHid, kb * 16, lane);
            load_b_trans(b, m.wt2, kHid, kb * 16, nb * 8, lane);
            mma_bf16(c, a, b);
        }
        int col = nb * 8 + 2 * t;
        float p00 = c[0] + b2[col], p01 = c[1] + b2[col + 1], p10 = c[2] + b2[col], p11 = c[3] + b2[col + 1];
        *reinterpret_cast<uint32_t*>(P2 + g * kHid + col) = pack_bf16x2(p00, p01);
        *reinterpret_cast<uint32_t*>(P2 + (g + 8) * kHid + col) = pack_bf16x2(p10, p11);
        *reinterpret_cast<uint32_t*>(H2 + g * kHid + col) = pack_bf16x2(gelu_f(p00), gelu_f(p01));
        *reinterpret_cast<uint32_t*>(H2 + (g + 8) * kHid + col) = pack_bf16x2(gelu_f(p10), gelu_f(p11));
    }
    __syncwarp();
    // layer 3 and the loss gradient dY = 2 (y - t) / (4 n)
    {
        float c[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        for (int kb = 0; kb < kHid / 16; ++kb) {
            load_a_rowmajor(a, H2, kHid, kb * 16, lane);
            load_b_trans(b, m.wt3, kHid, kb * 16, 0, lane);
            mma_bf16(c, a, b);
        }
        float d[4], lsum = 0.0f;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            int row = g + (q >> 1) * 8, col = 2 * t + (q & 1);
            float y = c[q] + b3[col];
            float dv = 0.0f;
            if (col < kOut && r0 + row < n) {
                float tv = (rows[(size_t)idx[r0 + row] * kSampleFloats + kFeat + col] - m.tmean[col]) / m.tstd[col];
                float diff = y - tv;
                lsum += diff * diff;
                dv = 2.0f * diff * inv;
            }
            d[q] = dv;
        }
        for (int o = 16; o > 0; o >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
        if (lane == 0) atomicAdd(loss, lsum);
        for (int e = lane; e < kTileY; e += 32) DY[e] = __float2bfloat16_rn(0.0f);
        __syncwarp();
        DY[g * 16 + 2 * t] = __float2bfloat16_rn(d[0]);
        DY[g * 16 + 2 * t + 1] = __float2bfloat16_rn(d[1]);
        DY[(g + 8) * 16 + 2 * t] = __float2bfloat16_rn(d[2]);
        DY[(g + 8) * 16 + 2 * t + 1] = __float2bfloat16_rn(d[3]);
        add_colsum(gb3, 0, d, lane);
    }
    __syncwarp();
    // dW3 = H2^T dY  (128 x 8)
    for (int mb = 0; mb < kHid / 16; ++mb) {
        float c[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        load_a_trans(a, H2, kHid, mb * 16, 0, lane);
        load_b_rowmajor(b, DY, 16, 0, 0, lane);
        mma_bf16(c, a, b);
        int row = mb * 16 + g, col = 2 * t;
        atomicAdd(gw3 + row * kOutPad + col, c[0]);
        atomicAdd(gw3 + row * kOutPad + col + 1, c[1]);
        atomicAdd(gw3 + (row + 8) * kOutPad + col, c[2]);
        atomicAdd(gw3 + (row + 8) * kOutPad + col + 1, c[3]);
    }
    // dH2 = (dY W3^T) * gelu'(P2)   (K = 8 outputs, padded to 16 with zeros)
    for (int nb = 0; nb < kHid / 8; ++nb) {
        float c[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        load_a_rowmajor(a, DY, 16, 0, lane);
        load_b_trans(b, m.wb3, kOutPad, 0, nb * 8, lane);
        b[1] = 0u;                                   // k = 8..15 are padding
        mma_bf16(c, a, b);
        int col = nb * 8 + 2 * t;
        c[0] *= gelu_grad(bf(P2, g * kHid + col));
        c[1] *= gelu_grad(bf(P2, g * kHid + col + 1));
        c[2] *= gelu_grad(bf(P2, (g + 8) * kHid + col));
        c[3] *= gelu_grad(bf(P2, (g + 8) * kHid + col + 1));
        *reinterpret_cast<uint32_t*>(D2 + g * kHid + col) = pack_bf16x2(c[0], c[1]);
        *reinterpret_cast<uint32_t*>(D2 + (g + 8) * kHid + col) = pack_bf16x2(c[2], c[3]);
        add_colsum(gb2, nb * 8, c, lane);
    }
    __syncwarp();
    // dW2 = H1^T dH2  (128 x 128)
    for (int mb = 0; mb < kHid / 16; ++mb) {
        load_a_trans(a, H1, kHid, mb * 16, 0, lane);
        for (int nb = 0; nb < kHid / 8; ++nb) {
            float c[4] = {0.0f, 0.0f, 0.0f, 0.0f};
            load_b_rowmajor(b, D2, kHid, 0, nb * 8, lane);
            mma_bf16(c, a, b);
            int row = mb * 16 + g, col = nb * 8 + 2 * t;
            atomicAdd(gw2 + row * kHid + col, c[0]);
            atomicAdd(gw2 + row * kHid + col + 1, c[1]);
            atomicAdd(gw2 + (row + 8) * kHid + col, c[2]);
            atomicAdd(gw2 + (row + 8) * kHid + col + 1, c[3]);
        }
    }
    // dH1 = (dH2 W2^T) * gelu'(P1)
    for (int nb = 0; nb < kHid / 8; ++nb) {
        float c[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        for (int kb = 0; kb < kHid / 16; ++kb) {
            load_a_rowmajor(a, D2, kHid, kb * 16, lane);
            load_b_trans(b, m.wb2, kHid, kb * 16, nb * 8, lane);
            mma_bf16(c, a, b);
        }
        int col = nb * 8 + 2 * t;
        c[0] *= gelu_grad(bf(P1, g * kHid + col));
        c[1] *= gelu_grad(bf(P1, g * kHid + col + 1));
        c[2] *= gelu_grad(bf(P1, (g + 8) * kHid + col));
        c[3] *= gelu_grad(bf(P1, (g + 8) * kHid + col + 1));
        *reinterpret_cast<uint32_t*>(D1 + g * kHid + col) = pack_bf16x2(c[0], c[1]);
        *reinterpret_cast<uint32_t*>(D1 + (g + 8) * kHid + col) = pack_bf16x2(c[2], c[3]);
        add_colsum(gb1, nb * 8, c, lane);
    }
    __syncwarp();
    // dW1 = X^T dH1  (32 x 128)
    for (int mb = 0; mb < kFeat / 16; ++mb) {
        load_a_trans(a, X, kFeat, mb * 16, 0, lane);
        for (int nb = 0; nb < kHid / 8; ++nb) {
            float c[4] = {0.0f, 0.0f, 0.0f, 0.0f};
            load_b_rowmajor(b, D1, kHid, 0, nb * 8, lane);
            mma_bf16(c, a, b);
            int row = mb * 16 + g, col = nb * 8 + 2 * t;
            atomicAdd(gw1 + row * kHid + col, c[0]);
            atomicAdd(gw1 + row * kHid + col + 1, c[1]);
            atomicAdd(gw1 + (row + 8) * kHid + col, c[2]);
            atomicAdd(gw1 + (row + 8) * kHid + col + 1, c[3]);
        }
    }
}

// BF16 copies of the FP32 parameters: transposed (forward) and row-major (backward)
__global__ void k_mlp_refresh(const float* p, __nv_bfloat16* wt1, __nv_bfloat16* wt2, __nv_bfloat16* wt3,
                              __nv_bfloat16* wb1, __nv_bfloat16* wb2, __nv_bfloat16* wb3) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < kW1 + kW2 + kW3; i += gridDim.x * blockDim.x) {
        if (i < kW1) {
            int r = i / kHid, c = i % kHid;                 // w1[r][c], r < 32
            __nv_bfloat16 v = __float2bfloat16_rn(p[i]);
            wb1[i] = v;
            wt1[c * kFeat + r] = v;
        } else if (i < kW1 + kW2) {
            int j = i - kW1, r = j / kHid, c = j % kHid;
            __nv_bfloat16 v = __float2bfloat16_rn(p[i]);
            wb2[j] = v;
            wt2[c * kHid + r] = v;
        } else {
            int j = i - kW1 - kW2, r = j / kOutPad, c = j % kOutPad;
            __nv_bfloat16 v = __float2bfloat16_rn(p[i]);
            wb3[j] = v;
            wt3[c * kHid + r] = v;
        }
    }
}

// Adam (beta1 0.9, beta2 0.999, eps 1e-8) on the flat parameter vector; clears grad
__global__ void k_mlp_adam(float* p, float* grad, float* mom, float* vel, int n, float lr, float bc1, float bc2) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float gi = grad[i];
        grad[i] = 0.0f;
        bool pad = false;
        if (i >= kW1 + kW2 && i < kW1 + kW2 + kW3) pad = ((i - kW1 - kW2) % kOutPad) >= kOut;
        if (i >= kW1 + kW2 + kW3 + 2 * kHid) pad = (i - (kW1 + kW2 + kW3 + 2 * kHid)) >= kOut;
        if (pad) continue;
        float mi = 0.9f * mom[i] + 0.1f * gi;
        float vi = 0.999f * vel[i] + 0.001f * gi * gi;
        mom[i] = mi;
        vel[i] = vi;
        p[i] -= lr * (mi / bc1) / (sqrtf(vi / bc2) + 1e-8f);
    }
}

// batch inference: out[r][0..3] = MLP(feats[r]) in target units
__global__ void __launch_bounds__(128) k_mlp_forward(MlpDev m, const float* feats, int n, float* out) {
    __shared__ __align__(16) __nv_bfloat16 sx[4][16 * kFeat];
    __shared__ __align__(16) __nv_bfloat16 sh[4][2][16 * kHid];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int r0 = (blockIdx.x * 4 + wib) * 16;
    if (r0 >= n) return;
    for (int e = lane; e < 16 * kFeat; e += 32) {
        int r = e / kFeat, f = e % kFeat;
        float v = r0 + r < n ? (feats[(size_t)(r0 + r) * kFeat + f] - m.fmean[f]) / m.fstd[f] : 0.0f;
        sx[wib][e] = __float2bfloat16_rn(v);
    }
    __syncwarp();
    float y[4];
    mlp_infer16(m, sx[wib], sh[wib][0], sh[wib][1], y, lane);
    const int g = lane >> 2, t = lane & 3;
    if (t < 2) {
        int c0 = 2 * t;
        if (r0 + g < n) {
            out[(size_t)(r0 + g) * kOut + c0] = y[0] * m.tstd[c0] + m.tmean[c0];
            out[(size_t)(r0 + g) * kOut + c0 + 1] = y[1] * m.tstd[c0 + 1] + m.tmean[c0 + 1];
        }
        if (r0 + g + 8 < n) {
            out[(size_t)(r0 + g + 8) * kOut + c0] = y[2] * m.tstd[c0] + m.tmean[c0];
            out[(size_t)(r0 + g + 8) * kOut + c0 + 1] = y[3] * m.tstd[c0 + 1] + m.tmean[c0 + 1];
        }
    }
}

}  // namespace dg

// ------------------------------------------------------------ host side
struct dbox_mlp {
    int device = 0;
    float* p = nullptr;           // kNParams
    float* grad = nullptr;
    float* mom = nullptr;
    float* vel = nullptr;
    float* norm = nullptr;        // fmean 32, fstd 32, tmean 4, tstd 4
    __nv_bfloat16* wbuf = nullptr;  // wt1 wt2 wt3 wb1 wb2 wb3
    float* loss = nullptr;
    int step = 0;
};

namespace {

const int kNorm = 2 * dg::kFeat + 2 * dg::kOut;

dg::MlpDev mlp_dev(const dbox_mlp* m) {
    dg::MlpDev d;
    d.p = m->p;
    d.wt1 = m->wbuf;
    d.wt2 = d.wt1 + dg::kW1;
    d.wt3 = d.wt2 + dg::kW2;
    d.wb1 = d.wt3 + dg::kW3;
    d.wb2 = d.wb1 + dg::kW1;
    d.wb3 = d.wb2 + dg::kW2;
    d.fmean = m->norm;
    d.fstd = m->norm + dg::kFeat;
    d.tmean = m->norm + 2 * dg::kFeat;
    d.tstd = m->norm + 2 * dg::kFeat + dg::kOut;
    return d;
}

int cuerr(cudaError_t e, const char* what) {
    if (e == cudaSuccess) return DBOX_OK;
    char buf[256];
    snprintf(buf, sizeof(buf), "%s: %s", what, cudaGetErrorString(e));
    return dbox_set_error(DBOX_ERR_CUDA, buf);
}
#define MCU(call) do { int r_ = cuerr((call), #call); if (r_) return r_; } while (0)

int refresh(dbox_mlp* m) {
    dg::MlpDev d = mlp_dev(m);
    dg::k_mlp_refresh<<<64, 256>>>(m->p, const_cast<__nv_bfloat16*>(d.wt1), const_cast<__nv_bfloat16*>(d.wt2),
                                   const_cast<__nv_bfloat16*>(d.wt3), const_cast<__nv_bfloat16*>(d.wb1),
                                   const_cast<__nv_bfloat16*>(d.wb2), const_cast<__nv_bfloat16*>(d.wb3));
    return cuerr(cudaGetLastError(), "k_mlp_refresh");
}

size_t train_smem() { return sizeof(__nv_bfloat16) * dg::kTrainWarps * dg::kWarpTrainElems; }

// gradient of one batch (rows idx[0..n)) added into m->grad; loss sum into m->loss
int run_batch(dbox_mlp* m, const float* rows, const int* idx, int n) {
    if (n <= 0) return DBOX_OK;
    int tiles = (n + 15) / 16;
    int blocks = (tiles + dg::kTrainWarps - 1) / dg::kTrainWarps;
    dg::k_mlp_train<<<blocks, dg::kTrainWarps * 32, train_smem()>>>(mlp_dev(m), m->grad, rows, idx, n, m->loss);
    return cuerr(cudaGetLastError(), "k_mlp_train");
}

// n host samples (features n x 32, targets n x 4) interleaved into one device buffer
int upload_rows(int n, const float* feats, const float* targets, float** out) {
    std::vector<float> h((size_t)n * dg::kSampleFloats);
    for (int i = 0; i < n; ++i) {
        memcpy(&h[(size_t)i * dg::kSampleFloats], feats + (size_t)i * dg::kFeat, sizeof(float) * dg::kFeat);
        memcpy(&h[(size_t)i * dg::kSampleFloats + dg::kFeat], targets + (size_t)i * dg::kOut, sizeof(float) * dg::kOut);
    }
    int r = cuerr(cudaMalloc(out, sizeof(float) * h.size()), "upload samples");
    if (r) return r;
    return cuerr(cudaMemcpy(*out, h.data(), sizeof(float) * h.size(), cudaMemcpyHostToDevice), "upload samples");
}

}  // namespace

const dg::MlpDev* dbox_mlp_device_view(const dbox_mlp* m, dg::MlpDev* out) {
    *out = mlp_dev(m);
    return out;
}

extern "C" {

int32_t dbox_mlp_create(dbox_mlp** out) {
    if (!out) return dbox_set_error(DBOX_ERR_INVALID, "dbox_mlp_create: null out");
    dbox_mlp* m = new dbox_mlp();
    cudaGetDevice(&m->device);
    bool ok = cudaMalloc(&m->p, sizeof(float) * dg::kNParams) == cudaSuccess &&
              cudaMalloc(&m->grad, sizeof(float) * dg::kNParams) == cudaSuccess &&
              cudaMalloc(&m->mom, sizeof(float) * dg::kNParams) == cudaSuccess &&
              cudaMalloc(&m->vel, sizeof(float) * dg::kNParams) == cudaSuccess &&
              cudaMalloc(&m->norm, sizeof(float) * kNorm) == cudaSuccess &&
              cudaMalloc(&m->wbuf, sizeof(__nv_bfloat16) * 2 * (dg::kW1 + dg::kW2 + dg::kW3)) == cudaSuccess &&
              cudaMalloc(&m->loss, sizeof(float)) == cudaSuccess;
    if (!ok) {
        dbox_mlp_destroy(m);
        return dbox_set_error(DBOX_ERR_CUDA, "dbox_mlp_create: device allocation failed");
    }
    cudaMemset(m->p, 0, sizeof(float) * dg::kNParams);
    cudaMemset(m->grad, 0, sizeof(float) * dg::kNParams);
    cudaMemset(m->mom, 0, sizeof(float) * dg::kNParams);
    cudaMemset(m->vel, 0, sizeof(float) * dg::kNParams);
    std::vector<float> norm(kNorm, 0.0f);
    for (int i = 0; i < dg::kFeat; ++i) norm[dg::kFeat + i] = 1.0f;
    for (int i = 0; i < dg::kOut; ++i) norm[2 * dg::kFeat + dg::kOut + i] = 1.0f;
    cudaMemcpy(m->norm, norm.data(), sizeof(float) * kNorm, cudaMemcpyHostToDevice);
    cudaFuncSetAttribute(dg::k_mlp_train, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)train_smem());
    int r = refresh(m);
    if (r) { dbox_mlp_destroy(m); return r; }
    *out = m;
    return DBOX_OK;
}

int32_t dbox_mlp_destroy(dbox_mlp* m) {
    if (!m) return DBOX_OK;
    cudaFree(m->p); cudaFree(m->grad); cudaFree(m->mom); cudaFree(m->vel);
    cudaFree(m->norm); cudaFree(m->wbuf); cudaFree(m->loss);
    delete m;
    return DBOX_OK;
}

int32_t dbox_mlp_set_params(dbox_mlp* m, const float* params, const float* norm) {
    if (!m) return dbox_set_error(DBOX_ERR_INVALID, "dbox_mlp_set_params: null model");
    if (params) MCU(cudaMemcpy(m->p, params, sizeof(float) * dg::kNParams, cudaMemcpyHostToDevice));
    if (norm) MCU(cudaMemcpy(m->norm, norm, sizeof(float) * kNorm, cudaMemcpyHostToDevice));
    m->step = 0;
    MCU(cudaMemset(m->mom, 0, sizeof(float) * dg::kNParams));
    MCU(cudaMemset(m->vel, 0, sizeof(float) * dg::kNParams));
    int r = refresh(m);
    if (r) return r;
    return cuerr(cudaDeviceSynchronize(), "dbox_mlp_set_params");
}

int32_t dbox_mlp_get_params(dbox_mlp* m, float* params, float* norm) {
    if (!m) return dbox_set_error(DBOX_ERR_INVALID, "dbox_mlp_get_params: null model");
    if (params) MCU(cudaMemcpy(params, m->p, sizeof(float) * dg::kNParams, cudaMemcpyDeviceToHost));
    if (norm) MCU(cudaMemcpy(norm, m->norm, sizeof(float) * kNorm, cudaMemcpyDeviceToHost));
    return DBOX_OK;
}

int32_t dbox_mlp_init(dbox_mlp* m, uint64_t seed) {
    if (!m) return dbox_set_error(DBOX_ERR_INVALID, "dbox_mlp_init: null model");
    // uniform fan-in scaling (+-sqrt(3 / fan_in)), zero biases, from a SplitMix64 stream
    std::vector<float> p(dg::kNParams, 0.0f);
    uint64_t s = seed;
    auto next = [&]() {
        s += 0x9E3779B97F4A7C15ull;
        uint64_t z = s;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        return (double)(z >> 11) * (1.0 / 9007199254740992.0);
    };
    auto fill = [&](int off, int rows, int cols, int used_cols, int fan_in) {
        double a = sqrt(3.0 / fan_in);
        for (int r = 0; r < rows; ++r)
            for (int c = 0; c < cols; ++c) p[off + r * cols + c] = c < used_cols ? (float)((2.0 * next() - 1.0) * a) : 0.0f;
    };
    fill(0, dg::kFeat, dg::kHid, dg::kHid, dg::kFeat);
    fill(dg::kW1, dg::kHid, dg::kHid, dg::kHid, dg::kHid);
    fill(dg::kW1 + dg::kW2, dg::kHid, dg::kOutPad, dg::kOut, dg::kHid);
    return dbox_mlp_set_params(m, p.data(), nullptr);
}

// Feature / target normalisation from n host samples (mean and standard deviation per column).
int32_t dbox_mlp_fit_normalization(dbox_mlp* m, int32_t n, const float* feats, const float* targets) {
    if (!m || n <= 0 || !feats || !targets) return dbox_set_error(DBOX_ERR_INVALID, "dbox_mlp_fit_normalization: bad arguments");
    std::vector<double> s(2 * dg::kFeat + 2 * dg::kOut, 0.0);
    for (int i = 0; i < n; ++i) {
        for (int f = 0; f < dg::kFeat; ++f) { double v = feats[(size_t)i * dg::kFeat + f]; s[f] += v; s[dg::kFeat + f] += v * v; }
        for (int o = 0; o < dg::kOut; ++o) {
            double v = targets[(size_t)i * dg::kOut + o];
            s[2 * dg::kFeat + o] += v;
            s[2 * dg::kFeat + dg::kOut + o] += v * v;
        }
    }
    std::vector<float> norm(kNorm);
    for (int f = 0; f < dg::kFeat; ++f) {
        double mu = s[f] / n, var = s[dg::kFeat + f] / n - mu * mu;
        norm[f] = (float)mu;
        norm[dg::kFeat + f] = (float)(var > 1e-12 ? sqrt(var) : 1.0);
    }
    for (int o = 0; o < dg::kOut; ++o) {
        double mu = s[2 * dg::kFeat + o] / n, var = s[2 * dg::kFeat + dg::kOut + o] / n - mu * mu;
        norm[2 * dg::kFeat + o] = (float)mu;
        norm[2 * dg::kFeat + dg::kOut + o] = (float)(var > 1e-12 ? sqrt(var) : 1.0);
    }
    return cuerr(cudaMemcpy(m->norm, norm.data(), sizeof(float) * kNorm, cudaMemcpyHostToDevice), "fit_normalization");
}

// Mean-squared-error gradient of one batch of n host samples (no update): grad[kNParams], *loss.
int32_t dbox_mlp_gradient(dbox_mlp* m, int32_t n, const float* feats, const float* targets, float* grad, float* loss) {
    if (!m || n <= 0 || !feats || !targets) return dbox_set_error(DBOX_ERR_INVALID, "dbox_mlp_gradient: bad arguments");
    float* drows = nullptr;
    int* di = nullptr;
    int r = upload_rows(n, feats, targets, &drows);
    if (r) return r;
    MCU(cudaMalloc(&di, sizeof(int) * (size_t)n));
    std::vector<int> idx(n);
    for (int i = 0; i < n; ++i) idx[i] = i;
    cudaMemcpy(di, idx.data(), sizeof(int) * (size_t)n, cudaMemcpyHostToDevice);
    cudaMemset(m->grad, 0, sizeof(float) * dg::kNParams);
    cudaMemset(m->loss, 0, sizeof(float));
    r = run_batch(m, drows, di, n);
    if (!r) r = cuerr(cudaDeviceSynchronize(), "dbox_mlp_gradient");
    if (!r && grad) r = cuerr(cudaMemcpy(grad, m->grad, sizeof(float) * dg::kNParams, cudaMemcpyDeviceToHost), "grad");
    float l = 0.0f;
    if (!r) r = cuerr(cudaMemcpy(&l, m->loss, sizeof(float), cudaMemcpyDeviceToHost), "loss");
    if (loss) *loss = l / (4.0f * (float)n);
    cudaMemset(m->grad, 0, sizeof(float) * dg::kNParams);
    cudaFree(drows); cudaFree(di);
    return r;
}

// Adam training on n device-resident samples (kSampleFloats each: 32 features, 4 targets):
// `epochs` passes in shuffled batches; epoch_loss[e] gets the mean squared error of epoch e
// in normalised units.
int32_t dbox_mlp_train_device(dbox_mlp* m, int32_t n, const float* rows, int32_t epochs, int32_t batch, float lr,
                              uint64_t seed, float* epoch_loss) {
    if (!m || n <= 0 || !rows || epochs <= 0 || batch <= 0)
        return dbox_set_error(DBOX_ERR_INVALID, "dbox_mlp_train_device: bad arguments");
    int* di = nullptr;
    MCU(cudaMalloc(&di, sizeof(int) * (size_t)n));
    std::vector<int> idx(n);
    for (int i = 0; i < n; ++i) idx[i] = i;
    uint64_t s = seed ^ 0x2545F4914F6CDD1Dull;
    int r = DBOX_OK;
    for (int e = 0; e < epochs && !r; ++e) {
        for (int i = n - 1; i > 0; --i) {          // Fisher-Yates with an xorshift64 stream
            s ^= s << 13; s ^= s >> 7; s ^= s << 17;
            int j = (int)(s % (uint64_t)(i + 1));
            std::swap(idx[i], idx[j]);
        }
        cudaMemcpy(di, idx.data(), sizeof(int) * (size_t)n, cudaMemcpyHostToDevice);
        cudaMemset(m->loss, 0, sizeof(float));
        for (int b0 = 0; b0 < n && !r; b0 += batch) {
            int nb = std::min(batch, n - b0);
            r = run_batch(m, rows, di + b0, nb);
            if (r) break;
            ++m->step;
            float bc1 = 1.0f - powf(0.9f, (float)m->step), bc2 = 1.0f - powf(0.999f, (float)m->step);
            dg::k_mlp_adam<<<64, 256>>>(m->p, m->grad, m->mom, m->vel, dg::kNParams, lr, bc1, bc2);
            r = cuerr(cudaGetLastError(), "k_mlp_adam");
            if (!r) r = refresh(m);
        }
        if (!r) r = cuerr(cudaDeviceSynchronize(), "dbox_mlp_train_device");
        if (!r && epoch_loss) {
            float l = 0.0f;
            cudaMemcpy(&l, m->loss, sizeof(float), cudaMemcpyDeviceToHost);
            // per-batch losses are means over (nb * 4); the sum below is over all n * 4 entries
            epoch_loss[e] = l / (4.0f * (float)n);
        }
    }
    cudaFree(di);
    return r;
}

// Same, from host arrays.
int32_t dbox_mlp_train(dbox_mlp* m, int32_t n, const float* feats, const float* targets, int32_t epochs,
                       int32_t batch, float lr, uint64_t seed, float* epoch_loss) {
    if (!m || n <= 0 || !feats || !targets) return dbox_set_error(DBOX_ERR_INVALID, "dbox_mlp_train: bad arguments");
    float* drows = nullptr;
    int r = upload_rows(n, feats, targets, &drows);
    if (r) return r;
    r = dbox_mlp_train_device(m, n, drows, epochs, batch, lr, seed, epoch_loss);
    cudaFree(drows);
    return r;
}

// Batch inference: out[n x 4] = predicted impulses for n host feature rows.
int32_t dbox_mlp_forward(dbox_mlp* m, int32_t n, const float* feats, float* out) {
    if (!m || n <= 0 || !feats || !out) return dbox_set_error(DBOX_ERR_INVALID, "dbox_mlp_forward: bad arguments");
    float *df = nullptr, *dout = nullptr;
    MCU(cudaMalloc(&df, sizeof(float) * (size_t)n * dg::kFeat));
    MCU(cudaMalloc(&dout, sizeof(float) * (size_t)n * dg::kOut));
    cudaMemcpy(df, feats, sizeof(float) * (size_t)n * dg::kFeat, cudaMemcpyHostToDevice);
    int blocks = (n + 63) / 64;
    dg::k_mlp_forward<<<blocks, 128>>>(mlp_dev(m), df, n, dout);
    int r = cuerr(cudaGetLastError(), "k_mlp_forward");
    if (!r) r = cuerr(cudaMemcpy(out, dout, sizeof(float) * (size_t)n * dg::kOut, cudaMemcpyDeviceToHost), "forward out");
    cudaFree(df);
    cudaFree(dout);
    return r;
}

}  // extern "C"
