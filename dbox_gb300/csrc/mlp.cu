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
#include "tc.cuh"
#include "../../include/dbox_gpu.h"

static_assert(dg::kNParams == DBOX_MLP_PARAMS && dg::kSampleFloats == DBOX_MLP_SAMPLE, "header sizes");

extern "C" int dbox_set_error(int code, const char* msg);

namespace dg {

// ---------------------------------------------------------------- training on tcgen05
// One CTA (8 warps) per SM takes 128-sample tiles in turn.  Per tile, one thread issues the
// tensor-core MMAs of the forward and backward passes (accumulators in tensor memory,
// operands in shared memory), the warps run the epilogues (bias, GELU, loss, GELU
// derivative) between them, and the weight and bias gradients stay in tensor memory across
// all of the CTA's tiles; they leave the SM once, at the end.  Warp w and w + 4 read tensor
// memory lanes 32 (w % 4) .. +31, i.e. the tile's samples (or, for the gradients, hidden
// units) 32 (w % 4) .. +31, and split the columns between them.
//
//   forward   Z1 = X W1, H1 = gelu(Z1 + b1)            X: 128 x 32 (padded to 64), W1: 32 x 128
//             Z2 = H1 W2, H2 = gelu(Z2 + b2)           W2: 128 x 128 (gelu' kept for the backward)
//             Y = H2 W3 + b3, dY = 2 (Y - T) / (4 n)   W3: 128 x 4 (padded to 16)
//   backward  dW3 += H2^T dY, db3 += colsum dY
//             dZ2 = (dY W3^T) * gelu'(P2),  dW2 += H1^T dZ2,  db2 += colsum dZ2
//             dZ1 = (dZ2 W2^T) * gelu'(P1), dW1 += X^T dZ1,   db1 += colsum dZ1
// The transposed operands are the same shared-memory tiles read MN-major (see tc.cuh); column
// sums are MMAs against a tile of ones.
constexpr int kTcThreads = 256;
constexpr uint32_t kOffW1 = 0;          // W1^T [128 hidden][64] (features 32..63 zero)      16 KB
constexpr uint32_t kOffW2 = 16384;      // W2^T [128 out][128 in]                             32 KB
constexpr uint32_t kOffW3 = 49152;      // W3^T [16 out][128 hidden] (rows 4..15 zero)         4 KB
constexpr uint32_t kOffOnes = 53248;    // [16][128] ones                                      4 KB
constexpr uint32_t kOffX = 57344;       // X [128 samples][64] (features 32..63 zero)         16 KB
constexpr uint32_t kOffH1 = 73728;      // H1 [128][128], then dZ1                            32 KB
constexpr uint32_t kOffH2 = 106496;     // H2 [128][128], then dZ2                            32 KB
constexpr uint32_t kOffDY = 139264;     // dY [128][64] (columns 4..63 zero)                  16 KB
constexpr uint32_t kOffP1 = 155648;     // gelu'(Z1 + b1) (bf16, 272-byte rows)               34 KB
constexpr uint32_t kOffP2 = 190464;     // gelu'(Z2 + b2)                                     34 KB
constexpr uint32_t kPRow = 272;
constexpr uint32_t kTcSmemBytes = 225280 + 1024;   // + slack to align the base to 1024 bytes
// tensor-memory columns
constexpr uint32_t kTZ = 0, kTdW2 = 128, kTdW3 = 256, kTdW1 = 320, kTY = 384, kTdb2 = 400, kTdb1 = 416;
constexpr uint32_t kTCols = 512;

// A bijection of [0, n) standing in for a shuffled index array: a four-round Feistel network
// over the smallest even number of bits covering n, walked along its cycle until it lands
// back in [0, n) (each try lands there with probability above 1/4).
struct Perm {
    uint32_t half_bits, mask, n;
    uint32_t key[4];
};
__device__ __forceinline__ uint32_t perm_round(uint32_t r, uint32_t k) {
    uint32_t h = (r * 0x9E3779B1u) ^ k;
    h ^= h >> 15;
    h *= 0x2C1B3C6Du;
    h ^= h >> 12;
    return h;
}
__device__ __forceinline__ uint32_t perm_apply(const Perm& p, uint32_t x) {
    for (int walk = 0; walk < 128; ++walk) {
        uint32_t l = x >> p.half_bits, r = x & p.mask;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const uint32_t t = l ^ (perm_round(r, p.key[i]) & p.mask);
            l = r;
            r = t;
        }
        x = (l << p.half_bits) | r;
        if (x < p.n) return x;
    }
    return x % p.n;                                       // bounded: a repeat sample at worst
}

__device__ __forceinline__ void gelu_both(float x, float& h, float& g) {
    const float k0 = 0.7978845608028654f, k1 = 0.044715f;
    float t = tanhf(k0 * (x + k1 * x * x * x));
    h = 0.5f * x * (1.0f + t);
    g = 0.5f * (1.0f + t) + 0.5f * x * (1.0f - t * t) * k0 * (1.0f + 3.0f * k1 * x * x);
}
// 16 bf16 values into row `row`, columns c0 .. c0 + 15 of a swizzled tile of 128 rows
__device__ __forceinline__ void put16(uint8_t* tile, int row, int c0, const float* v) {
    uint4 a, b;
    a.x = pack_bf16x2(v[0], v[1]); a.y = pack_bf16x2(v[2], v[3]); a.z = pack_bf16x2(v[4], v[5]); a.w = pack_bf16x2(v[6], v[7]);
    b.x = pack_bf16x2(v[8], v[9]); b.y = pack_bf16x2(v[10], v[11]); b.z = pack_bf16x2(v[12], v[13]); b.w = pack_bf16x2(v[14], v[15]);
    *reinterpret_cast<uint4*>(tile + tc::sw128_offset(row, c0, 128)) = a;
    *reinterpret_cast<uint4*>(tile + tc::sw128_offset(row, c0 + 8, 128)) = b;
}
__device__ __forceinline__ void put16_rows(uint8_t* buf, int row, int c0, const float* v) {
    uint4 a, b;
    a.x = pack_bf16x2(v[0], v[1]); a.y = pack_bf16x2(v[2], v[3]); a.z = pack_bf16x2(v[4], v[5]); a.w = pack_bf16x2(v[6], v[7]);
    b.x = pack_bf16x2(v[8], v[9]); b.y = pack_bf16x2(v[10], v[11]); b.z = pack_bf16x2(v[12], v[13]); b.w = pack_bf16x2(v[14], v[15]);
    uint4* p = reinterpret_cast<uint4*>(buf + row * kPRow + c0 * 2);
    p[0] = a;
    p[1] = b;
}
__device__ __forceinline__ void get16_rows(const uint8_t* buf, int row, int c0, float* v) {
    const __nv_bfloat16* p = reinterpret_cast<const __nv_bfloat16*>(buf + row * kPRow + c0 * 2);
#pragma unroll
    for (int j = 0; j < 16; ++j) v[j] = __bfloat162float(p[j]);
}

// Forward + backward of MSE(MLP(x), t) / (n * 4) over n samples of `rows` (kSampleFloats per
// sample: features, then targets): samples idx[0 .. n), or, with idx NULL, the samples
// perm(offset + 0 .. n) of a shuffle; normalised with the model's statistics.  CTA b writes
// the gradient of its tiles to gpart[b * kNParams ..] (every entry, padding as zero; the
// partial rows are summed by the consumer), the sum of squared errors is added into *loss.
// *status gets 1 if a wait for the tensor core ran past its bound.  The next tile's samples
// are loaded while the current tile is in the tensor core.
__global__ void __launch_bounds__(kTcThreads, 1) k_mlp_train(MlpDev m, float* gpart, const float* rows, const int* idx,
                                                             int n, Perm perm, int offset, float* loss, int* status) {
    extern __shared__ uint8_t tc_smem_raw[];
    uint8_t* sm = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(tc_smem_raw) + 1023) & ~uintptr_t(1023));
    __shared__ uint64_t bar;
    __shared__ uint32_t tbase;
    __shared__ float s_db3[4], s_loss;
    __shared__ float s_bias[2 * kHid];                  // b1, b2
    __shared__ float s_fnorm[2 * kFeat];                // feature means, standard deviations
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int quad = warp & 3, half = warp >> 2;
    const int row = quad * 32 + lane;                    // sample (or hidden unit) of this thread's lane
    const uint32_t lane_off = (uint32_t)(quad * 32) << 16;
    const int ntiles = (n + 127) / 128;
    uint8_t* W1 = sm + kOffW1;
    uint8_t* W2 = sm + kOffW2;
    uint8_t* W3 = sm + kOffW3;
    uint8_t* ONES = sm + kOffOnes;
    uint8_t* X = sm + kOffX;
    uint8_t* H1 = sm + kOffH1;
    uint8_t* H2 = sm + kOffH2;
    uint8_t* DY = sm + kOffDY;
    uint8_t* P1 = sm + kOffP1;
    uint8_t* P2 = sm + kOffP2;
    const float* b1 = m.p + kW1 + kW2 + kW3;
    const float* b2 = b1 + kHid;
    const float* b3 = b2 + kHid;
    // weights and constant tiles (the zero padding of X and dY stays zero for every tile), 16
    // bytes at a time: eight consecutive columns of a row are one 16-byte chunk of the swizzle
    const uint4 z4 = make_uint4(0u, 0u, 0u, 0u);
    const uint32_t one2 = pack_bf16x2(1.0f, 1.0f);
    const uint4 ones4 = make_uint4(one2, one2, one2, one2);
#pragma unroll 4
    for (int i = tid; i < 128 * 8; i += kTcThreads) {
        const int r = i >> 3, c = (i & 7) * 8;
        const uint4 v = c < kFeat ? *reinterpret_cast<const uint4*>(m.wt1 + r * kFeat + c) : z4;
        *reinterpret_cast<uint4*>(W1 + tc::sw128_offset(r, c, 128)) = v;
        *reinterpret_cast<uint4*>(X + tc::sw128_offset(r, c, 128)) = z4;
        *reinterpret_cast<uint4*>(DY + tc::sw128_offset(r, c, 128)) = z4;
    }
#pragma unroll 8
    for (int i = tid; i < 128 * 16; i += kTcThreads) {
        const int r = i >> 4, c = (i & 15) * 8;
        *reinterpret_cast<uint4*>(W2 + tc::sw128_offset(r, c, 128)) = *reinterpret_cast<const uint4*>(m.wt2 + r * kHid + c);
    }
    for (int i = tid; i < 16 * 16; i += kTcThreads) {
        const int r = i >> 4, c = (i & 15) * 8;
        *reinterpret_cast<uint4*>(W3 + tc::sw128_offset(r, c, 16)) =
            r < kOutPad ? *reinterpret_cast<const uint4*>(m.wt3 + r * kHid + c) : z4;
        *reinterpret_cast<uint4*>(ONES + tc::sw128_offset(r, c, 16)) = ones4;
    }
    for (int i = tid; i < 2 * kHid; i += kTcThreads) s_bias[i] = b1[i];             // b1 then b2
    for (int i = tid; i < 2 * kFeat; i += kTcThreads) s_fnorm[i] = i < kFeat ? m.fmean[i] : m.fstd[i - kFeat];
    if (tid == 0) {
        tc::mbar_init(&bar);
        s_loss = 0.0f;
        s_db3[0] = s_db3[1] = s_db3[2] = s_db3[3] = 0.0f;
    }
    if (warp == 0) tc::tmem_alloc(&tbase, kTCols);
    tc::fence_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t T = tbase;
    const uint32_t aX = tc::smem_addr(X), aH1 = tc::smem_addr(H1), aH2 = tc::smem_addr(H2), aDY = tc::smem_addr(DY);
    const uint32_t aW1 = tc::smem_addr(W1), aW2 = tc::smem_addr(W2), aW3 = tc::smem_addr(W3), aON = tc::smem_addr(ONES);
    constexpr uint32_t kKK128 = tc::idesc_bf16(128, 128, 0, 0), kKK16 = tc::idesc_bf16(128, 16, 0, 0);
    constexpr uint32_t kKM128 = tc::idesc_bf16(128, 128, 0, 1), kMM128 = tc::idesc_bf16(128, 128, 1, 1);
    constexpr uint32_t kMM64 = tc::idesc_bf16(128, 64, 1, 1), kMK16 = tc::idesc_bf16(128, 16, 1, 0);
    uint32_t phase = 0;
    bool ok = true;
    auto wait_mma = [&]() {
        ok &= tc::mbar_wait(&bar, phase, 1 << 24);
        phase ^= 1u;
        tc::fence_after_sync();
    };
    // shared-memory writes and tensor-memory reads of the epilogue done before the next MMAs
    auto sync_for_mma = [&]() {
        tc::fence_async_smem();
        tc::fence_before_sync();
        __syncthreads();
        tc::fence_after_sync();
    };
    const float inv = 1.0f / (4.0f * (float)n);
    const int cbeg = half * 64;
    float lsum = 0.0f, db3[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    bool first = true;
    // this thread's row of a tile: half 0 features 0..15 and the targets, half 1 features 16..31
    auto fetch = [&](int tile, float* fv, float* tv) {
        const int r0 = tile * 128;
        const bool valid = tile < ntiles && r0 + row < n;
        const int sid = !valid ? 0 : (idx ? idx[r0 + row] : (int)perm_apply(perm, (uint32_t)(offset + r0 + row)));
        // a sample row is 144 bytes, so its four-float groups are 16-byte aligned
        const float4* sample = reinterpret_cast<const float4*>(rows + (size_t)sid * kSampleFloats);
        const float4 z = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const float4 v = valid ? sample[half * 4 + q] : z;
            fv[4 * q] = v.x; fv[4 * q + 1] = v.y; fv[4 * q + 2] = v.z; fv[4 * q + 3] = v.w;
        }
        const float4 t4 = valid && half == 0 ? sample[kFeat / 4] : z;
        tv[0] = t4.x; tv[1] = t4.y; tv[2] = t4.z; tv[3] = t4.w;
    };
    float fcur[16], tcur[kOut];
    fetch(blockIdx.x, fcur, tcur);
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int r0 = tile * 128;
        const bool valid = r0 + row < n;
        {   // inputs: half 0 writes features 0..15 of its row, half 1 features 16..31
            float v[16];
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                const int f = half * 16 + j;
                v[j] = valid ? (fcur[j] - s_fnorm[f]) / s_fnorm[kFeat + f] : 0.0f;
            }
            put16(X, row, half * 16, v);
        }
        float fnext[16], tnext[kOut];
        fetch(tile + gridDim.x, fnext, tnext);
        sync_for_mma();
        if (tid == 0) {                                   // Z1 = X W1 (K = 32)
            for (int ks = 0; ks < 2; ++ks) tc::mma(T + kTZ, tc::desc_k(aX, ks, 16384), tc::desc_k(aW1, ks, 16384), kKK128, ks > 0);
            tc::commit(&bar);
        }
        wait_mma();
        for (int c0 = cbeg; c0 < cbeg + 64; c0 += 16) {  // H1 = gelu(Z1 + b1), P1
            float z[16], h[16];
            tc::ld16(T + lane_off + kTZ + c0, z);
#pragma unroll
            for (int j = 0; j < 16; ++j) gelu_both(z[j] + s_bias[c0 + j], h[j], z[j]);   // z becomes gelu'
            put16(H1, row, c0, h);
            put16_rows(P1, row, c0, z);
        }
        sync_for_mma();
        if (tid == 0) {                                   // Z2 = H1 W2
            for (int ks = 0; ks < 8; ++ks) tc::mma(T + kTZ, tc::desc_k(aH1, ks, 16384), tc::desc_k(aW2, ks, 16384), kKK128, ks > 0);
            tc::commit(&bar);
        }
        wait_mma();
        for (int c0 = cbeg; c0 < cbeg + 64; c0 += 16) {  // H2 = gelu(Z2 + b2), P2
            float z[16], h[16];
            tc::ld16(T + lane_off + kTZ + c0, z);
#pragma unroll
            for (int j = 0; j < 16; ++j) gelu_both(z[j] + s_bias[kHid + c0 + j], h[j], z[j]);   // z becomes gelu'
            put16(H2, row, c0, h);
            put16_rows(P2, row, c0, z);
        }
        sync_for_mma();
        if (tid == 0) {                                   // Y = H2 W3 (N = 16)
            for (int ks = 0; ks < 8; ++ks) tc::mma(T + kTY, tc::desc_k(aH2, ks, 16384), tc::desc_k(aW3, ks, 2048), kKK16, ks > 0);
            tc::commit(&bar);
        }
        wait_mma();
        if (half == 0) {                                  // loss and dY = 2 (Y + b3 - T) / (4 n)
            float y[16];
            tc::ld16(T + lane_off + kTY, y);
            float d[4];
#pragma unroll
            for (int o = 0; o < kOut; ++o) {
                d[o] = 0.0f;
                if (valid) {
                    const float tv = (tcur[o] - m.tmean[o]) / m.tstd[o];
                    const float diff = y[o] + b3[o] - tv;
                    lsum += diff * diff;
                    d[o] = 2.0f * diff * inv;
                }
            }
            uint2 q;
            q.x = pack_bf16x2(d[0], d[1]);
            q.y = pack_bf16x2(d[2], d[3]);
            *reinterpret_cast<uint2*>(DY + tc::sw128_offset(row, 0, 128)) = q;
#pragma unroll
            for (int o = 0; o < kOut; ++o) db3[o] += d[o];
        }
        sync_for_mma();
        if (tid == 0) {
            // dW3 += H2^T dY (M = hidden, N = 64, K = samples); dH2 = dY W3^T (K = 16)
            for (int ks = 0; ks < 8; ++ks)
                tc::mma(T + kTdW3, tc::desc_mn(aH2, ks, 16384), tc::desc_mn(aDY, ks, 16384), kMM64, !first || ks > 0);
            tc::mma(T + kTZ, tc::desc_k(aDY, 0, 16384), tc::desc_mn(aW3, 0, 2048), kKM128, false);
            tc::commit(&bar);
        }
        wait_mma();
        for (int c0 = cbeg; c0 < cbeg + 64; c0 += 16) {  // dZ2 = dH2 * gelu'(P2), over H2
            float z[16], p[16];
            tc::ld16(T + lane_off + kTZ + c0, z);
            get16_rows(P2, row, c0, p);
#pragma unroll
            for (int j = 0; j < 16; ++j) z[j] *= p[j];
            put16(H2, row, c0, z);
        }
        sync_for_mma();
        if (tid == 0) {
            // dW2 += H1^T dZ2, db2 += dZ2^T 1, dH1 = dZ2 W2^T
            for (int ks = 0; ks < 8; ++ks) {
                tc::mma(T + kTdW2, tc::desc_mn(aH1, ks, 16384), tc::desc_mn(aH2, ks, 16384), kMM128, !first || ks > 0);
                tc::mma(T + kTdb2, tc::desc_mn(aH2, ks, 16384), tc::desc_k(aON, ks, 2048), kMK16, !first || ks > 0);
            }
            for (int ks = 0; ks < 8; ++ks) tc::mma(T + kTZ, tc::desc_k(aH2, ks, 16384), tc::desc_mn(aW2, ks, 16384), kKM128, ks > 0);
            tc::commit(&bar);
        }
        wait_mma();
        for (int c0 = cbeg; c0 < cbeg + 64; c0 += 16) {  // dZ1 = dH1 * gelu'(P1), over H1
            float z[16], p[16];
            tc::ld16(T + lane_off + kTZ + c0, z);
            get16_rows(P1, row, c0, p);
#pragma unroll
            for (int j = 0; j < 16; ++j) z[j] *= p[j];
            put16(H1, row, c0, z);
        }
        sync_for_mma();
        if (tid == 0) {
            // dW1^T += dZ1^T X (M = hidden, N = 64 features), db1 += dZ1^T 1
            for (int ks = 0; ks < 8; ++ks) {
                tc::mma(T + kTdW1, tc::desc_mn(aH1, ks, 16384), tc::desc_mn(aX, ks, 16384), kMM64, !first || ks > 0);
                tc::mma(T + kTdb1, tc::desc_mn(aH1, ks, 16384), tc::desc_k(aON, ks, 2048), kMK16, !first || ks > 0);
            }
            tc::commit(&bar);
        }
        wait_mma();
        first = false;
#pragma unroll
        for (int j = 0; j < 16; ++j) fcur[j] = fnext[j];
#pragma unroll
        for (int o = 0; o < kOut; ++o) tcur[o] = tnext[o];
        __syncthreads();                                  // the next tile rewrites X and the activations
    }
    // loss and db3: warp sums, then the block's
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
#pragma unroll
        for (int q = 0; q < kOut; ++q) db3[q] += __shfl_xor_sync(0xffffffffu, db3[q], o);
    }
    if (lane == 0 && half == 0) {
        atomicAdd(&s_loss, lsum);
#pragma unroll
        for (int q = 0; q < kOut; ++q) atomicAdd(&s_db3[q], db3[q]);
    }
    // the CTA's gradients, this thread's lane being hidden unit `row`, into the CTA's partial row
    float* gw1 = gpart + (size_t)blockIdx.x * kNParams;
    float* gw2 = gw1 + kW1;
    float* gw3 = gw2 + kW2;
    float* gb1 = gw3 + kW3;
    float* gb2 = gb1 + kHid;
    float* gb3 = gb2 + kHid;
    for (int c0 = cbeg; c0 < cbeg + 64; c0 += 16) {      // dW2[in = row][out]
        float v[16];
        tc::ld16(T + lane_off + kTdW2 + c0, v);
#pragma unroll
        for (int j = 0; j < 16; j += 4)
            *reinterpret_cast<float4*>(gw2 + row * kHid + c0 + j) = make_float4(v[j], v[j + 1], v[j + 2], v[j + 3]);
    }
    if (half == 0) {
        float v[16];
        tc::ld16(T + lane_off + kTdW3, v);                // dW3[hidden = row][0..3], padding zero
#pragma unroll
        for (int j = 0; j < kOutPad; ++j) gw3[row * kOutPad + j] = j < kOut ? v[j] : 0.0f;
        for (int c0 = 0; c0 < kFeat; c0 += 16) {          // dW1[feature][hidden = row]
            tc::ld16(T + lane_off + kTdW1 + c0, v);
#pragma unroll
            for (int j = 0; j < 16; ++j) gw1[(c0 + j) * kHid + row] = v[j];
        }
        tc::ld16(T + lane_off + kTdb2, v);
        gb2[row] = v[0];
    } else {
        float v[16];
        tc::ld16(T + lane_off + kTdb1, v);
        gb1[row] = v[0];
    }
    tc::fence_before_sync();
    __syncthreads();
    if (tid < kOutPad) gb3[tid] = tid < kOut ? s_db3[tid] : 0.0f;
    if (tid == 0) atomicAdd(loss, s_loss);
    if (!ok && lane == 0) atomicExch(status, 1);
    if (warp == 0) tc::tmem_free(T, kTCols);
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

// the gradient of a batch: the sum of the `parts` partial rows k_mlp_train wrote
__device__ __forceinline__ float grad_sum(const float* gpart, int parts, int i) {
    float g = 0.0f;
    for (int b = 0; b < parts; ++b) g += gpart[(size_t)b * kNParams + i];
    return g;
}
__global__ void k_mlp_reduce(const float* gpart, int parts, float* grad) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < kNParams; i += gridDim.x * blockDim.x)
        grad[i] = grad_sum(gpart, parts, i);
}

// Adam (beta1 0.9, beta2 0.999, eps 1e-8) on the flat parameter vector, its gradient the sum of
// the batch's partial rows, and the BF16 copies of the updated weights (as k_mlp_refresh
// writes them)
__global__ void k_mlp_adam(float* p, const float* gpart, int parts, float* mom, float* vel, int n, float lr, float bc1,
                           float bc2, __nv_bfloat16* wt1, __nv_bfloat16* wt2, __nv_bfloat16* wt3, __nv_bfloat16* wb1,
                           __nv_bfloat16* wb2, __nv_bfloat16* wb3) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float gi = grad_sum(gpart, parts, i);
        bool pad = false;
        if (i >= kW1 + kW2 && i < kW1 + kW2 + kW3) pad = ((i - kW1 - kW2) % kOutPad) >= kOut;
        if (i >= kW1 + kW2 + kW3 + 2 * kHid) pad = (i - (kW1 + kW2 + kW3 + 2 * kHid)) >= kOut;
        if (pad) continue;
        float mi = 0.9f * mom[i] + 0.1f * gi;
        float vi = 0.999f * vel[i] + 0.001f * gi * gi;
        mom[i] = mi;
        vel[i] = vi;
        const float pi = p[i] - lr * (mi / bc1) / (sqrtf(vi / bc2) + 1e-8f);
        p[i] = pi;
        if (i >= kW1 + kW2 + kW3) continue;
        const __nv_bfloat16 v = __float2bfloat16_rn(pi);
        if (i < kW1) {
            const int r = i / kHid, c = i % kHid;
            wb1[i] = v;
            wt1[c * kFeat + r] = v;
        } else if (i < kW1 + kW2) {
            const int j = i - kW1, r = j / kHid, c = j % kHid;
            wb2[j] = v;
            wt2[c * kHid + r] = v;
        } else {
            const int j = i - kW1 - kW2, r = j / kOutPad, c = j % kOutPad;
            wb3[j] = v;
            wt3[c * kHid + r] = v;
        }
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
    float* grad = nullptr;        // kNParams: a batch's gradient, for dbox_mlp_gradient
    float* gpart = nullptr;       // nsm x kNParams: per-CTA partial gradients of a batch
    float* mom = nullptr;
    float* vel = nullptr;
    float* norm = nullptr;        // fmean 32, fstd 32, tmean 4, tstd 4
    __nv_bfloat16* wbuf = nullptr;  // wt1 wt2 wt3 wb1 wb2 wb3
    float* loss = nullptr;
    int* status = nullptr;        // set by k_mlp_train when a tensor-core wait ran past its bound
    int nsm = 1;
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

// gradient of one batch (rows idx[0..n)) as partial rows in m->gpart (*parts of them); loss sum
// added into m->loss: one CTA per SM at most, each taking 128-sample tiles in turn
int run_batch(dbox_mlp* m, const float* rows, const int* idx, int n, int* parts, const dg::Perm& perm = dg::Perm(),
              int offset = 0) {
    *parts = 0;
    if (n <= 0) return DBOX_OK;
    const int tiles = (n + 127) / 128;
    const int blocks = tiles < m->nsm ? tiles : m->nsm;
    dg::k_mlp_train<<<blocks, dg::kTcThreads, dg::kTcSmemBytes>>>(mlp_dev(m), m->gpart, rows, idx, n, perm, offset,
                                                                 m->loss, m->status);
    *parts = blocks;
    return cuerr(cudaGetLastError(), "k_mlp_train");
}

// the shuffle of epoch e of n samples (dg::Perm), keyed from the training seed
dg::Perm make_perm(uint32_t n, uint64_t seed, int epoch) {
    dg::Perm p;
    int bits = 2;
    while (bits < 32 && (1ull << bits) < n) bits += 2;
    p.half_bits = (uint32_t)(bits / 2);
    p.mask = (1u << p.half_bits) - 1u;
    p.n = n;
    uint64_t s = seed ^ (0x9E3779B97F4A7C15ull * (uint64_t)(epoch + 1));
    for (int i = 0; i < 4; ++i) {                     // SplitMix64
        s += 0x9E3779B97F4A7C15ull;
        uint64_t z = s;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        p.key[i] = (uint32_t)(z ^ (z >> 31));
    }
    return p;
}

// a wait for the tensor core that ran past its bound in any training launch since the last check
int check_train_status(dbox_mlp* m) {
    int st = 0;
    int r = cuerr(cudaMemcpy(&st, m->status, sizeof(int), cudaMemcpyDeviceToHost), "training status");
    if (r) return r;
    if (st) {
        cudaMemset(m->status, 0, sizeof(int));
        return dbox_set_error(DBOX_ERR_TIMEOUT, "k_mlp_train: a tensor-core wait ran past its bound");
    }
    return DBOX_OK;
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
              cudaMalloc(&m->loss, sizeof(float)) == cudaSuccess &&
              cudaMalloc(&m->status, sizeof(int)) == cudaSuccess;
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
    cudaMemset(m->status, 0, sizeof(int));
    cudaDeviceGetAttribute(&m->nsm, cudaDevAttrMultiProcessorCount, m->device);
    if (m->nsm < 1) m->nsm = 1;
    if (cudaMalloc(&m->gpart, sizeof(float) * dg::kNParams * (size_t)m->nsm) != cudaSuccess) {
        dbox_mlp_destroy(m);
        return dbox_set_error(DBOX_ERR_CUDA, "dbox_mlp_create: device allocation failed");
    }
    cudaFuncSetAttribute(dg::k_mlp_train, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dg::kTcSmemBytes);
    int r = refresh(m);
    if (r) { dbox_mlp_destroy(m); return r; }
    *out = m;
    return DBOX_OK;
}

int32_t dbox_mlp_destroy(dbox_mlp* m) {
    if (!m) return DBOX_OK;
    cudaFree(m->p); cudaFree(m->grad); cudaFree(m->gpart); cudaFree(m->mom); cudaFree(m->vel);
    cudaFree(m->norm); cudaFree(m->wbuf); cudaFree(m->loss); cudaFree(m->status);
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
    cudaMemset(m->loss, 0, sizeof(float));
    int parts = 0;
    r = run_batch(m, drows, di, n, &parts);
    if (!r) {
        dg::k_mlp_reduce<<<(dg::kNParams + 255) / 256, 256>>>(m->gpart, parts, m->grad);
        r = cuerr(cudaGetLastError(), "k_mlp_reduce");
    }
    if (!r) r = cuerr(cudaDeviceSynchronize(), "dbox_mlp_gradient");
    if (!r) r = check_train_status(m);
    if (!r && grad) r = cuerr(cudaMemcpy(grad, m->grad, sizeof(float) * dg::kNParams, cudaMemcpyDeviceToHost), "grad");
    float l = 0.0f;
    if (!r) r = cuerr(cudaMemcpy(&l, m->loss, sizeof(float), cudaMemcpyDeviceToHost), "loss");
    if (loss) *loss = l / (4.0f * (float)n);
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
    if (reinterpret_cast<uintptr_t>(rows) & 15u)
        return dbox_set_error(DBOX_ERR_INVALID, "dbox_mlp_train_device: rows must be 16-byte aligned");
    int r = DBOX_OK;
    dg::MlpDev d = mlp_dev(m);
    for (int e = 0; e < epochs && !r; ++e) {
        const dg::Perm perm = make_perm((uint32_t)n, seed, e);   // this epoch's shuffle, applied on the device
        cudaMemset(m->loss, 0, sizeof(float));
        for (int b0 = 0; b0 < n && !r; b0 += batch) {
            int nb = std::min(batch, n - b0);
            int parts = 0;
            r = run_batch(m, rows, nullptr, nb, &parts, perm, b0);
            if (r) break;
            ++m->step;
            float bc1 = 1.0f - powf(0.9f, (float)m->step), bc2 = 1.0f - powf(0.999f, (float)m->step);
            dg::k_mlp_adam<<<(dg::kNParams + 255) / 256, 256>>>(m->p, m->gpart, parts, m->mom, m->vel, dg::kNParams, lr, bc1, bc2,
                                        const_cast<__nv_bfloat16*>(d.wt1), const_cast<__nv_bfloat16*>(d.wt2),
                                        const_cast<__nv_bfloat16*>(d.wt3), const_cast<__nv_bfloat16*>(d.wb1),
                                        const_cast<__nv_bfloat16*>(d.wb2), const_cast<__nv_bfloat16*>(d.wb3));
            r = cuerr(cudaGetLastError(), "k_mlp_adam");
        }
        if (!r) r = cuerr(cudaDeviceSynchronize(), "dbox_mlp_train_device");
        if (!r) r = check_train_status(m);
        if (!r && epoch_loss) {
            float l = 0.0f;
            cudaMemcpy(&l, m->loss, sizeof(float), cudaMemcpyDeviceToHost);
            // per-batch losses are means over (nb * 4); the sum below is over all n * 4 entries
            epoch_loss[e] = l / (4.0f * (float)n);
        }
    }
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
