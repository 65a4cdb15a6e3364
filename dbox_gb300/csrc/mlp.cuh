// Learned warm start: a 32 -> 128 -> 128 -> 4 multilayer perceptron (GELU, BF16 weights and
// activations, FP32 accumulation) that predicts the normal and tangent impulses of the two
// manifold points of a contact whose points are new this step.  The network runs on the
// tensor cores through warp-level mma.sync (m16n8k16, bf16 x bf16 -> f32); a batch is a
// 16-row tile per warp.  This header holds the parameter layout, the fragment helpers and
// the one-warp inference used inside the solver; training is in mlp.cu.
#pragma once
#include <cuda_bf16.h>
#include <stdint.h>

namespace dg {

constexpr int kFeat = 32;        // input features per contact
constexpr int kHid = 128;        // hidden width (two layers)
constexpr int kOut = 4;          // normalImpulse0, tangentImpulse0, normalImpulse1, tangentImpulse1
constexpr int kOutPad = 8;       // output columns padded to one n8 tile
constexpr int kSampleFloats = kFeat + kOut;   // one training sample: features then targets

// Parameters.  FP32 master copies are what Adam updates; the BF16 copies feed the tensor
// cores: wt* are the transposes (N x K, row-major) used by the forward pass, w* the
// K x N row-major copies used to propagate gradients backwards.
struct MlpParams {
    float* w1;    // 32 x 128
    float* w2;    // 128 x 128
    float* w3;    // 128 x 8 (columns 4..7 stay zero)
    float* b1;    // 128
    float* b2;    // 128
    float* b3;    // 8
};
constexpr int kW1 = kFeat * kHid, kW2 = kHid * kHid, kW3 = kHid * kOutPad;
constexpr int kNParams = kW1 + kW2 + kW3 + kHid + kHid + kOutPad;   // flat FP32 layout in this order

struct MlpDev {
    const float* p;                  // kNParams FP32 (w1, w2, w3, b1, b2, b3)
    const __nv_bfloat16* wt1;        // 128 x 32
    const __nv_bfloat16* wt2;        // 128 x 128
    const __nv_bfloat16* wt3;        // 8 x 128
    const __nv_bfloat16* wb1;        // 32 x 128
    const __nv_bfloat16* wb2;        // 128 x 128
    const __nv_bfloat16* wb3;        // 128 x 8
    const float* fmean;              // 32: feature normalisation x' = (x - mean) / std
    const float* fstd;
    const float* tmean;              // 4: target normalisation
    const float* tstd;
};

__device__ __forceinline__ uint32_t pack_bf16x2(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&v);
}
__device__ __forceinline__ uint32_t pack_raw(__nv_bfloat16 lo, __nv_bfloat16 hi) {
    __nv_bfloat162 v;
    v.x = lo;
    v.y = hi;
    return *reinterpret_cast<uint32_t*>(&v);
}

// D = A (16x16, row) * B (16x8, col) + C on the tensor cores; fragments per PTX ISA m16n8k16:
// gid = lane / 4, tig = lane % 4;  a: (gid, 2tig..+1), (gid+8, 2tig..), (gid, 2tig+8..), (gid+8, 2tig+8..);
// b: (k = 2tig..+1, n = gid), (k = 2tig+8.., n = gid);  c: (gid, 2tig..+1), (gid+8, 2tig..+1).
__device__ __forceinline__ void mma_bf16(float c[4], const uint32_t a[4], const uint32_t b[2]) {
    asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                 "{%0,%1,%2,%3};"
                 : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
                 : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// GELU, tanh form: 0.5 x (1 + tanh(sqrt(2/pi) (x + 0.044715 x^3)))
__device__ __forceinline__ float gelu_f(float x) {
    const float k0 = 0.7978845608028654f, k1 = 0.044715f;
    return 0.5f * x * (1.0f + tanhf(k0 * (x + k1 * x * x * x)));
}
__device__ __forceinline__ float gelu_grad(float x) {
    const float k0 = 0.7978845608028654f, k1 = 0.044715f;
    float u = k0 * (x + k1 * x * x * x);
    float t = tanhf(u);
    return 0.5f * (1.0f + t) + 0.5f * x * (1.0f - t * t) * k0 * (1.0f + 3.0f * k1 * x * x);
}

// A fragment of a 16 x 16 bf16 tile at (row0, col0) of a row-major shared array with `ld`
// elements per row.
__device__ __forceinline__ void load_a_rowmajor(uint32_t a[4], const __nv_bfloat16* s, int ld, int col0, int lane) {
    const int g = lane >> 2, t = lane & 3;
    const __nv_bfloat16* r0 = s + g * ld + col0 + 2 * t;
    const __nv_bfloat16* r1 = s + (g + 8) * ld + col0 + 2 * t;
    a[0] = *reinterpret_cast<const uint32_t*>(r0);
    a[1] = *reinterpret_cast<const uint32_t*>(r1);
    a[2] = *reinterpret_cast<const uint32_t*>(r0 + 8);
    a[3] = *reinterpret_cast<const uint32_t*>(r1 + 8);
}
// B fragment (k16 x n8 at k0, n0) when B[k][n] = M[n][k] for a row-major M with `ld`
// elements per row (pairs along k are contiguous)
__device__ __forceinline__ void load_b_trans(uint32_t b[2], const __nv_bfloat16* m, int ld, int k0, int n0, int lane) {
    const int g = lane >> 2, t = lane & 3;
    const __nv_bfloat16* r = m + (n0 + g) * ld + k0 + 2 * t;
    b[0] = *reinterpret_cast<const uint32_t*>(r);
    b[1] = *reinterpret_cast<const uint32_t*>(r + 8);
}

// One warp: y[16][4] = MLP(x[16][32]) for 16 rows of normalised features held in shared
// memory (bf16, row-major 16 x 32).  scratch: 2 x 16 x 128 bf16 (8 KB).  Rows beyond the
// caller's count are computed and ignored.  Outputs are the normalised targets; the
// caller applies tmean / tstd.
__device__ __forceinline__ void mlp_infer16(const MlpDev& m, const __nv_bfloat16* x, __nv_bfloat16* h1,
                                            __nv_bfloat16* h2, float y[4], int lane) {
    const int g = lane >> 2, t = lane & 3;
    const float* b1 = m.p + kW1 + kW2 + kW3;
    const float* b2 = b1 + kHid;
    const float* b3 = b2 + kHid;
    // layer 1: 16 x 32 -> 16 x 128
    uint32_t a[4];
    for (int nb = 0; nb < kHid / 8; ++nb) {
        float c[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
        for (int kb = 0; kb < kFeat / 16; ++kb) {
            uint32_t b[2];
            load_a_rowmajor(a, x, kFeat, kb * 16, lane);
            load_b_trans(b, m.wt1, kFeat, kb * 16, nb * 8, lane);
            mma_bf16(c, a, b);
        }
        const int col = nb * 8 + 2 * t;
        float bb0 = b1[col], bb1 = b1[col + 1];
        *reinterpret_cast<uint32_t*>(h1 + g * kHid + col) = pack_bf16x2(gelu_f(c[0] + bb0), gelu_f(c[1] + bb1));
        *reinterpret_cast<uint32_t*>(h1 + (g + 8) * kHid + col) = pack_bf16x2(gelu_f(c[2] + bb0), gelu_f(c[3] + bb1));
    }
    __syncwarp();
    // layer 2: 16 x 128 -> 16 x 128
    for (int nb = 0; nb < kHid / 8; ++nb) {
        float c[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll 4
        for (int kb = 0; kb < kHid / 16; ++kb) {
            uint32_t b[2];
            load_a_rowmajor(a, h1, kHid, kb * 16, lane);
            load_b_trans(b, m.wt2, kHid, kb * 16, nb * 8, lane);
            mma_bf16(c, a, b);
        }
        const int col = nb * 8 + 2 * t;
        float bb0 = b2[col], bb1 = b2[col + 1];
        *reinterpret_cast<uint32_t*>(h2 + g * kHid + col) = pack_bf16x2(gelu_f(c[0] + bb0), gelu_f(c[1] + bb1));
        *reinterpret_cast<uint32_t*>(h2 + (g + 8) * kHid + col) = pack_bf16x2(gelu_f(c[2] + bb0), gelu_f(c[3] + bb1));
    }
    __syncwarp();
    // layer 3: 16 x 128 -> 16 x 8 (columns 0..3 used)
    float c[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll 4
    for (int kb = 0; kb < kHid / 16; ++kb) {
        uint32_t b[2];
        load_a_rowmajor(a, h2, kHid, kb * 16, lane);
        load_b_trans(b, m.wt3, kHid, kb * 16, 0, lane);
        mma_bf16(c, a, b);
    }
    // lane (g, t) holds rows g and g + 8, columns 2t and 2t + 1
    y[0] = c[0] + b3[2 * t];
    y[1] = c[1] + b3[2 * t + 1];
    y[2] = c[2] + b3[2 * t];
    y[3] = c[3] + b3[2 * t + 1];
}

}  // namespace dg
