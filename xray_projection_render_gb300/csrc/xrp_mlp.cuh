// xrp_mlp.cuh -- the learned proposal network on tensor cores.
//
// A 3x64 MLP (64 inputs -> 64 -> 64 -> 64 -> 1 logit, ReLU) with BF16
// weights and activations, FP32 accumulation, evaluated 32 rows per warp with
// mma.sync.m16n8k16 (BF16 x BF16 -> FP32).  Rows are ray segments; the logit
// says how likely the segment holds a density transition.
//
// Fragment layouts are those of the PTX ISA for m16n8k16 with 16-bit A/B:
// groupID g = lane >> 2, thread-in-group t = lane & 3;
//   A (16x16, row major): a0 = A[g][2t..2t+1], a1 = A[g+8][2t..2t+1],
//                         a2 = A[g][2t+8..], a3 = A[g+8][2t+8..]
//   B (16x8):             b0 = B[2t..2t+1][g], b1 = B[2t+8..2t+9][g]
//   C/D (16x8, f32):      c0 = C[g][2t], c1 = C[g][2t+1], c2 = C[g+8][2t], c3 = C[g+8][2t+1]
// so the D fragments of one layer are, after ReLU and BF16 packing, exactly
// the A fragments of the next (K of the next layer = N of this one).
#pragma once
#include <cuda_bf16.h>
#include <stdint.h>

namespace xrp {

constexpr int kMlpIn = 64;
constexpr int kMlpHid = 64;
constexpr int kMlpLd = 72;  // padded shared-memory row stride (bf16 elements)

// FP32 parameter block layout (master copy and gradients).
struct MlpLayout {
    static constexpr int W1 = 0;                         // [64 out][64 in]
    static constexpr int B1 = W1 + kMlpHid * kMlpIn;     // [64]
    static constexpr int W2 = B1 + kMlpHid;              // [64][64]
    static constexpr int B2 = W2 + kMlpHid * kMlpHid;
    static constexpr int W3 = B2 + kMlpHid;
    static constexpr int B3 = W3 + kMlpHid * kMlpHid;
    static constexpr int W4 = B3 + kMlpHid;              // [64]
    static constexpr int B4 = W4 + kMlpHid;              // [1]
    static constexpr int N = B4 + 1;
};

#if defined(__CUDACC__)

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);  // .x = lo (low half), .y = hi
    return *reinterpret_cast<uint32_t*>(&v);
}

__device__ __forceinline__ void mma_bf16(float* d, const uint32_t* a, const uint32_t* b) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
        "{%8,%9}, {%0,%1,%2,%3};"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// Shared-memory parameter image used by inference: BF16 weights stored
// [out][in] with padded rows (so B^T rows are contiguous in K), FP32 biases
// and output weights.
struct MlpShared {
    __nv_bfloat16 w[3][kMlpHid * kMlpLd];
    float b[3][kMlpHid];
    float w4[kMlpHid];
    float b4;
};

// One layer on 32 rows: acc[m][n][4] = A(32x64) * W^T, with A given as the
// A fragments of two 16-row tiles (af[m][kb][4]) and W in shared memory
// ([out][in], padded).  Output fragments are FP32 (bias not added).
__device__ __forceinline__ void mlp_layer(const uint32_t (&af)[2][4][4],
                                          const __nv_bfloat16* __restrict__ w, float (&acc)[2][8][4]) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll
    for (int m = 0; m < 2; m++)
#pragma unroll
        for (int n = 0; n < 8; n++)
#pragma unroll
            for (int q = 0; q < 4; q++) acc[m][n][q] = 0.0f;
#pragma unroll
    for (int n = 0; n < 8; n++) {
        const __nv_bfloat16* wr = w + (n * 8 + g) * kMlpLd;
#pragma unroll
        for (int kb = 0; kb < 4; kb++) {
            uint32_t b[2];
            b[0] = *reinterpret_cast<const uint32_t*>(wr + kb * 16 + 2 * t);
            b[1] = *reinterpret_cast<const uint32_t*>(wr + kb * 16 + 8 + 2 * t);
            mma_bf16(acc[0][n], af[0][kb], b);
            mma_bf16(acc[1][n], af[1][kb], b);
        }
    }
}

// Bias + ReLU + BF16 packing of layer outputs into the next layer's A
// fragments.
__device__ __forceinline__ void mlp_relu_pack(const float (&acc)[2][8][4], const float* __restrict__ bias,
                                              uint32_t (&af)[2][4][4]) {
    const int lane = threadIdx.x & 31, t = lane & 3;
#pragma unroll
    for (int m = 0; m < 2; m++)
#pragma unroll
        for (int kb = 0; kb < 4; kb++) {
            const int n0 = 2 * kb, n1 = 2 * kb + 1;
            const float ba = bias[n0 * 8 + 2 * t], bb = bias[n0 * 8 + 2 * t + 1];
            const float bc = bias[n1 * 8 + 2 * t], bd = bias[n1 * 8 + 2 * t + 1];
            af[m][kb][0] = pack_bf16(fmaxf(acc[m][n0][0] + ba, 0.f), fmaxf(acc[m][n0][1] + bb, 0.f));
            af[m][kb][1] = pack_bf16(fmaxf(acc[m][n0][2] + ba, 0.f), fmaxf(acc[m][n0][3] + bb, 0.f));
            af[m][kb][2] = pack_bf16(fmaxf(acc[m][n1][0] + bc, 0.f), fmaxf(acc[m][n1][1] + bd, 0.f));
            af[m][kb][3] = pack_bf16(fmaxf(acc[m][n1][2] + bc, 0.f), fmaxf(acc[m][n1][3] + bd, 0.f));
        }
}

// A fragments of 32 input rows staged in shared memory ([row][kMlpLd] bf16).
__device__ __forceinline__ void mlp_load_a(const __nv_bfloat16* __restrict__ x, uint32_t (&af)[2][4][4]) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll
    for (int m = 0; m < 2; m++)
#pragma unroll
        for (int kb = 0; kb < 4; kb++) {
            const __nv_bfloat16* r0 = x + (m * 16 + g) * kMlpLd + kb * 16 + 2 * t;
            const __nv_bfloat16* r1 = r0 + 8 * kMlpLd;
            af[m][kb][0] = *reinterpret_cast<const uint32_t*>(r0);
            af[m][kb][1] = *reinterpret_cast<const uint32_t*>(r1);
            af[m][kb][2] = *reinterpret_cast<const uint32_t*>(r0 + 8);
            af[m][kb][3] = *reinterpret_cast<const uint32_t*>(r1 + 8);
        }
}

// Inference on one 16-row tile held in shared memory (`x`, kMlpLd stride),
// overwritten in place by the hidden activations: rows only feed their own
// outputs, so each layer reads its A fragments, the warp synchronises, and
// the outputs go back to the same rows.  Keeps one tile's accumulators live
// (about 50 registers) so the march around it does not spill.  Returns the
// output-layer partial sums of rows g and g+8 over this thread's columns.
__device__ __forceinline__ void mlp_tile16(const MlpShared& P, __nv_bfloat16* x, float& p0, float& p1) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    float acc[8][4];
#pragma unroll 1
    for (int l = 0; l < 3; l++) {
        uint32_t af[4][4];
#pragma unroll
        for (int kb = 0; kb < 4; kb++) {
            const __nv_bfloat16* r0 = x + g * kMlpLd + kb * 16 + 2 * t;
            const __nv_bfloat16* r1 = r0 + 8 * kMlpLd;
            af[kb][0] = *reinterpret_cast<const uint32_t*>(r0);
            af[kb][1] = *reinterpret_cast<const uint32_t*>(r1);
            af[kb][2] = *reinterpret_cast<const uint32_t*>(r0 + 8);
            af[kb][3] = *reinterpret_cast<const uint32_t*>(r1 + 8);
        }
        const __nv_bfloat16* w = P.w[l];
#pragma unroll
        for (int n = 0; n < 8; n++) {
#pragma unroll
            for (int q = 0; q < 4; q++) acc[n][q] = 0.0f;
            const __nv_bfloat16* wr = w + (n * 8 + g) * kMlpLd;
#pragma unroll
            for (int kb = 0; kb < 4; kb++) {
                uint32_t b[2];
                b[0] = *reinterpret_cast<const uint32_t*>(wr + kb * 16 + 2 * t);
                b[1] = *reinterpret_cast<const uint32_t*>(wr + kb * 16 + 8 + 2 * t);
                mma_bf16(acc[n], af[kb], b);
            }
        }
        if (l == 2) break;
        const float* bias = P.b[l];
        __syncwarp();
#pragma unroll
        for (int n = 0; n < 8; n++) {
            const int c = n * 8 + 2 * t;
            const float b0 = bias[c], b1 = bias[c + 1];
            *reinterpret_cast<uint32_t*>(x + g * kMlpLd + c) =
                pack_bf16(fmaxf(acc[n][0] + b0, 0.f), fmaxf(acc[n][1] + b1, 0.f));
            *reinterpret_cast<uint32_t*>(x + (g + 8) * kMlpLd + c) =
                pack_bf16(fmaxf(acc[n][2] + b0, 0.f), fmaxf(acc[n][3] + b1, 0.f));
        }
        __syncwarp();
    }
    p0 = 0.f;
    p1 = 0.f;
#pragma unroll
    for (int n = 0; n < 8; n++) {
        const int c0 = n * 8 + 2 * t, c1 = c0 + 1;
        p0 += fmaxf(acc[n][0] + P.b[2][c0], 0.f) * P.w4[c0] + fmaxf(acc[n][1] + P.b[2][c1], 0.f) * P.w4[c1];
        p1 += fmaxf(acc[n][2] + P.b[2][c0], 0.f) * P.w4[c0] + fmaxf(acc[n][3] + P.b[2][c1], 0.f) * P.w4[c1];
    }
}

// Logits of the 32 rows in `x` (shared memory, 32 x kMlpLd bf16, clobbered):
// returns, in lane r, the logit of row r.
__device__ __forceinline__ float mlp_forward_warp(const MlpShared& P, __nv_bfloat16* x) {
    const int lane = threadIdx.x & 31;
    float part[2][2];  // [m][row g / g+8]
    // one copy of the tile code (instruction cache), two tiles
    float q0 = 0.f, q1 = 0.f;
#pragma unroll 1
    for (int m = 0; m < 2; m++) {
        float p0, p1;
        mlp_tile16(P, x + m * 16 * kMlpLd, p0, p1);
        if (m == 0) {
            q0 = p0;
            q1 = p1;
        } else {
            part[1][0] = p0;
            part[1][1] = p1;
        }
    }
    part[0][0] = q0;
    part[0][1] = q1;
#pragma unroll
    for (int m = 0; m < 2; m++)
#pragma unroll
        for (int h = 0; h < 2; h++) {
            part[m][h] += __shfl_xor_sync(0xffffffffu, part[m][h], 1);
            part[m][h] += __shfl_xor_sync(0xffffffffu, part[m][h], 2);
        }
    // row r = m*16 + h*8 + g lives in lanes 4g..4g+3; gather it into lane r
    const int m = lane >> 4, h = (lane >> 3) & 1, gg = lane & 7;
    float v0 = __shfl_sync(0xffffffffu, part[0][0], gg * 4);
    float v1 = __shfl_sync(0xffffffffu, part[0][1], gg * 4);
    float v2 = __shfl_sync(0xffffffffu, part[1][0], gg * 4);
    float v3 = __shfl_sync(0xffffffffu, part[1][1], gg * 4);
    float v = m == 0 ? (h == 0 ? v0 : v1) : (h == 0 ? v2 : v3);
    return v + P.b4;
}

#endif  // __CUDACC__

// Positional features of a segment from its end points (world units):
// per coordinate c of (a, b): c, sin(pi c 2^f), cos(pi c 2^f) for f = 0..3;
// then the direction b - a scaled to unit length, a constant 1 and zeros.
template <class F>
XRP_HD void segment_features(const float* a, const float* b, F&& put) {
    float p[6] = {a[0], a[1], a[2], b[0], b[1], b[2]};
    int k = 0;
#pragma unroll
    for (int c = 0; c < 6; c++) {
        put(k++, p[c]);
        float s, co;
        // base angle pi*c, then double-angle recurrences
#if defined(__CUDA_ARCH__)
        __sincosf(3.14159265358979f * p[c], &s, &co);
#else
        s = sinf(3.14159265358979f * p[c]);
        co = cosf(3.14159265358979f * p[c]);
#endif
#pragma unroll
        for (int f = 0; f < 4; f++) {
            put(k++, s);
            put(k++, co);
            float s2 = 2.0f * s * co, c2 = fmaf(2.0f * co, co, -1.0f);
            s = s2;
            co = c2;
        }
    }
    float dx = b[0] - a[0], dy = b[1] - a[1], dz = b[2] - a[2];
    float n = sqrtf(dx * dx + dy * dy + dz * dz);
    float in = n > 0.f ? 1.0f / n : 0.f;
    put(k++, dx * in);
    put(k++, dy * in);
    put(k++, dz * in);
    put(k++, 1.0f);
    while (k < kMlpIn) put(k++, 0.0f);
}

}  // namespace xrp
