// xrp_train.cuh -- training of the proposal MLP on tensor cores.
//
// One block of 4 warps handles 128 rows (segments) of a batch: forward with
// mma.sync (BF16 operands, FP32 accumulation), weighted binary cross-entropy
// on the logits, and backward: input gradients dz_l = dz_{l+1} W_{l+1} and
// weight gradients dW = dz^T z as m16n8k16 products too.  Gradients are
// summed per block in shared memory and added to the FP32 gradient buffer
// with one atomic per parameter per block; Adam then updates the FP32 master
// weights and their BF16 copy.
#pragma once
#include "xrp_mlp.cuh"

namespace xrp {

constexpr int kTrainWarps = 4;
constexpr int kTrainRows = 32 * kTrainWarps;

struct TrainShared {
    __nv_bfloat16 x[kTrainRows * kMlpLd];
    __nv_bfloat16 z1[kTrainRows * kMlpLd];
    __nv_bfloat16 z2[kTrainRows * kMlpLd];
    __nv_bfloat16 dz[kTrainRows * kMlpLd];
    __nv_bfloat16 w[3][kMlpHid * kMlpLd];   // W_l as [out][in]
    __nv_bfloat16 wt[3][kMlpHid * kMlpLd];  // W_l^T as [in][out] (W1^T unused)
    float b[3][kMlpHid];
    float w4[kMlpHid];
    float b4;
    float grad[MlpLayout::N];
    float loss;
};

#if defined(__CUDACC__)

__device__ __forceinline__ uint32_t pack2(__nv_bfloat16 lo, __nv_bfloat16 hi) {
    return (uint32_t)__bfloat16_as_ushort(lo) | ((uint32_t)__bfloat16_as_ushort(hi) << 16);
}

// gW[n][i] += sum over the warp's 32 rows of dz[r][n] * z[r][i] (tensor
// cores, K = rows), accumulated into shared FP32 `gw` ([n][i], 64 x 64).
__device__ __forceinline__ void weight_grad(const __nv_bfloat16* dz, const __nv_bfloat16* z, float* gw) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    for (int mt = 0; mt < 4; mt++) {
        float acc[8][4];
#pragma unroll
        for (int n = 0; n < 8; n++)
#pragma unroll
            for (int q = 0; q < 4; q++) acc[n][q] = 0.f;
#pragma unroll
        for (int ks = 0; ks < 2; ks++) {
            const int r0 = ks * 16 + 2 * t;
            const int nr = mt * 16 + g;
            uint32_t a[4];
            a[0] = pack2(dz[(r0)*kMlpLd + nr], dz[(r0 + 1) * kMlpLd + nr]);
            a[1] = pack2(dz[(r0)*kMlpLd + nr + 8], dz[(r0 + 1) * kMlpLd + nr + 8]);
            a[2] = pack2(dz[(r0 + 8) * kMlpLd + nr], dz[(r0 + 9) * kMlpLd + nr]);
            a[3] = pack2(dz[(r0 + 8) * kMlpLd + nr + 8], dz[(r0 + 9) * kMlpLd + nr + 8]);
#pragma unroll
            for (int nt = 0; nt < 8; nt++) {
                const int ic = nt * 8 + g;
                uint32_t b[2];
                b[0] = pack2(z[(r0)*kMlpLd + ic], z[(r0 + 1) * kMlpLd + ic]);
                b[1] = pack2(z[(r0 + 8) * kMlpLd + ic], z[(r0 + 9) * kMlpLd + ic]);
                mma_bf16(acc[nt], a, b);
            }
        }
#pragma unroll
        for (int nt = 0; nt < 8; nt++) {
            const int row = mt * 16 + g, col = nt * 8 + 2 * t;
            atomicAdd(&gw[row * kMlpIn + col], acc[nt][0]);
            atomicAdd(&gw[row * kMlpIn + col + 1], acc[nt][1]);
            atomicAdd(&gw[(row + 8) * kMlpIn + col], acc[nt][2]);
            atomicAdd(&gw[(row + 8) * kMlpIn + col + 1], acc[nt][3]);
        }
    }
}

// Store FP32 D-layout values (rows g, g+8 of two m-tiles, 8 n-tiles) as BF16
// rows of `dst` (the warp's 32-row region).
__device__ __forceinline__ void store_rows(const float (&v)[2][8][4], __nv_bfloat16* dst) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll
    for (int m = 0; m < 2; m++)
#pragma unroll
        for (int n = 0; n < 8; n++) {
            const int c = n * 8 + 2 * t;
            *reinterpret_cast<uint32_t*>(dst + (m * 16 + g) * kMlpLd + c) = pack_bf16(v[m][n][0], v[m][n][1]);
            *reinterpret_cast<uint32_t*>(dst + (m * 16 + g + 8) * kMlpLd + c) = pack_bf16(v[m][n][2], v[m][n][3]);
        }
}

// dz (FP32, D layout) -> A fragments for the product dz * W
__device__ __forceinline__ void pack_a(const float (&v)[2][8][4], uint32_t (&af)[2][4][4]) {
#pragma unroll
    for (int m = 0; m < 2; m++)
#pragma unroll
        for (int kb = 0; kb < 4; kb++) {
            af[m][kb][0] = pack_bf16(v[m][2 * kb][0], v[m][2 * kb][1]);
            af[m][kb][1] = pack_bf16(v[m][2 * kb][2], v[m][2 * kb][3]);
            af[m][kb][2] = pack_bf16(v[m][2 * kb + 1][0], v[m][2 * kb + 1][1]);
            af[m][kb][3] = pack_bf16(v[m][2 * kb + 1][2], v[m][2 * kb + 1][3]);
        }
}

// Multiply D-layout values by the ReLU derivative read from BF16 activation
// rows (z > 0) and sum columns into the bias gradient (shared atomics).
__device__ __forceinline__ void relu_back(float (&v)[2][8][4], const __nv_bfloat16* z, float* gb) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll
    for (int n = 0; n < 8; n++) {
        const int c = n * 8 + 2 * t;
        float s0 = 0.f, s1 = 0.f;
#pragma unroll
        for (int m = 0; m < 2; m++) {
            const __nv_bfloat16* r0 = z + (m * 16 + g) * kMlpLd + c;
            const __nv_bfloat16* r1 = r0 + 8 * kMlpLd;
            v[m][n][0] = __bfloat162float(r0[0]) > 0.f ? v[m][n][0] : 0.f;
            v[m][n][1] = __bfloat162float(r0[1]) > 0.f ? v[m][n][1] : 0.f;
            v[m][n][2] = __bfloat162float(r1[0]) > 0.f ? v[m][n][2] : 0.f;
            v[m][n][3] = __bfloat162float(r1[1]) > 0.f ? v[m][n][3] : 0.f;
            s0 += v[m][n][0] + v[m][n][2];
            s1 += v[m][n][1] + v[m][n][3];
        }
        // sum over the 8 row groups (lanes with the same t)
        for (int o = 4; o < 32; o <<= 1) {
            s0 += __shfl_xor_sync(0xffffffffu, s0, o);
            s1 += __shfl_xor_sync(0xffffffffu, s1, o);
        }
        if (g == 0) {
            atomicAdd(&gb[c], s0);
            atomicAdd(&gb[c + 1], s1);
        }
    }
}

#if defined(XRP_MLP_KERNELS)
// One training pass over `rows` rows (row r is X[idx[r]], or X[r] without
// an index) of BF16 features ([.][64]) and 0/1 labels y.  Adds the gradient
// of inv_batch * sum_r w_r * BCE(sigmoid(logit_r), y_r), w_r = pos_weight for
// positive rows and 1 otherwise, to `grad` and the loss to `loss`;
// optionally writes the logits.
__global__ void __launch_bounds__(kTrainRows)
    k_mlp_train(const float* __restrict__ params, const __nv_bfloat16* __restrict__ X,
                const float* __restrict__ y, const int* __restrict__ idx, int rows, float pos_weight,
                float inv_batch, float* __restrict__ grad, float* __restrict__ loss,
                float* __restrict__ logits_out) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    TrainShared& S = *reinterpret_cast<TrainShared*>(smem_raw);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, g = lane >> 2, t = lane & 3;
    const int row0 = blockIdx.x * kTrainRows;
    // parameters -> shared (BF16 weights, FP32 biases), zero the block gradient
    for (int q = tid; q < kMlpHid * kMlpIn; q += blockDim.x) {
        int o = q / kMlpIn, i = q % kMlpIn;
        for (int l = 0; l < 3; l++) {
            const float* W = params + (l == 0 ? MlpLayout::W1 : l == 1 ? MlpLayout::W2 : MlpLayout::W3);
            __nv_bfloat16 wv = __float2bfloat16_rn(W[q]);
            S.w[l][o * kMlpLd + i] = wv;
            S.wt[l][i * kMlpLd + o] = wv;
        }
    }
    for (int q = tid; q < kMlpHid; q += blockDim.x) {
        S.b[0][q] = params[MlpLayout::B1 + q];
        S.b[1][q] = params[MlpLayout::B2 + q];
        S.b[2][q] = params[MlpLayout::B3 + q];
        S.w4[q] = params[MlpLayout::W4 + q];
    }
    if (tid == 0) {
        S.b4 = params[MlpLayout::B4];
        S.loss = 0.f;
    }
    for (int q = tid; q < MlpLayout::N; q += blockDim.x) S.grad[q] = 0.f;
    for (int q = tid; q < kTrainRows * kMlpIn / 2; q += blockDim.x) {
        int r = q / (kMlpIn / 2), c = q % (kMlpIn / 2);
        int gr = row0 + r;
        uint32_t v = 0;
        if (gr < rows) {
            size_t src = idx ? (size_t)idx[gr] : (size_t)gr;
            v = reinterpret_cast<const uint32_t*>(X + src * kMlpIn)[c];
        }
        reinterpret_cast<uint32_t*>(S.x + r * kMlpLd)[c] = v;
    }
    __syncthreads();
    __nv_bfloat16* xw = S.x + warp * 32 * kMlpLd;
    __nv_bfloat16* z1w = S.z1 + warp * 32 * kMlpLd;
    __nv_bfloat16* z2w = S.z2 + warp * 32 * kMlpLd;
    __nv_bfloat16* dzw = S.dz + warp * 32 * kMlpLd;
    // ---- forward
    uint32_t af[2][4][4];
    float acc[2][8][4];
    mlp_load_a(xw, af);
    mlp_layer(af, S.w[0], acc);
    mlp_relu_pack(acc, S.b[0], af);
    // z1 rows (post-ReLU BF16) for the weight gradient of layer 2
#pragma unroll
    for (int m = 0; m < 2; m++)
#pragma unroll
        for (int kb = 0; kb < 4; kb++) {
            const int c = kb * 16 + 2 * t;
            *reinterpret_cast<uint32_t*>(z1w + (m * 16 + g) * kMlpLd + c) = af[m][kb][0];
            *reinterpret_cast<uint32_t*>(z1w + (m * 16 + g + 8) * kMlpLd + c) = af[m][kb][1];
            *reinterpret_cast<uint32_t*>(z1w + (m * 16 + g) * kMlpLd + c + 8) = af[m][kb][2];
            *reinterpret_cast<uint32_t*>(z1w + (m * 16 + g + 8) * kMlpLd + c + 8) = af[m][kb][3];
        }
    mlp_layer(af, S.w[1], acc);
    mlp_relu_pack(acc, S.b[1], af);
#pragma unroll
    for (int m = 0; m < 2; m++)
#pragma unroll
        for (int kb = 0; kb < 4; kb++) {
            const int c = kb * 16 + 2 * t;
            *reinterpret_cast<uint32_t*>(z2w + (m * 16 + g) * kMlpLd + c) = af[m][kb][0];
            *reinterpret_cast<uint32_t*>(z2w + (m * 16 + g + 8) * kMlpLd + c) = af[m][kb][1];
            *reinterpret_cast<uint32_t*>(z2w + (m * 16 + g) * kMlpLd + c + 8) = af[m][kb][2];
            *reinterpret_cast<uint32_t*>(z2w + (m * 16 + g + 8) * kMlpLd + c + 8) = af[m][kb][3];
        }
    mlp_layer(af, S.w[2], acc);  // z3 pre-activation (bias not yet added)
    // z3 = relu(acc + b3); logits per row (rows g, g+8 of each m-tile)
    float z3[2][8][4];
    float part[2][2] = {{0.f, 0.f}, {0.f, 0.f}};
#pragma unroll
    for (int m = 0; m < 2; m++)
#pragma unroll
        for (int n = 0; n < 8; n++) {
            const int c0 = n * 8 + 2 * t, c1 = c0 + 1;
            z3[m][n][0] = fmaxf(acc[m][n][0] + S.b[2][c0], 0.f);
            z3[m][n][1] = fmaxf(acc[m][n][1] + S.b[2][c1], 0.f);
            z3[m][n][2] = fmaxf(acc[m][n][2] + S.b[2][c0], 0.f);
            z3[m][n][3] = fmaxf(acc[m][n][3] + S.b[2][c1], 0.f);
            part[m][0] += z3[m][n][0] * S.w4[c0] + z3[m][n][1] * S.w4[c1];
            part[m][1] += z3[m][n][2] * S.w4[c0] + z3[m][n][3] * S.w4[c1];
        }
    float dlog[2][2];
#pragma unroll
    for (int m = 0; m < 2; m++)
#pragma unroll
        for (int h = 0; h < 2; h++) {
            float p = part[m][h];
            p += __shfl_xor_sync(0xffffffffu, p, 1);
            p += __shfl_xor_sync(0xffffffffu, p, 2);
            const float logit = p + S.b4;
            const int r = row0 + warp * 32 + m * 16 + h * 8 + g;
            float yy = 0.f, ww = 0.f;
            if (r < rows) {
                yy = y[idx ? idx[r] : r];
                ww = yy > 0.5f ? pos_weight : 1.0f;
            }
            // BCE with logits: softplus(l) - y l ; d/dl = sigmoid(l) - y
            const float sp = fmaxf(logit, 0.f) + log1pf(expf(-fabsf(logit)));
            const float sg = 1.0f / (1.0f + expf(-logit));
            dlog[m][h] = ww * (sg - yy) * inv_batch;
            if (t == 0) {
                atomicAdd(&S.loss, ww * (sp - yy * logit) * inv_batch);
                if (logits_out && r < rows) logits_out[r] = logit;
            }
        }
    // output layer gradients
    float gb4 = 0.f;
#pragma unroll
    for (int m = 0; m < 2; m++) gb4 += dlog[m][0] + dlog[m][1];
    if (t == 0) atomicAdd(&S.grad[MlpLayout::B4], gb4);
#pragma unroll
    for (int n = 0; n < 8; n++) {
        const int c = n * 8 + 2 * t;
        float s0 = 0.f, s1 = 0.f;
#pragma unroll
        for (int m = 0; m < 2; m++) {
            s0 += dlog[m][0] * z3[m][n][0] + dlog[m][1] * z3[m][n][2];
            s1 += dlog[m][0] * z3[m][n][1] + dlog[m][1] * z3[m][n][3];
        }
        for (int o = 4; o < 32; o <<= 1) {
            s0 += __shfl_xor_sync(0xffffffffu, s0, o);
            s1 += __shfl_xor_sync(0xffffffffu, s1, o);
        }
        if (g == 0) {
            atomicAdd(&S.grad[MlpLayout::W4 + c], s0);
            atomicAdd(&S.grad[MlpLayout::W4 + c + 1], s1);
        }
    }
    // dz3 (pre-activation) = dlogit * w4 * relu'(z3)
    float dz[2][8][4];
#pragma unroll
    for (int m = 0; m < 2; m++)
#pragma unroll
        for (int n = 0; n < 8; n++) {
            const int c0 = n * 8 + 2 * t, c1 = c0 + 1;
            dz[m][n][0] = z3[m][n][0] > 0.f ? dlog[m][0] * S.w4[c0] : 0.f;
            dz[m][n][1] = z3[m][n][1] > 0.f ? dlog[m][0] * S.w4[c1] : 0.f;
            dz[m][n][2] = z3[m][n][2] > 0.f ? dlog[m][1] * S.w4[c0] : 0.f;
            dz[m][n][3] = z3[m][n][3] > 0.f ? dlog[m][1] * S.w4[c1] : 0.f;
        }
    // b3 gradient
#pragma unroll
    for (int n = 0; n < 8; n++) {
        const int c = n * 8 + 2 * t;
        float s0 = dz[0][n][0] + dz[0][n][2] + dz[1][n][0] + dz[1][n][2];
        float s1 = dz[0][n][1] + dz[0][n][3] + dz[1][n][1] + dz[1][n][3];
        for (int o = 4; o < 32; o <<= 1) {
            s0 += __shfl_xor_sync(0xffffffffu, s0, o);
            s1 += __shfl_xor_sync(0xffffffffu, s1, o);
        }
        if (g == 0) {
            atomicAdd(&S.grad[MlpLayout::B3 + c], s0);
            atomicAdd(&S.grad[MlpLayout::B3 + c + 1], s1);
        }
    }
    // layer 3: dW3 = dz3^T z2 ; dz2 = dz3 W3 (through W3^T rows) * relu'(z2)
    store_rows(dz, dzw);
    __syncwarp();
    weight_grad(dzw, z2w, S.grad + MlpLayout::W3);
    pack_a(dz, af);
    mlp_layer(af, S.wt[2], dz);
    relu_back(dz, z2w, S.grad + MlpLayout::B2);
    __syncwarp();
    store_rows(dz, dzw);
    __syncwarp();
    weight_grad(dzw, z1w, S.grad + MlpLayout::W2);
    pack_a(dz, af);
    mlp_layer(af, S.wt[1], dz);
    relu_back(dz, z1w, S.grad + MlpLayout::B1);
    __syncwarp();
    store_rows(dz, dzw);
    __syncwarp();
    weight_grad(dzw, xw, S.grad + MlpLayout::W1);
    __syncthreads();
    for (int q = tid; q < MlpLayout::N; q += blockDim.x) atomicAdd(&grad[q], S.grad[q]);
    if (tid == 0) atomicAdd(loss, S.loss);
}

// Adam on the FP32 master parameters; clears the gradient.
__global__ void k_mlp_adam(float* __restrict__ params, float* __restrict__ grad, float* __restrict__ m1,
                           float* __restrict__ m2, int n, float lr, float b1, float b2, float eps,
                           float c1, float c2) {
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
        float gq = grad[q];
        float a = b1 * m1[q] + (1.f - b1) * gq;
        float v = b2 * m2[q] + (1.f - b2) * gq * gq;
        m1[q] = a;
        m2[q] = v;
        params[q] -= lr * (a * c1) / (sqrtf(v * c2) + eps);
        grad[q] = 0.f;
    }
}

#endif  // XRP_MLP_KERNELS

#endif  // __CUDACC__

}  // namespace xrp
