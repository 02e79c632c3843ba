// xrp_train_tc.cuh -- the proposal network's training step on Blackwell's
// fifth-generation tensor cores (tcgen05).
//
// One CTA of 128 threads owns 128 rows (segments) of a batch; thread t is row
// t, and row t is TMEM lane t of the accumulator.  Every product is one
// tcgen05.mma group issued by a single thread: BF16 operands in shared
// memory, FP32 accumulator in TMEM (128 lanes x 64 columns), completion
// signalled on an mbarrier by tcgen05.commit, results read back with
// tcgen05.ld (each warp its 32 lanes):
//   forward   Z_l = relu(Z_{l-1} W_l^T + b_l)          M 128, N 64, K 64
//   backward  dZ_{l-1} = (dZ_l W_l) * relu'(Z_{l-1})   M 128, N 64, K 64
//             dW_l = dZ_l^T Z_{l-1}                    M 128 (64 used), N 64, K 128
// The rounding points are those of the FP64 oracle's emulation (oracle/mlp.py):
// activations and the backward dZ in BF16, Z3 and the head in FP32.
//
// Shared-memory operands use the canonical K-major layout without swizzle:
// 8-row x 16-byte core matrices, core matrices adjacent along K 128 bytes
// apart (leading byte offset), 8-row groups K/8 * 128 bytes apart (stride
// byte offset).  A K = 16 step of the MMA advances the start address by two
// core matrices (256 bytes).
#pragma once
#include "xrp_mlp.cuh"

namespace xrp {

constexpr int kTcRows = 128;  // rows per CTA = TMEM lanes = threads

// Operand tiles (bf16, K-major core-matrix layout) and block parameters.
struct TrainTcShared {
    __nv_bfloat16 x[kTcRows * 64];    // A of layer 1: rows x in
    __nv_bfloat16 z1[kTcRows * 64];   // A of layer 2
    __nv_bfloat16 z2[kTcRows * 64];   // A of layer 3
    __nv_bfloat16 xt[64 * kTcRows];   // B of dW1: in x rows
    __nv_bfloat16 z1t[64 * kTcRows];  // B of dW2
    __nv_bfloat16 z2t[64 * kTcRows];  // B of dW3
    __nv_bfloat16 w[3][64 * 64];      // B of the forward products: W_l [out][in]
    __nv_bfloat16 wt[2][64 * 64];     // B of the backward products: W2^T, W3^T [in][out]
    __nv_bfloat16 dz[kTcRows * 64];   // A of dZ W: rows x out
    __nv_bfloat16 dzt[kTcRows * kTcRows];  // A of dW: out x rows (out 64..127 zero)
    float b[3][64];
    float w4[64];
    float b4;
    float loss;
    unsigned long long mbar;
    uint32_t tmem;
};

#if defined(__CUDACC__) && defined(XRP_MLP_KERNELS)

// byte offset of element (r, k) of a K-major tile whose rows are kw wide
__device__ __forceinline__ uint32_t tc_off(int r, int k, int kw) {
    return (uint32_t)((r >> 3) * (kw * 16) + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

__device__ __forceinline__ uint32_t tc_smem(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor: start address, leading and stride byte
// offsets (16-byte units), descriptor version 1, no swizzle.
__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::f16: FP32 accumulator (bits 4-5 = 1), BF16
// A and B (bits 7-9, 10-12 = 1), both K-major, N >> 3 at bit 17, M >> 4 at
// bit 24: M = 128, N = 64.
constexpr uint32_t kTcIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((64u >> 3) << 17) | ((128u >> 4) << 24);

__device__ __forceinline__ void tc_mma(uint32_t dtmem, uint64_t ad, uint64_t bd, uint32_t accumulate) {
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(dtmem),
        "l"(ad), "l"(bd), "r"(kTcIdesc), "r"(accumulate));
}

__device__ __forceinline__ void tc_commit(uint32_t mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
                 : "memory");
}

__device__ __forceinline__ bool tc_try_wait(uint32_t mbar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(mbar), "r"(parity)
        : "memory");
    return ok != 0;
}

// Waits for phase `parity` of the mbarrier for at most `limit` polls.
__device__ __forceinline__ bool tc_wait(uint32_t mbar, uint32_t parity, int limit) {
    for (int q = 0; q < limit; q++)
        if (tc_try_wait(mbar, parity)) return true;
    return false;
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_proxy() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// 16 FP32 columns [col, col + 16) of this thread's TMEM lane.
__device__ __forceinline__ void tc_ld16(uint32_t taddr, float* v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, "
        "[%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
#pragma unroll
    for (int q = 0; q < 16; q++) v[q] = __uint_as_float(r[q]);
}

__device__ __forceinline__ void tc_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// The 64 accumulator columns of this thread's row.
__device__ __forceinline__ void tc_load_row(uint32_t tmem, float (&v)[64]) {
    const uint32_t lane_base = (uint32_t)((threadIdx.x >> 5) * 32) << 16;
#pragma unroll
    for (int c = 0; c < 64; c += 16) tc_ld16(tmem + lane_base + (uint32_t)c, v + c);
    tc_wait_ld();
}

// Row `r` of a 64-wide K-major tile from 64 floats (BF16 rounding).
__device__ __forceinline__ void tc_store_row(__nv_bfloat16* tile, int r, const float (&v)[64]) {
    unsigned char* base = reinterpret_cast<unsigned char*>(tile);
#pragma unroll
    for (int c = 0; c < 64; c += 8) {
        uint4 q;
        q.x = pack_bf16(v[c], v[c + 1]);
        q.y = pack_bf16(v[c + 2], v[c + 3]);
        q.z = pack_bf16(v[c + 4], v[c + 5]);
        q.w = pack_bf16(v[c + 6], v[c + 7]);
        *reinterpret_cast<uint4*>(base + tc_off(r, c, 64)) = q;
    }
}

// Column `r` of a transposed tile (64 rows, kTcRows wide): element (c, r).
__device__ __forceinline__ void tc_store_col(__nv_bfloat16* tile, int r, const float (&v)[64]) {
    unsigned char* base = reinterpret_cast<unsigned char*>(tile);
#pragma unroll
    for (int c = 0; c < 64; c++)
        *reinterpret_cast<__nv_bfloat16*>(base + tc_off(c, r, kTcRows)) = __float2bfloat16_rn(v[c]);
}

// Sum over the block's rows of v[c] (one value per thread and column) added
// to global `out[c]`: warp shuffles, one atomic per column per warp.
__device__ __forceinline__ void tc_colsum(const float (&v)[64], float* out) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int c = 0; c < 64; c++) {
        float s = v[c];
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) atomicAdd(&out[c], s);
    }
}

// Polls per wait before the step gives up (each poll may suspend the
// thread briefly): far beyond a product of microseconds.
constexpr int kTcPolls = 1 << 22;

// Tensor-core failures (a wait that ran out), read by the host after training.
__device__ unsigned g_mlp_tc_error;

// The training step on rows [blockIdx.x * 128, +128) of `rows` (row r is
// X[idx[r]] or X[r]; labels y): adds the gradient of
// inv_batch * sum_r w_r BCE(sigmoid(logit_r), y_r) (w_r = pos_weight for
// positive rows, 1 otherwise) to `grad` and the loss to `loss`; optionally
// writes the logits.  With `grad` null only the forward pass runs (the
// logits of validation rows; y and loss unused).
__global__ void __launch_bounds__(kTcRows, 1)
    k_mlp_train_tc(const float* __restrict__ params, const __nv_bfloat16* __restrict__ X,
                   const float* __restrict__ y, const int* __restrict__ idx, int rows, float pos_weight,
                   float inv_batch, float* __restrict__ grad, float* __restrict__ loss,
                   float* __restrict__ logits_out) {
    extern __shared__ __align__(1024) unsigned char tc_smem_raw[];
    TrainTcShared& S = *reinterpret_cast<TrainTcShared*>(
        tc_smem_raw + ((1024 - (tc_smem(tc_smem_raw) & 1023)) & 1023));
    const int t = threadIdx.x, warp = t >> 5;
    const int row = blockIdx.x * kTcRows + t;
    const bool valid = row < rows;

    // parameters: BF16 weights as B tiles, FP32 biases and head
    if (t < 64) {
        float wv[64];
        for (int l = 0; l < 3; l++) {
            const float* W = params + (l == 0 ? MlpLayout::W1 : l == 1 ? MlpLayout::W2 : MlpLayout::W3);
            for (int i = 0; i < 64; i++) wv[i] = W[t * 64 + i];  // row out = t of W_l
            tc_store_row(S.w[l], t, wv);
            if (l > 0) {
                for (int o = 0; o < 64; o++) wv[o] = W[o * 64 + t];  // row in = t of W_l^T
                tc_store_row(S.wt[l - 1], t, wv);
            }
        }
        S.b[0][t] = params[MlpLayout::B1 + t];
        S.b[1][t] = params[MlpLayout::B2 + t];
        S.b[2][t] = params[MlpLayout::B3 + t];
        S.w4[t] = params[MlpLayout::W4 + t];
    }
    // this thread's input row, in both orientations
    {
        float xv[64];
        if (valid) {
            const size_t src = idx ? (size_t)idx[row] : (size_t)row;
            const uint4* xr = reinterpret_cast<const uint4*>(X + src * kMlpIn);
#pragma unroll
            for (int c = 0; c < 8; c++) {
                const uint4 q = xr[c];
                const uint32_t u[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
                for (int h = 0; h < 4; h++) {
                    xv[8 * c + 2 * h] = __uint_as_float(u[h] << 16);
                    xv[8 * c + 2 * h + 1] = __uint_as_float(u[h] & 0xffff0000u);
                }
            }
        } else {
#pragma unroll
            for (int c = 0; c < 64; c++) xv[c] = 0.0f;
        }
        tc_store_row(S.x, t, xv);
        tc_store_col(S.xt, t, xv);
    }
    // rows 64..127 of the dW products' A stay zero
    for (int q = t; q < kTcRows * kTcRows / 2 / 8; q += kTcRows)
        reinterpret_cast<uint4*>(reinterpret_cast<unsigned char*>(S.dzt) + kTcRows * kTcRows)[q] =
            make_uint4(0, 0, 0, 0);
    if (t == 0) {
        S.b4 = params[MlpLayout::B4];
        S.loss = 0.0f;
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(tc_smem(&S.mbar)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 64;" ::"r"(tc_smem(&S.tmem))
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = S.tmem;
    const uint32_t mbar = tc_smem(&S.mbar);
    uint32_t phase = 0;
    bool ok = true;

    // one product: D = A B^T over `ksteps` K = 16 steps (A sbo, B sbo)
    auto product = [&](const void* a, uint32_t a_sbo, const void* b, uint32_t b_sbo, int ksteps) {
        tc_fence_proxy();  // this thread's operand writes, to the tensor core's proxy
        tc_fence_before();
        __syncthreads();
        if (t == 0) {
            tc_fence_after();
            const uint32_t sa = tc_smem(a), sb = tc_smem(b);
            for (int s = 0; s < ksteps; s++)
                tc_mma(tmem, tc_desc(sa + 256u * s, 128, a_sbo), tc_desc(sb + 256u * s, 128, b_sbo),
                       s > 0 ? 1u : 0u);
            tc_commit(mbar);
        }
        const bool done = tc_wait(mbar, phase, kTcPolls);
        phase ^= 1u;
        ok = __syncthreads_and(done ? 1 : 0) != 0 && ok;
        tc_fence_after();
    };

    float acc[64];
    // ---- forward
    product(S.x, 64 * 16, S.w[0], 64 * 16, 4);
    if (ok) {
        tc_load_row(tmem, acc);
#pragma unroll
        for (int c = 0; c < 64; c++) acc[c] = __bfloat162float(__float2bfloat16_rn(fmaxf(acc[c] + S.b[0][c], 0.0f)));
        tc_store_row(S.z1, t, acc);
        tc_store_col(S.z1t, t, acc);
        product(S.z1, 64 * 16, S.w[1], 64 * 16, 4);
    }
    if (ok) {
        tc_load_row(tmem, acc);
#pragma unroll
        for (int c = 0; c < 64; c++) acc[c] = __bfloat162float(__float2bfloat16_rn(fmaxf(acc[c] + S.b[1][c], 0.0f)));
        tc_store_row(S.z2, t, acc);
        tc_store_col(S.z2t, t, acc);
        product(S.z2, 64 * 16, S.w[2], 64 * 16, 4);
    }
    float dlog = 0.0f;  // d loss / d logit
    if (ok) {
        tc_load_row(tmem, acc);
        // head: z3 = relu(acc + b3) in FP32, logit, loss, dlogit
        float logit = S.b4;
#pragma unroll
        for (int c = 0; c < 64; c++) {
            acc[c] = fmaxf(acc[c] + S.b[2][c], 0.0f);
            logit = fmaf(acc[c], S.w4[c], logit);
        }
        if (logits_out && valid) logits_out[row] = logit;
        float yy = 0.0f, ww = 0.0f;
        if (valid && grad) {
            yy = y[idx ? idx[row] : row];
            ww = yy > 0.5f ? pos_weight : 1.0f;
        }
        const float sp = fmaxf(logit, 0.0f) + log1pf(expf(-fabsf(logit)));
        const float sg = 1.0f / (1.0f + expf(-logit));
        dlog = ww * (sg - yy) * inv_batch;
        atomicAdd(&S.loss, ww * (sp - yy * logit) * inv_batch);
    }
    if (ok && grad) {
        {
            float s = dlog;
            for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
            if ((t & 31) == 0) atomicAdd(&grad[MlpLayout::B4], s);
        }
        float g[64];
#pragma unroll
        for (int c = 0; c < 64; c++) g[c] = dlog * acc[c];
        tc_colsum(g, grad + MlpLayout::W4);
        // dz3 = dlogit w4 relu'(z3), then its bias gradient
#pragma unroll
        for (int c = 0; c < 64; c++) g[c] = acc[c] > 0.0f ? dlog * S.w4[c] : 0.0f;
        tc_colsum(g, grad + MlpLayout::B3);
        tc_store_row(S.dz, t, g);
        tc_store_col(S.dzt, t, g);
        product(S.dzt, kTcRows * 16, S.z2t, kTcRows * 16, 8);  // dW3
    }
    // backward through layers 3 and 2: dW_l from dZ_l^T Z_{l-1}, then
    // dZ_{l-1} = (dZ_l W_l) relu'(Z_{l-1})
    const __nv_bfloat16* zprev[2] = {S.z2, S.z1};  // Z_{l-1} rows for l = 3, 2
    const __nv_bfloat16* zprevt[2] = {S.z1t, S.xt};
    for (int l = 0; l < 2 && ok && grad; l++) {
        tc_load_row(tmem, acc);  // dW of layer 3 - l in lanes 0..63
        if (t < 64) {
            float* gw = grad + (l == 0 ? MlpLayout::W3 : MlpLayout::W2) + t * 64;
#pragma unroll
            for (int c = 0; c < 64; c++) atomicAdd(&gw[c], acc[c]);
        }
        product(S.dz, 64 * 16, S.wt[1 - l], 64 * 16, 4);  // dZ_l W_l
        if (!ok) break;
        tc_load_row(tmem, acc);
        const unsigned char* zr = reinterpret_cast<const unsigned char*>(zprev[l]);
#pragma unroll
        for (int c = 0; c < 64; c++) {
            const float z = __bfloat162float(*reinterpret_cast<const __nv_bfloat16*>(zr + tc_off(t, c, 64)));
            acc[c] = z > 0.0f ? acc[c] : 0.0f;
        }
        tc_colsum(acc, grad + (l == 0 ? MlpLayout::B2 : MlpLayout::B1));
        tc_store_row(S.dz, t, acc);
        tc_store_col(S.dzt, t, acc);
        product(S.dzt, kTcRows * 16, zprevt[l], kTcRows * 16, 8);  // dW of layer 2 - l
    }
    if (ok && grad) {
        tc_load_row(tmem, acc);  // dW1 in lanes 0..63
        if (t < 64) {
            float* gw = grad + MlpLayout::W1 + t * 64;
#pragma unroll
            for (int c = 0; c < 64; c++) atomicAdd(&gw[c], acc[c]);
        }
    } else if (!ok && t == 0) {
        atomicOr(&g_mlp_tc_error, 1u);
        tc_wait(mbar, phase, kTcPolls);  // a product still in flight, if any
    }
    tc_fence_before();
    __syncthreads();
    if (t == 0 && loss) atomicAdd(loss, S.loss);
    if (warp == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 64;" ::"r"(tmem) : "memory");
    }
}

#endif  // __CUDACC__ && XRP_MLP_KERNELS

}  // namespace xrp
