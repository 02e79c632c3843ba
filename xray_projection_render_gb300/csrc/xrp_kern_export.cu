// xrp_kern_export.cu -- volume export of any scene and device-side image
// finishing.
#include "xrp_launch.h"

namespace xrp {

// Volume export of any scene (main.go:549-635): density(x, y, z) with the
// multiplier at x = i/res*2-1 (same for y with j, z with k), [k][i][j]
// layout.  FP32 guarded evaluation, FP64 (reference arithmetic) when a
// decision is uncertain, so values equal the reference's rounded to FP32.
template <int DEPTH, bool DEFS>
__global__ void __launch_bounds__(256)
    k_voxelize_scene(const __grid_constant__ SceneDev S, int res, double dm, float* __restrict__ out,
                     unsigned* __restrict__ vmax_bits) {
    const long long total = (long long)res * res * res;
    unsigned local = 0u;  // ordered bits of the running maximum
    for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x) {
        const int k = (int)(idx / ((long long)res * res));
        const int i = (int)((idx / res) % res);
        const int j = (int)(idx % res);
        const double rf = (double)res;
        const double x = (double)i / rf * 2.0 - 1.0, y = (double)j / rf * 2.0 - 1.0,
                     z = (double)k / rf * 2.0 - 1.0;
        float r32 = density32<DEPTH, DEFS>(S, (float)x, (float)y, (float)z);
        double r = isunc(r32) ? density_hyb(S, x, y, z) : (double)r32;
        const float v = (float)(r * dm);
        out[idx] = v;
        const unsigned b = __float_as_uint(v);
        const unsigned ob = (b & 0x80000000u) ? ~b : (b | 0x80000000u);  // order-preserving
        local = ob > local ? ob : local;
    }
    local = __reduce_max_sync(0xffffffffu, local);
    if ((threadIdx.x & 31) == 0) atomicMax(vmax_bits, local);
}

// byte(v / max * 255) of the export (main.go:622-626), in FP64; values
// below zero give 0 and a zero maximum gives 0 (the reference divides by 0).
__global__ void k_volume_u8(const float* __restrict__ v, long long n, const unsigned* __restrict__ vmax_bits,
                            unsigned char* __restrict__ out) {
    const unsigned ob = *vmax_bits;
    const unsigned b = (ob & 0x80000000u) ? (ob & 0x7fffffffu) : ~ob;
    const double mx = (double)__uint_as_float(b);
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
        double t = mx > 0.0 ? (double)v[q] / mx * 255.0 : 0.0;
        out[q] = (unsigned char)(t <= 0.0 ? 0.0 : (t >= 255.0 ? 255.0 : t));
    }
}

cudaError_t launch_voxelize_scene(const SceneDev& S, int depth, bool defs, int res, double dm, float* out,
                                  unsigned* vmax_bits, unsigned char* u8, cudaStream_t st) {
    const long long total = (long long)res * res * res;
    long long blocks = (total + 255) / 256;
    if (blocks > 152LL * 32) blocks = 152LL * 32;
    if (blocks < 1) blocks = 1;
    cudaError_t e = cudaMemsetAsync(vmax_bits, 0, sizeof(unsigned), st);
    if (e != cudaSuccess) return e;
    if (depth == 0) {
        if (defs) k_voxelize_scene<0, true><<<(unsigned)blocks, 256, 0, st>>>(S, res, dm, out, vmax_bits);
        else k_voxelize_scene<0, false><<<(unsigned)blocks, 256, 0, st>>>(S, res, dm, out, vmax_bits);
    } else {
        if (defs) k_voxelize_scene<kMaxDepth, true><<<(unsigned)blocks, 256, 0, st>>>(S, res, dm, out, vmax_bits);
        else k_voxelize_scene<kMaxDepth, false><<<(unsigned)blocks, 256, 0, st>>>(S, res, dm, out, vmax_bits);
    }
    if (u8) k_volume_u8<<<(unsigned)blocks, 256, 0, st>>>(out, total, vmax_bits, u8);
    return cudaGetLastError();
}

// Image finishing on the device (main.go:482-506, cuda_path.go:104-130):
// gray = uint16(val * 0xffff) stored at PNG pixel (x = i, y = res-1-j),
// alpha = 0xffff, or with transparency 0xffff where val < 1 and 0 elsewhere,
// and each image's min and max.  32x32 tiles through shared memory so both
// the read (along j) and the flipped write (along x = i) are coalesced; a
// block walks a strip of kFinishTiles tiles along j and adds its min/max
// with one atomic pair (per-view atomics from every warp contend in L2).
constexpr int kFinishTiles = 8;
__global__ void __launch_bounds__(256)
    k_finish(const float* __restrict__ img, int res, int transparency, unsigned short* __restrict__ gray,
             unsigned short* __restrict__ alpha, unsigned* __restrict__ minmax_bits) {
    __shared__ float tile[32][33];
    __shared__ unsigned red[2][8];
    const int v = blockIdx.z;
    const int i0 = blockIdx.y * 32;
    const float* src = img + (size_t)v * res * res;
    const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8 threads
    unsigned lo = 0xffffffffu, hi = 0u;                       // ordered bits
    for (int tj = 0; tj < kFinishTiles; tj++) {
        const int j0 = (blockIdx.x * kFinishTiles + tj) * 32;
        if (j0 >= res) break;
        for (int r = ty; r < 32; r += 8) {
            const int i = i0 + r, j = j0 + tx;
            float val = 0.0f;
            if (i < res && j < res) {
                val = src[(size_t)i * res + j];
                const unsigned b = __float_as_uint(val);
                const unsigned ob = (b & 0x80000000u) ? ~b : (b | 0x80000000u);
                lo = ob < lo ? ob : lo;
                hi = ob > hi ? ob : hi;
            }
            tile[r][tx] = val;
        }
        __syncthreads();
        // output row y = res-1-j (j = j0 + c), column x = i (i = i0 + tx)
        for (int c = ty; c < 32; c += 8) {
            const int j = j0 + c, i = i0 + tx;
            if (i < res && j < res) {
                const float val = tile[tx][c];
                // uint16(float64(val) * 0xffff): the product is exact in FP64;
                // in FP32 it is p + e exactly (e by FMA), and truncation of
                // p + e is trunc(p), less one when p is whole and e < 0
                const float p = val * 65535.0f;
                const float e = fmaf(val, 65535.0f, -p);
                float t = truncf(p);
                if (t == p && e < 0.0f) t -= 1.0f;
                t = t <= 0.0f ? 0.0f : (t >= 65535.0f ? 65535.0f : t);
                const size_t o = (size_t)v * res * res + (size_t)(res - 1 - j) * res + i;
                gray[o] = (unsigned short)t;
                if (alpha) alpha[o] = transparency ? (val < 1.0f ? 0xffff : 0) : 0xffff;
            }
        }
        __syncthreads();
    }
    lo = __reduce_min_sync(0xffffffffu, lo);
    hi = __reduce_max_sync(0xffffffffu, hi);
    if (tx == 0) {
        red[0][ty] = lo;
        red[1][ty] = hi;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int q = 1; q < 8; q++) {
            lo = red[0][q] < lo ? red[0][q] : lo;
            hi = red[1][q] > hi ? red[1][q] : hi;
        }
        atomicMin(&minmax_bits[2 * v], lo);
        atomicMax(&minmax_bits[2 * v + 1], hi);
    }
}

// The same finishing for images whose side is a multiple of 4 and whose
// buffers are 16-byte (input) and 8-byte (outputs) aligned: 64x64 tiles,
// each thread issuing its tile's four 16-byte loads before it touches any
// (16 KB in flight per block, streaming loads: the images are read once)
// and writing four output pixels of a row with one 8-byte store.  A block
// walks kFinishVTiles tiles along j.
constexpr int kFinishVTiles = 4;
__global__ void __launch_bounds__(256)
    k_finish_v4(const float* __restrict__ img, int res, int transparency, unsigned short* __restrict__ gray,
                unsigned short* __restrict__ alpha, unsigned* __restrict__ minmax_bits) {
    __shared__ float tile[64][65];
    __shared__ unsigned red[2][8];
    const int v = blockIdx.z;
    const int i0 = blockIdx.y * 64;
    const float* src = img + (size_t)v * res * res;
    const int lx = threadIdx.x & 15, ly = threadIdx.x >> 4;  // 16 x 16 threads
    unsigned lo = 0xffffffffu, hi = 0u;                       // ordered bits
    for (int tj = 0; tj < kFinishVTiles; tj++) {
        const int j0 = (blockIdx.x * kFinishVTiles + tj) * 64;
        if (j0 >= res) break;
        const int j = j0 + 4 * lx;  // j < res implies j + 3 < res (res % 4 == 0)
        float4 q[4];
#pragma unroll
        for (int p = 0; p < 4; p++) {
            const int i = i0 + ly + 16 * p;
            q[p] = (i < res && j < res) ? __ldcs(reinterpret_cast<const float4*>(src + (size_t)i * res + j))
                                        : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        }
#pragma unroll
        for (int p = 0; p < 4; p++) {
            const int i = i0 + ly + 16 * p;
            const float e[4] = {q[p].x, q[p].y, q[p].z, q[p].w};
            if (i < res && j < res) {
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    const unsigned b = __float_as_uint(e[k]);
                    const unsigned ob = (b & 0x80000000u) ? ~b : (b | 0x80000000u);
                    lo = ob < lo ? ob : lo;
                    hi = ob > hi ? ob : hi;
                }
            }
            float* t = &tile[ly + 16 * p][4 * lx];
#pragma unroll
            for (int k = 0; k < 4; k++) t[k] = e[k];
        }
        __syncthreads();
        // output rows y = res-1-j (j = j0 + c), columns x = i0 + 4*lx .. +3
        const int i = i0 + 4 * lx;
#pragma unroll
        for (int p = 0; p < 4; p++) {
            const int c = ly + 16 * p;
            const int jj = j0 + c;
            if (jj < res && i < res) {
                unsigned short g[4], a[4];
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    const float val = tile[4 * lx + k][c];
                    // uint16(float64(val) * 0xffff), as in k_finish
                    const float pr = val * 65535.0f;
                    const float er = fmaf(val, 65535.0f, -pr);
                    float t = truncf(pr);
                    if (t == pr && er < 0.0f) t -= 1.0f;
                    t = t <= 0.0f ? 0.0f : (t >= 65535.0f ? 65535.0f : t);
                    g[k] = (unsigned short)t;
                    a[k] = transparency ? (val < 1.0f ? 0xffff : 0) : 0xffff;
                }
                const size_t o = (size_t)v * res * res + (size_t)(res - 1 - jj) * res + i;
                *reinterpret_cast<ushort4*>(gray + o) = make_ushort4(g[0], g[1], g[2], g[3]);
                if (alpha) *reinterpret_cast<ushort4*>(alpha + o) = make_ushort4(a[0], a[1], a[2], a[3]);
            }
        }
        __syncthreads();
    }
    lo = __reduce_min_sync(0xffffffffu, lo);
    hi = __reduce_max_sync(0xffffffffu, hi);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) {
        red[0][warp] = lo;
        red[1][warp] = hi;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < 8; w++) {
            lo = red[0][w] < lo ? red[0][w] : lo;
            hi = red[1][w] > hi ? red[1][w] : hi;
        }
        atomicMin(&minmax_bits[2 * v], lo);
        atomicMax(&minmax_bits[2 * v + 1], hi);
    }
}

__global__ void k_minmax_init(unsigned* mm, int n) {
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
        mm[2 * q] = 0xffffffffu;
        mm[2 * q + 1] = 0u;
    }
}

// Ordered bits back to floats, in place.
__global__ void k_minmax_final(unsigned* mm, int n) {
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < 2 * n; q += gridDim.x * blockDim.x) {
        const unsigned ob = mm[q];
        mm[q] = (ob & 0x80000000u) ? (ob & 0x7fffffffu) : ~ob;
    }
}

cudaError_t launch_finish(const float* img, int nviews, int res, int transparency, unsigned short* gray,
                          unsigned short* alpha, float* minmax, cudaStream_t st) {
    if (nviews <= 0 || res <= 0) return cudaSuccess;
    unsigned* mm = reinterpret_cast<unsigned*>(minmax);
    int ib = (nviews + 255) / 256;
    k_minmax_init<<<ib, 256, 0, st>>>(mm, nviews);
    const bool vec = res % 4 == 0 && ((uintptr_t)img & 15) == 0 && ((uintptr_t)gray & 7) == 0 &&
                     ((uintptr_t)alpha & 7) == 0;
    if (vec) {
        dim3 grid((res + 64 * kFinishVTiles - 1) / (64 * kFinishVTiles), (res + 63) / 64, nviews);
        k_finish_v4<<<grid, 256, 0, st>>>(img, res, transparency, gray, alpha, mm);
    } else {
        dim3 grid((res + 32 * kFinishTiles - 1) / (32 * kFinishTiles), (res + 31) / 32, nviews);
        k_finish<<<grid, 256, 0, st>>>(img, res, transparency, gray, alpha, mm);
    }
    k_minmax_final<<<(2 * nviews + 255) / 256, 256, 0, st>>>(mm, nviews);
    return cudaGetLastError();
}

}  // namespace xrp
