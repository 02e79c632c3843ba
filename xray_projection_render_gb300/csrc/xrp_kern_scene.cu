// xrp_kern_scene.cu -- the general-scene kernel (any object tree and
// deformation), one thread per pixel, specialised on the deepest
// tessellation nesting and on the presence of a deformation.
#include "xrp_launch.h"

namespace xrp {

// Minimum resident blocks per SM asked of the compiler (register budget)
// for the general-scene kernel, tuned on GB300.
#ifndef XRP_SCENE_MIN_BLOCKS
#define XRP_SCENE_MIN_BLOCKS 2
#endif

template <bool HIER, int DEPTH, bool DEFS>
__global__ void __launch_bounds__(256, XRP_SCENE_MIN_BLOCKS)
    k_render(const __grid_constant__ SceneDev S, const __grid_constant__ Lattice L,
             const __grid_constant__ RenderParams P, const ViewDev* __restrict__ views, int view0,
             int nviews, float* __restrict__ out, unsigned long long* __restrict__ stats) {
    const int res = P.res;
    const int tpr = (res + 15) >> 4;
    const int tpv = tpr * tpr;
    const int b = blockIdx.x;
    const int v = b / tpv;
    const int t = b - v * tpv;
    const int ti = t / tpr, tj = t - ti * tpr;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int i = (ti << 4) + ((warp >> 1) << 2) + (lane >> 3);
    const int j = (tj << 4) + ((warp & 1) << 3) + (lane & 7);
    RayStats st{0, 0};
    if (v < nviews && i < res && j < res) {
        float val = render_pixel<HIER, false, DEPTH, DEFS>(S, L, P, views[view0 + v], i, j, st);
        out[((size_t)v * res + i) * res + j] = val;
    }
    if (stats) {  // every lane reaches this point
        unsigned s = __reduce_add_sync(0xffffffffu, st.samples);
        unsigned f = __reduce_add_sync(0xffffffffu, st.fallbacks);
        if (lane == 0) {
            atomicAdd(&stats[0], (unsigned long long)s);
            if (f) atomicAdd(&stats[1], (unsigned long long)f);
        }
    }
}

// Batches of scenes (general path): every warp of a persistent grid takes
// 32-pixel tiles (tw x th) from a global counter, so scenes, resolutions
// and view counts of uneven size share one launch and balance across SMs
// without block barriers (rays differ in length; a block-wide tile would
// hold finished warps at a barrier).  Items are ordered by decreasing work
// and their tiles numbered consecutively; a tile's item is found by binary
// search on the items' first tile.  The tile's scene header, item
// parameters and view are staged in the warp's shared memory.
static_assert(sizeof(SceneDev) % 4 == 0 && sizeof(RenderParams) % 4 == 0 && sizeof(ViewDev) % 4 == 0,
              "staged structures are copied as 32-bit words");

struct BatchStage {
    SceneDev S;
    RenderParams P;
    ViewDev V;
};

template <bool HIER, int DEPTH, bool DEFS>
__global__ void __launch_bounds__(256, XRP_SCENE_MIN_BLOCKS)
    k_batch(const SceneDev* __restrict__ scenes, const BatchItemDev* __restrict__ items, int nitems,
            const ViewDev* __restrict__ views, const __grid_constant__ Lattice L, long long ntiles, int tw,
            int th, unsigned long long* __restrict__ counter, long long stride, long long limit,
            float* __restrict__ out) {
    __shared__ __align__(16) BatchStage stage[8];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    BatchStage& sg = stage[warp];
    for (;;) {
        long long t = -1;
        int item = 0;
        if (lane == 0) {
            unsigned long long k = atomicAdd(counter, 1ull);
            t = (long long)k < limit ? (long long)k * stride : ntiles;
            if (t >= ntiles) t = -1;
            if (t >= 0) {
                int lo = 0, hi = nitems - 1;
                while (lo < hi) {  // last item with tile0 <= t
                    int mid = (lo + hi + 1) >> 1;
                    if (items[mid].tile0 <= t) lo = mid;
                    else hi = mid - 1;
                }
                item = lo;
            }
        }
        t = __shfl_sync(0xffffffffu, t, 0);
        item = __shfl_sync(0xffffffffu, item, 0);
        if (t < 0) break;
        const BatchItemDev& B = items[item];
        const int res = B.P.res;
        const long long local = t - B.tile0;
        const int tpv = B.tiles_x * B.tiles_y;
        const int v = (int)(local / tpv);
        {
            const unsigned* src_s = reinterpret_cast<const unsigned*>(scenes + B.scene);
            const unsigned* src_p = reinterpret_cast<const unsigned*>(&B.P);
            const unsigned* src_v = reinterpret_cast<const unsigned*>(views + B.view0 + v);
            unsigned* ds_ = reinterpret_cast<unsigned*>(&sg.S);
            unsigned* dp_ = reinterpret_cast<unsigned*>(&sg.P);
            unsigned* dv_ = reinterpret_cast<unsigned*>(&sg.V);
            constexpr int ns = sizeof(SceneDev) / 4, np = sizeof(RenderParams) / 4, nv = sizeof(ViewDev) / 4;
            for (int q = lane; q < ns + np + nv; q += 32) {
                if (q < ns) ds_[q] = src_s[q];
                else if (q < ns + np) dp_[q - ns] = src_p[q - ns];
                else dv_[q - ns - np] = src_v[q - ns - np];
            }
        }
        __syncwarp();
        const int tt = (int)(local - (long long)v * tpv);
        const int ty = tt / B.tiles_x, tx = tt - ty * B.tiles_x;
        const int i = ty * th + lane / tw;
        const int j = tx * tw + lane % tw;
        if (i < res && j < res) {
            RayStats st{0, 0};
            float val = render_pixel<HIER, false, DEPTH, DEFS>(sg.S, L, sg.P, sg.V, i, j, st);
            out[B.out0 + ((long long)v * res + i) * res + j] = val;
        }
        __syncwarp();  // before the next tile overwrites the staged data
    }
}

template <bool HIER, int DEPTH, bool DEFS>
static cudaError_t launch_batch_t(const BatchLaunch& b, cudaStream_t st) {
    k_batch<HIER, DEPTH, DEFS><<<b.blocks, 256, 0, st>>>(b.scenes, b.items, b.nitems, b.views, b.L, b.ntiles,
                                                         b.tw, b.th, b.counter, b.stride, b.limit, b.out);
    return cudaGetLastError();
}

cudaError_t launch_batch(const BatchLaunch& b, cudaStream_t st) {
    if (b.blocks <= 0 || b.ntiles <= 0) return cudaSuccess;
    if (b.hier) {
        if (b.depth == 0) return b.defs ? launch_batch_t<true, 0, true>(b, st) : launch_batch_t<true, 0, false>(b, st);
        return b.defs ? launch_batch_t<true, 3, true>(b, st) : launch_batch_t<true, 3, false>(b, st);
    }
    if (b.depth == 0) return b.defs ? launch_batch_t<false, 0, true>(b, st) : launch_batch_t<false, 0, false>(b, st);
    return b.defs ? launch_batch_t<false, 3, true>(b, st) : launch_batch_t<false, 3, false>(b, st);
}

cudaError_t batch_blocks_per_sm(int depth, bool defs, bool hier, int* out) {
    const void* f;
    if (hier) {
        if (depth == 0) f = defs ? (const void*)k_batch<true, 0, true> : (const void*)k_batch<true, 0, false>;
        else f = defs ? (const void*)k_batch<true, 3, true> : (const void*)k_batch<true, 3, false>;
    } else {
        if (depth == 0) f = defs ? (const void*)k_batch<false, 0, true> : (const void*)k_batch<false, 0, false>;
        else f = defs ? (const void*)k_batch<false, 3, true> : (const void*)k_batch<false, 3, false>;
    }
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(out, f, 256, 0);
}

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
    dim3 grid((res + 32 * kFinishTiles - 1) / (32 * kFinishTiles), (res + 31) / 32, nviews);
    k_finish<<<grid, 256, 0, st>>>(img, res, transparency, gray, alpha, mm);
    k_minmax_final<<<(2 * nviews + 255) / 256, 256, 0, st>>>(mm, nviews);
    return cudaGetLastError();
}

cudaError_t launch_scene(const Prepared& pr, int view0, int nviews, bool hier, float* dout,
                         unsigned long long* stats, cudaStream_t st) {
    const int res = pr.P.res;
    const int tpr = (res + 15) / 16;
    long blocks = (long)nviews * tpr * tpr;
    if (blocks <= 0) return cudaSuccess;
    if (blocks > 0x7fffffffL) return cudaErrorInvalidConfiguration;
    dim3 grid((unsigned)blocks), block(256);
    const ViewDev* dviews = pr.views;
#define XRP_GEN(H, D, F) \
    k_render<H, D, F><<<grid, block, 0, st>>>(pr.S, pr.L, pr.P, dviews, view0, nviews, dout, stats)
#define XRP_GEN_D(H, F)                  \
    if (pr.depth == 0) XRP_GEN(H, 0, F); \
    else if (pr.depth == 1) XRP_GEN(H, 1, F); \
    else XRP_GEN(H, 3, F);
    if (hier) {
        if (pr.defs) { XRP_GEN_D(true, true) } else { XRP_GEN_D(true, false) }
    } else {
        if (pr.defs) { XRP_GEN_D(false, true) } else { XRP_GEN_D(false, false) }
    }
#undef XRP_GEN_D
#undef XRP_GEN
    return cudaGetLastError();
}

}  // namespace xrp
