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

// Batches of scenes (general path): a persistent grid takes 256-pixel tiles
// from a global counter, so scenes, resolutions and view counts of uneven
// size share one launch and balance across SMs.  Items are ordered by
// decreasing work and their tiles numbered consecutively; a tile's item is
// found by binary search on the items' first tile.
template <bool HIER, int DEPTH, bool DEFS>
__global__ void __launch_bounds__(256, XRP_SCENE_MIN_BLOCKS)
    k_batch(const SceneDev* __restrict__ scenes, const BatchItemDev* __restrict__ items, int nitems,
            const ViewDev* __restrict__ views, const __grid_constant__ Lattice L, long long ntiles, int tw,
            int th, unsigned long long* __restrict__ counter, long long stride, long long limit,
            float* __restrict__ out) {
    __shared__ long long s_tile;
    __shared__ int s_item;
    for (;;) {
        if (threadIdx.x == 0) {
            unsigned long long k = atomicAdd(counter, 1ull);
            long long t = (long long)k < limit ? (long long)k * stride : ntiles;
            if (t >= ntiles) t = -1;
            int item = 0;
            if (t >= 0) {
                int lo = 0, hi = nitems - 1;
                while (lo < hi) {  // last item with tile0 <= t
                    int mid = (lo + hi + 1) >> 1;
                    if (items[mid].tile0 <= t) lo = mid;
                    else hi = mid - 1;
                }
                item = lo;
            }
            s_tile = t;
            s_item = item;
        }
        __syncthreads();
        const long long t = s_tile;
        const int it = s_item;
        __syncthreads();
        if (t < 0) break;
        const BatchItemDev& B = items[it];
        const int res = B.P.res;
        const long long local = t - B.tile0;
        const int tpv = B.tiles_x * B.tiles_y;
        const int v = (int)(local / tpv);
        const int tt = (int)(local - (long long)v * tpv);
        const int ty = tt / B.tiles_x, tx = tt - ty * B.tiles_x;
        const int i = ty * th + threadIdx.x / tw;
        const int j = tx * tw + threadIdx.x % tw;
        if (i < res && j < res) {
            RayStats st{0, 0};
            float val = render_pixel<HIER, false, DEPTH, DEFS>(scenes[B.scene], L, B.P, views[B.view0 + v], i, j, st);
            out[B.out0 + ((long long)v * res + i) * res + j] = val;
        }
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
