// xrp_batch.cuh -- the batch kernel template (many scenes of uneven size in
// one persistent launch) and its launch helpers.  Each certificate mode is
// instantiated in its own translation unit (xrp_kern_batch*.cu) so that
// they compile in parallel.
#pragma once
#include "xrp_launch.h"

namespace xrp {

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

// TRACE: 0 plain integrator, 1 certificate tracing with ball certificates,
// 2 with ray certificates (every scene of the batch has an affine chain),
// 3 with curve certificates (some scene has a non-affine chain).
// Resident blocks per SM (register budget) measured on GB300 for tracing:
// 4 (64 registers). Ray bounds on the 64-scene batch: 4116 Mrays/s with 2
// blocks, 4591 with 3, 4809 with 4, 4841 with 5; ball certificates: 1678
// with 3, 1911 with 4 (spills cost less than the lost warps).
// XRP_BATCH_MERGE: tracing serves the warp's FP64 re-evaluations together.
#ifndef XRP_BATCH_MERGE
#define XRP_BATCH_MERGE 1
#endif
template <bool HIER, int DEPTH, bool DEFS, int TRACE>
__global__ void __launch_bounds__(256, (TRACE && DEPTH < 3) ? 4 : XRP_SCENE_MIN_BLOCKS)
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
        const unsigned wm = __ballot_sync(0xffffffffu, i < res && j < res);
        if (i < res && j < res) {
            float val;
            if constexpr (TRACE != 0) {
                // the warp's FP64 re-evaluations served together
                unsigned ev = 0;
                val = trace_pixel<HIER, DEPTH, DEFS, TRACE == 2, TRACE == 3, XRP_BATCH_MERGE != 0>(
                    sg.S, L, sg.P, sg.V, i, j, ev, wm);
            } else {
                RayStats st{0, 0};
                val = render_pixel<HIER, false, DEPTH, DEFS>(sg.S, L, sg.P, sg.V, i, j, st);
            }
            out[B.out0 + ((long long)v * res + i) * res + j] = val;
        }
        __syncwarp();  // before the next tile overwrites the staged data
    }
}

template <bool HIER, int DEPTH, bool DEFS, int TRACE>
cudaError_t launch_batch_t(const BatchLaunch& b, cudaStream_t st) {
    k_batch<HIER, DEPTH, DEFS, TRACE><<<b.blocks, 256, 0, st>>>(b.scenes, b.items, b.nitems, b.views, b.L,
                                                                b.ntiles, b.tw, b.th, b.counter, b.stride,
                                                                b.limit, b.out);
    return cudaGetLastError();
}

// Curve certificates (TRACE 3) serve deformed scenes only: DEFS is always on.
template <int TRACE>
cudaError_t launch_batch_mode(const BatchLaunch& b, cudaStream_t st) {
    if (b.depth == 0) {
        if (TRACE == 3 || b.defs) return b.hier ? launch_batch_t<true, 0, true, TRACE>(b, st) : launch_batch_t<false, 0, true, TRACE>(b, st);
        if constexpr (TRACE != 3)
            return b.hier ? launch_batch_t<true, 0, false, TRACE>(b, st) : launch_batch_t<false, 0, false, TRACE>(b, st);
    }
    if (TRACE == 3 || b.defs) return b.hier ? launch_batch_t<true, 3, true, TRACE>(b, st) : launch_batch_t<false, 3, true, TRACE>(b, st);
    if constexpr (TRACE != 3)
        return b.hier ? launch_batch_t<true, 3, false, TRACE>(b, st) : launch_batch_t<false, 3, false, TRACE>(b, st);
    return cudaErrorInvalidValue;
}

template <int TRACE>
const void* batch_fn_mode(int depth, bool defs, bool hier) {
    if (depth == 0) {
        if (TRACE == 3 || defs) return hier ? (const void*)k_batch<true, 0, true, TRACE> : (const void*)k_batch<false, 0, true, TRACE>;
        if constexpr (TRACE != 3)
            return hier ? (const void*)k_batch<true, 0, false, TRACE> : (const void*)k_batch<false, 0, false, TRACE>;
    }
    if (TRACE == 3 || defs) return hier ? (const void*)k_batch<true, 3, true, TRACE> : (const void*)k_batch<false, 3, true, TRACE>;
    if constexpr (TRACE != 3)
        return hier ? (const void*)k_batch<true, 3, false, TRACE> : (const void*)k_batch<false, 3, false, TRACE>;
    return nullptr;
}

// The four instantiations (xrp_kern_batch.cu, xrp_kern_batch_ball.cu,
// xrp_kern_batch_ray.cu, xrp_kern_batch_curve.cu).
cudaError_t launch_batch_plain(const BatchLaunch& b, cudaStream_t st);
cudaError_t launch_batch_ball(const BatchLaunch& b, cudaStream_t st);
cudaError_t launch_batch_ray(const BatchLaunch& b, cudaStream_t st);
cudaError_t launch_batch_curve(const BatchLaunch& b, cudaStream_t st);
const void* batch_fn_plain(int depth, bool defs, bool hier);
const void* batch_fn_ball(int depth, bool defs, bool hier);
const void* batch_fn_ray(int depth, bool defs, bool hier);
const void* batch_fn_curve(int depth, bool defs, bool hier);

}  // namespace xrp
