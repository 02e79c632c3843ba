// xrp_kern_scene.cu -- the general-scene kernel (any object tree and
// deformation), one thread per pixel, specialised on the deepest
// tessellation nesting and on the presence of a deformation.
#include "xrp_launch.h"

namespace xrp {

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
