// xrp_kern_trace_plain.cu -- the plain integrator over a general scene as a
// mode of the tracing kernel (k_trace, CERT 4): every lattice sample is
// evaluated in FP32 and the samples FP32 cannot decide go to the FP64 list
// (k_prop_fallback) instead of being re-evaluated inside the march.  A ray
// with a sample that found the list full is marched again by k_plain_redo
// (FP64 inside the march, as k_render does), which overwrites its optical
// depth before the exp pass.
#include <algorithm>

#include "xrp_trace.cuh"

namespace xrp {

cudaError_t launch_trace_plain(const Prepared& pr, int view0, int nviews, const PropParams& Q, float* dout,
                               cudaStream_t st) {
    return launch_trace_mode<4>(pr, view0, nviews, Q, dout, st);
}

// One thread per listed ray (grid-stride over the device-side count).
template <bool HIER, int DEPTH, bool DEFS>
__global__ void __launch_bounds__(256)
    k_plain_redo(const __grid_constant__ SceneDev S, const __grid_constant__ Lattice L,
                 const __grid_constant__ RenderParams P, const ViewDev* __restrict__ views, int view0,
                 const unsigned* __restrict__ redo, const unsigned* __restrict__ redo_count, unsigned cap,
                 float* __restrict__ T, unsigned long long* __restrict__ stats) {
    const unsigned n = min(*redo_count, cap);
    const long img = (long)P.res * P.res;
    for (unsigned q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
        const long r = redo[q];
        const int v = view0 + (int)(r / img);
        const long pix = r % img;
        const int i = (int)(pix / P.res), j = (int)(pix % P.res);
        RayStats rs{0, 0};
        T[r] = depth_pixel<HIER, DEPTH, DEFS>(S, L, P, views[v], i, j, rs);
        if (stats) {
            atomicAdd(&stats[kStatEvaluations], (unsigned long long)rs.samples);
            if (rs.fallbacks) atomicAdd(&stats[kStatFallbacks], (unsigned long long)rs.fallbacks);
        }
    }
}

cudaError_t launch_plain_redo(const Prepared& pr, int view0, const PropParams& Q, float* dout, unsigned cap,
                              int grid, cudaStream_t st) {
#define XRP_GEN(H, D, F)                                                                                  \
    k_plain_redo<H, D, F><<<grid, 256, 0, st>>>(pr.S, pr.L, pr.P, pr.views, view0, Q.redo, Q.redo_count, \
                                                cap, dout, Q.stats)
#define XRP_GEN_D(H, F)                       \
    if (pr.depth == 0) XRP_GEN(H, 0, F);      \
    else if (pr.depth == 1) XRP_GEN(H, 1, F); \
    else XRP_GEN(H, 3, F);
    if (pr.L.hierarchical) {
        if (pr.defs) { XRP_GEN_D(true, true) } else { XRP_GEN_D(true, false) }
    } else {
        if (pr.defs) { XRP_GEN_D(false, true) } else { XRP_GEN_D(false, false) }
    }
#undef XRP_GEN_D
#undef XRP_GEN
    return cudaGetLastError();
}

}  // namespace xrp
