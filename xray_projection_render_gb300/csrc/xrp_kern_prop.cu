// xrp_kern_prop.cu -- the proposal march's rendering kernels
// (xrp_proposal.cuh), specialised like the general-scene kernel.
#define XRP_PROP_RENDER_KERNELS
#include <algorithm>

#include "xrp_launch.h"

namespace xrp {

template <int DEPTH, bool DEFS>
static cudaError_t trace_t(const Prepared& pr, int view0, int nviews, const PropParams& Q, float* dout,
                           cudaStream_t st) {
    const int tpr = (pr.P.res + 15) / 16;
    long blocks = (long)nviews * tpr * tpr;
    if (blocks <= 0) return cudaSuccess;
    if (blocks > 0x7fffffffL) return cudaErrorInvalidConfiguration;
    if (pr.L.hierarchical)
        k_trace<DEPTH, DEFS, true><<<(unsigned)blocks, 256, 0, st>>>(pr.S, pr.L, pr.P, pr.views, view0, nviews, Q, dout);
    else
        k_trace<DEPTH, DEFS, false><<<(unsigned)blocks, 256, 0, st>>>(pr.S, pr.L, pr.P, pr.views, view0, nviews, Q, dout);
    return cudaGetLastError();
}

static cudaError_t march(const Prepared& pr, int view0, int nviews, const PropParams& Q, float* dout,
                         cudaStream_t st) {
    if (Q.trace) {
        if (pr.defs) {
            if (pr.depth == 0) return trace_t<0, true>(pr, view0, nviews, Q, dout, st);
            if (pr.depth == 1) return trace_t<1, true>(pr, view0, nviews, Q, dout, st);
            return trace_t<3, true>(pr, view0, nviews, Q, dout, st);
        }
        if (pr.depth == 0) return trace_t<0, false>(pr, view0, nviews, Q, dout, st);
        if (pr.depth == 1) return trace_t<1, false>(pr, view0, nviews, Q, dout, st);
        return trace_t<3, false>(pr, view0, nviews, Q, dout, st);
    }
    if (Q.mlp) return launch_prop_net(pr, view0, nviews, Q, dout, st);
    if (Q.refine) { XRP_PROP_DISPATCH(kPropRefine, dout) }
    XRP_PROP_DISPATCH(kPropDense, dout)
}

// March (optical depths), FP64 for the samples it left undecided, exp(-T).
cudaError_t launch_prop_render(const Prepared& pr, int view0, int nviews, const PropParams& Q,
                               float* dout, cudaStream_t st) {
    const long rays = (long)nviews * pr.P.res * pr.P.res;
    if (rays <= 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(Q.fb_count, 0, sizeof(unsigned), st);
    if (e != cudaSuccess) return e;
    if ((e = march(pr, view0, nviews, Q, dout, st)) != cudaSuccess) return e;
    static std::atomic<int> fb_grid[kMaxDevices];
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    int g = fb_grid[dev].load(std::memory_order_relaxed);
    if (!g) {
        int sms = 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        g = std::max(1, sms * 4);
        fb_grid[dev].store(g, std::memory_order_relaxed);
    }
    k_prop_fallback<<<g, 256, 0, st>>>(pr.S, pr.L, pr.P, pr.views, view0, Q.fb, Q.fb_count, Q.fb_cap,
                                      dout, Q.stats, Q.fb_overflow);
    long fin = (rays + 255) / 256;
    k_prop_finish<<<(unsigned)(fin < 65536 ? fin : 65536), 256, 0, st>>>(dout, rays);
    return cudaGetLastError();
}

}  // namespace xrp
