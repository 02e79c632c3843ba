// xrp_kern_prop.cu -- the proposal march's rendering kernels
// (xrp_proposal.cuh), specialised like the general-scene kernel.
#define XRP_PROP_RENDER_KERNELS
#include <algorithm>

#include "xrp_launch.h"

namespace xrp {

static cudaError_t march(const Prepared& pr, int view0, int nviews, const PropParams& Q, float* dout,
                         cudaStream_t st) {
    if (Q.trace) return launch_trace(pr, view0, nviews, Q, dout, st);
    if (Q.mlp) return launch_prop_net(pr, view0, nviews, Q, dout, st);
    if (Q.refine) { XRP_PROP_DISPATCH(kPropRefine, dout) }
    XRP_PROP_DISPATCH(kPropDense, dout)
}

// March (optical depths), FP64 for the samples it left undecided (and, in
// the plain mode, a second march of the rays that found the list full),
// exp(-T).
cudaError_t launch_prop_render(const Prepared& pr, int view0, int nviews, const PropParams& Q,
                               float* dout, cudaStream_t st) {
    const long rays = (long)nviews * pr.P.res * pr.P.res;
    if (rays <= 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(Q.fb_count, 0, sizeof(unsigned), st);
    if (e != cudaSuccess) return e;
    if (Q.trace == 4 && (e = cudaMemsetAsync(Q.redo_count, 0, sizeof(unsigned), st)) != cudaSuccess) return e;
    if ((e = march(pr, view0, nviews, Q, dout, st)) != cudaSuccess) return e;
    static std::atomic<int> fb_grid[kMaxDevices];
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    // one wave of resident blocks: every block of the grid-stride loop has
    // the same share of the list, so blocks beyond one wave would run as a
    // second, partly occupied wave
    int g = fb_grid[dev].load(std::memory_order_relaxed);
    if (!g) {
        int sms = 0, per_sm = 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_prop_fallback, 256, 0) != cudaSuccess ||
            per_sm < 1)
            per_sm = 1;
        g = std::max(1, sms * per_sm);
        fb_grid[dev].store(g, std::memory_order_relaxed);
    }
    k_prop_fallback<<<g, 256, 0, st>>>(pr.S, pr.L, pr.P, pr.views, view0, Q.fb, Q.fb_count, Q.fb_cap,
                                      dout, Q.stats, Q.fb_overflow);
    if (Q.trace == 4 && (e = launch_plain_redo(pr, view0, Q, dout, Q.redo_cap, g, st)) != cudaSuccess)
        return e;
    long fin = (rays + 255) / 256;
    k_prop_finish<<<(unsigned)(fin < 65536 ? fin : 65536), 256, 0, st>>>(dout, rays);
    return cudaGetLastError();
}

}  // namespace xrp
