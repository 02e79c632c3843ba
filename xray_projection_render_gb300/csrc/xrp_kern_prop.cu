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

// The march of one launch group: optical depths into `dout`, undecided
// samples onto Q's list (its counters reset first).
cudaError_t launch_prop_march(const Prepared& pr, int view0, int nviews, const PropParams& Q, float* dout,
                              cudaStream_t st) {
    const long rays = (long)nviews * pr.P.res * pr.P.res;
    if (rays <= 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(Q.fb_count, 0, sizeof(unsigned), st);
    if (e != cudaSuccess) return e;
    if (Q.trace == 4 && (e = cudaMemsetAsync(Q.redo_count, 0, sizeof(unsigned), st)) != cudaSuccess) return e;
    return march(pr, view0, nviews, Q, dout, st);
}

// The rest of a launch group: FP64 for the samples the march left
// undecided (and, in the plain mode, a second march of the rays that found
// the list full), exp(-T).  `blocks_per_sm` sizes the FP64 pass's grid (0:
// one full wave).
cudaError_t launch_prop_tail(const Prepared& pr, int view0, int nviews, const PropParams& Q, float* dout,
                             cudaStream_t st, int blocks_per_sm) {
    const long rays = (long)nviews * pr.P.res * pr.P.res;
    if (rays <= 0) return cudaSuccess;
    static std::atomic<int> sm_count[kMaxDevices], fb_per_sm[kMaxDevices];
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    // one wave of resident blocks: every block of the grid-stride loop has
    // the same share of the list, so blocks beyond one wave would run as a
    // second, partly occupied wave
    int sms = sm_count[dev].load(std::memory_order_relaxed), per_sm = fb_per_sm[dev].load(std::memory_order_relaxed);
    if (!sms) {
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_prop_fallback, 256, 0) != cudaSuccess ||
            per_sm < 1)
            per_sm = 1;
        fb_per_sm[dev].store(per_sm, std::memory_order_relaxed);
        sm_count[dev].store(sms, std::memory_order_relaxed);
    }
    const int g = std::max(1, sms * (blocks_per_sm > 0 ? std::min(blocks_per_sm, per_sm) : per_sm));
    k_prop_fallback<<<g, 256, 0, st>>>(pr.S, pr.L, pr.P, pr.views, view0, Q.fb, Q.fb_count, Q.fb_cap,
                                      dout, Q.stats, Q.fb_overflow);
    cudaError_t e;
    if (Q.trace == 4 && (e = launch_plain_redo(pr, view0, Q, dout, Q.redo_cap, g, st)) != cudaSuccess)
        return e;
    long fin = (rays + 255) / 256;
    k_prop_finish<<<(unsigned)(fin < 65536 ? fin : 65536), 256, 0, st>>>(dout, rays);
    return cudaGetLastError();
}

// March, FP64 pass and exp(-T) of one launch group on one stream.
cudaError_t launch_prop_render(const Prepared& pr, int view0, int nviews, const PropParams& Q,
                               float* dout, cudaStream_t st) {
    cudaError_t e = launch_prop_march(pr, view0, nviews, Q, dout, st);
    if (e != cudaSuccess) return e;
    return launch_prop_tail(pr, view0, nviews, Q, dout, st, 0);
}

}  // namespace xrp
