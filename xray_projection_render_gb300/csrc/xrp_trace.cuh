// xrp_trace.cuh -- launch helpers of certificate tracing (k_trace in
// xrp_proposal.cuh), instantiated per certificate kind in
// xrp_kern_trace.cu (balls), xrp_kern_trace_ray.cu (ray bounds),
// xrp_kern_trace_curve.cu (curve bounds) and xrp_kern_trace_plain.cu (no
// certificate: the plain integrator).
#pragma once
#include "xrp_launch.h"

namespace xrp {

template <int DEPTH, bool DEFS, int CERT>
cudaError_t trace_r(const Prepared& pr, int view0, int nviews, const PropParams& Q, float* dout,
                    cudaStream_t st) {
    const int tpr = (pr.P.res + 15) / 16;
    long blocks = (long)nviews * tpr * tpr;
    if (blocks <= 0) return cudaSuccess;
    if (blocks > 0x7fffffffL) return cudaErrorInvalidConfiguration;
    const size_t smem = (size_t)pr.S.nnodes * sizeof(Node);
    if (pr.L.hierarchical) {
        // curve certificates serve the simple integrator only
        if constexpr (CERT == 2 || CERT == 3) return cudaErrorInvalidValue;
        else
            k_trace<DEPTH, DEFS, true, CERT><<<(unsigned)blocks, 256, smem, st>>>(pr.S, pr.L, pr.P, pr.views,
                                                                                view0, nviews, Q, dout);
    } else
        k_trace<DEPTH, DEFS, false, CERT><<<(unsigned)blocks, 256, smem, st>>>(pr.S, pr.L, pr.P, pr.views, view0,
                                                                             nviews, Q, dout);
    return cudaGetLastError();
}

// CERT 2 and 3 (curve bounds) serve deformed scenes only: DEFS is always on.
template <int CERT>
cudaError_t launch_trace_mode(const Prepared& pr, int view0, int nviews, const PropParams& Q, float* dout,
                              cudaStream_t st) {
    constexpr bool kCurve = CERT == 2 || CERT == 3;
    if (kCurve || pr.defs) {
        if (pr.depth == 0) return trace_r<0, true, CERT>(pr, view0, nviews, Q, dout, st);
        if (pr.depth == 1) return trace_r<1, true, CERT>(pr, view0, nviews, Q, dout, st);
        return trace_r<3, true, CERT>(pr, view0, nviews, Q, dout, st);
    }
    if constexpr (!kCurve) {
        if (pr.depth == 0) return trace_r<0, false, CERT>(pr, view0, nviews, Q, dout, st);
        if (pr.depth == 1) return trace_r<1, false, CERT>(pr, view0, nviews, Q, dout, st);
        return trace_r<3, false, CERT>(pr, view0, nviews, Q, dout, st);
    }
    return cudaErrorInvalidValue;
}

}  // namespace xrp
