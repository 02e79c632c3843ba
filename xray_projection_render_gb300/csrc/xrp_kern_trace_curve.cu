// xrp_kern_trace_curve.cu -- certificate tracing with curve bounds (smooth
// non-affine deformation chains: gaussian, sigmoid), one thread per ray; a
// kernel with gyroid leaves only for the scenes that have no other leaf.
#include "xrp_trace.cuh"

namespace xrp {

cudaError_t launch_trace_curve(const Prepared& pr, int view0, int nviews, const PropParams& Q, float* dout,
                               cudaStream_t st) {
    if (pr.leaves == (1 << N_GYROID)) return launch_trace_mode<3>(pr, view0, nviews, Q, dout, st);
    return launch_trace_mode<2>(pr, view0, nviews, Q, dout, st);
}

}  // namespace xrp
