// xrp_kern_trace_ray.cu -- certificate tracing with ray bounds (affine
// deformation chains), one thread per ray.
#include "xrp_trace.cuh"

namespace xrp {

cudaError_t launch_trace_ray(const Prepared& pr, int view0, int nviews, const PropParams& Q, float* dout,
                             cudaStream_t st) {
    return launch_trace_mode<1>(pr, view0, nviews, Q, dout, st);
}

}  // namespace xrp
