// xrp_kern_trace.cu -- certificate tracing (k_trace in xrp_proposal.cuh),
// one thread per ray, specialised on tessellation depth, deformation,
// integrator and certificate kind (ray bounds for affine chains, curve
// bounds for other deformation chains, balls on request).  Its own translation unit so it compiles in parallel with the
// segment march.
#include "xrp_trace.cuh"

namespace xrp {

// Ray- and curve-certificate kernels live in xrp_kern_trace_ray.cu and
// xrp_kern_trace_curve.cu, the plain kernels in xrp_kern_trace_plain.cu.
cudaError_t launch_trace_ray(const Prepared& pr, int view0, int nviews, const PropParams& Q, float* dout,
                             cudaStream_t st);
cudaError_t launch_trace_curve(const Prepared& pr, int view0, int nviews, const PropParams& Q, float* dout,
                               cudaStream_t st);
cudaError_t launch_trace_plain(const Prepared& pr, int view0, int nviews, const PropParams& Q, float* dout,
                               cudaStream_t st);

cudaError_t launch_trace(const Prepared& pr, int view0, int nviews, const PropParams& Q, float* dout,
                         cudaStream_t st) {
    if (Q.trace == 4) return launch_trace_plain(pr, view0, nviews, Q, dout, st);
    if (Q.trace == 1 && pr.S.affine) return launch_trace_ray(pr, view0, nviews, Q, dout, st);
    // curve certificates for the simple integrator; the hierarchical one
    // refines every crossing over fine samples, where the curve bound's
    // extra arithmetic does not pay (gyroid: balls 370 against 345 Mrays/s)
    if (Q.trace == 1 && pr.defs && !pr.L.hierarchical) return launch_trace_curve(pr, view0, nviews, Q, dout, st);
    return launch_trace_mode<0>(pr, view0, nviews, Q, dout, st);
}

}  // namespace xrp
