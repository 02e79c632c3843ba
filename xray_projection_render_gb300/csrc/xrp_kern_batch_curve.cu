// xrp_kern_batch_curve.cu -- the batch kernel with certificate tracing,
// curve certificates (some scene of the batch has a non-affine chain).
#include "xrp_batch.cuh"

namespace xrp {

cudaError_t launch_batch_curve(const BatchLaunch& b, cudaStream_t st) { return launch_batch_mode<3>(b, st); }
const void* batch_fn_curve(int depth, bool defs, bool hier) { return batch_fn_mode<3>(depth, defs, hier); }

}  // namespace xrp
