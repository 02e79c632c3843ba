// xrp_kern_batch_ball.cu -- the batch kernel with certificate tracing,
// ball certificates.
#include "xrp_batch.cuh"

namespace xrp {

cudaError_t launch_batch_ball(const BatchLaunch& b, cudaStream_t st) { return launch_batch_mode<1>(b, st); }
const void* batch_fn_ball(int depth, bool defs, bool hier) { return batch_fn_mode<1>(depth, defs, hier); }

}  // namespace xrp
