// xrp_kern_batch_ray.cu -- the batch kernel with certificate tracing,
// ray certificates (affine chains).
#include "xrp_batch.cuh"

namespace xrp {

cudaError_t launch_batch_ray(const BatchLaunch& b, cudaStream_t st) { return launch_batch_mode<2>(b, st); }
const void* batch_fn_ray(int depth, bool defs, bool hier) { return batch_fn_mode<2>(depth, defs, hier); }

}  // namespace xrp
