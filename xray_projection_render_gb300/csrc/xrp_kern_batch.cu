// xrp_kern_batch.cu -- the batch kernel with the plain integrator, and the
// dispatch over certificate modes (xrp_batch_* in xrp_engine.cu).
#include "xrp_batch.cuh"

namespace xrp {

cudaError_t launch_batch_plain(const BatchLaunch& b, cudaStream_t st) { return launch_batch_mode<0>(b, st); }
const void* batch_fn_plain(int depth, bool defs, bool hier) { return batch_fn_mode<0>(depth, defs, hier); }

cudaError_t launch_batch(const BatchLaunch& b, cudaStream_t st) {
    if (b.blocks <= 0 || b.ntiles <= 0) return cudaSuccess;
    if (b.trace == 3) return launch_batch_curve(b, st);
    if (b.trace == 2) return launch_batch_ray(b, st);
    if (b.trace == 1) return launch_batch_ball(b, st);
    return launch_batch_plain(b, st);
}

cudaError_t batch_blocks_per_sm(int depth, bool defs, bool hier, int trace, int* out) {
    const int d = depth == 0 ? 0 : 3;
    const void* f = trace == 3   ? batch_fn_curve(d, defs, hier)
                    : trace == 2 ? batch_fn_ray(d, defs, hier)
                    : trace == 1 ? batch_fn_ball(d, defs, hier)
                                 : batch_fn_plain(d, defs, hier);
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(out, f, 256, 0);
}

}  // namespace xrp
