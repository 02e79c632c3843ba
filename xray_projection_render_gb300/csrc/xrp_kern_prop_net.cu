// xrp_kern_prop_net.cu -- the proposal march with the network routing
// (xrp_proposal.cuh, mode kPropNet), in its own translation unit so the
// march variants compile in parallel.
#include "xrp_launch.h"

namespace xrp {

cudaError_t launch_prop_net(const Prepared& pr, int view0, int nviews, const PropParams& Q, float* dout,
                            cudaStream_t st) {
    XRP_PROP_DISPATCH(kPropNet, dout)
}

}  // namespace xrp
