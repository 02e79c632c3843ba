// xrp_train.cuh -- Adam for the proposal MLP.  The training step itself
// (forward and backward on the tcgen05 tensor cores) is xrp_train_tc.cuh;
// Adam updates the FP32 master weights from the gradients it accumulates.
#pragma once
#include "xrp_mlp.cuh"

namespace xrp {

#if defined(__CUDACC__)

#if defined(XRP_MLP_KERNELS)
// Adam on the FP32 master parameters; clears the gradient.
__global__ void k_mlp_adam(float* __restrict__ params, float* __restrict__ grad, float* __restrict__ m1,
                           float* __restrict__ m2, int n, float lr, float b1, float b2, float eps,
                           float c1, float c2) {
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
        float gq = grad[q];
        float a = b1 * m1[q] + (1.f - b1) * gq;
        float v = b2 * m2[q] + (1.f - b2) * gq * gq;
        m1[q] = a;
        m2[q] = v;
        params[q] -= lr * (a * c1) / (sqrtf(v * c2) + eps);
        grad[q] = 0.f;
    }
}

#endif  // XRP_MLP_KERNELS

#endif  // __CUDACC__

}  // namespace xrp
