// xrp_kern_train.cu -- training of the proposal network: the training-row
// generation march (k_propose with TRAIN), the forward/backward step on the
// tcgen05 tensor cores (xrp_train_tc.cuh, also the logits of validation
// rows) and Adam.
#define XRP_MLP_KERNELS
#include "xrp_launch.h"
#include "xrp_train_tc.cuh"

namespace xrp {

cudaError_t launch_prop_train(const Prepared& pr, int view0, int nviews, const PropParams& Q,
                              cudaStream_t st) {
    XRP_PROP_DISPATCH(kPropTrain, nullptr)
}

// dynamic shared memory of k_mlp_train_tc: its tiles plus room to align them to 1024 bytes
constexpr size_t kTcSmem = sizeof(TrainTcShared) + 1024;

cudaError_t mlp_kernel_attrs() {
    return cudaFuncSetAttribute(k_mlp_train_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTcSmem);
}

cudaError_t mlp_train_launch(cudaStream_t st, const float* params, const __nv_bfloat16* X,
                             const float* y, const int* idx, int rows, float pos_weight,
                             float inv_batch, float* grad, float* loss, float* logits) {
    int blocks = (rows + kTcRows - 1) / kTcRows;
    if (blocks <= 0) return cudaSuccess;
    k_mlp_train_tc<<<blocks, kTcRows, kTcSmem, st>>>(params, X, y, idx, rows, pos_weight, inv_batch, grad,
                                                     loss, logits);
    return cudaGetLastError();
}

cudaError_t mlp_tc_error(unsigned* out) {
    cudaError_t e = cudaMemcpyFromSymbol(out, g_mlp_tc_error, sizeof(unsigned));
    const unsigned zero = 0;
    if (e == cudaSuccess && *out) e = cudaMemcpyToSymbol(g_mlp_tc_error, &zero, sizeof(unsigned));
    return e;
}

cudaError_t mlp_adam_launch(cudaStream_t st, float* params, float* grad, float* m1, float* m2, int n,
                            float lr, float b1, float b2, float eps, float c1, float c2) {
    k_mlp_adam<<<(n + 255) / 256, 256, 0, st>>>(params, grad, m1, m2, n, lr, b1, b2, eps, c1, c2);
    return cudaGetLastError();
}

// Logits of validation rows: the forward pass of the tcgen05 step.
cudaError_t mlp_logits_launch(cudaStream_t st, const float* params, const __nv_bfloat16* X, int rows,
                              float* logits) {
    int blocks = (rows + kTcRows - 1) / kTcRows;
    if (blocks <= 0) return cudaSuccess;
    k_mlp_train_tc<<<blocks, kTcRows, kTcSmem, st>>>(params, X, nullptr, nullptr, rows, 1.0f, 0.0f, nullptr,
                                                     nullptr, logits);
    return cudaGetLastError();
}

}  // namespace xrp
