// xrp_kern_train.cu -- training of the proposal network: the training-row
// generation march (k_propose with TRAIN), the tensor-core forward/backward
// step, Adam, and the logits of validation rows.
#define XRP_MLP_KERNELS
#include "xrp_launch.h"

namespace xrp {

cudaError_t launch_prop_train(const Prepared& pr, int view0, int nviews, const PropParams& Q,
                              cudaStream_t st) {
    XRP_PROP_DISPATCH(kPropTrain, nullptr)
}

cudaError_t mlp_kernel_attrs() {
    cudaError_t e = cudaFuncSetAttribute(k_mlp_train, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)sizeof(TrainShared));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_mlp_logits, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)sizeof(PropShared));
    return e;
}

cudaError_t mlp_train_launch(cudaStream_t st, const float* params, const __nv_bfloat16* X,
                             const float* y, const int* idx, int rows, float pos_weight,
                             float inv_batch, float* grad, float* loss, float* logits) {
    int blocks = (rows + kTrainRows - 1) / kTrainRows;
    if (blocks <= 0) return cudaSuccess;
    k_mlp_train<<<blocks, kTrainRows, sizeof(TrainShared), st>>>(params, X, y, idx, rows, pos_weight,
                                                               inv_batch, grad, loss, logits);
    return cudaGetLastError();
}

cudaError_t mlp_adam_launch(cudaStream_t st, float* params, float* grad, float* m1, float* m2, int n,
                            float lr, float b1, float b2, float eps, float c1, float c2) {
    k_mlp_adam<<<(n + 255) / 256, 256, 0, st>>>(params, grad, m1, m2, n, lr, b1, b2, eps, c1, c2);
    return cudaGetLastError();
}

cudaError_t mlp_logits_launch(cudaStream_t st, const float* params, const __nv_bfloat16* X, int rows,
                              float* logits) {
    int tiles = (rows + 31) / 32;
    int blocks = (tiles + kPropWarps - 1) / kPropWarps;
    if (blocks > 4096) blocks = 4096;
    if (blocks <= 0) return cudaSuccess;
    k_mlp_logits<<<blocks, 32 * kPropWarps, sizeof(PropShared), st>>>(params, X, rows, logits);
    return cudaGetLastError();
}

}  // namespace xrp
