// xrp_launch.h -- what the engine's host code shares with the kernel
// translation units: the prepared render state and the launchers.
//
// The kernels are split over several translation units (general scenes,
// proposal march, training) so they compile in parallel; each unit owns its
// launchers, declared here.
#pragma once
#include <cuda_runtime.h>

#include <atomic>

#include "xrp_device.h"
#include "xrp_proposal.cuh"

namespace xrp {

// Minimum resident blocks per SM asked of the compiler (register budget)
// for the general-scene and batch kernels, measured on GB300: 3 (80
// registers) against 2 (128): gyroid 94 vs 72, lattice 140 vs 112 Mrays/s,
// plain batch 770 vs 591; the spills cost less than the lost warps.
#ifndef XRP_SCENE_MIN_BLOCKS
#define XRP_SCENE_MIN_BLOCKS 3
#endif

// Parameters of a voxel-grid root (no deformation), read by the voxel
// kernels from their constant bank so the march keeps few live registers.
struct VoxParams {
    cudaTextureObject_t tex;  // layered texture of the grid (gather path)
    const float* data;        // [z][x][y] (load path, FP64 re-evaluation)
    const double* data64;     // exact values when FP32 cannot hold them, else null
    int nx, ny, nz;
    int zero_guard;           // hierarchical integrator: guard the density == 0 test
    float scale[3];           // (N-1)/2
    float inv_scale[3];
    float band_w;             // world-space guard band of the inclusive [-1,1] test
    float band_zero;          // relative band of the zero test
    float inner_margin;       // clip margin of the bounds-free interior range
    float lo[3], hi[3];       // dilated support box
};

// Everything a render needs on the device except the volume data.
struct Prepared {
    SceneDev S;
    Lattice L;
    RenderParams P;
    const ViewDev* views = nullptr;
    bool volume_fast = false;
    cudaTextureObject_t tex = 0;  // layered texture of the root grid (0: use loads)
    VoxParams vq;                 // voxel-grid root parameters (volume_fast)
    int depth = kMaxDepth;        // kernel specialisation of general scenes
    bool defs = true;
    bool empty = false;  // no sample lattice or no support: every pixel is exp(-ff)
    int leaves = 0;      // leaf types of the scene, bit 1 << NodeType
};

// A proposal-march launch (see xrp_proposal.cuh); Q's scene-independent
// fields are filled in by the caller.
struct PropLaunch {
    PropParams Q;
    bool train = false;
    long long max_rays = 1LL << 23;  // rays per launch (bounds the FP64 list: 4 entries per ray,
                                     // and the plain mode's redo list: one per ray)
    // With `side`, the FP64 pass and exp of launch group g run on `side`
    // while group g + 1 marches on the call's stream: the lists alternate
    // between two slots (list, counter + overflow flag, redo list and its
    // counter), `done[s]` marks slot s's last tail, `groups` counts the
    // groups launched.  Null: one stream.
    cudaStream_t side = nullptr;
    uint2* fb_slot[2] = {nullptr, nullptr};
    unsigned* cnt_slot[2] = {nullptr, nullptr};
    unsigned* redo_slot[2] = {nullptr, nullptr};
    unsigned* redo_cnt_slot[2] = {nullptr, nullptr};
    cudaEvent_t marched = nullptr, done[2] = {nullptr, nullptr};
    int groups = 0;
};

// xrp_kern_scene.cu: k_render for general scenes.
cudaError_t launch_scene(const Prepared& pr, int view0, int nviews, bool hier, float* dout,
                         unsigned long long* stats, cudaStream_t st);

// One item of a batched render (several scenes, resolutions and view
// counts in one persistent launch): its scene, views, tiling and output.
struct BatchItemDev {
    int scene;            // index into the batch's SceneDev array
    int view0;            // first view in the batch's view array
    int nviews;
    int tiles_x, tiles_y; // tiles per view
    int pad;
    long long tile0;      // first global tile index
    long long out0;       // first output element
    RenderParams P;       // resolution, pixel table, flat field, multiplier
};

// Launch of the batch kernel: warp tiles of tw x th pixels (tw * th == 32),
// taken from a global counter by a persistent grid; the tiles visited are
// k * stride for k < limit (stride 1: all; larger strides sample the batch
// for the autotuner).
struct BatchLaunch {
    const SceneDev* scenes;
    const BatchItemDev* items;
    int nitems;
    const ViewDev* views;
    Lattice L;
    long long ntiles;
    int tw, th;
    int blocks;            // persistent grid size
    int depth;             // 0: no tessellation in the batch, else up to kMaxDepth
    bool defs, hier;
    int trace;             // certificate tracing: 0 off, 1 ball certificates, 2 ray certificates
    unsigned long long* counter;
    long long stride, limit;
    float* out;
};

// xrp_kern_batch.cu: the batch kernel and its occupancy.
cudaError_t launch_batch(const BatchLaunch& b, cudaStream_t st);
cudaError_t batch_blocks_per_sm(int depth, bool defs, bool hier, int trace, int* out);

// xrp_kern_export.cu: volume export of a scene and device-side image finishing.
cudaError_t launch_voxelize_scene(const SceneDev& S, int depth, bool defs, int res, double dm, float* out,
                                  unsigned* vmax_bits, unsigned char* u8, cudaStream_t st);
cudaError_t launch_finish(const float* img, int nviews, int res, int transparency, unsigned short* gray,
                          unsigned short* alpha, float* minmax, cudaStream_t st);

// xrp_kern_trace.cu: certificate tracing (k_trace); Q.trace 1: ray
// certificates where the scene's chain is affine, curve certificates for
// other deformation chains; 2: ball only.
cudaError_t launch_trace(const Prepared& pr, int view0, int nviews, const PropParams& Q, float* dout,
                         cudaStream_t st);

// xrp_kern_trace_plain.cu: the rays of the plain mode (Q.trace 4) whose
// samples found the FP64 list full, marched again into the optical depths
// `dout` (at most `cap` of the listed ones; `grid` blocks).
cudaError_t launch_plain_redo(const Prepared& pr, int view0, const PropParams& Q, float* dout, unsigned cap,
                              int grid, cudaStream_t st);

// xrp_kern_prop.cu: the proposal march (rendering).
cudaError_t launch_prop_march(const Prepared& pr, int view0, int nviews, const PropParams& Q, float* dout,
                              cudaStream_t st);
cudaError_t launch_prop_tail(const Prepared& pr, int view0, int nviews, const PropParams& Q, float* dout,
                             cudaStream_t st, int blocks_per_sm);
cudaError_t launch_prop_render(const Prepared& pr, int view0, int nviews, const PropParams& Q,
                               float* dout, cudaStream_t st);

// xrp_kern_prop_net.cu: the march with the network routing candidates.
cudaError_t launch_prop_net(const Prepared& pr, int view0, int nviews, const PropParams& Q, float* dout,
                            cudaStream_t st);

// xrp_kern_train.cu: training-row generation and the network's kernels.
cudaError_t launch_prop_train(const Prepared& pr, int view0, int nviews, const PropParams& Q,
                              cudaStream_t st);
cudaError_t mlp_kernel_attrs();
cudaError_t mlp_train_launch(cudaStream_t st, const float* params, const __nv_bfloat16* X,
                             const float* y, const int* idx, int rows, float pos_weight,
                             float inv_batch, float* grad, float* loss, float* logits);
cudaError_t mlp_adam_launch(cudaStream_t st, float* params, float* grad, float* m1, float* m2, int n,
                            float lr, float b1, float b2, float eps, float c1, float c2);
cudaError_t mlp_logits_launch(cudaStream_t st, const float* params, const __nv_bfloat16* X, int rows,
                              float* logits);
// Whether a tensor-core training step gave up waiting for its products since
// the last call (synchronous; clears the flag).
cudaError_t mlp_tc_error(unsigned* out);

constexpr int kMaxDevices = 64;  // per-device launch caches

// Grid of a persistent proposal launch: resident blocks x SMs (cached per
// kernel and device).
template <class K>
cudaError_t persistent_grid(K kern, size_t smem, int block, int* out) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int nb = 0, dev = 0, sms = 0;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, block, smem)) != cudaSuccess) return e;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
    *out = sms * (nb > 0 ? nb : 1);
    return cudaSuccess;
}

// One proposal-march launch, persistent grid (xrp_kern_prop.cu and
// xrp_kern_train.cu instantiate it).
template <int DEPTH, bool DEFS, int MODE>
cudaError_t launch_prop_t(const Prepared& pr, int view0, int nviews, const PropParams& Q,
                          float* dout, cudaStream_t st) {
    auto kern = k_propose<DEPTH, DEFS, MODE>;
    static std::atomic<int> grid_cache[kMaxDevices];  // per device; 0 until measured
    const size_t smem = sizeof(PropShared);
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    int gmax = grid_cache[dev].load(std::memory_order_relaxed);
    if (!gmax) {
        cudaError_t e = persistent_grid(kern, smem, 32 * kPropWarps, &gmax);
        if (e != cudaSuccess) return e;
        grid_cache[dev].store(gmax, std::memory_order_relaxed);
    }
    long rays = Q.rays ? (long)Q.nrays : (long)nviews * pr.P.res * pr.P.res;
    long need = (rays + 32 * kPropWarps - 1) / (32 * kPropWarps);  // 32 rays per warp batch
    long grid = need < gmax ? need : gmax;
    if (grid <= 0) return cudaSuccess;
    kern<<<(unsigned)grid, 32 * kPropWarps, smem, st>>>(pr.S, pr.L, pr.P, pr.views, view0, nviews, Q, dout);
    return cudaGetLastError();
}

#define XRP_PROP_DISPATCH(T, OUT)                                                   \
    if (pr.defs) {                                                                 \
        if (pr.depth == 0) return launch_prop_t<0, true, T>(pr, view0, nviews, Q, OUT, st);  \
        if (pr.depth == 1) return launch_prop_t<1, true, T>(pr, view0, nviews, Q, OUT, st);  \
        return launch_prop_t<3, true, T>(pr, view0, nviews, Q, OUT, st);                     \
    }                                                                              \
    if (pr.depth == 0) return launch_prop_t<0, false, T>(pr, view0, nviews, Q, OUT, st);     \
    if (pr.depth == 1) return launch_prop_t<1, false, T>(pr, view0, nviews, Q, OUT, st);     \
    return launch_prop_t<3, false, T>(pr, view0, nviews, Q, OUT, st);

}  // namespace xrp
