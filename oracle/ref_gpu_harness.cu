// ref_gpu_harness.cu -- timing harness of the reference's own GPU kernel.
//
// TEST INFRASTRUCTURE.  The kernel is not in this file: oracle/ref_gpu.py
// compiles the reference's unmodified cuda_backend.cu to a cubin
// (render_kernel, cuda_backend.cu:19-80), and this harness loads that cubin
// with the driver API and drives it the way RenderVolumeProjectionsCUDA
// (cuda_backend.cu:82-203) does: the volume in a 3D CUDA array of extent
// (ny, nx, nz), one float texture with linear filtering, clamped and
// normalised coordinates, 16 x 16 thread blocks over the image, and per
// camera a launch, a device synchronisation and a copy of the image back
// to pageable host memory.  The host steps are restated here (same calls,
// same order); none of the reference's code is compiled into this file.
//
//   ref_gpu_harness <cubin> <volume.f32> nx ny nz <cams.f32> ncams res ds
//                   flat_field warmup steps [images_out.f32]
//
// volume.f32: float32 [z][x][y]; cams.f32: ncams x 21 float32
// (XRayCameraParams).  Prints one JSON line: the end-to-end times of the
// whole call (allocation, upload, texture, launches, copies, frees) and the
// kernel-only times (all cameras launched back to back into a resident
// buffer, CUDA events around them).
#include <cuda.h>
#include <cuda_runtime.h>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

namespace {

struct CamParams {  // XRayCameraParams layout (cuda_backend.h:78-83)
    float eye[3];
    float view[16];
    float fov_y;
    float R;
};
static_assert(sizeof(CamParams) == 21 * sizeof(float), "camera layout");

// Itanium name of render_kernel(cudaTextureObject_t, XRayCameraParams, int,
// float, float, float, float*); the harness falls back to enumerating the
// module's functions.
const char* kKernelName = "_Z13render_kernely16XRayCameraParamsifffPf";

bool read_file(const char* path, std::vector<float>& out, size_t n) {
    FILE* f = fopen(path, "rb");
    if (!f) return false;
    out.resize(n);
    size_t got = fread(out.data(), sizeof(float), n, f);
    fclose(f);
    return got == n;
}

#define CK(x)                                                                       \
    do {                                                                            \
        cudaError_t e_ = (x);                                                       \
        if (e_ != cudaSuccess) {                                                    \
            fprintf(stderr, "%s failed: %s\n", #x, cudaGetErrorString(e_));         \
            return 1;                                                               \
        }                                                                           \
    } while (0)
#define DK(x)                                                                       \
    do {                                                                            \
        CUresult r_ = (x);                                                          \
        if (r_ != CUDA_SUCCESS) {                                                   \
            const char* s_ = nullptr;                                               \
            cuGetErrorString(r_, &s_);                                              \
            fprintf(stderr, "%s failed: %s\n", #x, s_ ? s_ : "?");                  \
            return 1;                                                               \
        }                                                                           \
    } while (0)

struct Args {
    int nx, ny, nz, ncams, res;
    float ds, ff;
};

CUfunction g_fn = nullptr;

int launch_camera(cudaTextureObject_t tex, const CamParams& cam, const Args& a, float* dimg, cudaStream_t st) {
    CamParams c = cam;
    int res = a.res;
    float ds = a.ds, ff = a.ff, chd = 1.74f;  // cube_half_diagonal of the reference's call
    void* params[] = {&tex, &c, &res, &ds, &ff, &chd, &dimg};
    unsigned g = (unsigned)((res + 15) / 16);
    DK(cuLaunchKernel(g_fn, g, g, 1, 16, 16, 1, 0, (CUstream)st, params, nullptr));
    return 0;
}

int make_volume(const std::vector<float>& vol, const Args& a, cudaArray_t* arr, cudaTextureObject_t* tex) {
    cudaChannelFormatDesc ch = cudaCreateChannelDesc<float>();
    cudaExtent ext = make_cudaExtent((size_t)a.ny, (size_t)a.nx, (size_t)a.nz);
    CK(cudaMalloc3DArray(arr, &ch, ext));
    cudaMemcpy3DParms p;
    memset(&p, 0, sizeof(p));
    p.srcPtr = make_cudaPitchedPtr((void*)vol.data(), (size_t)a.ny * sizeof(float), (size_t)a.ny, (size_t)a.nx);
    p.dstArray = *arr;
    p.extent = ext;
    p.kind = cudaMemcpyHostToDevice;
    CK(cudaMemcpy3D(&p));
    cudaResourceDesc rd;
    memset(&rd, 0, sizeof(rd));
    rd.resType = cudaResourceTypeArray;
    rd.res.array.array = *arr;
    cudaTextureDesc td;
    memset(&td, 0, sizeof(td));
    for (int k = 0; k < 3; k++) td.addressMode[k] = cudaAddressModeClamp;
    td.filterMode = cudaFilterModeLinear;
    td.readMode = cudaReadModeElementType;
    td.normalizedCoords = 1;
    CK(cudaCreateTextureObject(tex, &rd, &td, nullptr));
    return 0;
}

// One call with the reference's host sequence.
int call_e2e(const std::vector<float>& vol, const std::vector<CamParams>& cams, const Args& a, float* out_host) {
    cudaArray_t arr = nullptr;
    cudaTextureObject_t tex = 0;
    if (make_volume(vol, a, &arr, &tex)) return 1;
    const size_t img = (size_t)a.res * a.res;
    float* dimg = nullptr;
    CK(cudaMalloc(&dimg, img * sizeof(float)));
    for (int c = 0; c < a.ncams; c++) {
        if (launch_camera(tex, cams[c], a, dimg, 0)) return 1;
        CK(cudaDeviceSynchronize());
        CK(cudaMemcpy(out_host + c * img, dimg, img * sizeof(float), cudaMemcpyDeviceToHost));
    }
    CK(cudaFree(dimg));
    CK(cudaDestroyTextureObject(tex));
    CK(cudaFreeArray(arr));
    return 0;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 13) {
        fprintf(stderr, "usage: %s cubin volume.f32 nx ny nz cams.f32 ncams res ds flat_field warmup steps [out]\n",
                argv[0]);
        return 2;
    }
    Args a;
    a.nx = atoi(argv[3]);
    a.ny = atoi(argv[4]);
    a.nz = atoi(argv[5]);
    a.ncams = atoi(argv[7]);
    a.res = atoi(argv[8]);
    a.ds = (float)atof(argv[9]);
    a.ff = (float)atof(argv[10]);
    const int warmup = atoi(argv[11]), steps = atoi(argv[12]);
    // the kernel's FP32 loop `s += ds` must advance at s ~ R + 1.74: a step
    // below ~1e-5 could stall it, so such steps are refused
    if (a.nx <= 0 || a.ny <= 0 || a.nz <= 0 || a.ncams <= 0 || a.res <= 0 || !(a.ds >= 1e-5f) || steps <= 0 ||
        warmup < 0) {
        fprintf(stderr, "bad arguments\n");
        return 2;
    }
    std::vector<float> vol, camf;
    if (!read_file(argv[2], vol, (size_t)a.nx * a.ny * a.nz) || !read_file(argv[6], camf, (size_t)a.ncams * 21)) {
        fprintf(stderr, "cannot read inputs\n");
        return 2;
    }
    std::vector<CamParams> cams(a.ncams);
    memcpy(cams.data(), camf.data(), camf.size() * sizeof(float));

    CK(cudaSetDevice(0));
    CK(cudaFree(0));  // primary context, shared with the driver API below
    CUmodule mod;
    DK(cuModuleLoad(&mod, argv[1]));
    if (cuModuleGetFunction(&g_fn, mod, kKernelName) != CUDA_SUCCESS) {
        unsigned n = 0;
        DK(cuModuleGetFunctionCount(&n, mod));
        std::vector<CUfunction> fs(n);
        DK(cuModuleEnumerateFunctions(fs.data(), n, mod));
        for (CUfunction f : fs) {
            const char* name = nullptr;
            if (cuFuncGetName(&name, f) == CUDA_SUCCESS && name && strstr(name, "render_kernel")) g_fn = f;
        }
        if (!g_fn) {
            fprintf(stderr, "render_kernel not found in %s\n", argv[1]);
            return 1;
        }
    }
    const size_t img = (size_t)a.res * a.res;
    std::vector<float> out_host(img * a.ncams);

    // end to end, the reference's call sequence
    std::vector<double> e2e_ms;
    for (int it = 0; it < warmup + steps; it++) {
        auto t0 = std::chrono::steady_clock::now();
        if (call_e2e(vol, cams, a, out_host.data())) return 1;
        auto t1 = std::chrono::steady_clock::now();
        if (it >= warmup) e2e_ms.push_back(std::chrono::duration<double, std::milli>(t1 - t0).count());
    }
    if (argc > 13) {
        FILE* f = fopen(argv[13], "wb");
        if (!f || fwrite(out_host.data(), sizeof(float), out_host.size(), f) != out_host.size()) return 1;
        fclose(f);
    }

    // kernel only: volume resident, every camera into its own image
    cudaArray_t arr = nullptr;
    cudaTextureObject_t tex = 0;
    if (make_volume(vol, a, &arr, &tex)) return 1;
    float* dall = nullptr;
    CK(cudaMalloc(&dall, img * a.ncams * sizeof(float)));
    float* flush = nullptr;
    const size_t flush_n = (size_t)64 << 20;  // 256 MiB, larger than L2
    CK(cudaMalloc(&flush, flush_n * sizeof(float)));
    cudaStream_t st;
    CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    std::vector<double> k_ms;
    for (int it = 0; it < warmup + steps; it++) {
        CK(cudaMemsetAsync(flush, it & 0xff, flush_n * sizeof(float), st));
        CK(cudaEventRecord(e0, st));
        for (int c = 0; c < a.ncams; c++)
            if (launch_camera(tex, cams[c], a, dall + c * img, st)) return 1;
        CK(cudaEventRecord(e1, st));
        CK(cudaEventSynchronize(e1));
        float ms = 0;
        CK(cudaEventElapsedTime(&ms, e0, e1));
        if (it >= warmup) k_ms.push_back(ms);
    }
    printf("{\"rays\": %lld, \"e2e_ms\": [", (long long)img * a.ncams);
    for (size_t k = 0; k < e2e_ms.size(); k++) printf("%s%.4f", k ? ", " : "", e2e_ms[k]);
    printf("], \"kernel_ms\": [");
    for (size_t k = 0; k < k_ms.size(); k++) printf("%s%.4f", k ? ", " : "", k_ms[k]);
    printf("]}\n");
    cudaFree(flush);
    cudaFree(dall);
    cudaDestroyTextureObject(tex);
    cudaFreeArray(arr);
    cuModuleUnload(mod);
    return 0;
}
