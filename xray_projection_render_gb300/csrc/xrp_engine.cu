// xrp_engine.cu -- CUDA kernels and the C ABI of libcuda_render.so.
//
// One thread marches one pixel's ray over the reference's FP64 sample lattice
// with the FP32 guarded evaluator of xrp_device.h; a block covers a 16x16
// pixel tile (each warp an 8x4 sub-tile, so neighbouring rays of a warp stay
// spatially coherent for the voxel gathers and the primitive candidate
// lists).  Views are processed in chunks so that the copy of one chunk's
// images to the host overlaps the rendering of the next.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/xrp.h"
#include "xrp_launch.h"
#include "xrp_scene.h"

using namespace xrp;

// ---------------------------------------------------------------------------
// errors
// ---------------------------------------------------------------------------

static thread_local std::string t_err;
static thread_local uint64_t t_stats[2] = {0, 0};

static int fail(int code, const char* fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    t_err = buf;
    return code;
}

static int cuda_fail(int code, const char* what, cudaError_t e) {
    return fail(code, "%s: %s", what, cudaGetErrorString(e));
}

// ---------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------

// Gather of the 2x2 texels around (u, v) from layer `layer` of a 2D layered
// texture (hand-written tld4; CUDA C++ exposes gather for plain 2D only).
// With u, v at the centre of a texel quad the footprint is exact; the four
// values come back unfiltered, in the order (u0,v1), (u1,v1), (u1,v0), (u0,v0).
__device__ __forceinline__ float4 gather_a2d(cudaTextureObject_t tex, int layer, float u, float v) {
    float4 r;
    asm volatile("tld4.r.a2d.v4.f32.f32 {%0, %1, %2, %3}, [%4, {%5, %6, %7, %7}];"
                 : "=f"(r.x), "=f"(r.y), "=f"(r.z), "=f"(r.w)
                 : "l"(tex), "r"(layer), "f"(u), "f"(v));
    return r;
}



// FP64 density of sample s of pixel (i, j) (VoxelGrid.Density at the
// reference's own position, objects.go:789-855, main.go:148-150).
// Throughput probe of the texture path: every thread issues `iters` tld4
// gathers on a small layered texture (resident in L1), so the rate measures
// the TEX unit, the binding unit of the voxel kernel.  Coordinates cycle
// over texel-quad centres in bounds.
__global__ void __launch_bounds__(256) k_gather_probe(cudaTextureObject_t tex, int iters, float* sink) {
    // four independent chains per thread; each coordinate depends on the
    // previous gather of its chain (times 0, which is not folded without
    // fast math), so no gather can be hoisted or merged
    float a0 = 0.0f, a1 = 0.0f, a2 = 0.0f, a3 = 0.0f;
    const float u0 = 1.0f + (float)(threadIdx.x & 7), v0 = 1.0f + (float)((threadIdx.x >> 3) & 7);
    for (int k = 0; k < iters; k += 4) {
        const float4 g0 = gather_a2d(tex, 0, u0 + a0 * 0.0f, v0);
        const float4 g1 = gather_a2d(tex, 1, u0 + 1.0f + a1 * 0.0f, v0);
        const float4 g2 = gather_a2d(tex, 0, u0 + 2.0f + a2 * 0.0f, v0 + 1.0f);
        const float4 g3 = gather_a2d(tex, 1, u0 + 3.0f + a3 * 0.0f, v0 + 1.0f);
        a0 += g0.x + g0.w;
        a1 += g1.x + g1.w;
        a2 += g2.x + g2.w;
        a3 += g3.x + g3.w;
    }
    sink[blockIdx.x * blockDim.x + threadIdx.x] = a0 + a1 + a2 + a3;
}

__device__ __forceinline__ double vox_sample64_inl(const VoxParams& Q, const ViewDev& V,
                                                   const double* xs, int i, int j, double s) {
    Ray64 r;
    setup_ray64(V, xs, i, j, r);
    double x = xrp::dadd(r.o[0], xrp::dmul(r.d[0], s));
    double y = xrp::dadd(r.o[1], xrp::dmul(r.d[1], s));
    double z = xrp::dadd(r.o[2], xrp::dmul(r.d[2], s));
    Volume vol;
    vol.data = Q.data;
    vol.data64 = Q.data64;
    vol.nx = Q.nx;
    vol.ny = Q.ny;
    vol.nz = Q.nz;
    return voxel64(vol, x, y, z);
}

__device__ __noinline__ double vox_sample64(const VoxParams& Q, const ViewDev& V, const double* xs,
                                            int i, int j, double s) {
    return vox_sample64_inl(Q, V, xs, i, j, s);
}

// Trilinear value at grid point u (interior: no bounds test).  TEX: the 8
// taps come from two gathers of the layered texture (layer = z slice, width
// ny, height nx, point sampling, clamp to edge so x1 = min(x0+1, N-1) as in
// objects.go:822-830); otherwise from eight loads.
template <bool TEX>
__device__ __forceinline__ float vox_inner(const VoxParams& Q, float ux, float uy, float uz) {
    int x0 = min(max((int)floorf(ux), 0), Q.nx - 2);
    int y0 = min(max((int)floorf(uy), 0), Q.ny - 2);
    int z0 = min(max((int)floorf(uz), 0), Q.nz - 2);
    float wx = ux - (float)x0, wy = uy - (float)y0, wz = uz - (float)z0;
    float v000, v001, v010, v011, v100, v101, v110, v111;
    if constexpr (TEX) {
        float gu = (float)y0 + 1.0f, gv = (float)x0 + 1.0f;
        float4 g0 = gather_a2d(Q.tex, z0, gu, gv);
        float4 g1 = gather_a2d(Q.tex, z0 + 1, gu, gv);
        v000 = g0.w; v010 = g0.z; v100 = g0.x; v110 = g0.y;
        v001 = g1.w; v011 = g1.z; v101 = g1.x; v111 = g1.y;
    } else {
        const long NY = Q.ny, NXY = (long)Q.nx * Q.ny;
        const float* p0 = Q.data + z0 * NXY + x0 * NY + y0;
        const float* p1 = p0 + NXY;
        v000 = __ldg(p0); v010 = __ldg(p0 + 1); v100 = __ldg(p0 + NY); v110 = __ldg(p0 + NY + 1);
        v001 = __ldg(p1); v011 = __ldg(p1 + 1); v101 = __ldg(p1 + NY); v111 = __ldg(p1 + NY + 1);
    }
    float v = trilerp(wx, wy, wz, v000, v001, v010, v011, v100, v101, v110, v111);
    if (Q.zero_guard) {
        float amax = fmaxf(fmaxf(fmaxf(fabsf(v000), fabsf(v001)), fmaxf(fabsf(v010), fabsf(v011))),
                           fmaxf(fmaxf(fabsf(v100), fabsf(v101)), fmaxf(fabsf(v110), fabsf(v111))));
        if (amax > 0.0f && fabsf(v) <= Q.band_zero * amax) return xnan();
    }
    return v;
}

template <bool TEX>
struct VoxSampler {
    const VoxParams& Q;
    const ViewDev* V;
    const double* xs;
    float uc[3], du[3];
    int i, j;
    static constexpr bool kHasInner = true;
    __device__ __forceinline__ float f32(float t) const {
        float ux = fmaf(du[0], t, uc[0]), uy = fmaf(du[1], t, uc[1]), uz = fmaf(du[2], t, uc[2]);
        float mx = fminf(ux, (float)(Q.nx - 1) - ux) * Q.inv_scale[0];
        float my = fminf(uy, (float)(Q.ny - 1) - uy) * Q.inv_scale[1];
        float mz = fminf(uz, (float)(Q.nz - 1) - uz) * Q.inv_scale[2];
        float m = fminf(mx, fminf(my, mz));
        if (m < -Q.band_w) return 0.0f;
        if (!(m > Q.band_w)) return xnan();
        return vox_inner<TEX>(Q, ux, uy, uz);
    }
    __device__ __forceinline__ float f32_inner(float t) const {
        return vox_inner<TEX>(Q, fmaf(du[0], t, uc[0]), fmaf(du[1], t, uc[1]), fmaf(du[2], t, uc[2]));
    }
    __device__ __forceinline__ double f64(double s) const { return vox_sample64(Q, *V, xs, i, j, s); }
    __device__ __forceinline__ double f64_inline(double s) const {
        return vox_sample64_inl(Q, *V, xs, i, j, s);
    }
};

// Voxel-grid root: one thread per pixel, same tiling as k_render.
template <bool TEX, bool HIER>
__global__ void __launch_bounds__(256, 4)
    k_voxel(const __grid_constant__ VoxParams Q, const __grid_constant__ Lattice L,
            const __grid_constant__ RenderParams P, const ViewDev* __restrict__ views, int view0,
            int nviews, float* __restrict__ out, unsigned long long* __restrict__ stats) {
    const int res = P.res;
    const int tpr = (res + 15) >> 4;
    const int tpv = tpr * tpr;
    const int b = blockIdx.x;
    const int v = b / tpv;
    const int t = b - v * tpv;
    const int ti = t / tpr, tj = t - ti * tpr;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int i = (ti << 4) + ((warp >> 1) << 2) + (lane >> 3);
    const int j = (tj << 4) + ((warp & 1) << 3) + (lane & 7);
    RayStats st{0, 0};
    if (v < nviews && i < res && j < res) {
        const ViewDev* V = views + view0 + v;
        Ray r;
        VoxSampler<TEX> smp{Q, V, P.xs, {0, 0, 0}, {0, 0, 0}, i, j};
        {
            Ray64 r64;
            setup_ray64_fast(*V, P.xs, i, j, r64);
            setup_ray32(r64, L.s_c, r);
            for (int a = 0; a < 3; a++) {
                double sc = (double)Q.scale[a];
                smp.uc[a] = (float)((fma(r64.d[a], L.s_c, r64.o[a]) + 1.0) * sc);
                smp.du[a] = (float)(r64.d[a] * sc);
            }
        }
        float acc = HIER ? march_hier(L, Q.lo, Q.hi, r, smp, st)
                         : march_simple(L, Q.lo, Q.hi, r, smp, st, Q.inner_margin);
        float w = HIER ? P.density_multiplier : P.density_multiplier * L.ds32;
        out[((size_t)v * res + i) * res + j] = expf(-fmaf(w, acc, P.flat_field));
    }
    if (stats) {
        unsigned s1 = __reduce_add_sync(0xffffffffu, st.samples);
        unsigned f1 = __reduce_add_sync(0xffffffffu, st.fallbacks);
        if (lane == 0) {
            atomicAdd(&stats[0], (unsigned long long)s1);
            if (f1) atomicAdd(&stats[1], (unsigned long long)f1);
        }
    }
}

// Reference voxelizer semantics (cuda_backend.cu:208-252): one voxel per
// thread, cylinders staged in shared memory.
__global__ void __launch_bounds__(256)
    k_voxelize(const CylinderParams* __restrict__ cyl, int ncyl, int res, float dm,
               const int* __restrict__ cell_off, const int* __restrict__ cell_idx, int grid_dim,
               int use_smem, float* __restrict__ out) {
    extern __shared__ CylinderParams s_cyl[];
    const bool spatial = cell_off != nullptr;
    if (use_smem) {
        for (int k = threadIdx.x; k < ncyl; k += blockDim.x) s_cyl[k] = cyl[k];
        __syncthreads();
    }
    long total = (long)res * res * res;
    for (long idx = (long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (long)gridDim.x * blockDim.x) {
        int k = (int)(idx / ((long)res * res));
        int i = (int)((idx / res) % res);
        int j = (int)(idx % res);
        float rf = (float)res;
        float x = (float)i / rf * 2.0f - 1.0f;
        float y = (float)j / rf * 2.0f - 1.0f;
        float z = (float)k / rf * 2.0f - 1.0f;
        int c0 = 0, c1 = ncyl;
        if (spatial) {
            float cs = 2.0f / (float)grid_dim;
            int cx = (int)((x + 1.0f) / cs), cy = (int)((y + 1.0f) / cs), cz = (int)((z + 1.0f) / cs);
            cx = min(max(cx, 0), grid_dim - 1);
            cy = min(max(cy, 0), grid_dim - 1);
            cz = min(max(cz, 0), grid_dim - 1);
            int cell = (cz * grid_dim + cy) * grid_dim + cx;
            c0 = cell_off[cell];
            c1 = cell_off[cell + 1];
        }
        float dens = 0.0f;
        for (int q = c0; q < c1; q++) {
            const CylinderParams c = spatial ? cyl[cell_idx[q]] : (use_smem ? s_cyl[q] : cyl[q]);
            float vx = c.p1[0] - c.p0[0], vy = c.p1[1] - c.p0[1], vz = c.p1[2] - c.p0[2];
            float wx = x - c.p0[0], wy = y - c.p0[1], wz = z - c.p0[2];
            float vv = vx * vx + vy * vy + vz * vz;
            if (vv == 0.0f) continue;
            float tt = (wx * vx + wy * vy + wz * vz) / vv;
            if (tt < 0.0f || tt > 1.0f) continue;
            float dx = wx - vx * tt, dy = wy - vy * tt, dz = wz - vz * tt;
            if (dx * dx + dy * dy + dz * dz < c.radius * c.radius) dens += c.rho;
        }
        dens *= dm;
        dens = fminf(fmaxf(dens, 0.0f), 1.0f);
        out[idx] = dens;
    }
}

// ---------------------------------------------------------------------------
// per-device engine state
// ---------------------------------------------------------------------------

namespace {

struct Engine {
    int device = -1;
    cudaStream_t compute = nullptr, copy = nullptr;
    cudaStream_t side = nullptr;  // highest priority: FP64 passes beside the next march
    cudaMemPool_t pool = nullptr;
    std::mutex mtx;
    unsigned long long* stats = nullptr;  // 2 counters
    bool ok = false;
    std::string init_error;
};

std::mutex g_engines_mtx;
std::map<int, std::unique_ptr<Engine>> g_engines;

Engine* engine_for_current(int* code) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        *code = cuda_fail(3, "cudaGetDevice", e);
        return nullptr;
    }
    std::lock_guard<std::mutex> g(g_engines_mtx);
    auto it = g_engines.find(dev);
    if (it != g_engines.end()) return it->second.get();
    auto E = std::make_unique<Engine>();
    E->device = dev;
    cudaMemPoolProps props;
    memset(&props, 0, sizeof(props));
    props.allocType = cudaMemAllocationTypePinned;
    props.handleTypes = cudaMemHandleTypeNone;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    int prio_least = 0, prio_greatest = 0;
    cudaDeviceGetStreamPriorityRange(&prio_least, &prio_greatest);
    if ((e = cudaStreamCreateWithFlags(&E->compute, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaStreamCreateWithFlags(&E->copy, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaStreamCreateWithPriority(&E->side, cudaStreamNonBlocking, prio_greatest)) != cudaSuccess ||
        (e = cudaMemPoolCreate(&E->pool, &props)) != cudaSuccess ||
        (e = cudaMalloc(&E->stats, 2 * sizeof(unsigned long long))) != cudaSuccess) {
        *code = cuda_fail(3, "engine initialisation", e);
        return nullptr;
    }
    uint64_t thr = UINT64_MAX;
    cudaMemPoolSetAttribute(E->pool, cudaMemPoolAttrReleaseThreshold, &thr);
    E->ok = true;
    Engine* raw = E.get();
    g_engines[dev] = std::move(E);
    return raw;
}

// Stream-ordered allocation from the engine pool, freed on the same stream.
struct PoolBuf {
    void* p = nullptr;
    cudaStream_t s = nullptr;
    cudaError_t alloc(Engine* E, size_t n, cudaStream_t st) {
        s = st;
        return cudaMallocFromPoolAsync(&p, n ? n : 16, E->pool, st);
    }
    ~PoolBuf() {
        if (p) cudaFreeAsync(p, s);
    }
};

// A voxel grid as a 2D layered texture (layer = z slice, width ny, height
// nx), point-sampled with clamp-to-edge addressing, for the gather sampler.
struct LayeredTex {
    cudaArray_t arr = nullptr;
    cudaTextureObject_t tex = 0;
    ~LayeredTex() { release(); }
    void release() {
        if (tex) cudaDestroyTextureObject(tex);
        if (arr) cudaFreeArray(arr);
        tex = 0;
        arr = nullptr;
    }
    // Returns cudaSuccess and leaves tex == 0 when the grid does not fit the
    // layered-texture limits (the load path is used then).
    cudaError_t create(const float* data, int nx, int ny, int nz, cudaStream_t st) {
        release();
        int dev = 0, mw = 0, mh = 0, ml = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&mw, cudaDevAttrMaxTexture2DLayeredWidth, dev);
        cudaDeviceGetAttribute(&mh, cudaDevAttrMaxTexture2DLayeredHeight, dev);
        cudaDeviceGetAttribute(&ml, cudaDevAttrMaxTexture2DLayeredLayers, dev);
        if (ny > mw || nx > mh || nz > ml || nx < 2 || ny < 2 || nz < 2) return cudaSuccess;
        cudaChannelFormatDesc fd = cudaCreateChannelDesc<float>();
        cudaError_t e = cudaMalloc3DArray(&arr, &fd, make_cudaExtent(ny, nx, nz), cudaArrayLayered);
        if (e != cudaSuccess) { arr = nullptr; return e; }
        cudaMemcpy3DParms cp;
        memset(&cp, 0, sizeof(cp));
        cp.srcPtr = make_cudaPitchedPtr((void*)data, (size_t)ny * sizeof(float), ny, nx);
        cp.dstArray = arr;
        cp.extent = make_cudaExtent(ny, nx, nz);
        cp.kind = cudaMemcpyDefault;
        if ((e = cudaMemcpy3DAsync(&cp, st)) != cudaSuccess) return e;
        cudaResourceDesc rd;
        memset(&rd, 0, sizeof(rd));
        rd.resType = cudaResourceTypeArray;
        rd.res.array.array = arr;
        cudaTextureDesc td;
        memset(&td, 0, sizeof(td));
        td.addressMode[0] = td.addressMode[1] = td.addressMode[2] = cudaAddressModeClamp;
        td.filterMode = cudaFilterModePoint;
        td.readMode = cudaReadModeElementType;
        td.normalizedCoords = 0;
        return cudaCreateTextureObject(&tex, &rd, &td, nullptr);
    }
};

// Gathers are the default for voxel-grid roots; XRP_VOLUME_PATH=loads selects
// the per-tap load path (both give the same results).
static bool volume_gathers_enabled() {
    const char* e = getenv("XRP_VOLUME_PATH");
    return !(e && strcmp(e, "loads") == 0);
}

// Host-side fault injection for the error paths (tests only; no GPU work
// fails): XRP_FAULT holds a comma-separated list of sites -- alloc (volume
// allocation, code 3), upload (volume upload, 4), tables (table upload, 5),
// output (image buffer allocation, 6), launch (kernel launch, 7), copy
// (image copy, 8) -- and each listed site reports the CUDA error it would
// see instead of calling CUDA.  Unset (the default) it injects nothing.
static cudaError_t injected(const char* site) {
    const char* e = getenv("XRP_FAULT");
    if (!e || !*e) return cudaSuccess;
    const size_t n = strlen(site);
    for (const char* p = e; *p;) {
        const char* q = strchr(p, ',');
        size_t len = q ? (size_t)(q - p) : strlen(p);
        if (len == n && strncmp(p, site, n) == 0) {
            if (!strcmp(site, "alloc") || !strcmp(site, "output")) return cudaErrorMemoryAllocation;
            if (!strcmp(site, "launch")) return cudaErrorLaunchFailure;
            return cudaErrorInvalidValue;  // upload, tables, copy
        }
        if (!q) break;
        p = q + 1;
    }
    return cudaSuccess;
}

// Packs small tables into one upload.
struct Tables {
    std::vector<unsigned char> host;
    size_t add(const void* src, size_t n, size_t align = 16) {
        size_t off = (host.size() + align - 1) / align * align;
        host.resize(off + n);
        if (n) memcpy(host.data() + off, src, n);
        return off;
    }
    template <class T>
    size_t add(const std::vector<T>& v) {
        return add(v.data(), v.size() * sizeof(T));
    }
};



void fill_voxparams(const HostPrepared& hp, const float* data, const double* data64,
                    cudaTextureObject_t tex, VoxParams& q) {
    memset(&q, 0, sizeof(q));
    const Volume& v = hp.vols[0];
    q.tex = tex;
    q.data = data;
    q.data64 = data64;
    q.nx = v.nx;
    q.ny = v.ny;
    q.nz = v.nz;
    q.zero_guard = hp.S.hier_zero_guard;
    for (int a = 0; a < 3; a++) {
        q.scale[a] = v.scale[a];
        q.inv_scale[a] = 1.0f / v.scale[a];
        q.lo[a] = hp.S.sup_lo[a];
        q.hi[a] = hp.S.sup_hi[a];
    }
    q.band_w = v.band_w;
    q.band_zero = hp.fs.nodes[hp.fs.root].f[0];
    q.inner_margin = 4.0f * v.band_w + 2e-4f;
}

// Offsets of one render's tables inside their packed upload.
struct TableLayout {
    size_t nodes, n64, child, cells, items, defs, clear, vols, views, xs, xsf, s64, t32, fs, f64, ft32;
};

// Packs the scene image, the cameras, the pixel table and the sample
// lattice of a prepared render into one host buffer.
TableLayout pack_tables(const HostPrepared& hp, const std::vector<ViewDev>& views, Tables& T) {
    const FlatScene& fs = hp.fs;
    const HostLattice& hl = hp.hl;
    TableLayout o;
    o.nodes = T.add(fs.nodes);
    o.n64 = T.add(fs.nodes64);
    o.child = T.add(fs.child);
    o.cells = T.add(fs.cells);
    o.items = T.add(fs.items);
    o.defs = T.add(fs.defs);
    o.clear = T.add(fs.clear);
    o.vols = T.add(hp.vols);
    o.views = T.add(views);
    o.xs = T.add(hp.xs);
    o.xsf = T.add(hp.xsf);
    o.s64 = T.add(hl.s64);
    o.t32 = T.add(hl.t32);
    o.fs = T.add(hl.fstart);
    o.f64 = T.add(hl.f64);
    o.ft32 = T.add(hl.ft32);
    return o;
}

// Points a Prepared render at tables packed by pack_tables and uploaded to
// the device address `base` (a pool buffer, or the no-allocation array).
void bind_tables(const HostPrepared& hp, const std::vector<ViewDev>& views, const unsigned char* base,
                 const TableLayout& o, cudaTextureObject_t tex, const float* vol0, const double* vol64_0,
                 Prepared& out) {
    const FlatScene& fs = hp.fs;
    const HostLattice& hl = hp.hl;
    out.S = hp.S;
    SceneDev& S = out.S;
    S.nodes = (const Node*)(base + o.nodes);
    S.nodes64 = (const Node64*)(base + o.n64);
    S.child = (const int32_t*)(base + o.child);
    S.cells = (const int32_t*)(base + o.cells);
    S.items = (const int32_t*)(base + o.items);
    S.clear = (const float*)(base + o.clear);
    S.defs = (const DefStep*)(base + o.defs);
    S.vols = (const Volume*)(base + o.vols);
    // tracing kernels stage node tables of up to 32 KB in shared memory
    S.nnodes = fs.nodes.size() * sizeof(Node) <= 32768 ? (int32_t)fs.nodes.size() : 0;
    out.L = hl.hdr;
    Lattice& L = out.L;
    L.s64 = (const double*)(base + o.s64);
    L.t32 = (const float*)(base + o.t32);
    L.fstart = (const int32_t*)(base + o.fs);
    L.f64 = (const double*)(base + o.f64);
    L.ft32 = (const float*)(base + o.ft32);
    out.P = hp.P;
    out.P.nviews = (int)views.size();
    out.P.xs = (const double*)(base + o.xs);
    out.P.xsf = (const float*)(base + o.xsf);
    out.views = (const ViewDev*)(base + o.views);
    out.volume_fast = hp.volume_fast;
    out.depth = fs.depth;
    out.defs = !fs.defs.empty();
    out.tex = hp.volume_fast ? tex : 0;
    out.empty = hl.hdr.K <= 0;
    out.leaves = 0;
    for (const Node& n : fs.nodes)
        if (n.type >= N_SPHERE && n.type <= N_GYROID) out.leaves |= 1 << n.type;
    if (hp.volume_fast) fill_voxparams(hp, vol0, vol64_0, out.tex, out.vq);
}

// Everything a render needs on the device except the volume data.
int prepare(Engine* E, const HostScene& hs, const std::vector<const float*>& vol_dev,
            const std::vector<const double*>& vol64_dev, const std::vector<ViewDev>& views,
            int res, int integration, double ds, double R, double ff, double dm, double fov_max,
            cudaStream_t st, PoolBuf& tab, Prepared& out, cudaTextureObject_t tex, bool tracing = false,
            bool fine_lists = false) {
    HostPrepared hp;
    try {
        hp = prepare_host(hs, res, integration, ds, R, ff, dm, fov_max, tracing, fine_lists);
    } catch (const std::exception& ex) {
        return fail(2, "%s", ex.what());
    }
    for (size_t k = 0; k < hp.vols.size(); k++) {
        hp.vols[k].data = vol_dev[k];
        hp.vols[k].data64 = vol64_dev[k];
    }
    Tables T;
    const TableLayout o = pack_tables(hp, views, T);
    cudaError_t e = tab.alloc(E, T.host.size(), st);
    if (e != cudaSuccess) return cuda_fail(3, "table allocation", e);
    if ((e = injected("tables")) == cudaSuccess)
        e = cudaMemcpyAsync(tab.p, T.host.data(), T.host.size(), cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return cuda_fail(5, "table upload", e);
    bind_tables(hp, views, (const unsigned char*)tab.p, o, tex, vol_dev.empty() ? nullptr : vol_dev[0],
                vol64_dev.empty() ? nullptr : vol64_dev[0], out);
    return 0;
}

}  // namespace

// ---------------------------------------------------------------------------
// launch
// ---------------------------------------------------------------------------

// The list of samples a march leaves to FP64 (k_prop_fallback), reused by
// every launch of a call: four (ray, sample) entries per ray of a launch of
// pl.max_rays rays, with its counter and overflow flag.
// XRP_FALLBACK_LIST (a test hook) sets a smaller capacity, which exercises
// the overflow paths.
// With `slots` 2 the list, counter and flag come twice (pl.fb_slot,
// pl.cnt_slot), for the overlapped launch groups.
static int alloc_fallback_list(Engine* E, PropLaunch& pl, PoolBuf& fb, PoolBuf& fbc, cudaStream_t st,
                               int slots = 1) {
    unsigned fb_cap = (unsigned)std::max<long long>(1 << 20, (1LL << 23) * 4);
    if (const char* c = getenv("XRP_FALLBACK_LIST"))
        if (*c) fb_cap = (unsigned)std::min<long long>(fb_cap, std::max(1LL, atoll(c)));
    cudaError_t e;
    if ((e = fb.alloc(E, (size_t)slots * fb_cap * sizeof(uint2), st)) != cudaSuccess ||
        (e = fbc.alloc(E, (size_t)slots * 2 * sizeof(unsigned), st)) != cudaSuccess)
        return cuda_fail(3, "fallback list", e);
    if ((e = cudaMemsetAsync(fbc.p, 0, (size_t)slots * 2 * sizeof(unsigned), st)) != cudaSuccess)
        return cuda_fail(7, "fallback list reset", e);
    for (int k = 0; k < slots; k++) {
        pl.fb_slot[k] = (uint2*)fb.p + (size_t)k * fb_cap;
        pl.cnt_slot[k] = (unsigned*)fbc.p + 2 * k;
    }
    pl.Q.fb = pl.fb_slot[0];
    pl.Q.fb_count = pl.cnt_slot[0];
    pl.Q.fb_overflow = pl.cnt_slot[0] + 1;
    pl.Q.fb_cap = fb_cap;
    return 0;
}

// Whether a launch group found the FP64 list full (either slot).
static cudaError_t list_overflowed(const PropLaunch& pl, cudaStream_t st, unsigned* ovf) {
    unsigned h[2] = {0, 0};
    cudaError_t e = cudaSuccess;
    for (int k = 0; k < 2 && e == cudaSuccess; k++)
        if (pl.cnt_slot[k]) e = cudaMemcpyAsync(&h[k], pl.cnt_slot[k] + 1, sizeof(unsigned), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    *ovf = h[0] | h[1];
    return e;
}

// Events of the overlapped launch groups (PropLaunch::side).
struct OverlapEvents {
    cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
    cudaError_t create(PropLaunch& pl, cudaStream_t side) {
        for (auto& x : ev) {
            cudaError_t e = cudaEventCreateWithFlags(&x, cudaEventDisableTiming);
            if (e != cudaSuccess) return e;
        }
        pl.marched = ev[0];
        pl.done[0] = ev[1];
        pl.done[1] = ev[2];
        pl.side = side;
        return cudaSuccess;
    }
    ~OverlapEvents() {
        for (auto x : ev)
            if (x) cudaEventDestroy(x);
    }
};

// Overlapping each launch group's FP64 pass with the next group's march:
// on unless XRP_FB_OVERLAP is 0.
static bool overlap_enabled() {
    const char* c = getenv("XRP_FB_OVERLAP");
    return !(c && c[0] == '0');
}

static cudaError_t launch_prop(const Prepared& pr, int view0, int nviews, PropLaunch& pl, float* dout,
                               cudaStream_t st) {
    if (pl.train) return launch_prop_train(pr, view0, nviews, pl.Q, st);
    if (!pl.side) return launch_prop_render(pr, view0, nviews, pl.Q, dout, st);
    // group g uses list slot g & 1; its march waits until the FP64 pass of
    // group g - 2 (the slot's previous user) is done with the list, and its
    // tail runs on the side stream once the march is
    const int k = pl.groups & 1;
    PropParams Q = pl.Q;
    Q.fb = pl.fb_slot[k];
    Q.fb_count = pl.cnt_slot[k];
    Q.fb_overflow = pl.cnt_slot[k] + 1;
    if (Q.trace == 4) {
        Q.redo = pl.redo_slot[k];
        Q.redo_count = pl.redo_cnt_slot[k];
    }
    cudaError_t e;
    if (pl.groups >= 2 && (e = cudaStreamWaitEvent(st, pl.done[k], 0)) != cudaSuccess) return e;
    if ((e = launch_prop_march(pr, view0, nviews, Q, dout, st)) != cudaSuccess) return e;
    if ((e = cudaEventRecord(pl.marched, st)) != cudaSuccess ||
        (e = cudaStreamWaitEvent(pl.side, pl.marched, 0)) != cudaSuccess)
        return e;
    // one block of the FP64 pass per SM: it takes the registers one march
    // block frees, and the next group's march keeps the rest (two blocks:
    // lattice 515 against 533 Mrays/s, gyroid 1922 against 2036)
    if ((e = launch_prop_tail(pr, view0, nviews, Q, dout, pl.side, 1)) != cudaSuccess) return e;
    if ((e = cudaEventRecord(pl.done[k], pl.side)) != cudaSuccess) return e;
    pl.groups++;
    return cudaSuccess;
}

// The call's stream waits for every tail still on the side stream.
static cudaError_t join_side(const PropLaunch* pl, cudaStream_t st) {
    if (!pl || !pl->side) return cudaSuccess;
    for (int k = 0; k < 2 && k < pl->groups; k++) {
        cudaError_t e = cudaStreamWaitEvent(st, pl->done[k], 0);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

static cudaError_t launch(const Prepared& pr, int view0, int nviews, int integration, float* dout,
                          unsigned long long* stats, cudaStream_t st, PropLaunch* pl = nullptr) {
    if (pl) return launch_prop(pr, view0, nviews, *pl, dout, st);
    const ViewDev* dviews = pr.views;
    const int res = pr.P.res;
    const int tpr = (res + 15) / 16;
    long blocks = (long)nviews * tpr * tpr;
    if (blocks <= 0) return cudaSuccess;
    if (blocks > 0x7fffffffL) return cudaErrorInvalidConfiguration;
    dim3 grid((unsigned)blocks), block(256);
    bool hier = integration == XRP_INTEGRATE_HIERARCHICAL;
    if (pr.volume_fast) {
        bool tex = pr.vq.tex != 0;
        if (hier && tex) k_voxel<true, true><<<grid, block, 0, st>>>(pr.vq, pr.L, pr.P, dviews, view0, nviews, dout, stats);
        else if (hier) k_voxel<false, true><<<grid, block, 0, st>>>(pr.vq, pr.L, pr.P, dviews, view0, nviews, dout, stats);
        else if (tex) k_voxel<true, false><<<grid, block, 0, st>>>(pr.vq, pr.L, pr.P, dviews, view0, nviews, dout, stats);
        else k_voxel<false, false><<<grid, block, 0, st>>>(pr.vq, pr.L, pr.P, dviews, view0, nviews, dout, stats);
    } else {
        return launch_scene(pr, view0, nviews, hier, dout, stats, st);
    }
    return cudaGetLastError();
}

// Renders `views` into `out` (device or host memory).  Host output goes
// through two or three device chunk buffers so the copy of chunk c overlaps
// the rendering of the next chunks.
//
// plain_list: the plain integrator over a general scene (not the voxel-grid
// fast path) marches in the tracing kernel's plain mode, which leaves the
// samples FP32 cannot decide on a list for one FP64 pass instead of
// re-evaluating them inside the march (k_render: the FP64 state held across
// the loop costs registers and spills, and a warp waits on each lane's FP64
// evaluation).  Samples that find the list full are evaluated in place, so
// the call needs no overflow check and stays asynchronous.
static int render_views(Engine* E, const HostScene& hs, const std::vector<const float*>& vdev,
                        const std::vector<const double*>& v64, const std::vector<ViewDev>& views,
                        const xrp_render_opts& o, double fov_max, float* out, bool out_host,
                        cudaStream_t st, cudaStream_t st_copy, bool want_stats,
                        cudaTextureObject_t tex, PropLaunch* pl = nullptr, bool plain_list = false) {
    const int res = o.resolution;
    const int nviews = (int)views.size();
    PoolBuf tab;
    Prepared pr;
    // fine candidate lists from 2^25 rays: the march saves more than the
    // longer flattening costs (deformed lattice, plain: 171 -> 194 Mrays/s
    // for 0.1 -> 3.9 ms of host time per call)
    const bool fine = (long long)nviews * res * res >= (1LL << 25);
    int rc = prepare(E, hs, vdev, v64, views, res, o.integration, o.ds, o.R, o.flat_field,
                     o.density_multiplier, fov_max, st, tab, pr,
                     (o.flags & XRP_FLAG_VOLUME_LOADS) ? 0 : tex, pl && pl->Q.trace && pl->Q.trace != 4, fine);
    if (rc) return rc;
    unsigned long long* stats = nullptr;
    cudaError_t e;
    PropLaunch plain;
    PoolBuf lbuf, lcnt, lstats, rbuf, rcnt;
    // below 2^22 rays the list's extra launches cost more than the in-place
    // re-evaluation (one 512^2 view: 785 against 994 Mrays/s)
    const bool big = (long long)nviews * res * res >= (1LL << 22);
    const bool listed = plain_list && !pl && !pr.volume_fast && !(o.flags & XRP_FLAG_PLAIN_INPLACE) &&
                        ((o.flags & XRP_FLAG_PLAIN_LIST) || big);
    if (listed) {
        memset(&plain.Q, 0, sizeof(plain.Q));
        plain.Q.trace = 4;
        if (o.integration == XRP_INTEGRATE_HIERARCHICAL) plain.max_rays = 1LL << 21;
        const int slots = (long long)nviews * res * res > plain.max_rays ? 2 : 1;
        if ((rc = alloc_fallback_list(E, plain, lbuf, lcnt, st, slots))) return rc;
        // one slot per ray of the largest launch (the view split below)
        const long long img_rays = (long long)res * res;
        const long long redo_rays =
            std::min<long long>(nviews, std::max<long long>(1, plain.max_rays / img_rays)) * img_rays;
        if (redo_rays > 0xffffffffLL) return fail(2, "too many rays per launch for the redo list");
        if ((e = rbuf.alloc(E, (size_t)slots * redo_rays * sizeof(unsigned), st)) != cudaSuccess ||
            (e = rcnt.alloc(E, (size_t)slots * sizeof(unsigned), st)) != cudaSuccess)
            return cuda_fail(3, "redo list", e);
        for (int k = 0; k < slots; k++) {
            plain.redo_slot[k] = (unsigned*)rbuf.p + (size_t)k * redo_rays;
            plain.redo_cnt_slot[k] = (unsigned*)rcnt.p + k;
        }
        plain.Q.redo = plain.redo_slot[0];
        plain.Q.redo_count = plain.redo_cnt_slot[0];
        plain.Q.redo_cap = (unsigned)redo_rays;
        if (want_stats) {
            if ((e = lstats.alloc(E, kStatCount * sizeof(unsigned long long), st)) != cudaSuccess)
                return cuda_fail(3, "stats buffer", e);
            if ((e = cudaMemsetAsync(lstats.p, 0, kStatCount * sizeof(unsigned long long), st)) != cudaSuccess)
                return cuda_fail(7, "stats reset", e);
            plain.Q.stats = (unsigned long long*)lstats.p;
        }
        pl = &plain;
    } else if (want_stats) {
        if ((e = cudaMemsetAsync(E->stats, 0, 2 * sizeof(unsigned long long), st)) != cudaSuccess)
            return cuda_fail(7, "stats reset", e);
        stats = E->stats;
    }
    const size_t img = (size_t)res * res;
    const int tpv = ((res + 15) / 16) * ((res + 15) / 16);
    int max_views_per_launch = std::max(1, (int)(0x7fffffffL / tpv));
    if (pl) max_views_per_launch = std::max(1, std::min<int>(max_views_per_launch, (int)(pl->max_rays / (long long)img)));
    // two list slots: each launch group's FP64 pass beside the next march
    // (the side stream and its events live for this call only)
    OverlapEvents ovl;
    if (pl) {
        pl->side = nullptr;
        pl->groups = 0;
    }
    if (pl && !pl->train && pl->fb_slot[1] && nviews > max_views_per_launch && overlap_enabled()) {
        pl->groups = 0;
        if ((e = ovl.create(*pl, E->side)) != cudaSuccess) return cuda_fail(7, "overlap events", e);
    }
    if (!out_host) {
        for (int v0 = 0; v0 < nviews; v0 += max_views_per_launch) {
            int n = std::min(max_views_per_launch, nviews - v0);
            if ((e = injected("launch")) != cudaSuccess ||
                (e = launch(pr, v0, n, o.integration, out + (size_t)v0 * img, stats, st, pl)) != cudaSuccess) {
                join_side(pl, st);
                return cuda_fail(7, "kernel launch", e);
            }
        }
        if ((e = join_side(pl, st)) != cudaSuccess) return cuda_fail(7, "kernel launch", e);
    } else {
        size_t chunk = std::max<size_t>(1, std::min<size_t>((size_t)nviews, ((size_t)64 << 20) / (img * 4)));
        chunk = std::min<size_t>(chunk, (size_t)max_views_per_launch);
        int nchunks = (int)((nviews + chunk - 1) / chunk);
        // chunk buffers: two, or three when the FP64 passes run on the side
        // stream (a chunk is copied only after its pass, and the march that
        // reuses its buffer would wait for that copy with two)
        const int nbuf = (pl && pl->side) ? 3 : 2;
        PoolBuf buf[3];
        for (int b = 0; b < std::min(nbuf, nchunks); b++)
            if ((e = injected("output")) != cudaSuccess ||
                (e = buf[b].alloc(E, chunk * img * sizeof(float), st)) != cudaSuccess) {
                join_side(pl, st);
                return cuda_fail(6, "image buffer allocation", e);
            }
        cudaEvent_t kev[3], cev[3];
        for (int b = 0; b < 3; b++) {
            cudaEventCreateWithFlags(&kev[b], cudaEventDisableTiming);
            cudaEventCreateWithFlags(&cev[b], cudaEventDisableTiming);
        }
        auto launch_chunk = [&](int c) -> cudaError_t {
            int b = c % nbuf;
            if (c >= nbuf) cudaStreamWaitEvent(st, cev[b], 0);
            int v0 = (int)(c * chunk);
            int n = (int)std::min(chunk, (size_t)(nviews - v0));
            cudaError_t le = injected("launch");
            if (le == cudaSuccess) le = launch(pr, v0, n, o.integration, (float*)buf[b].p, stats, st, pl);
            // overlapped groups finish on the side stream
            cudaEventRecord(kev[b], (pl && pl->side) ? pl->side : st);
            return le;
        };
        int code = 0;
        if ((e = launch_chunk(0)) != cudaSuccess) code = cuda_fail(7, "kernel launch", e);
        for (int c = 0; c < nchunks && !code; c++) {
            if (c + 1 < nchunks && (e = launch_chunk(c + 1)) != cudaSuccess) {
                code = cuda_fail(7, "kernel launch", e);
                break;
            }
            int b = c % nbuf;
            int v0 = (int)(c * chunk);
            size_t n = std::min(chunk, (size_t)(nviews - v0));
            cudaStreamWaitEvent(st_copy, kev[b], 0);
            if ((e = injected("copy")) == cudaSuccess)
                e = cudaMemcpyAsync(out + (size_t)v0 * img, buf[b].p, n * img * sizeof(float),
                                    cudaMemcpyDeviceToHost, st_copy);
            if (e != cudaSuccess) {
                code = cuda_fail(8, "image copy", e);
                break;
            }
            cudaEventRecord(cev[b], st_copy);
        }
        cudaError_t e0 = join_side(pl, st);
        cudaError_t e1 = cudaStreamSynchronize(st_copy);
        cudaError_t e2 = cudaStreamSynchronize(st);
        if (e2 == cudaSuccess) e2 = e0;
        for (int b = 0; b < 3; b++) {
            cudaEventDestroy(kev[b]);
            cudaEventDestroy(cev[b]);
        }
        if (code) return code;
        if (e2 != cudaSuccess) return cuda_fail(7, "kernel execution", e2);
        if (e1 != cudaSuccess) return cuda_fail(8, "image copy", e1);
    }
    if (listed) {
        if (want_stats) {
            unsigned long long h[kStatCount];
            if ((e = cudaMemcpyAsync(h, lstats.p, sizeof(h), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
                (e = cudaStreamSynchronize(st)) != cudaSuccess)
                return cuda_fail(7, "stats read", e);
            t_stats[0] = h[kStatEvaluations];
            t_stats[1] = h[kStatFallbacks];
        }
        return 0;
    }
    if (want_stats) {
        unsigned long long h[2] = {0, 0};
        if ((e = cudaMemcpyAsync(h, E->stats, sizeof(h), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
            (e = cudaStreamSynchronize(st)) != cudaSuccess)
            return cuda_fail(7, "stats read", e);
        t_stats[0] = h[0];
        t_stats[1] = h[1];
    }
    return 0;
}

// ---------------------------------------------------------------------------
// scenes
// ---------------------------------------------------------------------------

struct xrp_scene {
    HostScene hs;
    std::vector<void*> owned;  // device allocations (cudaMalloc)
    std::vector<const float*> vdev;
    std::vector<const double*> v64;
    int device = -1;
    double sup_lo[3], sup_hi[3];
    std::unique_ptr<LayeredTex> tex;  // root voxel grid as a layered texture
    bool tex_tried = false;
};

static void scene_free(xrp_scene* s) {
    if (!s) return;
    for (void* p : s->owned) cudaFree(p);
    delete s;
}

// Builds the layered texture of a voxel-grid root once per scene.
static int scene_texture(xrp_scene* s, cudaStream_t st) {
    if (s->tex_tried) return 0;
    s->tex_tried = true;
    const HNode& r = s->hs.nodes[s->hs.root];
    if (r.type != N_VOXEL || !s->hs.defs.empty() || !volume_gathers_enabled()) return 0;
    const HVolume& v = s->hs.vols[r.vol];
    auto t = std::make_unique<LayeredTex>();
    cudaError_t e = t->create(s->vdev[r.vol], v.nx, v.ny, v.nz, st);
    if (e != cudaSuccess) return cuda_fail(3, "volume texture", e);
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return cuda_fail(4, "volume texture copy", e);
    if (t->tex) s->tex = std::move(t);
    return 0;
}

static bool opts_ok(const xrp_render_opts* o, std::string& why) {
    if (!o) { why = "null options"; return false; }
    if (o->resolution <= 0) { why = "resolution must be > 0"; return false; }
    if (!(o->ds > 0) || !std::isfinite(o->ds)) { why = "ds must be > 0 and finite"; return false; }
    if (!std::isfinite(o->R)) { why = "R must be finite"; return false; }
    if (o->integration != XRP_INTEGRATE_SIMPLE && o->integration != XRP_INTEGRATE_HIERARCHICAL) {
        why = "unknown integration method";
        return false;
    }
    double samples = 3.48 / o->ds;
    if (samples > 5.0e7) { why = "ds too small (more than 5e7 samples per ray)"; return false; }
    return true;
}

static std::vector<ViewDev> views_from(const xrp_camera* cams, int n, double* fov_max) {
    std::vector<ViewDev> v(n);
    *fov_max = 0;
    for (int k = 0; k < n; k++) {
        view_from_camera(cams[k].eye, cams[k].camera, cams[k].fov_deg, v[k]);
        *fov_max = std::max(*fov_max, std::fabs(cams[k].fov_deg));
    }
    return v;
}

extern "C" {

const char* xrp_last_error(void) { return t_err.c_str(); }

int xrp_version(void) { return 100; }

int xrp_cameras_from_angles(const double* az_polar, int n, double R, double fov_deg, xrp_camera* out) {
    if (!az_polar || !out) return fail(1, "null pointer");
    if (n < 0) return fail(2, "negative count");
    for (int k = 0; k < n; k++) {
        camera_from_angles(az_polar[2 * k], az_polar[2 * k + 1], R, out[k].eye, out[k].camera);
        out[k].fov_deg = fov_deg;
    }
    return 0;
}

int xrp_scene_create(const char* object_json, const char* deformation_json,
                     const xrp_volume_desc* volumes, int num_volumes, xrp_scene** out) {
    if (!object_json || !out) return fail(1, "null pointer");
    if (num_volumes < 0 || (num_volumes > 0 && !volumes)) return fail(1, "bad volume list");
    *out = nullptr;
    int code = 0;
    Engine* E = engine_for_current(&code);
    if (!E) return code;
    std::unique_ptr<xrp_scene, void (*)(xrp_scene*)> s(new xrp_scene(), scene_free);
    s->device = E->device;
    std::vector<HVolume> ext(num_volumes);
    for (int k = 0; k < num_volumes; k++) {
        const xrp_volume_desc& d = volumes[k];
        if (!d.data) return fail(1, "volume %d: null data", k);
        if (d.nx <= 0 || d.ny <= 0 || d.nz <= 0) return fail(2, "volume %d: bad sizes", k);
        ext[k].nx = d.nx;
        ext[k].ny = d.ny;
        ext[k].nz = d.nz;
        if (d.on_device) {
            ext[k].ext = d.data;
        } else {
            size_t n = (size_t)d.nx * d.ny * d.nz;
            ext[k].data.assign(d.data, d.data + n);
        }
    }
    try {
        s->hs = load_scene(object_json, deformation_json, ext);
        RenderGeometry g;
        FlatScene fs = flatten(s->hs, g, false);  // validates depth and types
        for (int a = 0; a < 3; a++) {
            s->sup_lo[a] = fs.sup_lo[a];
            s->sup_hi[a] = fs.sup_hi[a];
        }
    } catch (const std::exception& ex) {
        return fail(2, "%s", ex.what());
    }
    for (auto& v : s->hs.vols) {
        size_t n = (size_t)v.nx * v.ny * v.nz;
        if (v.ext) {
            s->vdev.push_back(v.ext);
        } else {
            void* p = nullptr;
            cudaError_t e = cudaMalloc(&p, n * sizeof(float));
            if (e != cudaSuccess) return cuda_fail(3, "volume allocation", e);
            s->owned.push_back(p);
            if ((e = cudaMemcpy(p, v.data.data(), n * sizeof(float), cudaMemcpyHostToDevice)) != cudaSuccess)
                return cuda_fail(4, "volume upload", e);
            s->vdev.push_back((const float*)p);
            std::vector<float>().swap(v.data);
        }
        if (!v.data64.empty()) {
            void* p = nullptr;
            cudaError_t e = cudaMalloc(&p, n * sizeof(double));
            if (e != cudaSuccess) return cuda_fail(3, "volume allocation", e);
            s->owned.push_back(p);
            if ((e = cudaMemcpy(p, v.data64.data(), n * sizeof(double), cudaMemcpyHostToDevice)) != cudaSuccess)
                return cuda_fail(4, "volume upload", e);
            s->v64.push_back((const double*)p);
            std::vector<double>().swap(v.data64);
        } else {
            s->v64.push_back(nullptr);
        }
    }
    *out = s.release();
    return 0;
}

void xrp_scene_destroy(xrp_scene* scene) { scene_free(scene); }

int xrp_scene_support(const xrp_scene* s, double lo[3], double hi[3]) {
    if (!s || !lo || !hi) return fail(1, "null pointer");
    for (int a = 0; a < 3; a++) {
        lo[a] = s->sup_lo[a];
        hi[a] = s->sup_hi[a];
    }
    return 0;
}

int xrp_scene_min_feature_size(const xrp_scene* s, double* out) {
    if (!s || !out) return fail(1, "null pointer");
    *out = min_feature_size(s->hs);
    return 0;
}

int xrp_render(xrp_scene* s, const xrp_camera* views, int nviews, const xrp_render_opts* o, float* out) {
    if (!s || !views || !o || !out) return fail(1, "null pointer");
    std::string why;
    if (nviews <= 0) return fail(2, "num_views must be > 0");
    if (!opts_ok(o, why)) return fail(2, "%s", why.c_str());
    int code = 0;
    Engine* E = engine_for_current(&code);
    if (!E) return code;
    if (E->device != s->device) return fail(2, "scene belongs to device %d", s->device);
    double fov_max;
    std::vector<ViewDev> v = views_from(views, nviews, &fov_max);
    std::lock_guard<std::mutex> g(E->mtx);
    int rc = scene_texture(s, E->compute);
    if (rc) return rc;
    return render_views(E, s->hs, s->vdev, s->v64, v, *o, fov_max, out, true, E->compute, E->copy,
                        (o->flags & XRP_FLAG_STATS) != 0, s->tex ? s->tex->tex : 0, nullptr, true);
}

int xrp_render_device(xrp_scene* s, const xrp_camera* views, int nviews, const xrp_render_opts* o,
                      float* out_device, void* stream) {
    if (!s || !views || !o || !out_device) return fail(1, "null pointer");
    std::string why;
    if (nviews <= 0) return fail(2, "num_views must be > 0");
    if (!opts_ok(o, why)) return fail(2, "%s", why.c_str());
    int code = 0;
    Engine* E = engine_for_current(&code);
    if (!E) return code;
    if (E->device != s->device) return fail(2, "scene belongs to device %d", s->device);
    double fov_max;
    std::vector<ViewDev> v = views_from(views, nviews, &fov_max);
    int rc = scene_texture(s, (cudaStream_t)stream);
    if (rc) return rc;
    // stats use the engine's shared counters and need a synchronisation
    return render_views(E, s->hs, s->vdev, s->v64, v, *o, fov_max, out_device, false,
                        (cudaStream_t)stream, (cudaStream_t)stream, false,
                        s->tex ? s->tex->tex : 0, nullptr, true);
}

int xrp_last_stats(uint64_t* samples, uint64_t* fp64_samples) {
    if (samples) *samples = t_stats[0];
    if (fp64_samples) *fp64_samples = t_stats[1];
    return 0;
}

void xrp_release_cache(void) {
    std::lock_guard<std::mutex> g(g_engines_mtx);
    for (auto& kv : g_engines) {
        std::lock_guard<std::mutex> g2(kv.second->mtx);
        cudaStreamSynchronize(kv.second->compute);
        cudaStreamSynchronize(kv.second->copy);
        cudaMemPoolTrimTo(kv.second->pool, 0);
    }
}

int xrp_voxelize_scene(xrp_scene* s, int res, double dm, float* out_f32, unsigned char* out_u8) {
    if (!s || (!out_f32 && !out_u8)) return fail(1, "null pointer");
    if (res <= 0 || res > 2048) return fail(2, "res must be in [1, 2048]");
    int code = 0;
    Engine* E = engine_for_current(&code);
    if (!E) return code;
    if (E->device != s->device) return fail(2, "scene belongs to device %d", s->device);
    std::lock_guard<std::mutex> g(E->mtx);
    cudaStream_t st = E->compute;
    // the error analysis of the default camera (R 4, fov 40) covers grid
    // points (|p| <= 1, one FP32 rounding)
    std::vector<ViewDev> views(1);
    memset(views.data(), 0, sizeof(ViewDev));
    PoolBuf tab, vol, vmax, u8;
    Prepared pr;
    int rc = prepare(E, s->hs, s->vdev, s->v64, views, 8, XRP_INTEGRATE_SIMPLE, 0.01, 4.0, 0.0, 1.0, 40.0, st,
                     tab, pr, 0);
    if (rc) return rc;
    const size_t nvox = (size_t)res * res * res;
    cudaError_t e;
    if ((e = vol.alloc(E, nvox * sizeof(float), st)) != cudaSuccess || (e = vmax.alloc(E, 16, st)) != cudaSuccess ||
        (out_u8 && (e = u8.alloc(E, nvox, st)) != cudaSuccess))
        return cuda_fail(3, "volume allocation", e);
    e = launch_voxelize_scene(pr.S, pr.depth == 0 ? 0 : kMaxDepth, pr.defs, res, dm, (float*)vol.p,
                              (unsigned*)vmax.p, out_u8 ? (unsigned char*)u8.p : nullptr, st);
    if (e != cudaSuccess) return cuda_fail(5, "voxelizer kernel", e);
    if (out_f32 && (e = cudaMemcpyAsync(out_f32, vol.p, nvox * sizeof(float), cudaMemcpyDeviceToHost, st)) != cudaSuccess)
        return cuda_fail(6, "volume copy", e);
    if (out_u8 && (e = cudaMemcpyAsync(out_u8, u8.p, nvox, cudaMemcpyDeviceToHost, st)) != cudaSuccess)
        return cuda_fail(6, "volume copy", e);
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return cuda_fail(5, "voxelizer kernel", e);
    return 0;
}

int xrp_finish_images(const float* d_images, int nviews, int res, int transparency, uint16_t* d_gray,
                      uint16_t* d_alpha, float* d_minmax, void* stream) {
    if (!d_images || !d_gray || !d_minmax) return fail(1, "null pointer");
    if (nviews <= 0 || res <= 0) return fail(2, "bad sizes");
    if (nviews > 65535) return fail(2, "at most 65535 views per call");
    cudaError_t e = launch_finish(d_images, nviews, res, transparency, (unsigned short*)d_gray,
                                  (unsigned short*)d_alpha, d_minmax, (cudaStream_t)stream);
    if (e != cudaSuccess) return cuda_fail(7, "finishing kernel", e);
    return 0;
}

int xrp_probe_gather_rate(double* gathers_per_s) {
    if (!gathers_per_s) return fail(1, "null pointer");
    int code = 0;
    Engine* E = engine_for_current(&code);
    if (!E) return code;
    std::lock_guard<std::mutex> g(E->mtx);
    cudaStream_t st = E->compute;
    std::vector<float> host(32 * 32 * 2);
    for (size_t k = 0; k < host.size(); k++) host[k] = (float)(k % 7);
    PoolBuf dv, sink;
    cudaError_t e;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, E->device);
    const int blocks = sms * 8, iters = 8192;
    if ((e = dv.alloc(E, host.size() * sizeof(float), st)) != cudaSuccess ||
        (e = sink.alloc(E, (size_t)blocks * 256 * sizeof(float), st)) != cudaSuccess)
        return cuda_fail(3, "probe buffers", e);
    if ((e = cudaMemcpyAsync(dv.p, host.data(), host.size() * sizeof(float), cudaMemcpyHostToDevice, st)) != cudaSuccess)
        return cuda_fail(4, "probe upload", e);
    LayeredTex t;
    if ((e = t.create((const float*)dv.p, 32, 32, 2, st)) != cudaSuccess || !t.tex) return cuda_fail(3, "probe texture", e);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float ms = 0.0f;
    for (int rep = 0; rep < 3; rep++) {
        cudaEventRecord(e0, st);
        k_gather_probe<<<blocks, 256, 0, st>>>(t.tex, iters, (float*)sink.p);
        cudaEventRecord(e1, st);
        if ((e = cudaEventSynchronize(e1)) != cudaSuccess) break;
        cudaEventElapsedTime(&ms, e0, e1);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (e != cudaSuccess || (e = cudaGetLastError()) != cudaSuccess) return cuda_fail(7, "probe kernel", e);
    *gathers_per_s = (double)blocks * 256 * iters / (ms * 1e-3);
    return 0;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// batched rendering
// ---------------------------------------------------------------------------

struct xrp_batch {
    int device = -1;
    void* tables = nullptr;   // scenes, views, pixel tables, lattice, items (cudaMalloc)
    float* out = nullptr;     // all items' images
    unsigned long long* counter = nullptr;
    std::vector<long long> offset;  // per item (caller's order)
    std::vector<long long> size;
    BatchLaunch bl;
    cudaStream_t cap = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaEvent_t rendered = nullptr;  // recorded after each replay, on its stream
    xrp_batch_info info;
};

static void batch_free(xrp_batch* b) {
    if (!b) return;
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    // cudaFree waits for the device, so no replay can still use the images
    if (b->tables) cudaFree(b->tables);
    if (b->counter) cudaFree(b->counter);
    if (b->out) {  // back to the engine pool
        if (b->cap) cudaFreeAsync(b->out, b->cap);
        else cudaFree(b->out);
    }
    if (b->cap) cudaStreamDestroy(b->cap);
    if (b->rendered) cudaEventDestroy(b->rendered);
    delete b;
}

// Items' tiling for a tile shape, in work order; returns the tile count.
static long long batch_tiling(std::vector<BatchItemDev>& items, int tw, int th) {
    long long t0 = 0;
    for (auto& it : items) {
        const int res = it.P.res;
        it.tiles_x = (res + tw - 1) / tw;
        it.tiles_y = (res + th - 1) / th;
        it.tile0 = t0;
        t0 += (long long)it.nviews * it.tiles_x * it.tiles_y;
    }
    return t0;
}

extern "C" {

int xrp_batch_create(const xrp_batch_item* items, int n, const xrp_render_opts* o, int autotune,
                     xrp_batch** out) {
    if (!items || !o || !out) return fail(1, "null pointer");
    *out = nullptr;
    if (n <= 0) return fail(2, "num_items must be > 0");
    xrp_render_opts oo = *o;
    for (int k = 0; k < n; k++) {
        if (!items[k].scene || !items[k].views) return fail(1, "null pointer in item %d", k);
        if (items[k].num_views <= 0 || items[k].resolution <= 0) return fail(2, "item %d: bad sizes", k);
    }
    oo.resolution = items[0].resolution;
    std::string why;
    if (!opts_ok(&oo, why)) return fail(2, "%s", why.c_str());
    int code = 0;
    Engine* E = engine_for_current(&code);
    if (!E) return code;
    for (int k = 0; k < n; k++)
        if (items[k].scene->device != E->device) return fail(2, "item %d: scene belongs to device %d", k, items[k].scene->device);
    auto t_start = std::chrono::steady_clock::now();
    std::unique_ptr<xrp_batch, void (*)(xrp_batch*)> B(new xrp_batch(), batch_free);
    B->device = E->device;
    memset(&B->info, 0, sizeof(B->info));
    // work order: largest items first, so the tail of the launch is small
    std::vector<int> order(n);
    for (int k = 0; k < n; k++) order[k] = k;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
        return (double)items[a].num_views * items[a].resolution * items[a].resolution >
               (double)items[b].num_views * items[b].resolution * items[b].resolution;
    });
    // flatten every scene for its cameras; one sample lattice (shared ds, R)
    std::vector<HostPrepared> hps(n);
    std::vector<std::vector<ViewDev>> vws(n);
    int depth = 0;
    bool defs = false, affine = true;
    // flattening is independent per item: host threads share the items
    std::vector<std::string> errs(n);
    {
        std::atomic<int> next{0};
        auto work = [&]() {
            for (int q; (q = next.fetch_add(1)) < n;) {
                const xrp_batch_item& it = items[order[q]];
                double fov_max;
                vws[q] = views_from(it.views, it.num_views, &fov_max);
                try {
                    // fine candidate lists: a batch flattens once and replays
                    hps[q] = prepare_host(it.scene->hs, it.resolution, oo.integration, oo.ds, oo.R,
                                          oo.flat_field, oo.density_multiplier, fov_max,
                                          (oo.flags & XRP_FLAG_TRACE) != 0, true);
                } catch (const std::exception& ex) {
                    errs[q] = ex.what();
                    if (errs[q].empty()) errs[q] = "flattening failed";
                }
            }
        };
        const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
        const int nth = (int)std::min<unsigned>(std::min<unsigned>(hw, 16u), (unsigned)n);
        std::vector<std::thread> pool;
        for (int k = 1; k < nth; k++) pool.emplace_back(work);
        work();
        for (auto& th : pool) th.join();
    }
    for (int q = 0; q < n; q++) {
        const xrp_batch_item& it = items[order[q]];
        if (!errs[q].empty()) return fail(2, "item %d: %s", order[q], errs[q].c_str());
        for (size_t v = 0; v < hps[q].vols.size(); v++) {
            hps[q].vols[v].data = it.scene->vdev[v];
            hps[q].vols[v].data64 = it.scene->v64[v];
        }
        depth = std::max(depth, hps[q].fs.depth);
        defs = defs || !hps[q].fs.defs.empty();
        affine = affine && hps[q].fs.affine;
    }
    const HostLattice& hl = hps[0].hl;
    // one upload: per item its scene tables, views and pixel table, then the
    // lattice, the SceneDev array and the item array (patched with addresses)
    Tables T;
    struct Off { size_t nodes, n64, child, cells, items, defs, vols, xs, clear, xsf; };
    std::vector<Off> off(n);
    std::vector<ViewDev> allv;  // every item's views, in work order
    std::vector<int> view0(n);
    for (int q = 0; q < n; q++) {
        const FlatScene& fs = hps[q].fs;
        off[q] = {T.add(fs.nodes), T.add(fs.nodes64), T.add(fs.child), T.add(fs.cells), T.add(fs.items),
                  T.add(fs.defs), T.add(hps[q].vols), T.add(hps[q].xs), T.add(fs.clear),
                  T.add(hps[q].xsf)};
        view0[q] = (int)allv.size();
        allv.insert(allv.end(), vws[q].begin(), vws[q].end());
    }
    size_t o_views = T.add(allv);
    size_t o_s64 = T.add(hl.s64), o_t32 = T.add(hl.t32), o_fs = T.add(hl.fstart);
    size_t o_f64 = T.add(hl.f64), o_ft32 = T.add(hl.ft32);
    std::vector<SceneDev> sdev(n);
    std::vector<BatchItemDev> idev(n);
    size_t o_scenes = T.add(sdev), o_items = T.add(idev);
    cudaError_t e = cudaMalloc(&B->tables, T.host.size());
    if (e != cudaSuccess) return cuda_fail(3, "batch tables", e);
    unsigned char* base = (unsigned char*)B->tables;
    long long out_total = 0;
    std::vector<long long> out0(n);
    for (int q = 0; q < n; q++) {
        const xrp_batch_item& it = items[order[q]];
        SceneDev S = hps[q].S;
        S.nodes = (const Node*)(base + off[q].nodes);
        S.nodes64 = (const Node64*)(base + off[q].n64);
        S.child = (const int32_t*)(base + off[q].child);
        S.cells = (const int32_t*)(base + off[q].cells);
        S.items = (const int32_t*)(base + off[q].items);
        S.clear = (const float*)(base + off[q].clear);
        S.defs = (const DefStep*)(base + off[q].defs);
        S.vols = (const Volume*)(base + off[q].vols);
        sdev[q] = S;
        BatchItemDev& I = idev[q];
        memset(&I, 0, sizeof(I));
        I.scene = q;
        I.view0 = view0[q];
        I.nviews = it.num_views;
        I.P = hps[q].P;
        I.P.nviews = it.num_views;
        I.P.xs = (const double*)(base + off[q].xs);
        I.P.xsf = (const float*)(base + off[q].xsf);
        I.out0 = out_total;
        out0[q] = out_total;
        out_total += (long long)it.num_views * it.resolution * it.resolution;
    }
    const ViewDev* vbase = (const ViewDev*)(base + o_views);
    memcpy(T.host.data() + o_scenes, sdev.data(), sdev.size() * sizeof(SceneDev));
    Lattice L = hl.hdr;
    L.s64 = (const double*)(base + o_s64);
    L.t32 = (const float*)(base + o_t32);
    L.fstart = (const int32_t*)(base + o_fs);
    L.f64 = (const double*)(base + o_f64);
    L.ft32 = (const float*)(base + o_ft32);
    B->offset.resize(n);
    B->size.resize(n);
    for (int q = 0; q < n; q++) {
        B->offset[order[q]] = out0[q];
        B->size[order[q]] = (long long)items[order[q]].num_views * items[order[q]].resolution * items[order[q]].resolution;
    }
    if ((e = cudaStreamCreateWithFlags(&B->cap, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaEventCreateWithFlags(&B->rendered, cudaEventDisableTiming)) != cudaSuccess)
        return cuda_fail(3, "batch stream", e);
    // the images come from the engine's pool: memory released by an earlier
    // batch is reused already mapped (copies out of freshly mapped device
    // memory ran at 20-60 GB/s against ~190 GB/s once warm)
    if ((e = cudaMallocFromPoolAsync((void**)&B->out, (size_t)std::max<long long>(out_total, 1) * sizeof(float),
                                     E->pool, B->cap)) != cudaSuccess ||
        (e = cudaStreamSynchronize(B->cap)) != cudaSuccess)
        return cuda_fail(3, "batch output", e);
    if ((e = cudaMalloc(&B->counter, sizeof(unsigned long long))) != cudaSuccess)
        return cuda_fail(3, "batch counter", e);
    int sms = 0, occ = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, E->device);
    const bool hier = oo.integration == XRP_INTEGRATE_HIERARCHICAL;
    // ray certificates when every scene's chain is affine, curve
    // certificates otherwise, ball certificates on request
    const int trace = !(oo.flags & XRP_FLAG_TRACE) ? 0 : (oo.flags & XRP_FLAG_BALL) ? 1 : affine ? 2 : 3;
    const int kdepth = depth == 0 ? 0 : kMaxDepth;
    if ((e = batch_blocks_per_sm(kdepth, defs, hier, trace, &occ)) != cudaSuccess)
        return cuda_fail(7, "batch occupancy", e);
    occ = std::max(occ, 1);
    BatchLaunch bl;
    memset(&bl, 0, sizeof(bl));
    bl.scenes = (const SceneDev*)(base + o_scenes);
    bl.items = (const BatchItemDev*)(base + o_items);
    bl.nitems = n;
    bl.views = vbase;
    bl.L = L;
    bl.depth = kdepth;
    bl.defs = defs;
    bl.hier = hier;
    bl.trace = trace;
    bl.counter = B->counter;
    bl.out = B->out;
    auto upload = [&](int tw, int th) -> cudaError_t {
        bl.tw = tw;
        bl.th = th;
        bl.ntiles = batch_tiling(idev, tw, th);
        memcpy(T.host.data() + o_items, idev.data(), idev.size() * sizeof(BatchItemDev));
        cudaError_t ue = cudaMemcpyAsync(B->tables, T.host.data(), T.host.size(), cudaMemcpyHostToDevice, B->cap);
        if (ue == cudaSuccess) ue = cudaStreamSynchronize(B->cap);
        return ue;
    };
    // autotuner: tile shapes x grid sizes, timed on the same sampled tiles
    static const int shapes[4][2] = {{8, 4}, {4, 8}, {16, 2}, {32, 1}};  // warp tiles
    int best_s = 0, best_b = occ;
    const int grids[2] = {occ, std::max(1, occ / 2)};
    int ncand = 0;
    if (autotune && out_total > 0) {
        cudaEvent_t e0, e1;
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        float best = 3.0e38f;
        for (int si = 0; si < 4; si++) {
            if ((e = upload(shapes[si][0], shapes[si][1])) != cudaSuccess) return cuda_fail(4, "batch tables", e);
            for (int gi = 0; gi < 2 && (gi == 0 || grids[1] != grids[0]); gi++) {
                BatchLaunch t = bl;
                t.blocks = grids[gi] * sms;
                t.limit = std::min<long long>(t.ntiles, 131072);
                t.stride = std::max<long long>(1, t.ntiles / t.limit);
                float ms = 0;
                for (int rep = 0; rep < 2; rep++) {
                    cudaMemsetAsync(B->counter, 0, sizeof(unsigned long long), B->cap);
                    cudaEventRecord(e0, B->cap);
                    e = launch_batch(t, B->cap);
                    cudaEventRecord(e1, B->cap);
                    if (e != cudaSuccess) break;
                    if ((e = cudaEventSynchronize(e1)) != cudaSuccess) break;
                    cudaEventElapsedTime(&ms, e0, e1);
                }
                if (e != cudaSuccess) {
                    cudaEventDestroy(e0);
                    cudaEventDestroy(e1);
                    return cuda_fail(7, "batch autotune", e);
                }
                if (ncand < 8) B->info.tune_ms[ncand] = ms;
                ncand++;
                if (ms < best) {
                    best = ms;
                    best_s = si;
                    best_b = grids[gi];
                }
            }
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
    }
    if ((e = upload(shapes[best_s][0], shapes[best_s][1])) != cudaSuccess) return cuda_fail(4, "batch tables", e);
    bl.blocks = best_b * sms;
    bl.stride = 1;
    bl.limit = bl.ntiles;
    B->bl = bl;
    // capture: counter reset + persistent launch
    if ((e = cudaStreamBeginCapture(B->cap, cudaStreamCaptureModeThreadLocal)) != cudaSuccess)
        return cuda_fail(7, "graph capture", e);
    cudaError_t e1 = cudaMemsetAsync(B->counter, 0, sizeof(unsigned long long), B->cap);
    cudaError_t e2 = launch_batch(B->bl, B->cap);
    e = cudaStreamEndCapture(B->cap, &B->graph);
    if (e1 != cudaSuccess || e2 != cudaSuccess || e != cudaSuccess)
        return cuda_fail(7, "graph capture", e != cudaSuccess ? e : (e1 != cudaSuccess ? e1 : e2));
    if ((e = cudaGraphInstantiate(&B->exec, B->graph, 0)) != cudaSuccess) return cuda_fail(7, "graph instantiate", e);
    B->info.rays = out_total;
    B->info.tiles = bl.ntiles;
    B->info.tile_w = shapes[best_s][0];
    B->info.tile_h = shapes[best_s][1];
    B->info.blocks_per_sm = best_b;
    B->info.num_sms = sms;
    B->info.tune_candidates = ncand;
    B->info.build_ms = (float)std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_start).count();
    *out = B.release();
    return 0;
}

int xrp_batch_render(xrp_batch* b, void* stream) {
    if (!b) return fail(1, "null pointer");
    cudaError_t e = cudaGraphLaunch(b->exec, (cudaStream_t)stream);
    if (e == cudaSuccess) e = cudaEventRecord(b->rendered, (cudaStream_t)stream);
    if (e != cudaSuccess) return cuda_fail(7, "graph launch", e);
    return 0;
}

const float* xrp_batch_output(const xrp_batch* b) { return b ? b->out : nullptr; }

long long xrp_batch_item_offset(const xrp_batch* b, int k) {
    if (!b || k < 0 || k >= (int)b->offset.size()) return -1;
    return b->offset[k];
}

// A copy on the batch's own stream, ordered after the last replay by its
// event (whatever stream the replay ran on), then a wait for that stream.
int xrp_batch_copy_item(const xrp_batch* b, int k, float* out_host) {
    if (!b || !out_host) return fail(1, "null pointer");
    if (k < 0 || k >= (int)b->offset.size()) return fail(2, "item %d out of range", k);
    cudaError_t e = cudaStreamWaitEvent(b->cap, b->rendered, 0);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(out_host, b->out + b->offset[k], (size_t)b->size[k] * sizeof(float),
                            cudaMemcpyDeviceToHost, b->cap);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->cap);
    if (e != cudaSuccess) return cuda_fail(8, "batch copy", e);
    return 0;
}

int xrp_batch_get_info(const xrp_batch* b, xrp_batch_info* out) {
    if (!b || !out) return fail(1, "null pointer");
    *out = b->info;
    return 0;
}

void xrp_batch_destroy(xrp_batch* b) { batch_free(b); }

}  // extern "C"

// ---------------------------------------------------------------------------
// learned proposal
// ---------------------------------------------------------------------------

struct xrp_proposal {
    int device = -1;
    float* params = nullptr;  // device, FP32 master parameters (MlpLayout)
    float tau = 0.0f;
    int segment = 64;
    float fc[3] = {0, 0, 0}, fs[3] = {1, 1, 1};  // feature normalisation
    xrp_proposal_info info;
};

static thread_local uint64_t t_prop_stats[kStatCount] = {0};

namespace {

uint64_t splitmix(uint64_t& s) {
    uint64_t z = (s += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

double unit_rand(uint64_t& s) { return (double)(splitmix(s) >> 11) * (1.0 / 9007199254740992.0); }

bool proposal_scene_ok(const xrp_scene* s, const xrp_render_opts* o, std::string& why) {
    if (o->integration != XRP_INTEGRATE_SIMPLE && !(o->flags & XRP_FLAG_TRACE)) {
        why = "the segment march supports the simple integrator only (certificate tracing both)";
        return false;
    }
    for (const HNode& n : s->hs.nodes)
        if (n.type == N_VOXEL) {
            why = "the proposal march supports analytic scenes only (no voxel grids)";
            return false;
        }
    return true;
}

// Feature normalisation from the dilated support box.
void feature_frame(const SceneDev& S, float fc[3], float fs[3]) {
    for (int a = 0; a < 3; a++) {
        float lo = S.sup_lo[a], hi = S.sup_hi[a];
        if (!(hi > lo) || hi - lo > 1e30f) {
            fc[a] = 0.0f;
            fs[a] = 1.0f;
        } else {
            fc[a] = 0.5f * (lo + hi);
            fs[a] = 2.0f / (hi - lo);
        }
    }
}

// Rows of training data: candidate segments of `nrays` random rays.
int gen_rows(Engine* E, const Prepared& pr, int nviews, int res, int segment, const float fc[3],
             const float fs[3], long nrays, uint64_t& rng, cudaStream_t st, PoolBuf& rays_buf, PoolBuf& X,
             PoolBuf& y, PoolBuf& cnt, unsigned cap, unsigned* count_out) {
    std::vector<int> rays(3 * (size_t)nrays);
    for (long r = 0; r < nrays; r++) {
        rays[3 * r] = (int)(splitmix(rng) % (uint64_t)nviews);
        rays[3 * r + 1] = (int)(splitmix(rng) % (uint64_t)res);
        rays[3 * r + 2] = (int)(splitmix(rng) % (uint64_t)res);
    }
    cudaError_t e;
    if ((e = rays_buf.alloc(E, rays.size() * sizeof(int), st)) != cudaSuccess ||
        (e = X.alloc(E, (size_t)cap * kMlpIn * sizeof(__nv_bfloat16), st)) != cudaSuccess ||
        (e = y.alloc(E, (size_t)cap * sizeof(float), st)) != cudaSuccess ||
        (e = cnt.alloc(E, sizeof(unsigned), st)) != cudaSuccess)
        return cuda_fail(3, "proposal training buffers", e);
    if ((e = cudaMemcpyAsync(rays_buf.p, rays.data(), rays.size() * sizeof(int), cudaMemcpyHostToDevice, st)) != cudaSuccess ||
        (e = cudaMemsetAsync(cnt.p, 0, sizeof(unsigned), st)) != cudaSuccess)
        return cuda_fail(4, "proposal training upload", e);
    PropLaunch pl;
    memset(&pl.Q, 0, sizeof(pl.Q));
    pl.train = true;
    pl.Q.mc = segment;
    for (int a = 0; a < 3; a++) {
        pl.Q.fc[a] = fc[a];
        pl.Q.fs[a] = fs[a];
    }
    pl.Q.rays = (const int*)rays_buf.p;
    pl.Q.nrays = (int)nrays;
    pl.Q.X = (__nv_bfloat16*)X.p;
    pl.Q.y = (float*)y.p;
    pl.Q.count = (unsigned*)cnt.p;
    pl.Q.cap = cap;
    if ((e = launch_prop(pr, 0, nviews, pl, nullptr, st)) != cudaSuccess)
        return cuda_fail(7, "proposal training rows", e);
    unsigned c = 0;
    if ((e = cudaMemcpyAsync(&c, cnt.p, sizeof(unsigned), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
        (e = cudaStreamSynchronize(st)) != cudaSuccess)
        return cuda_fail(7, "proposal training rows", e);
    *count_out = std::min(c, cap);
    return 0;
}

cudaError_t mlp_attrs_once() {
    static std::mutex m;
    static std::map<int, bool> done;
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> g(m);
    if (done[dev]) return cudaSuccess;
    cudaError_t e = mlp_kernel_attrs();
    if (e == cudaSuccess) done[dev] = true;
    return e;
}

// He-uniform initialisation of the hidden layers, small output layer.
std::vector<float> mlp_init(uint64_t& rng) {
    std::vector<float> p(MlpLayout::N, 0.0f);
    auto fill = [&](int off, int n, double bound) {
        for (int k = 0; k < n; k++) p[off + k] = (float)((2.0 * unit_rand(rng) - 1.0) * bound);
    };
    fill(MlpLayout::W1, kMlpHid * kMlpIn, std::sqrt(6.0 / kMlpIn));
    fill(MlpLayout::W2, kMlpHid * kMlpHid, std::sqrt(6.0 / kMlpHid));
    fill(MlpLayout::W3, kMlpHid * kMlpHid, std::sqrt(6.0 / kMlpHid));
    fill(MlpLayout::W4, kMlpHid, std::sqrt(3.0 / kMlpHid));
    return p;
}

}  // namespace

extern "C" {

int xrp_mlp_param_count(void) { return MlpLayout::N; }

int xrp_mlp_grad(const float* params, const uint16_t* X, const float* y, int rows, float pos_weight,
                 float* grad, float* loss, float* logits) {
    if (!params || !X || !y) return fail(1, "null pointer");
    if (rows <= 0) return fail(2, "rows must be > 0");
    int code = 0;
    Engine* E = engine_for_current(&code);
    if (!E) return code;
    std::lock_guard<std::mutex> g(E->mtx);
    cudaStream_t st = E->compute;
    cudaError_t e = mlp_attrs_once();
    if (e != cudaSuccess) return cuda_fail(7, "training kernel attributes", e);
    PoolBuf dp, dX, dy, dg, dl, dlog;
    const size_t N = MlpLayout::N;
    if ((e = dp.alloc(E, N * 4, st)) != cudaSuccess || (e = dX.alloc(E, (size_t)rows * kMlpIn * 2, st)) != cudaSuccess ||
        (e = dy.alloc(E, (size_t)rows * 4, st)) != cudaSuccess || (e = dg.alloc(E, N * 4, st)) != cudaSuccess ||
        (e = dl.alloc(E, 4, st)) != cudaSuccess || (e = dlog.alloc(E, (size_t)rows * 4, st)) != cudaSuccess)
        return cuda_fail(3, "gradient buffers", e);
    if ((e = cudaMemcpyAsync(dp.p, params, N * 4, cudaMemcpyHostToDevice, st)) != cudaSuccess ||
        (e = cudaMemcpyAsync(dX.p, X, (size_t)rows * kMlpIn * 2, cudaMemcpyHostToDevice, st)) != cudaSuccess ||
        (e = cudaMemcpyAsync(dy.p, y, (size_t)rows * 4, cudaMemcpyHostToDevice, st)) != cudaSuccess ||
        (e = cudaMemsetAsync(dg.p, 0, N * 4, st)) != cudaSuccess || (e = cudaMemsetAsync(dl.p, 0, 4, st)) != cudaSuccess)
        return cuda_fail(4, "gradient upload", e);
    e = mlp_train_launch(st, (const float*)dp.p, (const __nv_bfloat16*)dX.p, (const float*)dy.p, nullptr,
                         rows, pos_weight, 1.0f / (float)rows, (float*)dg.p, (float*)dl.p, (float*)dlog.p);
    if (e != cudaSuccess) return cuda_fail(7, "training kernel launch", e);
    if (grad && (e = cudaMemcpyAsync(grad, dg.p, N * 4, cudaMemcpyDeviceToHost, st)) != cudaSuccess)
        return cuda_fail(7, "gradient read", e);
    if (loss && (e = cudaMemcpyAsync(loss, dl.p, 4, cudaMemcpyDeviceToHost, st)) != cudaSuccess)
        return cuda_fail(7, "loss read", e);
    if (logits && (e = cudaMemcpyAsync(logits, dlog.p, (size_t)rows * 4, cudaMemcpyDeviceToHost, st)) != cudaSuccess)
        return cuda_fail(7, "logit read", e);
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return cuda_fail(7, "training kernel", e);
    unsigned tc_err = 0;
    if ((e = mlp_tc_error(&tc_err)) != cudaSuccess) return cuda_fail(7, "training status", e);
    if (tc_err) return fail(7, "a tensor-core training step timed out waiting for its products");
    return 0;
}

int xrp_proposal_train(xrp_scene* s, const xrp_camera* views, int nviews, const xrp_render_opts* o,
                       const xrp_proposal_opts* po, xrp_proposal** out) {
    if (!s || !views || !o || !out) return fail(1, "null pointer");
    *out = nullptr;
    std::string why;
    if (nviews <= 0) return fail(2, "num_views must be > 0");
    if (!opts_ok(o, why) || !proposal_scene_ok(s, o, why)) return fail(2, "%s", why.c_str());
    xrp_proposal_opts d;
    memset(&d, 0, sizeof(d));
    if (po) d = *po;
    const int segment = d.segment ? d.segment : 64;
    if (segment < 32 || segment > 4096 || segment % 32) return fail(2, "segment must be a multiple of 32 in [32, 4096]");
    const long train_rays = d.train_rays > 0 ? d.train_rays : 65536;
    const long val_rays = d.val_rays > 0 ? d.val_rays : 32768;
    const int steps = d.steps > 0 ? d.steps : 2000;
    const int batch = d.batch > 0 ? d.batch : 4096;
    const float lr = d.lr > 0 ? d.lr : 2e-3f;
    const float pw = d.pos_weight > 0 ? d.pos_weight : 8.0f;
    const float tmargin = d.tau_margin;
    int code = 0;
    Engine* E = engine_for_current(&code);
    if (!E) return code;
    if (E->device != s->device) return fail(2, "scene belongs to device %d", s->device);
    double fov_max;
    std::vector<ViewDev> v = views_from(views, nviews, &fov_max);
    std::lock_guard<std::mutex> g(E->mtx);
    cudaStream_t st = E->compute;
    auto t_start = std::chrono::steady_clock::now();
    PoolBuf tab;
    Prepared pr;
    int rc = prepare(E, s->hs, s->vdev, s->v64, v, o->resolution, XRP_INTEGRATE_SIMPLE, o->ds, o->R,
                     o->flat_field, o->density_multiplier, fov_max, st, tab, pr, 0);
    if (rc) return rc;
    auto P = std::make_unique<xrp_proposal>();
    P->device = E->device;
    P->segment = segment;
    feature_frame(pr.S, P->fc, P->fs);
    memset(&P->info, 0, sizeof(P->info));
    P->info.segment = segment;
    uint64_t rng = d.seed ^ 0x5eedull;
    const long segs_per_ray = (pr.L.K + segment - 1) / segment + 1;
    const unsigned cap_t = (unsigned)std::min<long>(train_rays * segs_per_ray, 1L << 22);
    const unsigned cap_v = (unsigned)std::min<long>(val_rays * segs_per_ray, 1L << 22);
    PoolBuf rays_t, X_t, y_t, c_t, rays_v, X_v, y_v, c_v;
    unsigned n_t = 0, n_v = 0;
    if (!pr.empty) {
        if ((rc = gen_rows(E, pr, nviews, o->resolution, segment, P->fc, P->fs, train_rays, rng, st, rays_t, X_t, y_t, c_t, cap_t, &n_t)))
            return rc;
        if ((rc = gen_rows(E, pr, nviews, o->resolution, segment, P->fc, P->fs, val_rays, rng, st, rays_v, X_v, y_v, c_v, cap_v, &n_v)))
            return rc;
    }
    cudaError_t e;
    if ((e = cudaMalloc(&P->params, MlpLayout::N * sizeof(float))) != cudaSuccess)
        return cuda_fail(3, "proposal parameters", e);
    std::unique_ptr<xrp_proposal, void (*)(xrp_proposal*)> guard(P.release(), xrp_proposal_destroy);
    xrp_proposal* Pp = guard.get();
    std::vector<float> init = mlp_init(rng);
    if ((e = cudaMemcpyAsync(Pp->params, init.data(), init.size() * 4, cudaMemcpyHostToDevice, st)) != cudaSuccess)
        return cuda_fail(4, "proposal parameters", e);
    if ((e = mlp_attrs_once()) != cudaSuccess) return cuda_fail(7, "training kernel attributes", e);
    std::vector<float> ylab;
    if (n_t > 0) {
        ylab.resize(n_t);
        if ((e = cudaMemcpyAsync(ylab.data(), y_t.p, n_t * 4, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
            (e = cudaStreamSynchronize(st)) != cudaSuccess)
            return cuda_fail(7, "training labels", e);
        for (float q : ylab) Pp->info.train_pos += q > 0.5f;
        Pp->info.train_rows = n_t;
        // Adam: batches drawn with replacement, linear decay of the rate
        const size_t N = MlpLayout::N;
        PoolBuf grad, m1, m2, idx, lossb;
        std::vector<int> hidx((size_t)steps * batch);
        for (auto& q : hidx) q = (int)(splitmix(rng) % n_t);
        if ((e = grad.alloc(E, N * 4, st)) != cudaSuccess || (e = m1.alloc(E, N * 4, st)) != cudaSuccess ||
            (e = m2.alloc(E, N * 4, st)) != cudaSuccess || (e = idx.alloc(E, hidx.size() * 4, st)) != cudaSuccess ||
            (e = lossb.alloc(E, (size_t)steps * 4, st)) != cudaSuccess)
            return cuda_fail(3, "training buffers", e);
        cudaMemsetAsync(grad.p, 0, N * 4, st);
        cudaMemsetAsync(m1.p, 0, N * 4, st);
        cudaMemsetAsync(m2.p, 0, N * 4, st);
        cudaMemsetAsync(lossb.p, 0, (size_t)steps * 4, st);
        if ((e = cudaMemcpyAsync(idx.p, hidx.data(), hidx.size() * 4, cudaMemcpyHostToDevice, st)) != cudaSuccess)
            return cuda_fail(4, "training batches", e);
        double b1p = 1.0, b2p = 1.0;
        for (int it = 0; it < steps && e == cudaSuccess; it++) {
            e = mlp_train_launch(st, Pp->params, (const __nv_bfloat16*)X_t.p, (const float*)y_t.p,
                                 (const int*)idx.p + (size_t)it * batch, batch, pw, 1.0f / (float)batch,
                                 (float*)grad.p, (float*)lossb.p + it, nullptr);
            b1p *= 0.9;
            b2p *= 0.999;
            float rate = lr * (1.0f - 0.9f * (float)it / (float)steps);
            if (e == cudaSuccess)
                e = mlp_adam_launch(st, Pp->params, (float*)grad.p, (float*)m1.p, (float*)m2.p, (int)N, rate,
                                    0.9f, 0.999f, 1e-8f, (float)(1.0 / (1.0 - b1p)), (float)(1.0 / (1.0 - b2p)));
        }
        if (e != cudaSuccess) return cuda_fail(7, "training launch", e);
        std::vector<float> hl(steps);
        if ((e = cudaMemcpyAsync(hl.data(), lossb.p, (size_t)steps * 4, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
            (e = cudaStreamSynchronize(st)) != cudaSuccess)
            return cuda_fail(7, "training", e);
        unsigned tc_err = 0;
        if ((e = mlp_tc_error(&tc_err)) != cudaSuccess) return cuda_fail(7, "training status", e);
        if (tc_err) return fail(7, "a tensor-core training step timed out waiting for its products");
        int tail = std::max(1, steps / 10);
        double sl = 0;
        for (int k = steps - tail; k < steps; k++) sl += hl[k];
        Pp->info.final_loss = (float)(sl / tail);
    }
    float tau = std::log(pw) + tmargin;
    if (n_v > 0 && n_t > 0) {
        PoolBuf lg;
        if ((e = lg.alloc(E, (size_t)n_v * 4, st)) != cudaSuccess) return cuda_fail(3, "validation buffers", e);
        e = mlp_logits_launch(st, Pp->params, (const __nv_bfloat16*)X_v.p, (int)n_v, (float*)lg.p);
        if (e != cudaSuccess) return cuda_fail(7, "validation launch", e);
        std::vector<float> hl(n_v), hy(n_v);
        if ((e = cudaMemcpyAsync(hl.data(), lg.p, (size_t)n_v * 4, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
            (e = cudaMemcpyAsync(hy.data(), y_v.p, (size_t)n_v * 4, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
            (e = cudaStreamSynchronize(st)) != cudaSuccess)
            return cuda_fail(7, "validation", e);
        long long npos = 0;
        for (unsigned k = 0; k < n_v; k++) npos += hy[k] > 0.5f;
        // routing threshold: a candidate goes dense when the network's
        // (class-weight corrected) probability of a transition exceeds 1/2
        tau = std::log(pw) + tmargin;
        long long acc = 0;
        for (unsigned k = 0; k < n_v; k++) acc += (hl[k] <= tau);
        Pp->info.val_rows = n_v;
        Pp->info.val_pos = npos;
        Pp->info.val_accepted = acc;
    }
    Pp->tau = tau;
    Pp->info.tau = tau;
    Pp->info.train_ms = (float)std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_start).count();
    *out = guard.release();
    return 0;
}

int xrp_proposal_get_info(const xrp_proposal* p, xrp_proposal_info* out) {
    if (!p || !out) return fail(1, "null pointer");
    *out = p->info;
    return 0;
}

int xrp_proposal_params(const xrp_proposal* p, float* out, int n) {
    if (!p || !out) return fail(1, "null pointer");
    if (n < MlpLayout::N) return fail(2, "need %d floats", MlpLayout::N);
    cudaError_t e = cudaMemcpy(out, p->params, MlpLayout::N * sizeof(float), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(7, "parameter read", e);
    return 0;
}

int xrp_proposal_set_tau(xrp_proposal* p, float tau) {
    if (!p) return fail(1, "null pointer");
    p->tau = tau;
    return 0;
}

void xrp_proposal_destroy(xrp_proposal* p) {
    if (!p) return;
    if (p->params) cudaFree(p->params);
    delete p;
}

// Curve certificates evaluate fewer samples than balls, but one curve
// evaluation costs about 4.2 ball evaluations on GB300 (fitted on the two
// gyroid scenes: scale 8, 7.4 against 44.7 evaluations per ray, curves
// 2058 against balls 1516 Mrays/s; scale 0.1, 21.4 against 73.2, curves 701
// against balls 892).  For a call of many rays over a non-affine chain the
// simple integrator's tracing counts both kinds' evaluations on up to four
// of the call's views at 64^2 and takes the cheaper: 2 (balls) or 1.
static int probe_certificate_kind(Engine* E, xrp_scene* s, const std::vector<ViewDev>& v, const xrp_render_opts& o,
                                  double fov_max, cudaStream_t st, int* kind) {
    *kind = 1;
    const int n = std::min<int>(4, (int)v.size());
    std::vector<ViewDev> pv;
    for (int q = 0; q < n; q++) pv.push_back(v[(size_t)q * v.size() / n]);
    xrp_render_opts po = o;
    po.resolution = 64;
    PoolBuf img, sb;
    cudaError_t e;
    if ((e = img.alloc(E, (size_t)n * 64 * 64 * sizeof(float), st)) != cudaSuccess ||
        (e = sb.alloc(E, 2 * kStatCount * sizeof(unsigned long long), st)) != cudaSuccess)
        return cuda_fail(3, "certificate probe", e);
    if ((e = cudaMemsetAsync(sb.p, 0, 2 * kStatCount * sizeof(unsigned long long), st)) != cudaSuccess)
        return cuda_fail(7, "certificate probe", e);
    for (int t = 1; t <= 2; t++) {
        PropLaunch pl;
        memset(&pl.Q, 0, sizeof(pl.Q));
        pl.Q.trace = t;
        pl.Q.mc = 64;
        pl.Q.stats = (unsigned long long*)sb.p + (t - 1) * kStatCount;
        PoolBuf fb, fbc;
        int rc = alloc_fallback_list(E, pl, fb, fbc, st);
        if (rc) return rc;
        rc = render_views(E, s->hs, s->vdev, s->v64, pv, po, fov_max, (float*)img.p, false, st, st, false, 0, &pl);
        if (rc) return rc;
    }
    unsigned long long h[2 * kStatCount];
    if ((e = cudaMemcpyAsync(h, sb.p, sizeof(h), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
        (e = cudaStreamSynchronize(st)) != cudaSuccess)
        return cuda_fail(7, "certificate probe", e);
    const double curve = (double)h[kStatEvaluations], ball = (double)h[kStatCount + kStatEvaluations];
    if (ball < 4.2 * curve) *kind = 2;
    return 0;
}

// Whether the scene's deformation chain has a non-affine step.
static bool chain_non_affine(const HostScene& hs) {
    for (const HDef& d : hs.defs)
        if (d.type != D_LINEAR && d.type != D_AFFINE && d.type != D_RIGID) return true;
    return false;
}

static int render_proposal(xrp_scene* s, const xrp_proposal* prop, int segment, const xrp_camera* views,
                           int nviews, const xrp_render_opts* o, float* out, bool out_host, void* stream) {
    if (!s || !views || !o || !out) return fail(1, "null pointer");
    std::string why;
    if (nviews <= 0) return fail(2, "num_views must be > 0");
    if (!opts_ok(o, why) || !proposal_scene_ok(s, o, why)) return fail(2, "%s", why.c_str());
    if (segment == 0) segment = prop ? prop->segment : 64;
    if (segment < 32 || segment > 4096 || segment % 32) return fail(2, "segment must be a multiple of 32 in [32, 4096]");
    int code = 0;
    Engine* E = engine_for_current(&code);
    if (!E) return code;
    if (E->device != s->device) return fail(2, "scene belongs to device %d", s->device);
    if (prop && prop->device != s->device) return fail(2, "proposal belongs to device %d", prop->device);
    if (prop && (o->flags & XRP_FLAG_TRACE)) return fail(2, "certificate tracing takes no proposal network");
    double fov_max;
    std::vector<ViewDev> v = views_from(views, nviews, &fov_max);
    std::unique_lock<std::mutex> g(E->mtx, std::defer_lock);
    if (out_host) g.lock();
    cudaStream_t st = out_host ? E->compute : (cudaStream_t)stream;
    const bool want_stats = (o->flags & XRP_FLAG_STATS) != 0;
    PoolBuf sb;
    PropLaunch pl;
    memset(&pl.Q, 0, sizeof(pl.Q));
    pl.Q.mc = segment;
    pl.Q.refine = (o->flags & XRP_FLAG_NO_REFINE) ? 0 : 1;
    pl.Q.trace = !(o->flags & XRP_FLAG_TRACE) ? 0 : (o->flags & XRP_FLAG_BALL) ? 2 : 1;
    pl.Q.min_piece = 8;
    if (prop) {
        pl.Q.mlp = prop->params;
        pl.Q.tau = prop->tau;
        for (int a = 0; a < 3; a++) {
            pl.Q.fc[a] = prop->fc[a];
            pl.Q.fs[a] = prop->fs[a];
        }
    }
    cudaError_t e;
    if (want_stats) {
        if ((e = sb.alloc(E, kStatCount * sizeof(unsigned long long), st)) != cudaSuccess)
            return cuda_fail(3, "stats buffer", e);
        if ((e = cudaMemsetAsync(sb.p, 0, kStatCount * sizeof(unsigned long long), st)) != cudaSuccess)
            return cuda_fail(7, "stats reset", e);
        pl.Q.stats = (unsigned long long*)sb.p;
    }
    // list of samples for FP64 re-evaluation (per launch of at most
    // pl.max_rays rays; reused): four entries per ray (the deformed lattice
    // leaves about one undecided sample per ray; an overflow costs a plain
    // re-render of the whole call).  The hierarchical integrator refines
    // every boundary crossing into ten fine samples next to the boundary,
    // where undecided samples gather (several per ray on the lattice): the
    // same list for a quarter of the rays, sixteen entries per ray.
    if (o->integration == XRP_INTEGRATE_HIERARCHICAL) pl.max_rays = 1LL << 21;
    PoolBuf fb, fbc;
    const int slots = (long long)nviews * o->resolution * o->resolution > pl.max_rays ? 2 : 1;
    int lrc = alloc_fallback_list(E, pl, fb, fbc, st, slots);
    if (lrc) return lrc;
    xrp_render_opts oo = *o;
    if (pl.Q.trace == 1 && o->integration == XRP_INTEGRATE_SIMPLE && chain_non_affine(s->hs) &&
        (long long)nviews * o->resolution * o->resolution >= (1LL << 22)) {
        int kind = 1;
        if ((lrc = probe_certificate_kind(E, s, v, *o, fov_max, st, &kind))) return lrc;
        pl.Q.trace = kind;
    }
    int rc = render_views(E, s->hs, s->vdev, s->v64, v, oo, fov_max, out, out_host, st,
                          out_host ? E->copy : st, false, 0, &pl);
    if (rc) return rc;
    // an overflowed list (more undecided samples in one launch than it
    // holds) is not expected; the plain integrator then renders the call
    unsigned ovf = 0;
    if ((e = list_overflowed(pl, st, &ovf)) != cudaSuccess) return cuda_fail(7, "proposal march", e);
    if (ovf) {
        rc = render_views(E, s->hs, s->vdev, s->v64, v, oo, fov_max, out, out_host, st,
                          out_host ? E->copy : st, false, 0, nullptr);
        if (rc) return rc;
    }
    if (want_stats) {
        unsigned long long h[kStatCount];
        if ((e = cudaMemcpyAsync(h, sb.p, sizeof(h), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
            (e = cudaStreamSynchronize(st)) != cudaSuccess)
            return cuda_fail(7, "stats read", e);
        for (int q = 0; q < kStatCount; q++) t_prop_stats[q] = h[q];
        t_prop_stats[kStatOverflows] = ovf ? 1 : 0;
    }
    return 0;
}

int xrp_render_proposal(xrp_scene* s, const xrp_proposal* prop, int segment, const xrp_camera* views,
                        int nviews, const xrp_render_opts* o, float* out) {
    return render_proposal(s, prop, segment, views, nviews, o, out, true, nullptr);
}

int xrp_render_proposal_device(xrp_scene* s, const xrp_proposal* prop, int segment, const xrp_camera* views,
                               int nviews, const xrp_render_opts* o, float* out_device, void* stream) {
    return render_proposal(s, prop, segment, views, nviews, o, out_device, false, stream);
}

int xrp_proposal_last_stats(uint64_t out[11]) {
    if (!out) return fail(1, "null pointer");
    for (int q = 0; q < kStatCount; q++) out[q] = t_prop_stats[q];
    return 0;
}

// ---------------------------------------------------------------------------
// reference ABI
// ---------------------------------------------------------------------------

int RenderVolumeProjectionsCUDA(const float* volume, int nx, int ny, int nz,
                                const XRayCameraParams* cams, int ncams, int res, float ds,
                                float flat_field, float* out_images) {
    if (!volume || !cams || !out_images) return fail(1, "null pointer");
    if (nx <= 0 || ny <= 0 || nz <= 0 || res <= 0 || ncams <= 0) return fail(2, "bad sizes");
    if (!(ds > 0.0f) || !std::isfinite(ds)) return fail(2, "ds must be > 0 and finite");
    if ((double)3.48 / (double)ds > 5.0e7) return fail(2, "ds too small");
    size_t nvox = (size_t)nx * ny * nz;
    if (nvox / nx / ny != (size_t)nz) return fail(2, "volume too large");
    int code = 0;
    Engine* E = engine_for_current(&code);
    if (!E) return code;
    std::lock_guard<std::mutex> g(E->mtx);
    cudaStream_t st = E->compute;
    PoolBuf dvol;
    LayeredTex tex;
    cudaError_t e;
    if (volume_gathers_enabled()) {
        // the gather path reads the grid from the texture only; the FP64
        // re-evaluation of uncertain samples reads the linear copy below
        if ((e = tex.create(volume, nx, ny, nz, st)) != cudaSuccess) return cuda_fail(3, "volume texture", e);
    }
    if ((e = injected("alloc")) != cudaSuccess || (e = dvol.alloc(E, nvox * sizeof(float), st)) != cudaSuccess)
        return cuda_fail(3, "volume allocation", e);
    if ((e = injected("upload")) != cudaSuccess ||
        (e = cudaMemcpyAsync(dvol.p, volume, nvox * sizeof(float), cudaMemcpyHostToDevice, st)) != cudaSuccess)
        return cuda_fail(4, "volume upload", e);
    HostScene hs = volume_scene((const float*)dvol.p, nx, ny, nz);
    std::vector<const float*> vdev{(const float*)dvol.p};
    std::vector<const double*> v64{nullptr};
    size_t img = (size_t)res * res;
    // cameras that share R share one sample lattice (main.go:465)
    int c0 = 0;
    while (c0 < ncams) {
        int c1 = c0 + 1;
        while (c1 < ncams && cams[c1].R == cams[c0].R) c1++;
        std::vector<ViewDev> views(c1 - c0);
        double fov_max = 0;
        for (int c = c0; c < c1; c++) {
            double eye[3], m[16];
            for (int a = 0; a < 3; a++) eye[a] = (double)cams[c].eye[a];
            for (int r = 0; r < 4; r++)
                for (int k = 0; k < 4; k++) m[k * 4 + r] = (double)cams[c].view[r * 4 + k];
            view_from_camera(eye, m, (double)cams[c].fov_y, views[c - c0]);
            fov_max = std::max(fov_max, std::fabs((double)cams[c].fov_y));
        }
        xrp_render_opts o;
        memset(&o, 0, sizeof(o));
        o.resolution = res;
        o.integration = XRP_INTEGRATE_SIMPLE;
        o.ds = (double)ds;
        o.R = (double)cams[c0].R;
        o.flat_field = (double)flat_field;
        o.density_multiplier = 1.0;
        int rc = render_views(E, hs, vdev, v64, views, o, fov_max, out_images + (size_t)c0 * img, true,
                              st, E->copy, false, tex.tex);
        if (rc) return rc;
        c0 = c1;
    }
    return 0;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// render without device allocation
// ---------------------------------------------------------------------------
//
// For callers that must not allocate device memory -- host frameworks whose
// allocator owns the whole device, or services whose device-memory budget is
// fixed up front.  The per-call tables (scene
// image, sample lattice, pixel table, cameras) live in the static array
// below instead of a stream-ordered pool allocation; the volume and the
// images are the caller's device buffers.  Every GPU that loads the library
// reserves this array until the process exits.
static constexpr size_t kNoAllocScratchBytes = (size_t)1 << 20;  // 1 MiB
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

static std::mutex g_noalloc_mtx;
static std::map<int, unsigned char*> g_noalloc_addr;  // device -> address of the array

// Device address of the scratch array on the current device, looked up once
// per device (host code cannot use the symbol itself as a device address).
static int noalloc_scratch(unsigned char** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_fail(3, "cudaGetDevice", e);
    std::lock_guard<std::mutex> g(g_noalloc_mtx);
    auto it = g_noalloc_addr.find(dev);
    if (it != g_noalloc_addr.end()) {
        *out = it->second;
        return 0;
    }
    unsigned char* p = nullptr;
    e = cudaGetSymbolAddress((void**)&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) return cuda_fail(3, "scratch symbol address", e);
    g_noalloc_addr[dev] = p;
    *out = p;
    return 0;
}

extern "C" int xrp_render_volume_noalloc(const float* d_volume, int nx, int ny, int nz,
                                         const XRayCameraParams* cams, int ncams, int res,
                                         float ds, float flat_field, float* d_out, void* stream) {
    if (!d_volume || !cams || !d_out) return fail(1, "null pointer");
    if (nx <= 0 || ny <= 0 || nz <= 0 || res <= 0 || ncams <= 0) return fail(2, "bad sizes");
    if (!(ds > 0.0f) || !std::isfinite(ds)) return fail(2, "ds must be > 0 and finite");
    for (int c = 1; c < ncams; c++)
        if (cams[c].R != cams[0].R) return fail(2, "all cameras of one call must share R");
    unsigned char* base = nullptr;
    int rc = noalloc_scratch(&base);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    std::vector<ViewDev> views(ncams);
    double fov_max = 0;
    for (int c = 0; c < ncams; c++) {
        double eye[3], m[16];
        for (int a = 0; a < 3; a++) eye[a] = (double)cams[c].eye[a];
        for (int r = 0; r < 4; r++)
            for (int k = 0; k < 4; k++) m[k * 4 + r] = (double)cams[c].view[r * 4 + k];
        view_from_camera(eye, m, (double)cams[c].fov_y, views[c]);
        fov_max = std::max(fov_max, std::fabs((double)cams[c].fov_y));
    }
    HostScene hs = volume_scene(d_volume, nx, ny, nz);
    HostPrepared hp;
    try {
        hp = prepare_host(hs, res, XRP_INTEGRATE_SIMPLE, (double)ds, (double)cams[0].R,
                          (double)flat_field, 1.0, fov_max);
    } catch (const std::exception& ex) {
        return fail(2, "%s", ex.what());
    }
    hp.vols[0].data = d_volume;
    hp.vols[0].data64 = nullptr;
    Tables T;
    const TableLayout o = pack_tables(hp, views, T);
    if (T.host.size() > kNoAllocScratchBytes)
        return fail(2, "this call needs %zu bytes of tables; the no-allocation entry point holds "
                       "at most %zu (fewer cameras, a smaller resolution or a larger ds fit)",
                    T.host.size(), kNoAllocScratchBytes);
    // every byte the kernel reads is written here, so nothing needs clearing;
    // the copy reads the pageable host buffer before the call returns
    cudaError_t e = cudaMemcpyAsync(base, T.host.data(), T.host.size(), cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return cuda_fail(5, "table upload", e);
    // per-tap loads: a texture would need an array allocation
    Prepared pr;
    bind_tables(hp, views, base, o, 0, d_volume, nullptr, pr);
    const int tpv = ((res + 15) / 16) * ((res + 15) / 16);
    const int per_launch = std::max(1, (int)(0x7fffffffL / tpv));
    size_t img = (size_t)res * res;
    for (int v0 = 0; v0 < ncams; v0 += per_launch) {
        int n = std::min(per_launch, ncams - v0);
        if ((e = launch(pr, v0, n, XRP_INTEGRATE_SIMPLE, d_out + (size_t)v0 * img, nullptr, st)) != cudaSuccess)
            return cuda_fail(7, "kernel launch", e);
    }
    return 0;
}

extern "C" {

static int voxelize(const CylinderParams* cyl, int ncyl, int res, float dm, int grid_dim,
                    const int* off, const int* idx, int nidx, float* out, bool spatial) {
    int code = 0;
    Engine* E = engine_for_current(&code);
    if (!E) return spatial ? 3 : 2;
    std::lock_guard<std::mutex> g(E->mtx);
    cudaStream_t st = E->compute;
    size_t nvox = (size_t)res * res * res;
    PoolBuf dcyl, dout, doff, didx;
    cudaError_t e;
    int c_alloc = spatial ? 3 : 2, c_copy = spatial ? 4 : 3, c_valloc = spatial ? 3 : 4;
    if ((e = dcyl.alloc(E, (size_t)ncyl * sizeof(CylinderParams), st)) != cudaSuccess)
        return cuda_fail(c_alloc, "cylinder allocation", e);
    if ((e = cudaMemcpyAsync(dcyl.p, cyl, (size_t)ncyl * sizeof(CylinderParams), cudaMemcpyHostToDevice, st)) != cudaSuccess)
        return cuda_fail(c_copy, "cylinder upload", e);
    if ((e = dout.alloc(E, nvox * sizeof(float), st)) != cudaSuccess)
        return cuda_fail(c_valloc, "volume allocation", e);
    if (spatial) {
        size_t ncell = (size_t)grid_dim * grid_dim * grid_dim + 1;
        if ((e = doff.alloc(E, ncell * sizeof(int), st)) != cudaSuccess ||
            (e = didx.alloc(E, (size_t)std::max(nidx, 1) * sizeof(int), st)) != cudaSuccess)
            return cuda_fail(3, "cell list allocation", e);
        if ((e = cudaMemcpyAsync(doff.p, off, ncell * sizeof(int), cudaMemcpyHostToDevice, st)) != cudaSuccess ||
            (nidx > 0 && (e = cudaMemcpyAsync(didx.p, idx, (size_t)nidx * sizeof(int), cudaMemcpyHostToDevice, st)) != cudaSuccess))
            return cuda_fail(4, "cell list upload", e);
    }
    int use_smem = (!spatial && (size_t)ncyl * sizeof(CylinderParams) <= 48 * 1024) ? 1 : 0;
    size_t smem = use_smem ? (size_t)ncyl * sizeof(CylinderParams) : 0;
    long blocks = (long)((nvox + 255) / 256);
    blocks = std::min<long>(blocks, 152L * 64);
    k_voxelize<<<(unsigned)std::max<long>(blocks, 1), 256, smem, st>>>(
        (const CylinderParams*)dcyl.p, ncyl, res, dm, spatial ? (const int*)doff.p : nullptr,
        spatial ? (const int*)didx.p : nullptr, grid_dim, use_smem, (float*)dout.p);
    if ((e = cudaGetLastError()) != cudaSuccess || (e = cudaStreamSynchronize(st)) != cudaSuccess)
        return cuda_fail(5, "voxelizer kernel", e);
    if ((e = cudaMemcpyAsync(out, dout.p, nvox * sizeof(float), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
        (e = cudaStreamSynchronize(st)) != cudaSuccess)
        return cuda_fail(6, "volume copy", e);
    return 0;
}

int AssembleVoxelGridCUDA(const CylinderParams* cylinders, int num_cylinders, int res,
                          float density_multiplier, float* out_volume) {
    if (!cylinders || !out_volume || num_cylinders <= 0 || res <= 0) return fail(1, "bad arguments");
    return voxelize(cylinders, num_cylinders, res, density_multiplier, 0, nullptr, nullptr, 0,
                    out_volume, false);
}

int AssembleVoxelGridSpatialCUDA(const CylinderParams* cylinders, int num_cylinders, int res,
                                 float density_multiplier, int grid_dim, const int* cell_offsets,
                                 const int* cyl_indices, int num_cyl_indices, float* out_volume) {
    if (!cylinders || !out_volume || !cell_offsets || !cyl_indices) return fail(1, "null pointer");
    if (num_cylinders <= 0 || res <= 0 || grid_dim <= 0 || num_cyl_indices < 0) return fail(2, "bad sizes");
    // the device reads cyl_indices[cell_offsets[c] .. cell_offsets[c+1]) and
    // cylinders[cyl_indices[q]]: check the lists before any device access
    long ncell = (long)grid_dim * grid_dim * grid_dim;
    if (grid_dim > 1024) return fail(2, "grid_dim too large");
    for (long c = 0; c < ncell; c++)
        if (cell_offsets[c] < 0 || cell_offsets[c] > cell_offsets[c + 1]) return fail(2, "bad cell offsets");
    if (cell_offsets[ncell] > num_cyl_indices) return fail(2, "cell offsets exceed the index list");
    for (int q = 0; q < num_cyl_indices; q++)
        if (cyl_indices[q] < 0 || cyl_indices[q] >= num_cylinders) return fail(2, "bad cylinder index");
    return voxelize(cylinders, num_cylinders, res, density_multiplier, grid_dim, cell_offsets,
                    cyl_indices, num_cyl_indices, out_volume, true);
}

}  // extern "C"
