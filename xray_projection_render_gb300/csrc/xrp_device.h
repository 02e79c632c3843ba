// xrp_device.h -- scene image and per-sample / per-ray evaluation, shared by
// the CUDA kernels and (for logic tests only) a host build.
//
// Two evaluators live here:
//   * an FP32 evaluator with guard bands: every discontinuous predicate of the
//     reference (strict `<` on a sphere, inclusive bounds of a unit cell, the
//     floor of a tessellation fold, ...) is decided in FP32 only when the FP32
//     margin is farther from the decision boundary than a precomputed error
//     bound; otherwise it reports "uncertain" (NaN);
//   * an FP64 evaluator that repeats the reference's arithmetic operation by
//     operation (no contraction: __dmul_rn/__dadd_rn on the device), used for
//     the uncertain samples only.
// The reference semantics restated here are objects/objects.go:63-72 (sphere),
// 171-179 (box), 247-255 (parallelepiped), 334-350 (cylinder), 422-438
// (collection), 458-464 (unit cell), 568-582 (tessellation), 789-855 (voxel
// grid), 1014-1032 (gyroid); deformations/deformations.go:29-38, 87-92,
// 136-141, 173-175, 210-222, 269-274; main.go:123-199 (density, deform and
// both integrators).
#pragma once
#include <math.h>
#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define XRP_HD __host__ __device__ __forceinline__
#define XRP_HDN static __host__ __device__ __noinline__
#else
#define XRP_HD inline
#define XRP_HDN static
#endif

namespace xrp {

// ---------------------------------------------------------------------------
// exact FP64 operations (one rounding each, never fused)
// ---------------------------------------------------------------------------
#if defined(__CUDA_ARCH__)
XRP_HD double dadd(double a, double b) { return __dadd_rn(a, b); }
XRP_HD double dsub(double a, double b) { return __dsub_rn(a, b); }
XRP_HD double dmul(double a, double b) { return __dmul_rn(a, b); }
XRP_HD double ddiv(double a, double b) { return __ddiv_rn(a, b); }
XRP_HD double drcp(double a) { return __drcp_rn(a); }  // 1.0 / a, correctly rounded as the division
XRP_HD double dsqrt(double a) { return __dsqrt_rn(a); }
XRP_HD float f_exp(float x) { return __expf(x); }
XRP_HD float f_rcp(float x) { return __frcp_rn(x); }
#else
XRP_HD double dadd(double a, double b) { return a + b; }
XRP_HD double dsub(double a, double b) { return a - b; }
XRP_HD double dmul(double a, double b) { return a * b; }
XRP_HD double ddiv(double a, double b) { return a / b; }
XRP_HD double drcp(double a) { return 1.0 / a; }
XRP_HD double dsqrt(double a) { return sqrt(a); }
XRP_HD float f_exp(float x) { return expf(x); }
XRP_HD float f_rcp(float x) { return 1.0f / x; }
#endif

XRP_HD float xnan() { return __builtin_nanf(""); }
XRP_HD int32_t f2i(float f) {
#if defined(__CUDA_ARCH__)
    return __float_as_int(f);
#else
    int32_t i;
    __builtin_memcpy(&i, &f, 4);
    return i;
#endif
}
XRP_HD bool isunc(float r) { return r != r; }

// sin and cos of one argument: Cody-Waite reduction to [-pi, pi] with a
// two-term 2*pi, then the SFU approximations (device) or libm (host).  The
// error of the reduction and of the approximations is folded into the gyroid
// guard band on the host side.
XRP_HD void f_sincos(float x, float* s, float* c) {
    const float inv2pi = 0.159154943091895f;
    const float twopi_hi = 6.28318548202514648f;      // float(2*pi)
    const float twopi_lo = -1.7484555314695172e-07f;  // 2*pi - twopi_hi
    float k = rintf(x * inv2pi);
    float r = fmaf(-k, twopi_hi, x);
    r = fmaf(-k, twopi_lo, r);
#if defined(__CUDA_ARCH__)
    __sincosf(r, s, c);
#else
    *s = sinf(r);
    *c = cosf(r);
#endif
}

// ---------------------------------------------------------------------------
// scene image
// ---------------------------------------------------------------------------
enum NodeType : int32_t {
    N_SPHERE = 1,
    N_BOX = 2,
    N_CYL = 3,
    N_PPD = 4,
    N_GYROID = 5,
    N_COLL = 6,
    N_TESS = 7,
    N_VOXEL = 8,
};

enum CollFlags : int32_t {
    C_GREEDY = 1,     // GreedyDensEval
    C_EXACT_SUM = 2,  // every partial sum of child densities is exact in FP32
    C_ACCEL = 4,      // per-cell candidate lists are present
    C_CLIP = 8,       // clip the sum to [0, 1] (every ObjectCollection)
    C_UNIFORM = 16,   // greedy, every child a leaf of the same FP32 density > 0
};

// Leaf parameter slots (Node.f).  RHO and BAND slots are shared by leaves.
enum : int { F_RHO = 27, F_BAND = 26, F_BAND2 = 25 };

// 16-byte aligned so that a leaf's parameters load as 128-bit vectors
// (f[0] sits at byte 16).
struct alignas(16) Node {
    int32_t type;
    int32_t a;      // COLL: first slot in the child list; TESS: unit-cell collection node; VOXEL: volume id
    int32_t b;      // COLL: number of children
    int32_t flags;  // COLL: CollFlags | (accel grid dim << 16) | (homogeneous leaf type << 8)
    float f[28];
};
static_assert(sizeof(Node) == 128, "Node must stay 128 bytes");

struct Node64 {
    double d[16];
};

struct Volume {
    const float* data;     // [z][x][y], FP32
    const double* data64;  // exact values when FP32 cannot hold them, else null
    int32_t nx, ny, nz;
    int32_t pad;
    float scale[3];        // (N-1)/2 per axis
    float band_w;          // world-space guard band for the inclusive [-1,1] test
};

enum DefType : int32_t { D_GAUSSIAN = 1, D_LINEAR, D_RIGID, D_SIGMOID, D_AFFINE };

struct DefStep {
    int32_t type;
    int32_t axis;  // sigmoid
    int32_t pad[2];
    float f[12];
    double d[12];
};

// Everything a kernel needs about one scene (passed by value).
struct SceneDev {
    const Node* nodes;
    const Node64* nodes64;
    const int32_t* child;   // child node ids of collections
    const int32_t* cells;   // accel: per collection, (G^3 + 1) offsets into items
    const int32_t* items;   // accel: node indices of each cell's listed children, in child order
    const float* clear;     // accel: per cell, distance to the nearest child not listed
    const Volume* vols;
    const DefStep* defs;
    int32_t root;
    int32_t ndefs;
    int32_t hier_zero_guard;  // 1: flag near-zero voxel values (hierarchical zero test)
    int32_t affine;           // 1: the deformation chain is affine and invertible (or empty)
    float sup_lo[3], sup_hi[3];  // dilated support box (FP32, world)
    // distance certificates (margin32): 1 / Lipschitz bound of the
    // deformation chain, and the absolute error allowance of a margin in
    // deformed coordinates (position error plus FP32 arithmetic)
    float inv_lip;
    float m_slack;
    // ray certificates (dens_ray32, affine chains): capsule radius in
    // deformed coordinates (m_slack plus the direction error over the span)
    float ray_slack;
    int32_t nnodes;  // node count when the tracing kernels stage the table in shared memory, else 0
    // curved-ray certificates (smooth non-affine chains): bounds on the
    // speed |dq/ds| and the acceleration |d^2 q/ds^2| of the deformed sample
    // point along a unit-speed ray
    float curve_vmax;
    float curve_acc;
};

// One view (camera) of a batch, prepared on the host.
struct ViewDev {
    double eye[3];
    double m[16];       // camera-to-world, column-major (mathgl layout)
    double inv_w;       // 1/m[15] when the last row is (0,0,0,w); else 0
    double f;           // focal length 1/tan(fov/2)
    int32_t general_w;  // 1: divide by the per-pixel w
    int32_t pad[3];
    // the same camera for the FP32 march, as (hi, lo) float pairs (general_w
    // == 0): direction before normalisation c0 * x_i + c1 * x_j + k, and the
    // eye
    float c0[6], c1[6], k[6], eye2[6];
};

// Sample lattice of one integrator run (same for every ray of a batch).
struct Lattice {
    const double* s64;    // simple: s_k; hierarchical: coarse right ends r_k
    const float* t32;     // float(s_k - s_c)
    const int32_t* fstart;  // hierarchical: fine sample range of coarse k
    const double* f64;    // hierarchical: fine positions
    const float* ft32;    // hierarchical: float(fine - s_c)
    int32_t K;            // number of (coarse) samples
    int32_t hierarchical;
    double s_c;           // reference point of the FP32 offsets
    double smin;
    double ds;            // simple: ds; hierarchical: DS
    double ds_fine;       // hierarchical: DS/10
    float ds32, dsf32;    // float(ds), float(ds_fine)
    float t_first;        // float(s_0 - s_c)
    float inv_ds;         // 1/ds (FP32, for clipping)
    float ds_hi, ds_lo;   // ds split so that t_k = t_first + k*(ds_hi + ds_lo)
    float s_c2[2];        // s_c as a (hi, lo) float pair
};

// FP32 offset of lattice sample k from s_c: t_first + k*ds with ds carried
// in two parts (error about 3 units of FP32 rounding of |t|, folded into the
// position error bound on the host).
XRP_HD float lattice_t(const Lattice& L, int k) {
    float kf = (float)k;
    return fmaf(kf, L.ds_hi, fmaf(kf, L.ds_lo, L.t_first));
}

struct RenderParams {
    int32_t res;
    int32_t nviews;
    float flat_field;
    float density_multiplier;
    const double* xs;     // pixel coordinate table i/(res/2)-1, length res
    const float* xsf;     // the same as (hi, lo) float pairs, length 2 res
};

// Four consecutive node parameters f[k..k+3], k a multiple of 4: one
// 128-bit load on the device.
struct alignas(16) F4 {
    float x, y, z, w;
};

XRP_HD F4 ld4(const float* p) {
#if defined(__CUDA_ARCH__)
    return *reinterpret_cast<const F4*>(p);
#else
    F4 r;
    memcpy(&r, p, sizeof(r));
    return r;
#endif
}

// ---------------------------------------------------------------------------
// FP32 guarded evaluation
// ---------------------------------------------------------------------------
// Returns the density (pre-multiplier) or NaN when a predicate is too close
// to its decision boundary for FP32 to decide.

// (f[24..27] holds F_BAND2, F_BAND, F_RHO: one vector load with the first.)
XRP_HD float sphere32(const float* f, float x, float y, float z) {
    const F4 a = ld4(f), t = ld4(f + 24);
    float dx = x - a.x, dy = y - a.y, dz = z - a.z;
    float m = fmaf(dz, dz, fmaf(dy, dy, dx * dx)) - a.w;
    if (m < -t.z) return t.w;
    if (m > t.z) return 0.0f;
    return xnan();
}

XRP_HD float box32(const float* f, float x, float y, float z) {
    const F4 a = ld4(f), c = ld4(f + 4), t = ld4(f + 24);
    float mx = a.w - fabsf(x - a.x);
    float my = c.x - fabsf(y - a.y);
    float mz = c.y - fabsf(z - a.z);
    float b = t.z;
    float mn = fminf(mx, fminf(my, mz));
    if (mn > b) return t.w;
    if (mn < -b) return 0.0f;
    return xnan();
}

XRP_HD float cyl32(const float* f, float x, float y, float z) {
    // a: p0, v.x; c: v.y, v.z, 1/|v|^2, r^2
    const F4 a = ld4(f), c4 = ld4(f + 4), t = ld4(f + 24);
    float wx = x - a.x, wy = y - a.y, wz = z - a.z;
    float c = fmaf(wz, c4.y, fmaf(wy, c4.x, wx * a.w)) * c4.z;
    float bc = t.y;
    if (c < -bc || c > 1.0f + bc) return 0.0f;
    float px = fmaf(-c, a.w, wx), py = fmaf(-c, c4.x, wy), pz = fmaf(-c, c4.y, wz);
    float m = fmaf(pz, pz, fmaf(py, py, px * px)) - c4.w;
    float bd = t.z;
    if (m > bd) return 0.0f;
    if (m < -bd && c > bc && c < 1.0f - bc) return t.w;
    return xnan();
}

XRP_HD float ppd32(const float* f, float x, float y, float z) {
    float wx = x - f[0], wy = y - f[1], wz = z - f[2];
    float qx = fmaf(f[5], wz, fmaf(f[4], wy, f[3] * wx));
    float qy = fmaf(f[8], wz, fmaf(f[7], wy, f[6] * wx));
    float qz = fmaf(f[11], wz, fmaf(f[10], wy, f[9] * wx));
    float b = f[F_BAND];
    // margin to the strict interval (0, 1) on each axis
    float mx = fminf(qx, 1.0f - qx), my = fminf(qy, 1.0f - qy), mz = fminf(qz, 1.0f - qz);
    float mn = fminf(mx, fminf(my, mz));
    if (mn > b) return f[F_RHO];
    if (mn < -b) return 0.0f;
    return xnan();
}

XRP_HD float gyroid32(const float* f, float x, float y, float z) {
    float X = (x - f[0]) * f[3], Y = (y - f[1]) * f[3], Z = (z - f[2]) * f[3];
    float sx, cx, sy, cy, sz, cz;
    f_sincos(X, &sx, &cx);
    f_sincos(Y, &sy, &cy);
    f_sincos(Z, &sz, &cz);
    float g = fmaf(sz, cx, fmaf(sy, cz, sx * cy));
    float m = f[4] - fabsf(g);
    if (m > f[F_BAND]) return f[F_RHO];
    if (m < -f[F_BAND]) return 0.0f;
    return xnan();
}

XRP_HD float voxel32(const Volume& V, float band_zero, float x, float y, float z, int zero_guard) {
    float b = V.band_w;
    float ax = fabsf(x), ay = fabsf(y), az = fabsf(z);
    float mx = fmaxf(ax, fmaxf(ay, az));
    if (mx > 1.0f + b) return 0.0f;
    if (!(mx < 1.0f - b)) return xnan();  // on the inclusive boundary, or NaN
    float ux = (x + 1.0f) * V.scale[0];
    float uy = (y + 1.0f) * V.scale[1];
    float uz = (z + 1.0f) * V.scale[2];
    float fx = floorf(ux), fy = floorf(uy), fz = floorf(uz);
    int x0 = (int)fx, y0 = (int)fy, z0 = (int)fz;
    float wx = ux - fx, wy = uy - fy, wz = uz - fz;
    x0 = x0 < 0 ? 0 : (x0 > V.nx - 1 ? V.nx - 1 : x0);
    y0 = y0 < 0 ? 0 : (y0 > V.ny - 1 ? V.ny - 1 : y0);
    z0 = z0 < 0 ? 0 : (z0 > V.nz - 1 ? V.nz - 1 : z0);
    int x1 = x0 + 1 > V.nx - 1 ? V.nx - 1 : x0 + 1;
    int y1 = y0 + 1 > V.ny - 1 ? V.ny - 1 : y0 + 1;
    int z1 = z0 + 1 > V.nz - 1 ? V.nz - 1 : z0 + 1;
    long NXY = (long)V.nx * V.ny, NY = V.ny;
    const float* r = V.data;
    float v000 = r[z0 * NXY + x0 * NY + y0];
    float v001 = r[z1 * NXY + x0 * NY + y0];
    float v010 = r[z0 * NXY + x0 * NY + y1];
    float v011 = r[z1 * NXY + x0 * NY + y1];
    float v100 = r[z0 * NXY + x1 * NY + y0];
    float v101 = r[z1 * NXY + x1 * NY + y0];
    float v110 = r[z0 * NXY + x1 * NY + y1];
    float v111 = r[z1 * NXY + x1 * NY + y1];
    float v00 = fmaf(wz, v001 - v000, v000);
    float v01 = fmaf(wz, v011 - v010, v010);
    float v10 = fmaf(wz, v101 - v100, v100);
    float v11 = fmaf(wz, v111 - v110, v110);
    float v0 = fmaf(wy, v01 - v00, v00);
    float v1 = fmaf(wy, v11 - v10, v10);
    float v = fmaf(wx, v1 - v0, v0);
    if (zero_guard) {
        // the hierarchical integrator tests density == 0: decide that only
        // when FP32 and FP64 cannot disagree
        float amax = fmaxf(fmaxf(fmaxf(fabsf(v000), fabsf(v001)), fmaxf(fabsf(v010), fabsf(v011))),
                           fmaxf(fmaxf(fabsf(v100), fabsf(v101)), fmaxf(fabsf(v110), fabsf(v111))));
        if (amax > 0.0f && fabsf(v) <= band_zero * amax) return xnan();
    }
    return v;
}

XRP_HD float leaf32(const Node& n, float x, float y, float z) {
    switch (n.type) {
    case N_SPHERE: return sphere32(n.f, x, y, z);
    case N_BOX: return box32(n.f, x, y, z);
    case N_CYL: return cyl32(n.f, x, y, z);
    case N_PPD: return ppd32(n.f, x, y, z);
    case N_GYROID: return gyroid32(n.f, x, y, z);
    default: return xnan();
    }
}

template <int D>
XRP_HD float coll32(const SceneDev& S, const Node& c, float x, float y, float z);

// A collection child: leaf, voxel grid or (nested) tessellation.
template <int D>
XRP_HD float item32(const SceneDev& S, int id, float x, float y, float z) {
    const Node& n = S.nodes[id];
    if (n.type <= N_GYROID) return leaf32(n, x, y, z);
    if (n.type == N_VOXEL) return voxel32(S.vols[n.a], n.f[0], x, y, z, S.hier_zero_guard);
    if (n.type == N_TESS) {
        if constexpr (D > 0) {
            // f[0..5] outer bounds, f[6] their band, f[7..12] unit-cell
            // bounds, f[13] their band, f[14..16] cell size, f[17..19] its
            // reciprocal, f[20..22] unit-cell origin, f[23] fold band
            const F4 f0 = ld4(n.f), f4 = ld4(n.f + 4), f8 = ld4(n.f + 8), f12 = ld4(n.f + 12);
            const F4 f16 = ld4(n.f + 16), f20 = ld4(n.f + 20);
            // outer inclusive bounds (objects.go:570)
            float mo = fminf(fminf(fminf(x - f0.x, f0.y - x), fminf(y - f0.z, f0.w - y)),
                             fminf(z - f4.x, f4.y - z));
            if (mo < -f4.z) return 0.0f;
            if (!(mo > f4.z)) return xnan();
            // fold into the unit cell (objects.go:574-579)
            float qx = (x - f20.x) * f16.y, qy = (y - f20.y) * f16.z, qz = (z - f20.z) * f16.w;
            float nx = floorf(qx), ny = floorf(qy), nz = floorf(qz);
            float bq = f20.w;
            float fr = fminf(fminf(fminf(qx - nx, 1.0f - (qx - nx)), fminf(qy - ny, 1.0f - (qy - ny))),
                             fminf(qz - nz, 1.0f - (qz - nz)));
            if (!(fr > bq)) return xnan();
            float fx = fmaf(-f12.z, nx, x), fy = fmaf(-f12.w, ny, y), fz = fmaf(-f16.x, nz, z);
            // unit-cell inclusive bounds (objects.go:460)
            float mu = fminf(fminf(fminf(fx - f4.w, f8.x - fx), fminf(fy - f8.y, f8.z - fy)),
                             fminf(fz - f8.w, f12.x - fz));
            if (mu < -f12.y) return 0.0f;
            if (!(mu > f12.y)) return xnan();
            return coll32<D - 1>(S, S.nodes[n.a], fx, fy, fz);
        } else {
            return xnan();
        }
    }
    return xnan();
}

// ObjectCollection.Density (objects.go:422-438) in FP32.
template <int D>
XRP_HD float coll32(const SceneDev& S, const Node& c, float x, float y, float z) {
    const int32_t* kids = S.child + c.a;
    int cnt = c.b;
    const int32_t* list = nullptr;
    if (c.flags & C_ACCEL) {
        int G = (c.flags >> 16) & 0xff;
        const F4 g0 = ld4(c.f), g4 = ld4(c.f + 4);  // grid origin, 1/cell size, cell base
        int ix = (int)floorf((x - g0.x) * g0.w);
        int iy = (int)floorf((y - g0.y) * g4.x);
        int iz = (int)floorf((z - g0.z) * g4.y);
        ix = ix < 0 ? 0 : (ix >= G ? G - 1 : ix);
        iy = iy < 0 ? 0 : (iy >= G ? G - 1 : iy);
        iz = iz < 0 ? 0 : (iz >= G ? G - 1 : iz);
        int cell_base = f2i(g4.z);
        const int32_t* off = S.cells + cell_base + (iz * G + iy) * G + ix;
        int s0 = off[0], s1 = off[1];
        list = S.items + s0;
        cnt = s1 - s0;
    }
    const bool greedy = (c.flags & C_GREEDY) != 0;
    float sum = 0.0f, sabs = 0.0f;
    const int homo = (c.flags >> 8) & 0xff;
    for (int k = 0; k < cnt; k++) {
        const int kid = list ? list[k] : kids[k];
        const Node& n = S.nodes[kid];
        float r;
        if (homo == N_CYL)
            r = cyl32(n.f, x, y, z);
        else if (homo == N_SPHERE)
            r = sphere32(n.f, x, y, z);
        else
            r = item32<D>(S, kid, x, y, z);
        if (isunc(r)) return r;
        if (greedy && r > 0.0f) return r;
        sum += r;
        sabs += fabsf(r);
    }
    if (!(c.flags & C_EXACT_SUM) && sabs > 0.0f && fabsf(sum) <= c.f[7] * sabs) return xnan();
    if (c.flags & C_CLIP) sum = fminf(fmaxf(sum, 0.0f), 1.0f);
    return sum;
}

// deform() (main.go:123-133) in FP32.
XRP_HD void deform32(const SceneDev& S, float& x, float& y, float& z) {
    for (int i = 0; i < S.ndefs; i++) {
        const DefStep& d = S.defs[i];
        const float* a = d.f;
        switch (d.type) {
        case D_GAUSSIAN: {
            float x0 = x - a[6], y0 = y - a[7], z0 = z - a[8];
            float r2 = fmaf(z0, z0, fmaf(y0, y0, x0 * x0));
            float dx = a[0] * f_exp(-r2 * a[3]);
            float dy = a[1] * f_exp(-r2 * a[4]);
            float dz = a[2] * f_exp(-r2 * a[5]);
            x += dx; y += dy; z += dz;
            break;
        }
        case D_LINEAR: {
            float nx = fmaf(a[4], z, fmaf(a[5], y, fmaf(a[0], x, x)));
            float ny = fmaf(a[3], z, fmaf(a[1], y, fmaf(a[5], x, y)));
            float nz = fmaf(a[2], z, fmaf(a[3], y, fmaf(a[4], x, z)));
            x = nx; y = ny; z = nz;
            break;
        }
        case D_RIGID: x += a[0]; y += a[1]; z += a[2]; break;
        case D_SIGMOID: {
            float* p = d.axis == 0 ? &x : (d.axis == 1 ? &y : &z);
            float e = f_exp(-(*p - a[1]) * a[2]);
            *p += a[0] * f_rcp(1.0f + e);
            break;
        }
        case D_AFFINE: {
            float nx = fmaf(a[2], z, fmaf(a[1], y, a[0] * x));
            float ny = fmaf(a[5], z, fmaf(a[4], y, a[3] * x));
            float nz = fmaf(a[8], z, fmaf(a[7], y, a[6] * x));
            x = nx; y = ny; z = nz;
            break;
        }
        default: break;
        }
    }
}

constexpr int kMaxDepth = 3;  // nested tessellations supported by the evaluators

// DEPTH: deepest tessellation nesting of the scene (kernels are specialised
// on it so that evaluator code a scene cannot reach is not compiled in);
// DEFS: whether a deformation is applied.
template <int DEPTH, bool DEFS>
XRP_HD float density32(const SceneDev& S, float x, float y, float z) {
    if constexpr (DEFS) deform32(S, x, y, z);
    const Node& r = S.nodes[S.root];
    if (r.type <= N_GYROID) return leaf32(r, x, y, z);
    if (r.type == N_COLL) return coll32<DEPTH>(S, r, x, y, z);
    return item32<DEPTH>(S, S.root, x, y, z);
}

// ---------------------------------------------------------------------------
// Distance certificates
// ---------------------------------------------------------------------------
// margin32 returns a lower bound on the world-space distance from a sample
// point to the nearest place where the density can change (a primitive
// surface, a container bound, a tessellation cell face).  Inside a ball of
// that radius the set of primitives containing the point is fixed, so the
// reference's FP64 density is the same value everywhere in it.  Each leaf
// bound is |max of the signed distances of the convex pieces it intersects|,
// which under-estimates the distance to the boundary inside and outside.

XRP_HD float leaf_margin(const Node& n, float x, float y, float z) {
    const float* f = n.f;
    switch (n.type) {
    case N_SPHERE: {
        float dx = x - f[0], dy = y - f[1], dz = z - f[2];
        float d = sqrtf(fmaf(dz, dz, fmaf(dy, dy, dx * dx)));
        return fabsf(d - f[4]);
    }
    case N_BOX: {
        float mx = f[3] - fabsf(x - f[0]);
        float my = f[4] - fabsf(y - f[1]);
        float mz = f[5] - fabsf(z - f[2]);
        return fabsf(fminf(mx, fminf(my, mz)));
    }
    case N_CYL: {
        float wx = x - f[0], wy = y - f[1], wz = z - f[2];
        float c = fmaf(wz, f[5], fmaf(wy, f[4], wx * f[3])) * f[6];
        float px = fmaf(-c, f[3], wx), py = fmaf(-c, f[4], wy), pz = fmaf(-c, f[5], wz);
        float pr = sqrtf(fmaf(pz, pz, fmaf(py, py, px * px)));
        float len = f[9];
        float sd = fmaxf(pr - f[8], fmaxf(-c * len, (c - 1.0f) * len));
        return fabsf(sd);
    }
    case N_PPD: {
        float wx = x - f[0], wy = y - f[1], wz = z - f[2];
        float sd = -3.0e38f;
        for (int a = 0; a < 3; a++) {
            const float* m = f + 3 + 3 * a;
            float q = fmaf(m[2], wz, fmaf(m[1], wy, m[0] * wx));
            float nrm = sqrtf(fmaf(m[2], m[2], fmaf(m[1], m[1], m[0] * m[0])));
            sd = fmaxf(sd, fmaxf(-q, q - 1.0f) / nrm);
        }
        return fabsf(sd);
    }
    case N_GYROID: {
        float X = (x - f[0]) * f[3], Y = (y - f[1]) * f[3], Z = (z - f[2]) * f[3];
        float sx, cx, sy, cy, sz, cz;
        f_sincos(X, &sx, &cx);
        f_sincos(Y, &sy, &cy);
        f_sincos(Z, &sz, &cz);
        float g = fmaf(sz, cx, fmaf(sy, cz, sx * cy));
        // |grad g| <= sqrt(6) |1/scale| (each component is a sum of two
        // products of sines and cosines)
        float m = fabsf(f[4] - fabsf(g)) - f[F_BAND];
        return fmaxf(m, 0.0f) / (2.4494898f * fabsf(f[3]));
    }
    default: return 0.0f;
    }
}

template <int D>
XRP_HD float collm32(const SceneDev& S, const Node& c, float x, float y, float z);

template <int D>
XRP_HD float itemm32(const SceneDev& S, int id, float x, float y, float z) {
    const Node& n = S.nodes[id];
    if (n.type <= N_GYROID) return leaf_margin(n, x, y, z);
    if (n.type == N_TESS) {
        if constexpr (D > 0) {
            const float* f = n.f;
            float mo = fminf(fminf(fminf(x - f[0], f[1] - x), fminf(y - f[2], f[3] - y)),
                             fminf(z - f[4], f[5] - z));
            if (mo <= 0.0f) return -mo;  // outside the outer bounds: zero up to the box
            float qx = (x - f[20]) * f[17], qy = (y - f[21]) * f[18], qz = (z - f[22]) * f[19];
            float nx = floorf(qx), ny = floorf(qy), nz = floorf(qz);
            // distance to the faces of this tessellation cell
            float fc = fminf(fminf(fminf(qx - nx, 1.0f - (qx - nx)) * fabsf(f[14]),
                                   fminf(qy - ny, 1.0f - (qy - ny)) * fabsf(f[15])),
                             fminf(qz - nz, 1.0f - (qz - nz)) * fabsf(f[16]));
            float m = fminf(mo, fc);
            float fx = fmaf(-f[14], nx, x), fy = fmaf(-f[15], ny, y), fz = fmaf(-f[16], nz, z);
            float mu = fminf(fminf(fminf(fx - f[7], f[8] - fx), fminf(fy - f[9], f[10] - fy)),
                             fminf(fz - f[11], f[12] - fz));
            if (mu <= 0.0f) return fminf(m, -mu);  // outside the unit-cell bounds: zero
            m = fminf(m, mu);
            return fminf(m, collm32<D - 1>(S, S.nodes[n.a], fx, fy, fz));
        }
    }
    return 0.0f;  // voxel grids and anything deeper: no certificate
}

// Collections: the density is a function of which children contain the
// point, so the nearest child boundary bounds it.  With candidate lists
// only the children overlapping the point's cell are listed; the others
// cannot reach inside the cell, so the distance to the cell's inner faces
// caps the bound.
template <int D>
XRP_HD float collm32(const SceneDev& S, const Node& c, float x, float y, float z) {
    const int32_t* kids = S.child + c.a;
    int cnt = c.b;
    const int32_t* list = nullptr;
    float m = 3.0e38f;
    if (c.flags & C_ACCEL) {
        int G = (c.flags >> 16) & 0xff;
        float ux = (x - c.f[0]) * c.f[3], uy = (y - c.f[1]) * c.f[4], uz = (z - c.f[2]) * c.f[5];
        int ix = (int)floorf(ux), iy = (int)floorf(uy), iz = (int)floorf(uz);
        ix = ix < 0 ? 0 : (ix >= G ? G - 1 : ix);
        iy = iy < 0 ? 0 : (iy >= G ? G - 1 : iy);
        iz = iz < 0 ? 0 : (iz >= G ? G - 1 : iz);
        // inner faces only (the outer cells extend to infinity by the clamp)
        if (ix > 0) m = fminf(m, (ux - (float)ix) / c.f[3]);
        if (ix < G - 1) m = fminf(m, ((float)(ix + 1) - ux) / c.f[3]);
        if (iy > 0) m = fminf(m, (uy - (float)iy) / c.f[4]);
        if (iy < G - 1) m = fminf(m, ((float)(iy + 1) - uy) / c.f[4]);
        if (iz > 0) m = fminf(m, (uz - (float)iz) / c.f[5]);
        if (iz < G - 1) m = fminf(m, ((float)(iz + 1) - uz) / c.f[5]);
        int cell_base = f2i(c.f[6]);
        const int cell = cell_base + (iz * G + iy) * G + ix;
        // unlisted children are beyond the cell's faces and beyond its clearance
        m = fmaxf(fmaxf(m, 0.0f), S.clear[cell]);
        const int32_t* off = S.cells + cell;
        int s0 = off[0], s1 = off[1];
        list = S.items + s0;
        cnt = s1 - s0;
    }
    for (int k = 0; k < cnt; k++) {
        m = fminf(m, itemm32<D>(S, list ? list[k] : kids[k], x, y, z));
    }
    return m;
}

// World-space certificate radius at a sample point (deformation applied
// here); 0 when nothing can be certified.
template <int DEPTH, bool DEFS>
XRP_HD float margin32(const SceneDev& S, float x, float y, float z) {
    if constexpr (DEFS) deform32(S, x, y, z);
    const Node& r = S.nodes[S.root];
    float m;
    if (r.type <= N_GYROID) m = leaf_margin(r, x, y, z);
    else if (r.type == N_COLL) m = collm32<DEPTH>(S, r, x, y, z);
    else m = itemm32<DEPTH>(S, S.root, x, y, z);
    m = fmaf(m, 0.9999f, -S.m_slack);
    return m > 0.0f ? m * S.inv_lip : 0.0f;
}

// ---------------------------------------------------------------------------
// Density and certificate radius in one traversal (certificate tracing):
// the same decisions as density32 and the same radius as margin32, with the
// deformation, folds and leaf geometry computed once.
// ---------------------------------------------------------------------------

XRP_HD float leaf_dm(const Node& n, float x, float y, float z, float& m) {
    const float* f = n.f;
    switch (n.type) {
    case N_SPHERE: {
        float dx = x - f[0], dy = y - f[1], dz = z - f[2];
        float d2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
        m = fabsf(sqrtf(d2) - f[4]);
        float q = d2 - f[3];
        if (q < -f[F_BAND]) return f[F_RHO];
        if (q > f[F_BAND]) return 0.0f;
        return xnan();
    }
    case N_BOX: {
        float mx = f[3] - fabsf(x - f[0]);
        float my = f[4] - fabsf(y - f[1]);
        float mz = f[5] - fabsf(z - f[2]);
        float mn = fminf(mx, fminf(my, mz));
        m = fabsf(mn);
        float b = f[F_BAND];
        if (mn > b) return f[F_RHO];
        if (mn < -b) return 0.0f;
        return xnan();
    }
    case N_CYL: {
        float wx = x - f[0], wy = y - f[1], wz = z - f[2];
        float c = fmaf(wz, f[5], fmaf(wy, f[4], wx * f[3])) * f[6];
        float px = fmaf(-c, f[3], wx), py = fmaf(-c, f[4], wy), pz = fmaf(-c, f[5], wz);
        float p2 = fmaf(pz, pz, fmaf(py, py, px * px));
        float len = f[9];
        m = fabsf(fmaxf(sqrtf(p2) - f[8], fmaxf(-c * len, (c - 1.0f) * len)));
        float bc = f[F_BAND2];
        if (c < -bc || c > 1.0f + bc) return 0.0f;
        float q = p2 - f[7];
        float bd = f[F_BAND];
        if (q > bd) return 0.0f;
        if (q < -bd && c > bc && c < 1.0f - bc) return f[F_RHO];
        return xnan();
    }
    case N_PPD: {
        float wx = x - f[0], wy = y - f[1], wz = z - f[2];
        float sd = -3.0e38f, mn = 3.0e38f;
        for (int a = 0; a < 3; a++) {
            const float* r = f + 3 + 3 * a;
            float q = fmaf(r[2], wz, fmaf(r[1], wy, r[0] * wx));
            float nrm = sqrtf(fmaf(r[2], r[2], fmaf(r[1], r[1], r[0] * r[0])));
            sd = fmaxf(sd, fmaxf(-q, q - 1.0f) / nrm);
            mn = fminf(mn, fminf(q, 1.0f - q));
        }
        m = fabsf(sd);
        float b = f[F_BAND];
        if (mn > b) return f[F_RHO];
        if (mn < -b) return 0.0f;
        return xnan();
    }
    case N_GYROID: {
        float X = (x - f[0]) * f[3], Y = (y - f[1]) * f[3], Z = (z - f[2]) * f[3];
        float sx, cx, sy, cy, sz, cz;
        f_sincos(X, &sx, &cx);
        f_sincos(Y, &sy, &cy);
        f_sincos(Z, &sz, &cz);
        float g = fmaf(sz, cx, fmaf(sy, cz, sx * cy));
        float q = f[4] - fabsf(g);
        m = fmaxf(fabsf(q) - f[F_BAND], 0.0f) / (2.4494898f * fabsf(f[3]));
        if (q > f[F_BAND]) return f[F_RHO];
        if (q < -f[F_BAND]) return 0.0f;
        return xnan();
    }
    default: m = 0.0f; return xnan();
    }
}

template <int D>
XRP_HD float coll_dm(const SceneDev& S, const Node& c, float x, float y, float z, float& m);

template <int D>
XRP_HD float item_dm(const SceneDev& S, int id, float x, float y, float z, float& m) {
    const Node& n = S.nodes[id];
    if (n.type <= N_GYROID) return leaf_dm(n, x, y, z, m);
    if (n.type == N_TESS) {
        if constexpr (D > 0) {
            const float* f = n.f;
            float mo = fminf(fminf(fminf(x - f[0], f[1] - x), fminf(y - f[2], f[3] - y)),
                             fminf(z - f[4], f[5] - z));
            if (mo <= 0.0f) m = -mo;
            if (mo < -f[6]) return 0.0f;
            if (!(mo > f[6])) { m = 0.0f; return xnan(); }
            float qx = (x - f[20]) * f[17], qy = (y - f[21]) * f[18], qz = (z - f[22]) * f[19];
            float nx = floorf(qx), ny = floorf(qy), nz = floorf(qz);
            float bq = f[23];
            float fr = fminf(fminf(fminf(qx - nx, 1.0f - (qx - nx)), fminf(qy - ny, 1.0f - (qy - ny))),
                             fminf(qz - nz, 1.0f - (qz - nz)));
            if (!(fr > bq)) { m = 0.0f; return xnan(); }
            float fc = fminf(fminf(fminf(qx - nx, 1.0f - (qx - nx)) * fabsf(f[14]),
                                   fminf(qy - ny, 1.0f - (qy - ny)) * fabsf(f[15])),
                             fminf(qz - nz, 1.0f - (qz - nz)) * fabsf(f[16]));
            float mm = fminf(mo, fc);
            float fx = fmaf(-f[14], nx, x), fy = fmaf(-f[15], ny, y), fz = fmaf(-f[16], nz, z);
            float mu = fminf(fminf(fminf(fx - f[7], f[8] - fx), fminf(fy - f[9], f[10] - fy)),
                             fminf(fz - f[11], f[12] - fz));
            if (mu < -f[13]) { m = fminf(mm, -mu); return 0.0f; }
            if (!(mu > f[13])) { m = 0.0f; return xnan(); }
            float mc;
            float r = coll_dm<D - 1>(S, S.nodes[n.a], fx, fy, fz, mc);
            m = fminf(fminf(mm, mu), mc);
            return r;
        }
    }
    m = 0.0f;  // voxel grids and anything deeper: density by the plain path
    if (n.type == N_VOXEL) return voxel32(S.vols[n.a], n.f[0], x, y, z, S.hier_zero_guard);
    return xnan();
}

template <int D>
XRP_HD float coll_dm(const SceneDev& S, const Node& c, float x, float y, float z, float& m) {
    const int32_t* kids = S.child + c.a;
    int cnt = c.b;
    const int32_t* list = nullptr;
    m = 3.0e38f;
    if (c.flags & C_ACCEL) {
        int G = (c.flags >> 16) & 0xff;
        float ux = (x - c.f[0]) * c.f[3], uy = (y - c.f[1]) * c.f[4], uz = (z - c.f[2]) * c.f[5];
        int ix = (int)floorf(ux), iy = (int)floorf(uy), iz = (int)floorf(uz);
        ix = ix < 0 ? 0 : (ix >= G ? G - 1 : ix);
        iy = iy < 0 ? 0 : (iy >= G ? G - 1 : iy);
        iz = iz < 0 ? 0 : (iz >= G ? G - 1 : iz);
        if (ix > 0) m = fminf(m, (ux - (float)ix) / c.f[3]);
        if (ix < G - 1) m = fminf(m, ((float)(ix + 1) - ux) / c.f[3]);
        if (iy > 0) m = fminf(m, (uy - (float)iy) / c.f[4]);
        if (iy < G - 1) m = fminf(m, ((float)(iy + 1) - uy) / c.f[4]);
        if (iz > 0) m = fminf(m, (uz - (float)iz) / c.f[5]);
        if (iz < G - 1) m = fminf(m, ((float)(iz + 1) - uz) / c.f[5]);
        int cell_base = f2i(c.f[6]);
        const int cell = cell_base + (iz * G + iy) * G + ix;
        // unlisted children are beyond the cell's faces and beyond its clearance
        m = fmaxf(fmaxf(m, 0.0f), S.clear[cell]);
        const int32_t* off = S.cells + cell;
        int s0 = off[0], s1 = off[1];
        list = S.items + s0;
        cnt = s1 - s0;
    }
    const bool greedy = (c.flags & C_GREEDY) != 0;
    float sum = 0.0f, sabs = 0.0f;
    bool unc = false, done = false;
    for (int k = 0; k < cnt; k++) {
        float mk;
        float r = item_dm<D>(S, list ? list[k] : kids[k], x, y, z, mk);
        m = fminf(m, mk);
        if (done) continue;  // greedy value fixed; radii of the rest still count
        if (isunc(r)) {
            unc = true;
            done = true;
            continue;
        }
        if (greedy && r > 0.0f) {
            sum = r;
            sabs = fabsf(r);
            done = true;
            continue;
        }
        sum += r;
        sabs += fabsf(r);
    }
    if (unc) return xnan();
    if (greedy && done) return sum;
    if (!(c.flags & C_EXACT_SUM) && sabs > 0.0f && fabsf(sum) <= c.f[7] * sabs) return xnan();
    if (c.flags & C_CLIP) sum = fminf(fmaxf(sum, 0.0f), 1.0f);
    return sum;
}

// density32 and margin32 at one point: returns the density (NaN when
// uncertain) and sets `m` to the world-space certificate radius.
template <int DEPTH, bool DEFS>
XRP_HD float dens_margin32(const SceneDev& S, float x, float y, float z, float& m) {
    if constexpr (DEFS) deform32(S, x, y, z);
    const Node& r = S.nodes[S.root];
    float rho;
    if (r.type <= N_GYROID) rho = leaf_dm(r, x, y, z, m);
    else if (r.type == N_COLL) rho = coll_dm<DEPTH>(S, r, x, y, z, m);
    else rho = item_dm<DEPTH>(S, S.root, x, y, z, m);
    m = fmaf(m, 0.9999f, -S.m_slack);
    m = m > 0.0f ? m * S.inv_lip : 0.0f;
    return rho;
}

}  // namespace xrp

#include "xrp_cert_ray.h"
#include "xrp_cert_curve.h"

namespace xrp {

// ---------------------------------------------------------------------------
// FP64 exact evaluation (reference arithmetic, operation by operation)
// ---------------------------------------------------------------------------

XRP_HD double sphere64(const double* d, double x, double y, double z) {
    x = dsub(x, d[0]);
    y = dsub(y, d[1]);
    z = dsub(z, d[2]);
    double r_2 = dadd(dadd(dmul(x, x), dmul(y, y)), dmul(z, z));
    if (r_2 < dmul(d[3], d[3])) return d[4];
    return 0.0;
}

XRP_HD double box64(const double* d, double x, double y, double z) {
    x = fabs(dsub(x, d[0]));
    y = fabs(dsub(y, d[1]));
    z = fabs(dsub(z, d[2]));
    if (x < dmul(0.5, d[3]) && y < dmul(0.5, d[4]) && z < dmul(0.5, d[5])) return d[6];
    return 0.0;
}

XRP_HD double ppd64(const double* d, double x, double y, double z) {
    double wx = dsub(x, d[0]), wy = dsub(y, d[1]), wz = dsub(z, d[2]);
    const double* m = &d[3];  // column-major
    double qx = dadd(dadd(dmul(m[0], wx), dmul(m[3], wy)), dmul(m[6], wz));
    double qy = dadd(dadd(dmul(m[1], wx), dmul(m[4], wy)), dmul(m[7], wz));
    double qz = dadd(dadd(dmul(m[2], wx), dmul(m[5], wy)), dmul(m[8], wz));
    if (qx > 0.0 && qx < 1.0 && qy > 0.0 && qy < 1.0 && qz > 0.0 && qz < 1.0) return d[12];
    return 0.0;
}

// Cylinder::Density (objects.go:334-350) in the reference's operation order.
// The per-cylinder terms come from the host, formed by the same operations:
// d[8..10] = p1 - p0, d[11] = |p1 - p0|^2, and d[12] = T with
// sqrt(s) < r exactly when s < T, so the square root is not taken.
XRP_HD double cyl64(const double* d, double x, double y, double z) {
    const double vx = d[8], vy = d[9], vz = d[10];
    double wx = dsub(x, d[0]), wy = dsub(y, d[1]), wz = dsub(z, d[2]);
    double wv = dadd(dadd(dmul(wx, vx), dmul(wy, vy)), dmul(wz, vz));
    double c = ddiv(wv, d[11]);
    if (c < 0.0 || c > 1.0) return 0.0;
    double dx = dsub(wx, dmul(vx, c)), dy = dsub(wy, dmul(vy, c)), dz = dsub(wz, dmul(vz, c));
    if (dadd(dadd(dmul(dx, dx), dmul(dy, dy)), dmul(dz, dz)) < d[12]) return d[7];
    return 0.0;
}

XRP_HD double gyroid64(const double* d, double x, double y, double z) {
    x = ddiv(dsub(x, d[0]), d[3]);
    y = ddiv(dsub(y, d[1]), d[3]);
    z = ddiv(dsub(z, d[2]), d[3]);
    double v = dadd(dadd(dmul(sin(x), cos(y)), dmul(sin(y), cos(z))), dmul(sin(z), cos(x)));
    if (fabs(v) < d[4]) return d[5];
    return 0.0;
}

XRP_HD double voxel64(const Volume& V, double x, double y, double z) {
    if (x < -1 || x > 1 || y < -1 || y > 1 || z < -1 || z > 1) return 0.0;
    // (v + 1) / 2: halving is exact, so the product by 0.5 is the quotient
    x = dmul(dadd(x, 1.0), 0.5);
    y = dmul(dadd(y, 1.0), 0.5);
    z = dmul(dadd(z, 1.0), 0.5);
    x = dmul(x, (double)(V.nx - 1));
    y = dmul(y, (double)(V.ny - 1));
    z = dmul(z, (double)(V.nz - 1));
    int x0 = (int)floor(x), y0 = (int)floor(y), z0 = (int)floor(z);
    int x1 = x0 + 1, y1 = y0 + 1, z1 = z0 + 1;
    if (x0 < 0) x0 = 0;
    if (y0 < 0) y0 = 0;
    if (z0 < 0) z0 = 0;
    if (x1 >= V.nx) x1 = V.nx - 1;
    if (y1 >= V.ny) y1 = V.ny - 1;
    if (z1 >= V.nz) z1 = V.nz - 1;
    // indices stay in range for inputs inside [-1,1]; clamp the upper side
    // too so that no input can address outside the grid
    if (x0 > V.nx - 1) x0 = V.nx - 1;
    if (y0 > V.ny - 1) y0 = V.ny - 1;
    if (z0 > V.nz - 1) z0 = V.nz - 1;
    double wx = dsub(x, (double)x0), wy = dsub(y, (double)y0), wz = dsub(z, (double)z0);
    long NXY = (long)V.nx * V.ny, NY = V.ny;
    long i000 = z0 * NXY + x0 * NY + y0, i001 = z1 * NXY + x0 * NY + y0;
    long i010 = z0 * NXY + x0 * NY + y1, i011 = z1 * NXY + x0 * NY + y1;
    long i100 = z0 * NXY + x1 * NY + y0, i101 = z1 * NXY + x1 * NY + y0;
    long i110 = z0 * NXY + x1 * NY + y1, i111 = z1 * NXY + x1 * NY + y1;
    double v000, v001, v010, v011, v100, v101, v110, v111;
    if (V.data64) {
        const double* r = V.data64;
        v000 = r[i000]; v001 = r[i001]; v010 = r[i010]; v011 = r[i011];
        v100 = r[i100]; v101 = r[i101]; v110 = r[i110]; v111 = r[i111];
    } else {
        const float* r = V.data;
        v000 = r[i000]; v001 = r[i001]; v010 = r[i010]; v011 = r[i011];
        v100 = r[i100]; v101 = r[i101]; v110 = r[i110]; v111 = r[i111];
    }
    double v00 = dadd(dmul(v000, dsub(1, wz)), dmul(v001, wz));
    double v01 = dadd(dmul(v010, dsub(1, wz)), dmul(v011, wz));
    double v10 = dadd(dmul(v100, dsub(1, wz)), dmul(v101, wz));
    double v11 = dadd(dmul(v110, dsub(1, wz)), dmul(v111, wz));
    double v0 = dadd(dmul(v00, dsub(1, wy)), dmul(v01, wy));
    double v1 = dadd(dmul(v10, dsub(1, wy)), dmul(v11, wy));
    return dadd(dmul(v0, dsub(1, wx)), dmul(v1, wx));
}

XRP_HD double leaf64(const SceneDev& S, int id, double x, double y, double z) {
    const double* d = S.nodes64[id].d;
    switch (S.nodes[id].type) {
    case N_SPHERE: return sphere64(d, x, y, z);
    case N_BOX: return box64(d, x, y, z);
    case N_CYL: return cyl64(d, x, y, z);
    case N_PPD: return ppd64(d, x, y, z);
    case N_GYROID: return gyroid64(d, x, y, z);
    default: return 0.0;
    }
}

template <int D>
XRP_HD double coll64(const SceneDev& S, int id, double x, double y, double z);

template <int D>
XRP_HD double item64(const SceneDev& S, int id, double x, double y, double z) {
    const Node& n = S.nodes[id];
    if (n.type <= N_GYROID) return leaf64(S, id, x, y, z);
    if (n.type == N_VOXEL) return voxel64(S.vols[n.a], x, y, z);
    if (n.type == N_TESS) {
        if constexpr (D > 0) {
            const double* t = S.nodes64[id].d;
            if (x < t[0] || x > t[1] || y < t[2] || y > t[3] || z < t[4] || z > t[5]) return 0.0;
            const double* u = &t[6];
            double dx = dsub(u[1], u[0]);
            x = dsub(x, dmul(dx, floor(ddiv(dsub(x, u[0]), dx))));
            double dy = dsub(u[3], u[2]);
            y = dsub(y, dmul(dy, floor(ddiv(dsub(y, u[2]), dy))));
            double dz = dsub(u[5], u[4]);
            z = dsub(z, dmul(dz, floor(ddiv(dsub(z, u[4]), dz))));
            if (x < u[0] || x > u[1] || y < u[2] || y > u[3] || z < u[4] || z > u[5]) return 0.0;
            return coll64<D - 1>(S, n.a, x, y, z);
        }
    }
    return 0.0;
}

template <int D>
XRP_HD double coll64(const SceneDev& S, int id, double x, double y, double z) {
    const Node& c = S.nodes[id];
    const int32_t* kids = S.child + c.a;
    const bool greedy = (c.flags & C_GREEDY) != 0;
    double density = 0.0;
    for (int k = 0; k < c.b; k++) {
        double rho = item64<D>(S, kids[k], x, y, z);
        if (greedy && rho > 0.0) return rho;
        density = dadd(density, rho);
    }
    if (c.flags & C_CLIP) {
        if (density < 0.0)
            density = 0.0;
        else if (density > 1.0)
            density = 1.0;
    }
    return density;
}

XRP_HD void deform64(const SceneDev& S, double& x, double& y, double& z) {
    for (int i = 0; i < S.ndefs; i++) {
        const DefStep& dd = S.defs[i];
        const double* a = dd.d;
        switch (dd.type) {
        case D_GAUSSIAN: {
            double x0 = dsub(x, a[6]), y0 = dsub(y, a[7]), z0 = dsub(z, a[8]);
            double r2 = dadd(dadd(dmul(x0, x0), dmul(y0, y0)), dmul(z0, z0));
            double dx = dmul(a[0], exp(ddiv(-r2, dmul(dmul(2.0, a[3]), a[3]))));
            double dy = dmul(a[1], exp(ddiv(-r2, dmul(dmul(2.0, a[4]), a[4]))));
            double dz = dmul(a[2], exp(ddiv(-r2, dmul(dmul(2.0, a[5]), a[5]))));
            x = dadd(x, dx); y = dadd(y, dy); z = dadd(z, dz);
            break;
        }
        case D_LINEAR: {
            double nx = dadd(dadd(dadd(x, dmul(a[0], x)), dmul(a[5], y)), dmul(a[4], z));
            double ny = dadd(dadd(dadd(y, dmul(a[5], x)), dmul(a[1], y)), dmul(a[3], z));
            double nz = dadd(dadd(dadd(z, dmul(a[4], x)), dmul(a[3], y)), dmul(a[2], z));
            x = nx; y = ny; z = nz;
            break;
        }
        case D_RIGID: x = dadd(x, a[0]); y = dadd(y, a[1]); z = dadd(z, a[2]); break;
        case D_SIGMOID: {
            double* p = dd.axis == 0 ? &x : (dd.axis == 1 ? &y : &z);
            double e = exp(ddiv(-dsub(*p, a[1]), a[2]));
            *p = dadd(*p, ddiv(a[0], dadd(1.0, e)));
            break;
        }
        case D_AFFINE: {
            double nx = dadd(dadd(dmul(a[0], x), dmul(a[1], y)), dmul(a[2], z));
            double ny = dadd(dadd(dmul(a[3], x), dmul(a[4], y)), dmul(a[5], z));
            double nz = dadd(dadd(dmul(a[6], x), dmul(a[7], y)), dmul(a[8], z));
            x = nx; y = ny; z = nz;
            break;
        }
        default: break;
        }
    }
}

// ---------------------------------------------------------------------------
// hybrid exact evaluation for uncertain samples
// ---------------------------------------------------------------------------
// The position pipeline (sample position, deformation, tessellation bounds
// and folds) runs in FP64 exactly as the reference does; each primitive is
// then first decided in FP32 at that FP64 point -- its guard band was sized
// for the much larger FP32 march error, so a certain FP32 decision equals the
// FP64 one -- and only primitives that stay undecided are evaluated in FP64.
// The value returned is the same as density64's, for a fraction of the FP64
// work (GB300 runs FP64 at a small fraction of its FP32 rate).

XRP_HD double leaf_rho64(const SceneDev& S, int id) {
    const double* d = S.nodes64[id].d;
    switch (S.nodes[id].type) {
    case N_SPHERE: return d[4];
    case N_BOX: return d[6];
    case N_CYL: return d[7];
    case N_PPD: return d[12];
    case N_GYROID: return d[5];
    default: return 0.0;
    }
}

// (xf, yf, zf): the point rounded to FP32, formed once per collection.
XRP_HD double leaf_hyb(const SceneDev& S, int id, double x, double y, double z, float xf, float yf, float zf) {
    float r = leaf32(S.nodes[id], xf, yf, zf);
    if (!isunc(r)) return r != 0.0f ? leaf_rho64(S, id) : 0.0;
    return leaf64(S, id, x, y, z);
}

XRP_HD double leaf_hyb(const SceneDev& S, int id, double x, double y, double z) {
    return leaf_hyb(S, id, x, y, z, (float)x, (float)y, (float)z);
}

template <int D>
XRP_HD double coll_hyb(const SceneDev& S, int id, double x, double y, double z);

// floor(a / b) as the reference forms it (the floor of the correctly rounded
// FP64 quotient), with ib32 = (float)(1 / b).  The FP32 quotient is within
// 3 * 2^-24 of a / b relatively ((float)a, ib32 and the product each round
// once), and the FP64 quotient within 2^-53, so when the FP32 value is more
// than 8 * 2^-24 |q| from an integer both floors agree; only then is the
// FP64 division (a long instruction sequence on GB300) skipped.
XRP_HD double floor_div64(double a, double b, float ib32) {
    const float qf = (float)a * ib32;
    const float err = fmaf(fabsf(qf), 8.0f * 5.9604645e-8f, 1e-30f);
    const float lo = floorf(qf - err), hi = floorf(qf + err);
    if (lo == hi) return (double)lo;
    return floor(ddiv(a, b));
}

template <int D>
XRP_HD double item_hyb(const SceneDev& S, int id, double x, double y, double z) {
    const Node& n = S.nodes[id];
    if (n.type <= N_GYROID) return leaf_hyb(S, id, x, y, z);
    if (n.type == N_VOXEL) return voxel64(S.vols[n.a], x, y, z);
    if (n.type == N_TESS) {
        if constexpr (D > 0) {
            const double* t = S.nodes64[id].d;
            if (x < t[0] || x > t[1] || y < t[2] || y > t[3] || z < t[4] || z > t[5]) return 0.0;
            const double* u = &t[6];
            const float* f = n.f;  // f[17..19]: (float)(1 / cell size) per axis
            double dx = dsub(u[1], u[0]);
            x = dsub(x, dmul(dx, floor_div64(dsub(x, u[0]), dx, f[17])));
            double dy = dsub(u[3], u[2]);
            y = dsub(y, dmul(dy, floor_div64(dsub(y, u[2]), dy, f[18])));
            double dz = dsub(u[5], u[4]);
            z = dsub(z, dmul(dz, floor_div64(dsub(z, u[4]), dz, f[19])));
            if (x < u[0] || x > u[1] || y < u[2] || y > u[3] || z < u[4] || z > u[5]) return 0.0;
            return coll_hyb<D - 1>(S, n.a, x, y, z);
        }
    }
    return 0.0;
}

// ObjectCollection.Density in FP64 over the candidate list of the point's
// cell (children outside it are exactly 0; order is kept, so greedy picks and
// FP64 sums equal the full loop's).
template <int D>
XRP_HD double coll_hyb(const SceneDev& S, int id, double x, double y, double z) {
    const Node& c = S.nodes[id];
    const int32_t* kids = S.child + c.a;
    int cnt = c.b;
    const int32_t* list = nullptr;
    const float xf = (float)x, yf = (float)y, zf = (float)z;
    if (c.flags & C_ACCEL) {
        int G = (c.flags >> 16) & 0xff;
        int ix = (int)floorf((xf - c.f[0]) * c.f[3]);
        int iy = (int)floorf((yf - c.f[1]) * c.f[4]);
        int iz = (int)floorf((zf - c.f[2]) * c.f[5]);
        ix = ix < 0 ? 0 : (ix >= G ? G - 1 : ix);
        iy = iy < 0 ? 0 : (iy >= G ? G - 1 : iy);
        iz = iz < 0 ? 0 : (iz >= G ? G - 1 : iz);
        const int32_t* off = S.cells + f2i(c.f[6]) + (iz * G + iy) * G + ix;
        list = S.items + off[0];
        cnt = off[1] - off[0];
    }
    const bool greedy = (c.flags & C_GREEDY) != 0;
    double density = 0.0;
    for (int k = 0; k < cnt; k++) {
        const int kid = list ? list[k] : kids[k];
        const double rho = S.nodes[kid].type <= N_GYROID ? leaf_hyb(S, kid, x, y, z, xf, yf, zf)
                                                         : item_hyb<D>(S, kid, x, y, z);
        if (greedy && rho > 0.0) return rho;
        density = dadd(density, rho);
    }
    if (c.flags & C_CLIP) {
        if (density < 0.0)
            density = 0.0;
        else if (density > 1.0)
            density = 1.0;
    }
    return density;
}

XRP_HD double density_hyb(const SceneDev& S, double x, double y, double z) {
    if (S.ndefs) deform64(S, x, y, z);
    if (S.nodes[S.root].type == N_COLL) return coll_hyb<kMaxDepth>(S, S.root, x, y, z);
    return item_hyb<kMaxDepth>(S, S.root, x, y, z);
}

// density() without the multiplier (main.go:137-140).
XRP_HD double density64(const SceneDev& S, double x, double y, double z) {
    if (S.ndefs) deform64(S, x, y, z);
    if (S.nodes[S.root].type == N_COLL) return coll64<kMaxDepth>(S, S.root, x, y, z);
    return item64<kMaxDepth>(S, S.root, x, y, z);
}

// ---------------------------------------------------------------------------
// per-ray setup and the two integrators
// ---------------------------------------------------------------------------

// FP64 ray exactly as the reference forms it (origin = eye, normalised
// direction), and its FP32 working copy: the point at s_c and the direction.
struct Ray64 {
    double o[3];
    double d[3];
};

struct Ray {
    float pc[3];   // float(o + d*s_c)
    float d32[3];  // float(d)
};

// main.go:457-465 and the Normalize() at main.go:145 / 160.
XRP_HD void setup_ray64(const ViewDev& V, const double* xs, int i, int j, Ray64& r) {
    double v0 = xs[i], v1 = xs[j], v2 = -V.f;
    const double* m = V.m;
    double t0 = dadd(dadd(dadd(dmul(m[0], v0), dmul(m[4], v1)), dmul(m[8], v2)), dmul(m[12], 1.0));
    double t1 = dadd(dadd(dadd(dmul(m[1], v0), dmul(m[5], v1)), dmul(m[9], v2)), dmul(m[13], 1.0));
    double t2 = dadd(dadd(dadd(dmul(m[2], v0), dmul(m[6], v1)), dmul(m[10], v2)), dmul(m[14], 1.0));
    double iw = V.inv_w;
    if (V.general_w) {
        double t3 = dadd(dadd(dadd(dmul(m[3], v0), dmul(m[7], v1)), dmul(m[11], v2)), dmul(m[15], 1.0));
        iw = drcp(t3);
    }
    double dx = dsub(dmul(t0, iw), V.eye[0]);
    double dy = dsub(dmul(t1, iw), V.eye[1]);
    double dz = dsub(dmul(t2, iw), V.eye[2]);
    double l = drcp(dsqrt(dadd(dadd(dmul(dx, dx), dmul(dy, dy)), dmul(dz, dz))));
    r.d[0] = dmul(dx, l);
    r.d[1] = dmul(dy, l);
    r.d[2] = dmul(dz, l);
    r.o[0] = V.eye[0];
    r.o[1] = V.eye[1];
    r.o[2] = V.eye[2];
}

// The ray of pixel (i, j) for the FP32 march: the direction to ~1e-13
// relative rather than in the reference's operation order.  An FP32
// reciprocal square root refined by one Newton step in FP64 replaces the
// FP64 square root and division (long instruction sequences on a GPU whose
// FP64 rate is a small fraction of FP32).  The positions it gives differ
// from the reference's by under 1e-12, inside the absolute term of the
// FP32 position error bound; the FP64 re-evaluation of undecided samples
// keeps setup_ray64.
XRP_HD void setup_ray64_fast(const ViewDev& V, const double* xs, int i, int j, Ray64& r) {
    const double v0 = xs[i], v1 = xs[j], v2 = -V.f;
    const double* m = V.m;
    const double t0 = fma(m[8], v2, fma(m[4], v1, fma(m[0], v0, m[12])));
    const double t1 = fma(m[9], v2, fma(m[5], v1, fma(m[1], v0, m[13])));
    const double t2 = fma(m[10], v2, fma(m[6], v1, fma(m[2], v0, m[14])));
    double iw = V.inv_w;
    if (V.general_w) iw = 1.0 / fma(m[11], v2, fma(m[7], v1, fma(m[3], v0, m[15])));
    const double dx = fma(t0, iw, -V.eye[0]);
    const double dy = fma(t1, iw, -V.eye[1]);
    const double dz = fma(t2, iw, -V.eye[2]);
    const double dd = fma(dz, dz, fma(dy, dy, dx * dx));
#if defined(__CUDA_ARCH__)
    double y = (double)rsqrtf((float)dd);
#else
    double y = (double)(1.0f / sqrtf((float)dd));
#endif
    y = y * fma(-0.5 * dd * y, y, 1.5);  // Newton: relative error ~1.5 e0^2
    r.d[0] = dx * y;
    r.d[1] = dy * y;
    r.d[2] = dz * y;
    r.o[0] = V.eye[0];
    r.o[1] = V.eye[1];
    r.o[2] = V.eye[2];
}

XRP_HD void setup_ray32(const Ray64& r64, double s_c, Ray& r) {
    for (int a = 0; a < 3; a++) {
        r.pc[a] = (float)fma(r64.d[a], s_c, r64.o[a]);
        r.d32[a] = (float)r64.d[a];
    }
}

// Double-float arithmetic (a value is hi + lo, |lo| <= ulp(hi)/2): products
// by FMA (exact error of a*b), sums by the two-sum.  About 44 significant
// bits, from FP32 instructions only; the rounded-to-nearest forms keep the
// device compiler from contracting the error terms.
struct DF {
    float hi, lo;
};

#if defined(__CUDA_ARCH__)
XRP_HD float df_rn_add(float a, float b) { return __fadd_rn(a, b); }
XRP_HD float df_rn_sub(float a, float b) { return __fsub_rn(a, b); }
XRP_HD float df_rn_mul(float a, float b) { return __fmul_rn(a, b); }
#else
XRP_HD float df_rn_add(float a, float b) { return a + b; }
XRP_HD float df_rn_sub(float a, float b) { return a - b; }
XRP_HD float df_rn_mul(float a, float b) { return a * b; }
#endif

XRP_HD DF df_norm(float s, float e) {  // |s| >= |e|
    const float r = df_rn_add(s, e);
    return {r, df_rn_sub(e, df_rn_sub(r, s))};
}

XRP_HD DF df_add(DF a, DF b) {
    const float s = df_rn_add(a.hi, b.hi);
    const float v = df_rn_sub(s, a.hi);
    float e = df_rn_add(df_rn_sub(a.hi, df_rn_sub(s, v)), df_rn_sub(b.hi, v));
    e = df_rn_add(e, df_rn_add(a.lo, b.lo));
    return df_norm(s, e);
}

XRP_HD DF df_mul(DF a, DF b) {
    const float p = df_rn_mul(a.hi, b.hi);
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, e));
    return df_norm(p, e);
}

// The ray of pixel (i, j) for the FP32 march without FP64 instructions
// (general_w == 0): the direction c0 x_i + c1 x_j + k (camera folded on the
// host), normalised by a reciprocal square root refined by one Newton step,
// all in double-float; then float(d) and float(o + d s_c).  Agrees with
// setup_ray64_fast + setup_ray32 up to ~1e-13 relative before the final
// rounding to FP32.
XRP_HD void setup_ray32_df(const ViewDev& V, const float* xsf, int i, int j, const float* s_c2, Ray& r) {
    const DF xi = {xsf[2 * i], xsf[2 * i + 1]}, xj = {xsf[2 * j], xsf[2 * j + 1]};
    DF d[3];
    for (int a = 0; a < 3; a++)
        d[a] = df_add(df_add(df_mul({V.c0[2 * a], V.c0[2 * a + 1]}, xi), df_mul({V.c1[2 * a], V.c1[2 * a + 1]}, xj)),
                      {V.k[2 * a], V.k[2 * a + 1]});
    const DF dd = df_add(df_add(df_mul(d[0], d[0]), df_mul(d[1], d[1])), df_mul(d[2], d[2]));
    // y0 ~ 1/sqrt(dd) to ~2^-22; y1 = y0 + y0 (1 - dd y0^2) / 2
    const float y0 = 1.0f / sqrtf(dd.hi);
    const DF y2 = df_norm(df_rn_mul(y0, y0), fmaf(y0, y0, -df_rn_mul(y0, y0)));
    const DF q = df_mul(dd, y2);  // ~1
    const float rres = df_rn_add(df_rn_sub(1.0f, q.hi), -q.lo);
    const DF y = df_norm(y0, df_rn_mul(df_rn_mul(0.5f, y0), rres));
    const DF sc = {s_c2[0], s_c2[1]};
    for (int a = 0; a < 3; a++) {
        const DF dn = df_mul(d[a], y);
        r.d32[a] = dn.hi;
        r.pc[a] = df_add({V.eye2[2 * a], V.eye2[2 * a + 1]}, df_mul(dn, sc)).hi;
    }
}

// The FP32 march's ray of pixel (i, j): FP32 instructions only for cameras
// without a per-pixel w, else the FP64 setup.
XRP_HD void setup_ray_march(const ViewDev& V, const RenderParams& P, const Lattice& L, int i, int j, Ray& r) {
    if (!V.general_w) {
        setup_ray32_df(V, P.xsf, i, j, L.s_c2, r);
        return;
    }
    Ray64 r64;
    setup_ray64_fast(V, P.xs, i, j, r64);
    setup_ray32(r64, L.s_c, r);
}

// FP64 density of sample s of pixel (i, j), positions formed exactly as the
// reference does (main.go:148-150).  The ray is recomputed here so that the
// FP32 march keeps no FP64 state live.
XRP_HD double sample64_pixel_inl(const SceneDev& S, const ViewDev& V, const double* xs, int i,
                                 int j, double s) {
    Ray64 r;
    setup_ray64(V, xs, i, j, r);
    double x = dadd(r.o[0], dmul(r.d[0], s));
    double y = dadd(r.o[1], dmul(r.d[1], s));
    double z = dadd(r.o[2], dmul(r.d[2], s));
    return density_hyb(S, x, y, z);
}

XRP_HDN double sample64_pixel(const SceneDev& S, const ViewDev& V, const double* xs, int i, int j,
                              double s) {
    return sample64_pixel_inl(S, V, xs, i, j, s);
}

// The pixel a sampler works for, for the FP64 re-evaluation.
struct PixelRef {
    const ViewDev* V;
    const double* xs;
    int i, j;
};

// Parameter interval [t0, t1] (offsets from s_c) where the ray is inside the
// dilated support box; t0 > t1 when it misses.
XRP_HD void clip_ray(const float* lo, const float* hi, const Ray& r, float& t0, float& t1) {
    t0 = -3.0e38f;
    t1 = 3.0e38f;
    for (int a = 0; a < 3; a++) {
        float dd = r.d32[a];
        float p = r.pc[a];
        if (dd != 0.0f) {
            float inv = 1.0f / dd;
            float ta = (lo[a] - p) * inv, tb = (hi[a] - p) * inv;
            t0 = fmaxf(t0, fminf(ta, tb));
            t1 = fminf(t1, fmaxf(ta, tb));
        } else if (p < lo[a] || p > hi[a]) {
            t0 = 1.0f;
            t1 = -1.0f;
        }
    }
}

struct KahanF {
    float s = 0.0f, c = 0.0f;
    XRP_HD void add(float v) {
        float y = v - c;
        float t = s + y;
        c = (t - s) - y;
        s = t;
    }
};

// Index range [k0, k1] of lattice samples that may lie inside the support.
XRP_HD bool sample_range(const Lattice& L, float t0, float t1, int K, int& k0, int& k1) {
    if (!(t0 <= t1)) return false;
    float a = (t0 - L.t_first) * L.inv_ds;
    float b = (t1 - L.t_first) * L.inv_ds;
    a = fmaxf(a, -4.0f);
    b = fminf(b, (float)K + 4.0f);
    k0 = (int)floorf(a) - 2;
    k1 = (int)ceilf(b) + 2;
    if (k0 < 0) k0 = 0;
    if (k1 > K - 1) k1 = K - 1;
    return k0 <= k1;
}

struct RayStats {
    uint32_t samples;
    uint32_t fallbacks;
};

// Samplers: density at lattice offset t (FP32, NaN when uncertain) and the
// exact FP64 density at reference position s.
template <int DEPTH, bool DEFS>
struct SceneSampler {
    const SceneDev& S;
    const Ray& r;
    PixelRef px;
    static constexpr bool kHasInner = false;
    XRP_HD float f32(float t) const {
        float x = fmaf(r.d32[0], t, r.pc[0]);
        float y = fmaf(r.d32[1], t, r.pc[1]);
        float z = fmaf(r.d32[2], t, r.pc[2]);
        return density32<DEPTH, DEFS>(S, x, y, z);
    }
    XRP_HD float f32_inner(float t) const { return f32(t); }
    XRP_HD double f64(double s) const { return sample64_pixel(S, *px.V, px.xs, px.i, px.j, s); }
    XRP_HD double f64_inline(double s) const {
        return sample64_pixel_inl(S, *px.V, px.xs, px.i, px.j, s);
    }
};

// A scene whose root is a voxel grid (no deformation): samples are formed
// directly in grid coordinates u = (p + 1) * (N - 1) / 2.
struct VolRay {
    float uc[3];  // float((p_c + 1) * scale)
    float du[3];  // float(d * scale)
};

XRP_HD void setup_volray(const Volume& V, const Ray64& r, double s_c, VolRay& vr) {
    for (int a = 0; a < 3; a++) {
        double sc = (double)V.scale[a];
        vr.uc[a] = (float)((fma(r.d[a], s_c, r.o[a]) + 1.0) * sc);
        vr.du[a] = (float)(r.d[a] * sc);
    }
}

// Trilinear interpolation of the 8 taps (objects.go:847-854), FP32.
XRP_HD float trilerp(float wx, float wy, float wz, float v000, float v001, float v010, float v011,
                     float v100, float v101, float v110, float v111) {
    float v00 = fmaf(wz, v001 - v000, v000);
    float v01 = fmaf(wz, v011 - v010, v010);
    float v10 = fmaf(wz, v101 - v100, v100);
    float v11 = fmaf(wz, v111 - v110, v110);
    float v0 = fmaf(wy, v01 - v00, v00);
    float v1 = fmaf(wy, v11 - v10, v10);
    return fmaf(wx, v1 - v0, v0);
}

// VoxelGrid.Density in grid coordinates, all dimensions >= 2, for a point
// known to lie inside [-1,1]^3 with margin (no bounds test).
XRP_HD float vol32_inner(const Volume& V, float band_zero, int zero_guard, float ux, float uy,
                         float uz) {
    float fx = floorf(ux), fy = floorf(uy), fz = floorf(uz);
    int x0 = (int)fx, y0 = (int)fy, z0 = (int)fz;
    x0 = x0 > V.nx - 2 ? V.nx - 2 : (x0 < 0 ? 0 : x0);
    y0 = y0 > V.ny - 2 ? V.ny - 2 : (y0 < 0 ? 0 : y0);
    z0 = z0 > V.nz - 2 ? V.nz - 2 : (z0 < 0 ? 0 : z0);
    float wx = ux - (float)x0, wy = uy - (float)y0, wz = uz - (float)z0;
    long NY = V.ny, NXY = (long)V.nx * V.ny;
    const float* p0 = V.data + z0 * NXY + x0 * NY + y0;
    const float* p1 = p0 + NXY;
#if defined(__CUDA_ARCH__)
    float v000 = __ldg(p0), v010 = __ldg(p0 + 1), v100 = __ldg(p0 + NY), v110 = __ldg(p0 + NY + 1);
    float v001 = __ldg(p1), v011 = __ldg(p1 + 1), v101 = __ldg(p1 + NY), v111 = __ldg(p1 + NY + 1);
#else
    float v000 = p0[0], v010 = p0[1], v100 = p0[NY], v110 = p0[NY + 1];
    float v001 = p1[0], v011 = p1[1], v101 = p1[NY], v111 = p1[NY + 1];
#endif
    float v = trilerp(wx, wy, wz, v000, v001, v010, v011, v100, v101, v110, v111);
    if (zero_guard) {
        float amax = fmaxf(fmaxf(fmaxf(fabsf(v000), fabsf(v001)), fmaxf(fabsf(v010), fabsf(v011))),
                           fmaxf(fmaxf(fabsf(v100), fabsf(v101)), fmaxf(fabsf(v110), fabsf(v111))));
        if (amax > 0.0f && fabsf(v) <= band_zero * amax) return xnan();
    }
    return v;
}

// World-space margin of grid point u to the inclusive [-1, 1]^3 bounds
// compared with the guard band: 0 outside, 1 inside, 2 uncertain.
XRP_HD int vol_bounds(const Volume& V, const float* inv_scale, float ux, float uy, float uz) {
    float mx = fminf(ux, (float)(V.nx - 1) - ux) * inv_scale[0];
    float my = fminf(uy, (float)(V.ny - 1) - uy) * inv_scale[1];
    float mz = fminf(uz, (float)(V.nz - 1) - uz) * inv_scale[2];
    float m = fminf(mx, fminf(my, mz));
    if (m < -V.band_w) return 0;
    if (m > V.band_w) return 1;
    return 2;
}

// VoxelGrid.Density in grid coordinates; all dimensions >= 2.
XRP_HD float vol32(const Volume& V, const float* inv_scale, float band_zero, int zero_guard,
                   float ux, float uy, float uz) {
    int b = vol_bounds(V, inv_scale, ux, uy, uz);
    if (b == 0) return 0.0f;
    if (b == 2) return xnan();
    return vol32_inner(V, band_zero, zero_guard, ux, uy, uz);
}

struct VolumeSampler {
    const SceneDev& S;
    const Volume& V;
    const VolRay& vr;
    PixelRef px;
    float inv_scale[3];
    float band_zero;
    static constexpr bool kHasInner = true;
    XRP_HD float f32(float t) const {
        return vol32(V, inv_scale, band_zero, S.hier_zero_guard, fmaf(vr.du[0], t, vr.uc[0]),
                     fmaf(vr.du[1], t, vr.uc[1]), fmaf(vr.du[2], t, vr.uc[2]));
    }
    XRP_HD float f32_inner(float t) const {
        return vol32_inner(V, band_zero, S.hier_zero_guard, fmaf(vr.du[0], t, vr.uc[0]),
                           fmaf(vr.du[1], t, vr.uc[1]), fmaf(vr.du[2], t, vr.uc[2]));
    }
    XRP_HD double f64(double s) const { return sample64_pixel(S, *px.V, px.xs, px.i, px.j, s); }
    XRP_HD double f64_inline(double s) const {
        return sample64_pixel_inl(S, *px.V, px.xs, px.i, px.j, s);
    }
};

// Sample range [a, b] that lies inside the box [lo+m, hi-m] (m > guard band
// plus the FP32 error of the clip itself): there the bounds test of the
// sampler always passes and is skipped.  Empty (a > b) when there is none.
XRP_HD void inner_range(const Lattice& L, const Ray& r, const float* lo, const float* hi, float m,
                        int k0, int k1, int& a, int& b) {
    float ilo[3] = {lo[0] + m, lo[1] + m, lo[2] + m};
    float ihi[3] = {hi[0] - m, hi[1] - m, hi[2] - m};
    float t0, t1;
    clip_ray(ilo, ihi, r, t0, t1);
    a = k1 + 1;
    b = k1;
    if (!(t0 < t1)) return;
    float fa = (t0 - L.t_first) * L.inv_ds, fb = (t1 - L.t_first) * L.inv_ds;
    fa = fmaxf(fa, (float)k0 - 4.0f);
    fb = fminf(fb, (float)k1 + 4.0f);
    a = (int)ceilf(fa) + 2;
    b = (int)floorf(fb) - 2;
    if (a < k0) a = k0;
    if (b > k1) b = k1;
}

// integrate_along_ray (main.go:144-154): returns the sum of densities over
// the lattice samples (pre-multiplier, pre-ds).
//
// Uncertain samples are not re-evaluated inside the loop: their indices go to
// a six-entry register buffer and the FP64 evaluation runs after the loop.
// A call site inside the loop would hold every loop value across a call and
// push the kernel into spills.  In the rare ray with more than six uncertain
// samples the march is repeated in FP32 to find the rest.  The sum's order
// changes, not its terms (Kahan-compensated either way).
struct Deferred {
    int n = 0;
    int b0 = 0, b1 = 0, b2 = 0, b3 = 0, b4 = 0, b5 = 0;
    XRP_HD void push(int k) {
        if (n == 0) b0 = k;
        else if (n == 1) b1 = k;
        else if (n == 2) b2 = k;
        else if (n == 3) b3 = k;
        else if (n == 4) b4 = k;
        else if (n == 5) b5 = k;
        n++;
    }
    XRP_HD int get(int q) const {
        return q == 0 ? b0 : q == 1 ? b1 : q == 2 ? b2 : q == 3 ? b3 : q == 4 ? b4 : b5;
    }
    static constexpr int kCap = 6;
};

template <class Sampler, bool INNER>
XRP_HD void march_range(const Lattice& L, const Sampler& smp, int k0, int k1, KahanF& acc,
                        Deferred& dq) {
    for (int k = k0; k <= k1; k++) {
        float t = lattice_t(L, k);
        float rho = INNER ? smp.f32_inner(t) : smp.f32(t);
        if (isunc(rho)) {
            dq.push(k);
            rho = 0.0f;
        }
        acc.add(rho);
    }
}

template <class Sampler>
XRP_HD float march_simple(const Lattice& L, const float* lo, const float* hi, const Ray& r,
                          const Sampler& smp, RayStats& st, float inner_margin = 0.0f) {
    float t0, t1;
    clip_ray(lo, hi, r, t0, t1);
    int k0, k1;
    KahanF acc;
    if (!sample_range(L, t0, t1, L.K, k0, k1)) return 0.0f;
    st.samples += (uint32_t)(k1 - k0 + 1);
    Deferred dq;
    int a = k1 + 1, b = k1;
    if constexpr (Sampler::kHasInner) inner_range(L, r, lo, hi, inner_margin, k0, k1, a, b);
    if (a <= b) {
        march_range<Sampler, false>(L, smp, k0, a - 1, acc, dq);
        march_range<Sampler, true>(L, smp, a, b, acc, dq);
        march_range<Sampler, false>(L, smp, b + 1, k1, acc, dq);
    } else {
        march_range<Sampler, false>(L, smp, k0, k1, acc, dq);
    }
    if (dq.n) {
        // FP64 for the buffered samples; when more than kCap were uncertain,
        // refill the buffer by scanning on from the last one evaluated (the
        // FP32 decisions repeat exactly, so the same samples are found)
        const int total = dq.n;
        st.fallbacks += (uint32_t)total;
        int done = 0;
        for (;;) {
            int nb = dq.n < Deferred::kCap ? dq.n : Deferred::kCap;
            for (int q = 0; q < nb; q++) acc.add((float)smp.f64_inline(L.s64[dq.get(q)]));
            done += nb;
            if (done >= total || nb == 0) break;
            int from = dq.get(nb - 1) + 1;
            dq.n = 0;
            for (int k = from; k <= k1 && dq.n < Deferred::kCap; k++) {
                float t = lattice_t(L, k);
                float rho = (k >= a && k <= b) ? smp.f32_inner(t) : smp.f32(t);
                if (isunc(rho)) dq.push(k);
            }
        }
    }
    return acc.s;
}

// integrate_hierarchical (main.go:159-199): returns sum(w*rho) with w in
// {DS, DS/10} (pre-multiplier).
template <class Sampler>
XRP_HD float march_hier(const Lattice& L, const float* lo, const float* hi, const Ray& r,
                        const Sampler& smp, RayStats& st) {
    float t0, t1;
    clip_ray(lo, hi, r, t0, t1);
    int k0, k1;
    KahanF acc;
    if (!sample_range(L, t0, t1, L.K, k0, k1)) return 0.0f;
    bool prev_zero = true;  // coarse samples before k0 are outside the support
    // One sample per iteration: a coarse sample that flips queues its
    // interval's fine samples m..me-1 (rho_c: its density), evaluated by the
    // next iterations, so lanes that flip at different coarse indices do not
    // serialise the warp on a nested loop.  Same terms, same order.
    int k = k0, m = 0, me = 0;
    float rho_c = 0.0f;
    while (k <= k1) {
        const bool fine = m < me;
        float rho = smp.f32(fine ? L.ft32[m] : lattice_t(L, k));
        if (isunc(rho)) {
            rho = (float)smp.f64(fine ? L.f64[m] : L.s64[k]);
            st.fallbacks++;
        }
        st.samples++;
        if (fine) {
            acc.add(rho * L.dsf32);
            if (++m < me) continue;
            acc.add(rho_c * L.dsf32);
            k++;
            continue;
        }
        const bool zero = (rho == 0.0f);
        if (zero != prev_zero) {
            prev_zero = zero;
            m = L.fstart[k];
            me = L.fstart[k + 1];
            if (m < me) {
                rho_c = rho;
                continue;
            }
            acc.add(rho * L.dsf32);
        } else {
            acc.add(rho * L.ds32);
        }
        k++;
    }
    return acc.s;
}

// One step of certificate tracing at lattice sample k (k <= k1): evaluates
// the density and its certificate there, adds the covered samples' terms to
// `acc` and advances k past them.  u: the ray's object-space direction (RAY).
template <int DEPTH, bool DEFS, bool RAY, bool CURVE = false, int LM = kLeafAll, class Unc>
XRP_HD void trace_step(const SceneDev& S, const Lattice& L, const Ray& ray, const RayDir& u, int& k, int k1,
                       float step, float istep, Unc&& unc, KahanF& acc, unsigned& evals) {
    const float tk = lattice_t(L, k);
    const float x = fmaf(ray.d32[0], tk, ray.pc[0]);
    const float y = fmaf(ray.d32[1], tk, ray.pc[1]);
    const float z = fmaf(ray.d32[2], tk, ray.pc[2]);
    float m;
    float rho;
    if constexpr (RAY) rho = dens_ray32<DEPTH, DEFS>(S, x, y, z, u, (float)(k1 - k + 1) * step, m);
    else if constexpr (CURVE) rho = dens_curve32<DEPTH, DEFS, LM>(S, x, y, z, ray.d32, m);
    else rho = dens_margin32<DEPTH, DEFS>(S, x, y, z, m);
    evals++;
    if (isunc(rho)) {
        acc.add(unc(k));
        k++;
        return;
    }
    const int jmp = (int)fminf(floorf(m * istep), (float)(k1 - k));
    acc.add(rho * (float)(jmp + 1));
    k += jmp + 1;
}

// Certificate tracing of one ray over lattice samples [k0, k1]: at sample k
// the density and the certificate radius m (dens_margin32); the samples
// k..k+j with j*ds <= m lie inside the ball around sample k, so they share
// its density and are counted at once.  With RAY (affine chains) m is the
// ray bound of dens_ray32 instead: the samples k..k+j with j*ds <= m lie on
// the certified segment.  `unc(k)` returns the value of a
// sample FP32 cannot decide (its FP64 density, or 0 when the caller
// re-evaluates it later).  Returns the Kahan-compensated sum of densities,
// the same terms as march_simple.  With CURVE (smooth non-affine chains)
// m is the curve bound of dens_curve32, compiled for the leaf types LM.
template <int DEPTH, bool DEFS, bool RAY, bool CURVE = false, int LM = kLeafAll, class Unc>
XRP_HD float trace_sum(const SceneDev& S, const Lattice& L, const Ray& ray, int k0, int k1, Unc&& unc,
                       unsigned& evals) {
    KahanF acc;
    const float step = L.ds32 * 1.00001f;  // world distance between samples, rounded up
    const float istep = (1.0f / step) * 0.999999f;  // rounded down
    RayDir u;
    if constexpr (RAY) u = ray_dir32(S, ray.d32);
    int k = k0;
    while (k <= k1) trace_step<DEPTH, DEFS, RAY, CURVE, LM>(S, L, ray, u, k, k1, step, istep, unc, acc, evals);
    return acc.s - acc.c;
}

// The plain integrator's sum over lattice samples [k0, k1] (main.go:144-154)
// without certificates: every sample is evaluated in FP32; `unc(k)` gives
// the value of a sample FP32 cannot decide (0 when it goes to the FP64
// list).  The loop holds no FP64 state, so it stays in registers.
template <int DEPTH, bool DEFS, class Unc>
XRP_HD float plain_sum(const SceneDev& S, const Lattice& L, const Ray& ray, int k0, int k1, Unc&& unc,
                       unsigned& evals) {
    KahanF acc;
    for (int k = k0; k <= k1; k++) {
        const float tk = lattice_t(L, k);
        float rho = density32<DEPTH, DEFS>(S, fmaf(ray.d32[0], tk, ray.pc[0]), fmaf(ray.d32[1], tk, ray.pc[1]),
                                           fmaf(ray.d32[2], tk, ray.pc[2]));
        if (isunc(rho)) rho = unc(k);
        acc.add(rho);
    }
    evals += (unsigned)(k1 - k0 + 1);
    return acc.s - acc.c;
}

// Certificate tracing of the hierarchical integrator (main.go:159-199):
// coarse samples k0..k1 (right ends, spacing DS).  A coarse sample whose
// zero-ness differs from its predecessor's is refined over its fine samples
// as march_hier does, each fine sample's ray or ball certificate covering
// the fine samples after it that lie within its radius; the coarse samples a
// certificate covers share the evaluated density, so none of them flips and
// each adds rho*DS.
// `unc(index, fine)` gives the value of an undecided coarse (fine = false,
// index into s64) or fine (fine = true, index into f64) sample.  Returns
// sum(w * rho) with w in {DS, DS/10}.  PLAIN: no certificates (every coarse
// sample evaluated), the plain hierarchical integrator.
// Tried and dropped: leaving an undecided coarse sample to the FP64 pass
// (refining the intervals on both sides of it whatever its zero-ness, and
// choosing the terms there) instead of re-evaluating it in place: the extra
// loop state spilled and grew the kernel (lattice 64.7 -> 61.0 Mrays/s,
// gyroid 364 -> 185).
// Merging the in-place FP64 re-evaluations of the hierarchical march
// (MERGE): a lane whose coarse sample FP32 cannot decide waits, and the
// warp's waiting lanes are served together, in one call, once
// XRP_MERGE_LANES of them wait, no other lane is still marching, or the
// first has waited XRP_MERGE_WAIT iterations.  On GB300 a warp's FP64
// instruction holds the narrow FP64 pipe however few lanes execute it, so
// one call for several lanes costs about what one call for one lane does.
#ifndef XRP_MERGE_LANES
#define XRP_MERGE_LANES 4
#endif
#ifndef XRP_MERGE_WAIT
#define XRP_MERGE_WAIT 32
#endif

template <int DEPTH, bool DEFS, bool RAY, bool CURVE = false, int LM = kLeafAll, bool PLAIN = false,
          bool MERGE = false, class Unc>
XRP_HD float trace_sum_hier(const SceneDev& S, const Lattice& L, const Ray& ray, int k0, int k1, Unc&& unc,
                            unsigned& evals, unsigned wmask = 0u) {
    KahanF acc;
    const float step = L.ds32 * 1.00001f;
    const float istep = (1.0f / step) * 0.999999f;  // rounded down
    const float stepf = L.dsf32 * 1.00001f;          // the fine samples' spacing, rounded up
    const float istepf = (1.0f / stepf) * 0.999999f;
    RayDir u;
    if constexpr (RAY) u = ray_dir32(S, ray.d32);
    bool prev_zero = true;  // coarse samples before k0 are outside the support
    int k = k0;
    // One sample per iteration, coarse or fine: a coarse sample that flips
    // queues its interval's fine samples q..qe-1, which the next iterations
    // evaluate before the march moves on (rho_c, jmp_c: the coarse sample's
    // density and jump).  Nested, the fine loop ran once per lane that
    // flipped at a given coarse index, serialising the warp.
    int q = 0, qe = 0;
    float rho_c = 0.0f;
    int jmp_c = 0;
    bool pend = false;  // MERGE: coarse sample k waits for its FP64 value
    int waited = 0;     // MERGE: iterations the warp's waiting lanes have waited
    (void)wmask;
    (void)waited;
    for (;;) {
        bool serve = false;
#if defined(__CUDA_ARCH__)
        if constexpr (MERGE) {
            if (!__any_sync(wmask, k <= k1)) break;
            const unsigned pm = __ballot_sync(wmask, pend);
            if (pm) {
                const unsigned busy = __ballot_sync(wmask, k <= k1 && !pend);
                serve = __popc(pm) >= XRP_MERGE_LANES || busy == 0u || ++waited >= XRP_MERGE_WAIT;
                if (serve) waited = 0;
            }
            if (k > k1) continue;
        } else
#endif
        if (k > k1) {
            break;
        }
        float rho, m = 0.0f;
        bool certified = true;  // rho came with a certificate radius m
        if (MERGE && pend) {
            if (!serve) continue;
            pend = false;
            rho = unc(k, false);  // every waiting lane of the warp at once
            certified = false;
        } else {
            const bool fine = q < qe;
            const float tk = fine ? L.ft32[q] : lattice_t(L, k);
            const float x = fmaf(ray.d32[0], tk, ray.pc[0]);
            const float y = fmaf(ray.d32[1], tk, ray.pc[1]);
            const float z = fmaf(ray.d32[2], tk, ray.pc[2]);
            // fine samples go through the certificate evaluation too: one call
            // site per iteration (with a plain evaluation for them, a warp whose
            // lanes mix coarse and fine samples ran both every iteration:
            // hierarchical lattice 53.8 against 64.7 Mrays/s, gyroid 342 against
            // 364), and with ray and ball certificates their radius skips the
            // fine samples it covers.
            if constexpr (PLAIN) rho = density32<DEPTH, DEFS>(S, x, y, z);
            else if constexpr (RAY)
                rho = dens_ray32<DEPTH, DEFS>(S, x, y, z, u, fine ? (float)(qe - q) * stepf : (float)(k1 - k + 1) * step,
                                              m);
            else if constexpr (CURVE) rho = dens_curve32<DEPTH, DEFS, LM>(S, x, y, z, ray.d32, m);
            else rho = dens_margin32<DEPTH, DEFS>(S, x, y, z, m);
            evals++;
            if (fine) {
                // the fine samples its certificate covers share its density (not
                // with curve certificates: there the skips ran slower, gyroid
                // 346 -> 319 Mrays/s, while the ball and ray certificates gained:
                // lattice 66.6 -> 77.6, cube 837 -> 917)
                int jf = 0;
                if (isunc(rho)) rho = unc(q, true);
                else if constexpr (!PLAIN && !CURVE) jf = (int)fminf(floorf(m * istepf), (float)(qe - 1 - q));
                acc.add(rho * L.dsf32 * (float)(jf + 1));
                q += jf + 1;
                if (q < qe) continue;
                // interval refined: the coarse sample's own term and its jump
                acc.add(rho_c * L.dsf32);
                if (jmp_c > 0) acc.add(rho_c * L.ds32 * (float)jmp_c);
                k += jmp_c + 1;
                continue;
            }
            if (isunc(rho)) {
                if constexpr (MERGE) {
                    pend = true;
                    continue;
                }
                rho = unc(k, false);
                certified = false;
            }
        }
        int jmp = 0;
        if constexpr (!PLAIN)
            if (certified) jmp = (int)fminf(floorf(m * istep), (float)(k1 - k));
        const bool zero = (rho == 0.0f);
        if (zero != prev_zero) {
            prev_zero = zero;
            q = L.fstart[k];
            qe = L.fstart[k + 1];
            if (q < qe) {
                rho_c = rho;
                jmp_c = jmp;
                continue;
            }
            acc.add(rho * L.dsf32);
        } else {
            acc.add(rho * L.ds32);
        }
        if (jmp > 0) acc.add(rho * L.ds32 * (float)jmp);
        k += jmp + 1;
    }
    return acc.s - acc.c;
}

#if defined(__CUDA_ARCH__)
// trace_sum with the warp's FP64 re-evaluations served together, as the
// hierarchical march's MERGE does (XRP_MERGE_LANES, XRP_MERGE_WAIT): a lane
// holds one undecided sample back and marches on, and a lane that meets a
// second one waits until the held one is served.  The held value joins the
// sum when served, so the terms are added in another order.  `wmask`: the
// lanes calling.
template <int DEPTH, bool DEFS, bool RAY, bool CURVE = false, int LM = kLeafAll, class Unc>
__device__ __forceinline__ float trace_sum_merged(const SceneDev& S, const Lattice& L, const Ray& ray, int k0,
                                                  int k1, Unc&& unc, unsigned& evals, unsigned wmask) {
    KahanF acc;
    const float step = L.ds32 * 1.00001f;
    const float istep = (1.0f / step) * 0.999999f;
    RayDir u;
    if constexpr (RAY) u = ray_dir32(S, ray.d32);
    int k = k0, held = -1, waited = 0;
    bool stalled = false;
    for (;;) {
        const unsigned pm = __ballot_sync(wmask, held >= 0);
        if (pm == 0u && !__any_sync(wmask, k <= k1)) break;
        if (pm) {
            const unsigned busy = __ballot_sync(wmask, k <= k1 && !stalled);
            if (__popc(pm) >= XRP_MERGE_LANES || busy == 0u || ++waited >= XRP_MERGE_WAIT) {
                waited = 0;
                if (held >= 0) {
                    acc.add(unc(held));  // every holding lane of the warp at once
                    held = -1;
                    stalled = false;
                }
            }
        }
        if (k > k1 || stalled) continue;
        const float tk = lattice_t(L, k);
        const float x = fmaf(ray.d32[0], tk, ray.pc[0]);
        const float y = fmaf(ray.d32[1], tk, ray.pc[1]);
        const float z = fmaf(ray.d32[2], tk, ray.pc[2]);
        float m;
        float rho;
        if constexpr (RAY) rho = dens_ray32<DEPTH, DEFS>(S, x, y, z, u, (float)(k1 - k + 1) * step, m);
        else if constexpr (CURVE) rho = dens_curve32<DEPTH, DEFS, LM>(S, x, y, z, ray.d32, m);
        else rho = dens_margin32<DEPTH, DEFS>(S, x, y, z, m);
        if (isunc(rho)) {
            if (held < 0) {
                held = k;
                k++;
                evals++;
            } else {
                stalled = true;  // evaluated again once the held sample is served
            }
            continue;
        }
        evals++;
        const int jmp = (int)fminf(floorf(m * istep), (float)(k1 - k));
        acc.add(rho * (float)(jmp + 1));
        k += jmp + 1;
    }
    return acc.s - acc.c;
}
#endif

// One pixel by certificate tracing, FP64 for undecided samples in place.
// MERGE (device): the warp's re-evaluations served together
// (trace_sum_merged, trace_sum_hier's MERGE); `wmask`: the lanes calling.
template <bool HIER, int DEPTH, bool DEFS, bool RAY, bool CURVE = false, bool MERGE = false>
XRP_HD float trace_pixel(const SceneDev& S, const Lattice& L, const RenderParams& P, const ViewDev& V,
                         int i, int j, unsigned& evals, unsigned wmask = 0u) {
    Ray r;
    setup_ray_march(V, P, L, i, j, r);
    float t0, t1;
    clip_ray(S.sup_lo, S.sup_hi, r, t0, t1);
    int k0, k1;
    float acc = 0.0f;
    const bool has = sample_range(L, t0, t1, L.K, k0, k1);
    unsigned wm = 0u;
#if defined(__CUDA_ARCH__)
    if constexpr (MERGE) wm = __ballot_sync(wmask, has);
#endif
    (void)wmask;
    (void)wm;
    if (has) {
        if constexpr (HIER) {
            acc = trace_sum_hier<DEPTH, DEFS, RAY, CURVE, kLeafAll, false, MERGE>(
                S, L, r, k0, k1,
                [&](int q, bool fine) {
                    return (float)sample64_pixel(S, V, P.xs, i, j, fine ? L.f64[q] : L.s64[q]);
                },
                evals, wm);
        } else {
            auto unc = [&](int k) { return (float)sample64_pixel(S, V, P.xs, i, j, L.s64[k]); };
#if defined(__CUDA_ARCH__)
            if constexpr (MERGE) acc = trace_sum_merged<DEPTH, DEFS, RAY, CURVE>(S, L, r, k0, k1, unc, evals, wm);
            else
#endif
                acc = trace_sum<DEPTH, DEFS, RAY, CURVE>(S, L, r, k0, k1, unc, evals);
        }
    }
    float w = HIER ? P.density_multiplier : P.density_multiplier * L.ds32;
    float T = fmaf(w, acc, P.flat_field);
    return expf(-T);
}

// Optical depth T = flat_field + multiplier * (sum) of pixel (i, j) of a
// general scene (main.go:146, 153, 175, 198), FP64 for undecided samples in
// the march.
template <bool HIER, int DEPTH, bool DEFS>
XRP_HD float depth_pixel(const SceneDev& S, const Lattice& L, const RenderParams& P, const ViewDev& V, int i,
                         int j, RayStats& st) {
    Ray r;
    setup_ray_march(V, P, L, i, j, r);
    PixelRef px{&V, P.xs, i, j};
    SceneSampler<DEPTH, DEFS> smp{S, r, px};
    float acc = HIER ? march_hier(L, S.sup_lo, S.sup_hi, r, smp, st) : march_simple(L, S.sup_lo, S.sup_hi, r, smp, st);
    float w = HIER ? P.density_multiplier : P.density_multiplier * L.ds32;
    return fmaf(w, acc, P.flat_field);
}

// One pixel: optical depth T = flat_field + multiplier * (sum), as
// transmittance exp(-T) (main.go:146, 153, 175, 198).
template <bool HIER, bool VOLUME, int DEPTH = kMaxDepth, bool DEFS = true>
XRP_HD float render_pixel(const SceneDev& S, const Lattice& L, const RenderParams& P,
                          const ViewDev& V, int i, int j, RayStats& st) {
    if constexpr (!VOLUME) {
        return expf(-depth_pixel<HIER, DEPTH, DEFS>(S, L, P, V, i, j, st));
    } else {
        Ray r;
        PixelRef px{&V, P.xs, i, j};
        const Volume& vol = S.vols[0];
        VolRay vr;
        {
            Ray64 r64;
            setup_ray64_fast(V, P.xs, i, j, r64);
            setup_ray32(r64, L.s_c, r);
            setup_volray(vol, r64, L.s_c, vr);
        }
        VolumeSampler smp{S, vol, vr, px,
                          {1.0f / vol.scale[0], 1.0f / vol.scale[1], 1.0f / vol.scale[2]},
                          S.nodes[S.root].f[0]};
        float acc = HIER ? march_hier(L, S.sup_lo, S.sup_hi, r, smp, st)
                         : march_simple(L, S.sup_lo, S.sup_hi, r, smp, st, 4.0f * vol.band_w + 2e-4f);
        float w = HIER ? P.density_multiplier : P.density_multiplier * L.ds32;
        float T = fmaf(w, acc, P.flat_field);
        return expf(-T);
    }
}

}  // namespace xrp
