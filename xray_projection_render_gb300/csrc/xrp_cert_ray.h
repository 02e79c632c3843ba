// xrp_cert_ray.h -- ray certificates (affine deformation chains): the
// distance along the ray before the density can change.  Part of
// xrp_device.h (included there after the ball certificates, whose leaf and
// container evaluators it uses); not a standalone header.
#pragma once

namespace xrp {

// ---------------------------------------------------------------------------
// Ray certificates.  When the deformation chain is affine (linear, affine,
// rigid or none) the samples ahead of a point lie on a straight line in
// object coordinates, w + u t, with u the chain's linear part applied to the
// ray direction (per unit of the ray parameter).  Instead of a ball around
// the sample, the bound is a ray parameter t before which the line cannot
// come within `eps` of a place where the density changes: the first
// crossing of each primitive's boundary inflated (outside) or shrunk
// (inside) by eps, of a tessellation cell face, of a candidate-list cell
// face.  All points within eps of the segment [w, w + u t] (a capsule) then
// have the density of the sample.  eps (SceneDev::ray_slack) covers the
// position error of the FP32 sample, the direction error over the sampled
// span and the FP32 arithmetic of the crossings, as m_slack does for balls.
// Every bound is also at least the ball bound (distance - eps) / |u|.
// ---------------------------------------------------------------------------
struct RayDir {
    float x, y, z;     // object-space direction per unit ray parameter
    float ix, iy, iz;  // reciprocals of the components (0 for a zero component)
    float a;           // |u|^2
    float il;          // 1 / |u|
    float eps;         // capsule radius (object units)
};

constexpr float kFar = 3.0e38f;
constexpr float kU32 = 5.9604645e-8f;  // 2^-24

// Reciprocal and reciprocal square root of the crossing arithmetic: the
// hardware approximations on the device (a few ulp; the final bound is
// scaled by 1 - 1e-5 and the capsule radius budgets relative errors of the
// crossings), exact division on the host build.
XRP_HD float frcp(float x) {
#if defined(__CUDA_ARCH__)
    return __fdividef(1.0f, x);
#else
    return 1.0f / x;
#endif
}

XRP_HD float frsqrt(float x) {
#if defined(__CUDA_ARCH__)
    return rsqrtf(x);
#else
    return 1.0f / sqrtf(x);
#endif
}

// Square root of the crossing arithmetic (relative error within 2^-23 on
// the device; the bounds that use it budget for it).
XRP_HD float fsqrt(float x) {
#if defined(__CUDA_ARCH__)
    float r;
    asm("sqrt.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
#else
    return sqrtf(x);
#endif
}

// A direction component this small counts as zero (the slab is parallel).
XRP_HD float rcp_dir(float d) { return fabsf(d) > 1e-30f ? frcp(d) : 0.0f; }

// Object-space direction of a ray (linear parts of an affine chain).
XRP_HD RayDir ray_dir32(const SceneDev& S, const float* d) {
    float x = d[0], y = d[1], z = d[2];
    for (int i = 0; i < S.ndefs; i++) {
        const DefStep& s = S.defs[i];
        const float* a = s.f;
        if (s.type == D_LINEAR) {
            float nx = fmaf(a[4], z, fmaf(a[5], y, fmaf(a[0], x, x)));
            float ny = fmaf(a[3], z, fmaf(a[1], y, fmaf(a[5], x, y)));
            float nz = fmaf(a[2], z, fmaf(a[3], y, fmaf(a[4], x, z)));
            x = nx; y = ny; z = nz;
        } else if (s.type == D_AFFINE) {
            float nx = fmaf(a[2], z, fmaf(a[1], y, a[0] * x));
            float ny = fmaf(a[5], z, fmaf(a[4], y, a[3] * x));
            float nz = fmaf(a[8], z, fmaf(a[7], y, a[6] * x));
            x = nx; y = ny; z = nz;
        }
    }
    RayDir u;
    u.x = x; u.y = y; u.z = z;
    u.ix = rcp_dir(x); u.iy = rcp_dir(y); u.iz = rcp_dir(z);
    u.a = fmaf(z, z, fmaf(y, y, x * x));
    u.il = 1.0f / sqrtf(u.a);
    u.eps = S.ray_slack;
    return u;
}

// Slab q + dq t inside (lo, hi), idq = 1/dq (0: parallel): exit parameter
// of the shrunk slab [lo + e, hi - e] for a point inside it.
XRP_HD float slab_exit(float q, float idq, float lo, float hi, float e) {
    if (idq > 0.0f) return (hi - e - q) * idq;
    if (idq < 0.0f) return (lo + e - q) * idq;
    return kFar;
}

// Slab q + dq t inside the inflated slab (lo - e, hi + e): narrows [tlo, thi].
XRP_HD void slab_clip(float q, float idq, float lo, float hi, float e, float& tlo, float& thi) {
    if (idq != 0.0f) {
        float a = (lo - e - q) * idq, b = (hi + e - q) * idq;
        tlo = fmaxf(tlo, fminf(a, b));
        thi = fminf(thi, fmaxf(a, b));
    } else if (!(q > lo - e && q < hi + e)) {
        tlo = kFar;
    }
}

// Spheres and cylinders: the line w + u t against a ball (3-D) or a disc
// (the projection of a cylinder across its axis) of radius R about the
// origin, from the closest approach tc = -b/a and the half chord
// sqrt(R^2 - h^2), h^2 = c2/a the squared distance of the line from the
// origin (c2 = |w x u|^2, stable near tangency).  `err` bounds the FP32
// error of the half chord (large only when the line is nearly tangent, where
// the ball bound takes over); a line within eps/2 of tangency to the
// inflated ball stays clear of the true one.  Outside, R = r + eps and the
// entry interval is widened by err; inside, R = r - eps and the exit is
// shrunk by it.

// Every partial bound below is clamped with fmaxf(., 0) before it enters a
// minimum, so that a NaN (never expected) can only shorten a jump.

// Sphere of radius r, point w from the centre at signed distance g.
XRP_HD float sphere_ray(float wx, float wy, float wz, float g, float r, const RayDir& u, float tcap) {
    const float eps = u.eps;
    const float ag = fabsf(g) - eps;
    if (!(ag > 0.0f)) return 0.0f;
    const float tb = ag * u.il;
    if (tb >= tcap) return tb;  // cannot lower the caller's minimum
    // inside: exit of the ball shrunk by eps; outside: entry of the ball
    // inflated by eps (one straight-line computation for both)
    const bool in = g < 0.0f;
    const float sg = in ? -1.0f : 1.0f;
    const float b = fmaf(wz, u.z, fmaf(wy, u.y, wx * u.x));
    const float cx = fmaf(wy, u.z, -wz * u.y), cy = fmaf(wz, u.x, -wx * u.z), cz = fmaf(wx, u.y, -wy * u.x);
    const float c2 = fmaf(cz, cz, fmaf(cy, cy, cx * cx));
    const float wl1 = fabsf(wx) + fabsf(wy) + fabsf(wz);
    const float R = fmaf(sg, eps, r);
    const float ia = u.il * u.il;
    const float h2 = c2 * ia;
    const float tc = -b * ia;
    const float ch = fsqrt(fmaxf(fmaf(R, R, -h2), 0.0f));
    const float err = 4.0f * kU32 * (fmaf(8.0f * wl1, R, 3.0f * R * R) * frcp(ch) + 4.0f * (wl1 + R));
    const float half = fmaf(sg, err, ch) * u.il;  // widened outside, shrunk inside
    float t = in ? tc + half : tc - half;
    // outside: moving away (the distance only grows), or within eps/2 of
    // tangency (never reaches the true ball)
    const float Rt = R - 0.5f * eps;
    if (!in && (!(b < 0.0f) || !(h2 < Rt * Rt))) t = kFar;
    return fmaxf(t, tb);
}

// Finite cylinder: w from p0, axial fraction c, perpendicular part p, radial
// and axial signed distances gr, ga (negative inside).
// Inside (g < -eps) the bound is the exit of the cylinder shrunk by eps,
// outside (g > eps) the entry of the cylinder inflated by eps: the axial
// slab and the radial chord are intervals of t either way, so both cases run
// the same straight-line code (lanes of a warp inside and outside struts do
// not diverge).
// v: the axis p1 - p0, ivv = 1/|v|^2, vl = |v|, bc: the band of c.
XRP_HD float cyl_ray(float vx, float vy, float vz, float ivv, float r, float vl, float bc, float c,
                     float px, float py, float pz, float gr, float ga, const RayDir& u, float tcap) {
    const float eps = u.eps;
    const float g = fmaxf(gr, ga);
    if (!(fabsf(g) > eps)) return 0.0f;
    const float tb = (fabsf(g) - eps) * u.il;
    if (tb >= tcap) return tb;  // cannot lower the caller's minimum
    const bool in = g < 0.0f;
    const float sg = in ? -1.0f : 1.0f;
    // axial: c + cu t inside (-es, 1 + es), es = +-(eps / |v| + band of c)
    const float cu = fmaf(u.z, vz, fmaf(u.y, vy, u.x * vx)) * ivv;
    const float icu = rcp_dir(cu);
    const float es = sg * fmaf(eps, vl * ivv, bc);
    float alo = -kFar, ahi = kFar;
    if (icu != 0.0f) {
        const float a1 = (-es - c) * icu, a2 = (1.0f + es - c) * icu;
        alo = fminf(a1, a2);
        ahi = fmaxf(a1, a2);
    } else if (!in && !(c > -es && c < 1.0f + es)) {
        alo = kFar;
    }
    // radial: the line's projection against the disc of radius r +- eps
    const float qx = fmaf(-cu, vx, u.x), qy = fmaf(-cu, vy, u.y), qz = fmaf(-cu, vz, u.z);
    const float a = fmaf(qz, qz, fmaf(qy, qy, qx * qx));
    float rlo = -kFar, rhi = kFar;
    if (a > 1e-12f * u.a) {
        const float b = fmaf(pz, qz, fmaf(py, qy, px * qx));
        const float cx = fmaf(py, qz, -pz * qy), cy = fmaf(pz, qx, -px * qz), cz = fmaf(px, qy, -py * qx);
        const float c2 = fmaf(cz, cz, fmaf(cy, cy, cx * cx));
        const float wl1 = fabsf(px) + fabsf(py) + fabsf(pz);
        const float R = fmaf(sg, eps, r);
        const float ia = frcp(a);
        const float h2 = c2 * ia;
        const float tc = -b * ia;
        const float ch = fsqrt(fmaxf(fmaf(R, R, -h2), 0.0f));
        const float err = 4.0f * kU32 * (fmaf(8.0f * wl1, R, 3.0f * R * R) * frcp(ch) + 4.0f * (wl1 + R));
        const float half = fmaf(sg, err, ch) * frsqrt(a);  // widened outside, shrunk inside
        rlo = tc - half;
        rhi = tc + half;
        // outside, a line within eps/2 of tangency never reaches the true disc
        const float Rt = R - 0.5f * eps;
        if (!in && !(h2 < Rt * Rt)) rlo = kFar;
    } else if (a > 0.0f) {  // nearly parallel to the axis: the radius changes at rate |u_perp|
        const float tr = (fabsf(gr) - eps) * frsqrt(a);
        if (in) rhi = tr;
        else if (gr > eps) rlo = tr;
    } else if (!in && gr > eps) {
        rlo = kFar;
    }
    float t;
    if (in) {
        t = fminf(ahi, rhi);
    } else {
        const float lo = fmaxf(fmaxf(alo, rlo), 0.0f), hi = fminf(ahi, rhi);
        t = lo <= hi ? lo : kFar;
    }
    return fmaxf(fmaxf(t, 0.0f), tb);
}

// Axis-aligned box of half sides h (F_BAND b): point w from the centre,
// mn = min(h - |w|).
XRP_HD float box_ray(const float* h, float wx, float wy, float wz, float mn, float b, const RayDir& u) {
    const float e = u.eps + b;
    if (!(fabsf(mn) > e)) return 0.0f;
    // inside: exit of the box shrunk by e; outside: entry of the box
    // inflated by e
    const bool in = mn > 0.0f;
    const float es = in ? -e : e;
    float lo = 0.0f, hi = kFar;
    slab_clip(wx, u.ix, -h[0], h[0], es, lo, hi);
    slab_clip(wy, u.iy, -h[1], h[1], es, lo, hi);
    slab_clip(wz, u.iz, -h[2], h[2], es, lo, hi);
    return in ? fmaxf(hi, 0.0f) : (lo <= hi ? lo : kFar);
}

// Leaf density (leaf_dm's decisions) and its ray bound t.  `tcap`: the
// caller's current minimum; a bound at or above it may be returned without
// its exact value (it cannot lower the minimum).
XRP_HD float leaf_dr(const Node& n, float x, float y, float z, const RayDir& u, float tcap, float& t) {
    const float* f = n.f;
    switch (n.type) {
    case N_SPHERE: {
        const F4 a = ld4(f), c4 = ld4(f + 4), tb = ld4(f + 24);  // centre, r^2; r; bands, rho
        float dx = x - a.x, dy = y - a.y, dz = z - a.z;
        float d2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
        t = sphere_ray(dx, dy, dz, fsqrt(d2) - c4.x, c4.x, u, tcap);
        float q = d2 - a.w;
        if (q < -tb.z) return tb.w;
        if (q > tb.z) return 0.0f;
        return xnan();
    }
    case N_BOX: {
        const F4 a = ld4(f), c4 = ld4(f + 4), tb = ld4(f + 24);  // centre, half sides; bands, rho
        const float h[3] = {a.w, c4.x, c4.y};
        float wx = x - a.x, wy = y - a.y, wz = z - a.z;
        float mn = fminf(h[0] - fabsf(wx), fminf(h[1] - fabsf(wy), h[2] - fabsf(wz)));
        float b = tb.z;
        t = box_ray(h, wx, wy, wz, mn, b, u);
        if (mn > b) return tb.w;
        if (mn < -b) return 0.0f;
        return xnan();
    }
    case N_CYL: {
        // a: p0, v.x; c4: v.y, v.z, 1/|v|^2, r^2; e: r, |v|; tb: bands, rho
        const F4 a = ld4(f), c4 = ld4(f + 4), e = ld4(f + 8), tb = ld4(f + 24);
        float wx = x - a.x, wy = y - a.y, wz = z - a.z;
        float c = fmaf(wz, c4.y, fmaf(wy, c4.x, wx * a.w)) * c4.z;
        float px = fmaf(-c, a.w, wx), py = fmaf(-c, c4.x, wy), pz = fmaf(-c, c4.y, wz);
        float p2 = fmaf(pz, pz, fmaf(py, py, px * px));
        float bc = tb.y;
        t = cyl_ray(a.w, c4.x, c4.y, c4.z, e.x, e.y, bc, c, px, py, pz, fsqrt(p2) - e.x,
                    fmaxf(-c, c - 1.0f) * e.y, u, tcap);
        if (c < -bc || c > 1.0f + bc) return 0.0f;
        float q = p2 - c4.w;
        float bd = tb.z;
        if (q > bd) return 0.0f;
        if (q < -bd && c > bc && c < 1.0f - bc) return tb.w;
        return xnan();
    }
    case N_PPD: {
        float wx = x - f[0], wy = y - f[1], wz = z - f[2];
        float b = f[F_BAND];
        float q[3], iqu[3], e[3];
        float mn = 3.0e38f, mrel = 3.0e38f;
        bool out = false;
        for (int a = 0; a < 3; a++) {
            const float* r = f + 3 + 3 * a;
            q[a] = fmaf(r[2], wz, fmaf(r[1], wy, r[0] * wx));
            iqu[a] = rcp_dir(fmaf(r[2], u.z, fmaf(r[1], u.y, r[0] * u.x)));
            e[a] = fmaf(u.eps, f[12 + a], b);
            float in = fminf(q[a], 1.0f - q[a]);
            mn = fminf(mn, in);
            mrel = fminf(mrel, in - e[a]);
            out = out || in < -e[a];
        }
        // inside (every slab at least e inside): exit of the shrunk slabs;
        // outside (some slab more than e outside): entry of the inflated
        // ones; else 0
        if (out || mrel > 0.0f) {
            float lo = 0.0f, hi = kFar;
            for (int a = 0; a < 3; a++) slab_clip(q[a], iqu[a], 0.0f, 1.0f, out ? e[a] : -e[a], lo, hi);
            t = out ? (lo <= hi ? lo : kFar) : fmaxf(hi, 0.0f);
        } else {
            t = 0.0f;
        }
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
        float m = fmaxf(fabsf(q) - f[F_BAND], 0.0f) / (2.4494898f * fabsf(f[3]));
        t = fmaxf(m - u.eps, 0.0f) * u.il;
        if (q > f[F_BAND]) return f[F_RHO];
        if (q < -f[F_BAND]) return 0.0f;
        return xnan();
    }
    default: t = 0.0f; return xnan();
    }
}

// Box [lo, hi] (per axis, interleaved lo0 hi0 lo1 hi1 ...): exit of the box
// shrunk by e for a point at least e inside, entry of the box inflated by e
// for a point more than e outside, else 0.  `in` is the point's smallest
// distance to a face (negative outside).
XRP_HD float bounds_ray(const float* b, float x, float y, float z, float in, float e, const RayDir& u) {
    if (!(fabsf(in) > e)) return 0.0f;
    const bool inside = in > 0.0f;
    const float es = inside ? -e : e;
    float lo = 0.0f, hi = kFar;
    slab_clip(x, u.ix, b[0], b[1], es, lo, hi);
    slab_clip(y, u.iy, b[2], b[3], es, lo, hi);
    slab_clip(z, u.iz, b[4], b[5], es, lo, hi);
    return inside ? fmaxf(hi, 0.0f) : (lo <= hi ? lo : kFar);
}

template <int D, bool UNI = false>
XRP_HD float coll_dr(const SceneDev& S, const Node& c, float x, float y, float z, const RayDir& u, float tcap,
                     float& t);

// item_dm's decisions; t: the ray bound (tessellations: the outer bounds,
// the cell faces of the fold and the unit-cell bounds cap the collection's).
template <int D>
XRP_HD float item_dr(const SceneDev& S, int id, float x, float y, float z, const RayDir& u, float tcap,
                     float& t) {
    const Node& n = S.nodes[id];
    if (n.type <= N_GYROID) return leaf_dr(n, x, y, z, u, tcap, t);
    if (n.type == N_TESS) {
        if constexpr (D > 0) {
            // node layout as in item32
            const F4 f0 = ld4(n.f), f4 = ld4(n.f + 4), f8 = ld4(n.f + 8), f12 = ld4(n.f + 12);
            const F4 f16 = ld4(n.f + 16), f20 = ld4(n.f + 20);
            const float ob[6] = {f0.x, f0.y, f0.z, f0.w, f4.x, f4.y};
            const float ub[6] = {f4.w, f8.x, f8.y, f8.z, f8.w, f12.x};
            float mo = fminf(fminf(fminf(x - ob[0], ob[1] - x), fminf(y - ob[2], ob[3] - y)),
                             fminf(z - ob[4], ob[5] - z));
            const float to = bounds_ray(ob, x, y, z, mo, u.eps + f4.z, u);
            if (mo < -f4.z) { t = to; return 0.0f; }  // outside: zero up to the bounds
            if (!(mo > f4.z)) { t = 0.0f; return xnan(); }
            float qx = (x - f20.x) * f16.y, qy = (y - f20.y) * f16.z, qz = (z - f20.z) * f16.w;
            float nx = floorf(qx), ny = floorf(qy), nz = floorf(qz);
            float bq = f20.w;
            float frx = qx - nx, fry = qy - ny, frz = qz - nz;
            float fr = fminf(fminf(fminf(frx, 1.0f - frx), fminf(fry, 1.0f - fry)), fminf(frz, 1.0f - frz));
            if (!(fr > bq)) { t = 0.0f; return xnan(); }
            // exit of this tessellation cell (q units; eps scaled by 1/cell
            // size; 1/(u f17) = (1/u) f14: f14 is the cell size, f17 its
            // reciprocal)
            float tc = fminf(fminf(fmaxf(slab_exit(frx, u.ix * f12.z, 0.0f, 1.0f, fmaf(u.eps, fabsf(f16.y), bq)), 0.0f),
                                   fmaxf(slab_exit(fry, u.iy * f12.w, 0.0f, 1.0f, fmaf(u.eps, fabsf(f16.z), bq)), 0.0f)),
                             fmaxf(slab_exit(frz, u.iz * f16.x, 0.0f, 1.0f, fmaf(u.eps, fabsf(f16.w), bq)), 0.0f));
            const float tt = fminf(to, tc);
            float fx = fmaf(-f12.z, nx, x), fy = fmaf(-f12.w, ny, y), fz = fmaf(-f16.x, nz, z);
            float mu = fminf(fminf(fminf(fx - ub[0], ub[1] - fx), fminf(fy - ub[2], ub[3] - fy)),
                             fminf(fz - ub[4], ub[5] - fz));
            if (mu < -f12.y) {  // outside the unit-cell bounds: zero up to them
                t = fminf(tt, bounds_ray(ub, fx, fy, fz, mu, u.eps + f12.y, u));
                return 0.0f;
            }
            if (!(mu > f12.y)) { t = 0.0f; return xnan(); }
            // Inside, the unit-cell bounds need no ray bound of their own: the
            // fold's period and origin are the unit cell's extent and lower
            // bounds (objects.go:574-579), so up to tc every sample folds into
            // this cell at least the fold band away from its faces, where the
            // inclusive unit-cell test (objects.go:460) holds.
            float tk;
            // unit cells are where uniform greedy collections occur (lattices)
            float r = coll_dr<D - 1, true>(S, S.nodes[n.a], fx, fy, fz, u, fminf(tt, tcap), tk);
            t = fminf(tt, tk);
            return r;
        }
    }
    t = 0.0f;  // voxel grids and anything deeper: density by the plain path
    if (n.type == N_VOXEL) return voxel32(S.vols[n.a], n.f[0], x, y, z, S.hier_zero_guard);
    return xnan();
}

// Uniform greedy collections (every child a leaf of the same density > 0):
// the decisions of coll_dm; inside a child (for certain) the density is
// that child's whatever the others do, so its exit alone bounds the ray (no
// list-cell cap, no other candidate).  `t` holds the list-cell cap on entry.
XRP_HD float coll_dr_uniform(const SceneDev& S, const int32_t* kids, const int32_t* list, int cnt, float x,
                             float y, float z, const RayDir& u, float tcap, float& t) {
    for (int k = 0; k < cnt; k++) {
        float tk;
        const float r = leaf_dr(S.nodes[list ? list[k] : kids[k]], x, y, z, u, tcap, tk);
        if (isunc(r)) {  // an undecided child before any certain one
            t = 0.0f;
            return r;
        }
        if (r > 0.0f) {
            t = tk;
            return r;
        }
        t = fminf(t, tk);
    }
    return 0.0f;  // outside every candidate (greedy sum of zeros, clipped)
}

// coll_dm's decisions; t: the minimum over the candidates, capped (with
// candidate lists) by the later of the exit from the point's list cell and
// the clearance of the unlisted children.
// UNI: the collection may be uniform (unit cells of tessellations); the
// uniform path is compiled only there, which keeps it out of the kernels of
// scenes without tessellations.
template <int D, bool UNI>
XRP_HD float coll_dr(const SceneDev& S, const Node& c, float x, float y, float z, const RayDir& u, float tcap,
                     float& t) {
    const int32_t* kids = S.child + c.a;
    int cnt = c.b;
    const int32_t* list = nullptr;
    t = kFar;
    if (c.flags & C_ACCEL) {
        int G = (c.flags >> 16) & 0xff;
        // f[0..2] grid origin, f[3..5] 1/cell size, f[6] cell base, f[8..10] cell size
        const F4 g0 = ld4(c.f), g4 = ld4(c.f + 4), g8 = ld4(c.f + 8);
        const float cf[11] = {g0.x, g0.y, g0.z, g0.w, g4.x, g4.y, g4.z, g4.w, g8.x, g8.y, g8.z};
        float ux = (x - cf[0]) * cf[3], uy = (y - cf[1]) * cf[4], uz = (z - cf[2]) * cf[5];
        int ix = (int)floorf(ux), iy = (int)floorf(uy), iz = (int)floorf(uz);
        ix = ix < 0 ? 0 : (ix >= G ? G - 1 : ix);
        iy = iy < 0 ? 0 : (iy >= G ? G - 1 : iy);
        iz = iz < 0 ? 0 : (iz >= G ? G - 1 : iz);
        // inner faces only (the outer cells extend to infinity by the clamp)
        float tc = kFar;
        {
            // grid units; 1/(u f3) = (1/u) f8 (f8: the cell size)
            const float dx = u.ix * cf[8], ex = u.eps * cf[3];
            if (dx > 0.0f && ix < G - 1) tc = fminf(tc, fmaxf(((float)(ix + 1) - ex - ux) * dx, 0.0f));
            if (dx < 0.0f && ix > 0) tc = fminf(tc, fmaxf(((float)ix + ex - ux) * dx, 0.0f));
            const float dy = u.iy * cf[9], ey = u.eps * cf[4];
            if (dy > 0.0f && iy < G - 1) tc = fminf(tc, fmaxf(((float)(iy + 1) - ey - uy) * dy, 0.0f));
            if (dy < 0.0f && iy > 0) tc = fminf(tc, fmaxf(((float)iy + ey - uy) * dy, 0.0f));
            const float dz = u.iz * cf[10], ez = u.eps * cf[5];
            if (dz > 0.0f && iz < G - 1) tc = fminf(tc, fmaxf(((float)(iz + 1) - ez - uz) * dz, 0.0f));
            if (dz < 0.0f && iz > 0) tc = fminf(tc, fmaxf(((float)iz + ez - uz) * dz, 0.0f));
        }
        int cell_base = f2i(cf[6]);
        const int cell = cell_base + (iz * G + iy) * G + ix;
        t = fmaxf(tc, fmaxf(S.clear[cell] - u.eps, 0.0f) * u.il);
        const int32_t* off = S.cells + cell;
        int s0 = off[0], s1 = off[1];
        list = S.items + s0;
        cnt = s1 - s0;
    }
    const bool greedy = (c.flags & C_GREEDY) != 0;
    if constexpr (UNI) {
        if (c.flags & C_UNIFORM) return coll_dr_uniform(S, kids, list, cnt, x, y, z, u, tcap, t);
    }
    float sum = 0.0f, sabs = 0.0f;
    bool unc = false, done = false;
    for (int k = 0; k < cnt; k++) {
        float tk;
        float r = item_dr<D>(S, list ? list[k] : kids[k], x, y, z, u, fminf(t, tcap), tk);
        t = fminf(t, tk);
        if (done) continue;  // greedy value fixed; bounds of the rest still count
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

// density32 at one point and the ray bound t (ray parameter units) of the
// samples ahead that share its density; affine chains only.  Bounds at or
// above `tcap` (the end of the caller's range) need not be exact.
template <int DEPTH, bool DEFS>
XRP_HD float dens_ray32(const SceneDev& S, float x, float y, float z, const RayDir& u, float tcap, float& t) {
    if constexpr (DEFS) deform32(S, x, y, z);
    const Node& r = S.nodes[S.root];
    float rho;
    if (r.type <= N_GYROID) rho = leaf_dr(r, x, y, z, u, tcap, t);
    else if (r.type == N_COLL) rho = coll_dr<DEPTH>(S, r, x, y, z, u, tcap, t);
    else rho = item_dr<DEPTH>(S, S.root, x, y, z, u, tcap, t);
    t = fmaxf(t, 0.0f) * 0.99999f;
    return rho;
}


}  // namespace xrp
