// xrp_cert_curve.h -- curved-ray certificates (smooth non-affine
// deformation chains).  Part of xrp_device.h (included there after the ray
// certificates); not a standalone header.
#pragma once

namespace xrp {

// ---------------------------------------------------------------------------
// Curved-ray certificates (smooth non-affine chains: gaussian, sigmoid).
// The deformed sample point q(s) of a ray then follows a curve, whose speed
// |q'| is at most `vmax` (the chain's Lipschitz bound) and whose
// acceleration |q''| is at most `acc` (host: chain rule over the steps).
// A ball of radius m around q(s0) holds the curve for s - s0 <= m / vmax;
// a gyroid leaf does better with a second-order bound on g(q(s)):
//   |g(s0 + tau) - g0 - g1 tau| <= M tau^2 / 2,  g1 = grad g . q'(s0),
//   M = |q'|^2 max|H g| + |grad g| |q''| <= 4 is^2 vmax^2 + sqrt(6) is acc,
// (is = 1/scale; every entry of the Hessian is a sum of at most two
// products of sines and cosines), so the band |g| < t is entered or left
// no earlier than the first root of that quadratic.  Near the band edge the
// bound grows like sqrt(gap / M) where the ball's grows like the gap.
// Selected by the CURVE flag of the tracing loops (CPU build; the device
// kernels use ball certificates for these chains).
// ---------------------------------------------------------------------------
struct CurveDir {
    float vx, vy, vz;  // q'(s) at the sample (object units per unit ray parameter)
    float vmax, acc;   // chain bounds on |q'| and |q''|
    float eps;         // absolute error allowance (m_slack)
};

// deform32 with the velocity: (x, y, z) <- def(p), (vx, vy, vz) <- J(p) v.
XRP_HD void deform_jvp32(const SceneDev& S, float& x, float& y, float& z, float& vx, float& vy, float& vz) {
    for (int i = 0; i < S.ndefs; i++) {
        const DefStep& d = S.defs[i];
        const float* a = d.f;
        switch (d.type) {
        case D_GAUSSIAN: {
            float x0 = x - a[6], y0 = y - a[7], z0 = z - a[8];
            float r2 = fmaf(z0, z0, fmaf(y0, y0, x0 * x0));
            float rv = fmaf(z0, vz, fmaf(y0, vy, x0 * vx));
            float ex = a[0] * f_exp(-r2 * a[3]);
            float ey = a[1] * f_exp(-r2 * a[4]);
            float ez = a[2] * f_exp(-r2 * a[5]);
            vx = fmaf(-2.0f * a[3] * ex, rv, vx);
            vy = fmaf(-2.0f * a[4] * ey, rv, vy);
            vz = fmaf(-2.0f * a[5] * ez, rv, vz);
            x += ex; y += ey; z += ez;
            break;
        }
        case D_LINEAR: {
            float nx = fmaf(a[4], z, fmaf(a[5], y, fmaf(a[0], x, x)));
            float ny = fmaf(a[3], z, fmaf(a[1], y, fmaf(a[5], x, y)));
            float nz = fmaf(a[2], z, fmaf(a[3], y, fmaf(a[4], x, z)));
            float mx = fmaf(a[4], vz, fmaf(a[5], vy, fmaf(a[0], vx, vx)));
            float my = fmaf(a[3], vz, fmaf(a[1], vy, fmaf(a[5], vx, vy)));
            float mz = fmaf(a[2], vz, fmaf(a[3], vy, fmaf(a[4], vx, vz)));
            x = nx; y = ny; z = nz;
            vx = mx; vy = my; vz = mz;
            break;
        }
        case D_RIGID: x += a[0]; y += a[1]; z += a[2]; break;
        case D_SIGMOID: {
            float* p = d.axis == 0 ? &x : (d.axis == 1 ? &y : &z);
            float* v = d.axis == 0 ? &vx : (d.axis == 1 ? &vy : &vz);
            float e = f_exp(-(*p - a[1]) * a[2]);
            float sg = f_rcp(1.0f + e);
            *v *= fmaf(a[0] * a[2], sg * (1.0f - sg), 1.0f);  // 1 + A sigma' / L
            *p += a[0] * sg;
            break;
        }
        case D_AFFINE: {
            float nx = fmaf(a[2], z, fmaf(a[1], y, a[0] * x));
            float ny = fmaf(a[5], z, fmaf(a[4], y, a[3] * x));
            float nz = fmaf(a[8], z, fmaf(a[7], y, a[6] * x));
            float mx = fmaf(a[2], vz, fmaf(a[1], vy, a[0] * vx));
            float my = fmaf(a[5], vz, fmaf(a[4], vy, a[3] * vx));
            float mz = fmaf(a[8], vz, fmaf(a[7], vy, a[6] * vx));
            x = nx; y = ny; z = nz;
            vx = mx; vy = my; vz = mz;
            break;
        }
        default: break;
        }
    }
}

// First tau > 0 at which D - w tau - M tau^2 / 2 can reach 0 (gap D > 0
// closing at speed w, curvature M > 0): the positive root, in the form
// without cancellation for each sign of w (moving away, the rationalised
// form would divide by a difference that FP32 can round to 0).
XRP_HD float gap_time(float D, float w, float M) {
    const float s = sqrtf(fmaf(w, w, 2.0f * M * D));
    return w >= 0.0f ? 2.0f * D / (w + s) : (s - w) / M;
}

// A ball margin m (object units) as a ray-parameter bound along the curve.
XRP_HD float curve_time(float m, const CurveDir& c) { return fmaxf(m - c.eps, 0.0f) / c.vmax; }

// Box b = (lo0, hi0, lo1, hi1, lo2, hi2) and a point inside it at least
// eps from every face: the first parameter at which the curve can reach a
// face, face by face (gap to the face, speed toward it, acceleration bound),
// at least the ball bound.
// Box b and a point outside it: entering needs every coordinate inside its
// slab (grown by eps), so the latest per-axis arrival bounds the entry.
XRP_HD float box_curve_entry(const float* b, float x, float y, float z, const CurveDir& c) {
    const float M = c.acc + 1e-20f;
    const float p[3] = {x, y, z}, v[3] = {c.vx, c.vy, c.vz};
    float t = 0.0f;
    for (int a = 0; a < 3; a++) {
        const float below = b[2 * a] - c.eps - p[a], above = p[a] - b[2 * a + 1] - c.eps;
        if (below > 0.0f) t = fmaxf(t, gap_time(below, v[a] + 1e-6f * c.vmax, M));
        if (above > 0.0f) t = fmaxf(t, gap_time(above, -v[a] + 1e-6f * c.vmax, M));
    }
    return t;
}

XRP_HD float box_curve_time(const float* b, float x, float y, float z, const CurveDir& c) {
    const float M = c.acc + 1e-20f;
    const float gaps[6] = {x - b[0] - c.eps, b[1] - x - c.eps, y - b[2] - c.eps,
                           b[3] - y - c.eps, z - b[4] - c.eps, b[5] - z - c.eps};
    const float w[6] = {-c.vx, c.vx, -c.vy, c.vy, -c.vz, c.vz};
    float t = kFar;
    for (int k = 0; k < 6; k++) {
        if (!(gaps[k] > 0.0f)) return 0.0f;
        t = fminf(t, gap_time(gaps[k], w[k] + 1e-6f * c.vmax, M));
    }
    return t;
}

// Slab lo < a < hi of a coordinate a(s) with a' = w at the sample and
// |a''| <= M: inside (at least e from both faces) the first exit, outside
// the first arrival at the slab (grown by e); 0 within e of a face.
XRP_HD float slab_curve(float a, float w, float lo, float hi, float e, float M, bool inside) {
    if (inside) {
        const float g0 = a - lo - e, g1 = hi - a - e;
        if (!(g0 > 0.0f && g1 > 0.0f)) return 0.0f;
        return fminf(gap_time(g0, -w, M), gap_time(g1, w, M));
    }
    if (a < lo - e) return gap_time(lo - e - a, w, M);
    if (a > hi + e) return gap_time(a - hi - e, -w, M);
    return 0.0f;
}

// Squared radius f = |w|^2 (3-D, or across a cylinder's axis) against r^2:
// f' = 2 w.v, |f''| <= 2 vmax^2 + 2 |w| acc with |w| <= r inside.  Inside
// (|w| < r - e): the first time f can reach (r - e)^2.  Outside the radius
// d = |w| has |d''| <= vmax^2 / r + acc while d >= r: the first time d can
// come down to r + e.
XRP_HD float radius_curve(float w2, float wv, float r, float e, float vmax, float acc, bool inside) {
    if (inside) {
        const float ri = r - e;
        const float gap = ri * ri - w2;
        if (!(ri > 0.0f && gap > 0.0f)) return 0.0f;
        return gap_time(gap, 2.0f * wv + 1e-6f * vmax * ri, fmaf(2.0f * r, acc, 2.0f * vmax * vmax) * 1.01f);
    }
    const float d = sqrtf(w2);
    const float gap = d - r - e;
    if (!(gap > 0.0f && r > 0.0f)) return 0.0f;
    return gap_time(gap, -wv / d + 1e-6f * vmax, fmaf(vmax, vmax / r, acc) * 1.01f + 1e-20f);
}

// Leaf density (leaf_dm's decisions) and its curve bound t: the ball bound,
// or better the second-order bound of the leaf's defining conditions
// (entry: the latest arrival over the violated conditions; exit: the
// earliest over all).
XRP_HD float gyroid_dc(const Node& n, float x, float y, float z, const CurveDir& c, float& t);

// The leaf types a curve-bound kernel is compiled for (bit 1 << NodeType):
// every leaf, or gyroids only (the tessellated gyroid scenes, whose kernel
// then carries no other leaf's code and fits the instruction cache better).
constexpr int kLeafAll = (1 << N_SPHERE) | (1 << N_BOX) | (1 << N_CYL) | (1 << N_PPD) | (1 << N_GYROID);
constexpr int kLeafGyroid = 1 << N_GYROID;

template <int LM = kLeafAll>
XRP_HD float leaf_dc(const Node& n, float x, float y, float z, const CurveDir& c, float& t) {
    if constexpr (LM == kLeafGyroid) return gyroid_dc(n, x, y, z, c, t);
    if (n.type == N_GYROID) return gyroid_dc(n, x, y, z, c, t);
    float m;
    const float rho = leaf_dm(n, x, y, z, m);
    t = curve_time(m, c);
    if (isunc(rho)) return rho;
    const float* f = n.f;
    const float e = c.eps;
    const float M = c.acc * 1.01f + 1e-20f;
    switch (n.type) {
    case N_SPHERE: {
        const float wx = x - f[0], wy = y - f[1], wz = z - f[2];
        const float w2 = fmaf(wz, wz, fmaf(wy, wy, wx * wx));
        const float wv = fmaf(wz, c.vz, fmaf(wy, c.vy, wx * c.vx));
        const float r = f[4], b = sqrtf(f[F_BAND]);  // band of d^2 - r^2 as a distance (upper bound)
        t = fmaxf(t, radius_curve(w2, wv, r, e + b, c.vmax, c.acc, w2 < r * r));
        return rho;
    }
    case N_BOX: {
        const float bb[6] = {f[0] - f[3], f[0] + f[3], f[1] - f[4], f[1] + f[4], f[2] - f[5], f[2] + f[5]};
        const float mn = fminf(f[3] - fabsf(x - f[0]), fminf(f[4] - fabsf(y - f[1]), f[5] - fabsf(z - f[2])));
        const float eb = e + f[F_BAND];
        float tt;
        if (mn > eb) {
            tt = kFar;
            const float p[3] = {x, y, z}, v[3] = {c.vx, c.vy, c.vz};
            for (int a = 0; a < 3; a++) tt = fminf(tt, slab_curve(p[a], v[a], bb[2 * a], bb[2 * a + 1], eb, M, true));
        } else if (mn < -eb) {
            tt = 0.0f;
            const float p[3] = {x, y, z}, v[3] = {c.vx, c.vy, c.vz};
            for (int a = 0; a < 3; a++) tt = fmaxf(tt, slab_curve(p[a], v[a], bb[2 * a], bb[2 * a + 1], eb, M, false));
        } else {
            tt = 0.0f;
        }
        t = fmaxf(t, tt);
        return rho;
    }
    case N_CYL: {
        // axis v (f[3..5]), 1/|v|^2 f[6], r f[8], |v| f[9]: axial coordinate
        // a = (q - p0).v/|v| in [0, |v|], radial part across the axis
        const float wx = x - f[0], wy = y - f[1], wz = z - f[2];
        const float il = f[9] * f[6];  // 1/|v|
        const float a = fmaf(wz, f[5], fmaf(wy, f[4], wx * f[3])) * il;
        const float va = fmaf(c.vz, f[5], fmaf(c.vy, f[4], c.vx * f[3])) * il;
        const float cc = a * il;
        const float px = fmaf(-cc, f[3], wx), py = fmaf(-cc, f[4], wy), pz = fmaf(-cc, f[5], wz);
        const float ca = va * il;
        const float qx = fmaf(-ca, f[3], c.vx), qy = fmaf(-ca, f[4], c.vy), qz = fmaf(-ca, f[5], c.vz);
        const float p2 = fmaf(pz, pz, fmaf(py, py, px * px));
        const float pv = fmaf(pz, qz, fmaf(py, qy, px * qx));
        const float r = f[8], br = sqrtf(f[F_BAND]);
        const float ea = e + f[F_BAND2] * f[9];  // band of c as an axial distance
        const bool in_r = p2 < r * r, in_a = a > 0.0f && a < f[9];
        float tt;
        if (rho != 0.0f || (in_r && in_a)) {  // inside both: the earlier exit
            tt = fminf(radius_curve(p2, pv, r, e + br, c.vmax, c.acc, true),
                       slab_curve(a, va, 0.0f, f[9], ea, M, true));
        } else {  // entering needs both: the later arrival of the violated ones
            tt = 0.0f;
            if (!in_r) tt = fmaxf(tt, radius_curve(p2, pv, r, e + br, c.vmax, c.acc, false));
            if (!in_a) tt = fmaxf(tt, slab_curve(a, va, 0.0f, f[9], ea, M, false));
        }
        t = fmaxf(t, tt);
        return rho;
    }
    case N_PPD: {
        const float wx = x - f[0], wy = y - f[1], wz = z - f[2];
        const float b = f[F_BAND];
        float q[3], qv[3], ea[3], Ma[3];
        float mrel = 3.0e38f;
        bool out = false;
        for (int k = 0; k < 3; k++) {
            const float* rr = f + 3 + 3 * k;
            q[k] = fmaf(rr[2], wz, fmaf(rr[1], wy, rr[0] * wx));
            qv[k] = fmaf(rr[2], c.vz, fmaf(rr[1], c.vy, rr[0] * c.vx));
            ea[k] = fmaf(e, f[12 + k], b);
            Ma[k] = M * f[12 + k];
            const float in = fminf(q[k], 1.0f - q[k]);
            mrel = fminf(mrel, in - ea[k]);
            out = out || in < -ea[k];
        }
        float tt = 0.0f;
        if (out) {
            for (int k = 0; k < 3; k++) tt = fmaxf(tt, slab_curve(q[k], qv[k], 0.0f, 1.0f, ea[k], Ma[k], false));
        } else if (mrel > 0.0f) {
            tt = kFar;
            for (int k = 0; k < 3; k++) tt = fminf(tt, slab_curve(q[k], qv[k], 0.0f, 1.0f, ea[k], Ma[k], true));
        }
        t = fmaxf(t, tt);
        return rho;
    }
    default: break;
    }
    return rho;
}

// The gyroid leaf: leaf_dm's decision and ball bound and the second-order
// curve bound from one set of sines and cosines.
XRP_HD float gyroid_dc(const Node& n, float x, float y, float z, const CurveDir& c, float& t) {
    const float* f = n.f;
    const float is = f[3], ais = fabsf(is);
    float X = (x - f[0]) * is, Y = (y - f[1]) * is, Z = (z - f[2]) * is;
    float sx, cx, sy, cy, sz, cz;
    f_sincos(X, &sx, &cx);
    f_sincos(Y, &sy, &cy);
    f_sincos(Z, &sz, &cz);
    const float g = fmaf(sz, cx, fmaf(sy, cz, sx * cy));
    // leaf_dm (N_GYROID): decision and ball bound
    const float q = f[4] - fabsf(g);
    const float m = fmaxf(fabsf(q) - f[F_BAND], 0.0f) / (2.4494898f * ais);
    t = curve_time(m, c);
    float rho;
    if (q > f[F_BAND]) rho = f[F_RHO];
    else if (q < -f[F_BAND]) rho = 0.0f;
    else return xnan();
    const float gX = fmaf(cx, cy, -sz * sx), gY = fmaf(cy, cz, -sx * sy), gZ = fmaf(cz, cx, -sy * sz);
    const float g1 = is * fmaf(gZ, c.vz, fmaf(gY, c.vy, gX * c.vx));
    // error of g1 (trigonometry, velocity, position) and of g (position slack)
    const float dg1 = fmaf(1e-5f, fabsf(g1), ais * c.vmax * fmaf(16.0f * ais, c.eps, 1e-5f));
    const float eg = 2.4494898f * ais * c.eps;
    const float Mg = fmaf(4.0f * is * is, c.vmax * c.vmax, 2.4494898f * ais * c.acc) * 1.01f + 1e-20f;
    const float th = f[4], band = f[F_BAND];
    float t2 = 0.0f;
    if (th - fabsf(g) > band) {  // inside |g| < th: both edges of the band
        const float T = th - band - eg;
        if (T - fabsf(g) > 0.0f)
            t2 = fminf(gap_time(T - g, g1 + dg1, Mg), gap_time(T + g, -g1 + dg1, Mg));
    } else {  // outside: the nearer edge
        const float T = th + band + eg;
        if (g > T) t2 = gap_time(g - T, -g1 + dg1, Mg);
        else if (g < -T) t2 = gap_time(-T - g, g1 + dg1, Mg);
    }
    t = fmaxf(t, t2);
    return rho;
}

template <int D, int LM = kLeafAll>
XRP_HD float coll_dc(const SceneDev& S, const Node& c, float x, float y, float z, const CurveDir& u, float& t);

// item_dm's decisions; the container distances become curve bounds.
template <int D, int LM = kLeafAll>
XRP_HD float item_dc(const SceneDev& S, int id, float x, float y, float z, const CurveDir& u, float& t) {
    const Node& n = S.nodes[id];
    if (n.type <= N_GYROID) return leaf_dc<LM>(n, x, y, z, u, t);
    if (n.type == N_TESS) {
        if constexpr (D > 0) {
            const float* f = n.f;
            float mo = fminf(fminf(fminf(x - f[0], f[1] - x), fminf(y - f[2], f[3] - y)),
                             fminf(z - f[4], f[5] - z));
            const float ob[6] = {f[0], f[1], f[2], f[3], f[4], f[5]};
            if (mo < -f[6]) {  // outside: zero until the curve can enter the bounds
                t = fmaxf(curve_time(-mo, u), box_curve_entry(ob, x, y, z, u));
                return 0.0f;
            }
            if (!(mo > f[6])) { t = 0.0f; return xnan(); }
            float qx = (x - f[20]) * f[17], qy = (y - f[21]) * f[18], qz = (z - f[22]) * f[19];
            float nx = floorf(qx), ny = floorf(qy), nz = floorf(qz);
            float bq = f[23];
            float fr = fminf(fminf(fminf(qx - nx, 1.0f - (qx - nx)), fminf(qy - ny, 1.0f - (qy - ny))),
                             fminf(qz - nz, 1.0f - (qz - nz)));
            if (!(fr > bq)) { t = 0.0f; return xnan(); }
            float fc = fminf(fminf(fminf(qx - nx, 1.0f - (qx - nx)) * fabsf(f[14]),
                                   fminf(qy - ny, 1.0f - (qy - ny)) * fabsf(f[15])),
                             fminf(qz - nz, 1.0f - (qz - nz)) * fabsf(f[16]));
            float fx = fmaf(-f[14], nx, x), fy = fmaf(-f[15], ny, y), fz = fmaf(-f[16], nz, z);
            float mu = fminf(fminf(fminf(fx - f[7], f[8] - fx), fminf(fy - f[9], f[10] - fy)),
                             fminf(fz - f[11], f[12] - fz));
            if (mu < -f[13]) { t = curve_time(fminf(fminf(mo, fc), -mu), u); return 0.0f; }
            if (!(mu > f[13])) { t = 0.0f; return xnan(); }
            float tk;
            float r = coll_dc<D - 1, LM>(S, S.nodes[n.a], fx, fy, fz, u, tk);
            // the outer bounds, the fold's cell and the unit-cell bounds, face
            // by face along the curve (their distances alone bound it too)
            const float ub[6] = {f[7], f[8], f[9], f[10], f[11], f[12]};
            float cb[6];
            for (int a = 0; a < 3; a++) {
                const float q0 = fmaf(a == 0 ? nx : (a == 1 ? ny : nz), f[14 + a], f[20 + a]);
                const float q1 = q0 + f[14 + a];
                cb[2 * a] = fminf(q0, q1);
                cb[2 * a + 1] = fmaxf(q0, q1);
            }
            // band of the fold (q units) as a world distance, per axis at most
            const float bw = bq * fmaxf(fabsf(f[14]), fmaxf(fabsf(f[15]), fabsf(f[16])));
            for (int a = 0; a < 6; a++) cb[a] += (a & 1) ? -bw : bw;
            const float tcon = fminf(fminf(box_curve_time(ob, x, y, z, u), box_curve_time(cb, x, y, z, u)),
                                     box_curve_time(ub, fx, fy, fz, u));
            t = fminf(fmaxf(tcon, curve_time(fminf(fminf(mo, fc), mu), u)), tk);
            return r;
        }
    }
    t = 0.0f;
    if (n.type == N_VOXEL) return voxel32(S.vols[n.a], n.f[0], x, y, z, S.hier_zero_guard);
    return xnan();
}

// coll_dm's decisions; the candidates' bounds, capped by the list cell's
// faces or clearance as curve bounds.
template <int D, int LM>
XRP_HD float coll_dc(const SceneDev& S, const Node& c, float x, float y, float z, const CurveDir& u, float& t) {
    const int32_t* kids = S.child + c.a;
    int cnt = c.b;
    const int32_t* list = nullptr;
    t = kFar;
    if (c.flags & C_ACCEL) {
        int G = (c.flags >> 16) & 0xff;
        float ux = (x - c.f[0]) * c.f[3], uy = (y - c.f[1]) * c.f[4], uz = (z - c.f[2]) * c.f[5];
        int ix = (int)floorf(ux), iy = (int)floorf(uy), iz = (int)floorf(uz);
        ix = ix < 0 ? 0 : (ix >= G ? G - 1 : ix);
        iy = iy < 0 ? 0 : (iy >= G ? G - 1 : iy);
        iz = iz < 0 ? 0 : (iz >= G ? G - 1 : iz);
        float m = 3.0e38f;
        if (ix > 0) m = fminf(m, (ux - (float)ix) / c.f[3]);
        if (ix < G - 1) m = fminf(m, ((float)(ix + 1) - ux) / c.f[3]);
        if (iy > 0) m = fminf(m, (uy - (float)iy) / c.f[4]);
        if (iy < G - 1) m = fminf(m, ((float)(iy + 1) - uy) / c.f[4]);
        if (iz > 0) m = fminf(m, (uz - (float)iz) / c.f[5]);
        if (iz < G - 1) m = fminf(m, ((float)(iz + 1) - uz) / c.f[5]);
        // the cell's inner faces along the curve (world distance = grid distance * cell size)
        float tf = kFar;
        {
            const float M = u.acc * 1.01f + 1e-20f;
            const float gu[3] = {ux, uy, uz}, vv[3] = {u.vx, u.vy, u.vz};
            const int ii[3] = {ix, iy, iz};
            for (int a = 0; a < 3; a++) {
                const float h = c.f[8 + a];
                if (ii[a] > 0) {
                    const float gap = (gu[a] - (float)ii[a]) * h - u.eps;
                    tf = gap > 0.0f ? fminf(tf, gap_time(gap, -vv[a] + 1e-6f * u.vmax, M)) : 0.0f;
                }
                if (ii[a] < G - 1) {
                    const float gap = ((float)(ii[a] + 1) - gu[a]) * h - u.eps;
                    tf = gap > 0.0f ? fminf(tf, gap_time(gap, vv[a] + 1e-6f * u.vmax, M)) : 0.0f;
                }
            }
        }
        const int cell = f2i(c.f[6]) + (iz * G + iy) * G + ix;
        t = fmaxf(fmaxf(curve_time(fmaxf(fmaxf(m, 0.0f), S.clear[cell]), u), fminf(tf, kFar)), 0.0f);
        const int32_t* off = S.cells + cell;
        list = S.items + off[0];
        cnt = off[1] - off[0];
    }
    const bool greedy = (c.flags & C_GREEDY) != 0;
    float sum = 0.0f, sabs = 0.0f;
    bool unc = false, done = false;
    // uniform greedy collections: inside a child (for certain) its exit alone
    // bounds the curve (see coll_dr_uniform)
    const bool uniform = (c.flags & C_UNIFORM) != 0;
    for (int k = 0; k < cnt; k++) {
        float tk;
        float r = item_dc<D, LM>(S, list ? list[k] : kids[k], x, y, z, u, tk);
        if (uniform && !unc && r > 0.0f) {
            t = tk;
            return r;
        }
        t = fminf(t, tk);
        if (done) continue;
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

// density32 at one point and the curve bound t (ray parameter units) of the
// samples ahead that share its density; d: the world ray direction.
template <int DEPTH, bool DEFS, int LM = kLeafAll>
XRP_HD float dens_curve32(const SceneDev& S, float x, float y, float z, const float* d, float& t) {
    CurveDir u;
    u.vx = d[0]; u.vy = d[1]; u.vz = d[2];
    if constexpr (DEFS) deform_jvp32(S, x, y, z, u.vx, u.vy, u.vz);
    u.vmax = S.curve_vmax;
    u.acc = S.curve_acc;
    u.eps = S.m_slack;
    const Node& r = S.nodes[S.root];
    float rho;
    if (r.type <= N_GYROID) rho = leaf_dc<LM>(r, x, y, z, u, t);
    else if (r.type == N_COLL) rho = coll_dc<DEPTH, LM>(S, r, x, y, z, u, t);
    else rho = item_dc<DEPTH, LM>(S, S.root, x, y, z, u, t);
    t = fmaxf(t, 0.0f) * 0.99999f;
    return rho;
}


}  // namespace xrp
