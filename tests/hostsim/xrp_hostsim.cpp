// xrp_hostsim.cpp -- TEST HARNESS ONLY: runs the engine's per-pixel code
// (xrp_device.h) on CPU threads so that its guard-band logic, flattening and
// lattices can be checked against the FP64 oracle without a GPU.  The product
// never loads this library; on the GPU the same code runs in xrp_engine.cu.
#include <cstring>
#include <thread>
#include <vector>

#include "../../xray_projection_render_gb300/csrc/xrp_device.h"
#include "../../xray_projection_render_gb300/csrc/xrp_scene.h"

using namespace xrp;

extern "C" __attribute__((visibility("default"))) int hs_render(
    const char* obj_json, const char* def_json, const float* vol, int nx, int ny, int nz,
    const double* cams, int ncams, int res, int integration, double ds, double R, double ff,
    double dm, float* out, unsigned long long* stats, int nthreads, const int* rays, long nrays,
    int force_general, int trace, int fine_lists, char* err, int errlen) {
    try {
        std::vector<HVolume> ext;
        if (vol) {
            HVolume v;
            v.nx = nx;
            v.ny = ny;
            v.nz = nz;
            v.data.assign(vol, vol + (size_t)nx * ny * nz);
            ext.push_back(v);
        }
        HostScene hs = load_scene(obj_json, def_json, ext);
        std::vector<ViewDev> views(ncams);
        double fov_max = 0;
        for (int c = 0; c < ncams; c++) {
            const double* p = cams + 20 * c;
            view_from_camera(p, p + 3, p[19], views[c]);
            fov_max = std::max(fov_max, std::fabs(p[19]));
        }
        HostPrepared hp = prepare_host(hs, res, integration, ds, R, ff, dm, fov_max, trace != 0, fine_lists != 0);
        for (size_t k = 0; k < hp.vols.size(); k++) {
            hp.vols[k].data = hs.vols[k].data.data();
            hp.vols[k].data64 = hs.vols[k].data64.empty() ? nullptr : hs.vols[k].data64.data();
        }
        SceneDev S = hp.S;
        S.nodes = hp.fs.nodes.data();
        S.nodes64 = hp.fs.nodes64.data();
        S.child = hp.fs.child.data();
        S.cells = hp.fs.cells.data();
        S.items = hp.fs.items.data();
        S.clear = hp.fs.clear.data();
        S.defs = hp.fs.defs.data();
        S.vols = hp.vols.data();
        Lattice L = hp.hl.hdr;
        L.s64 = hp.hl.s64.data();
        L.t32 = hp.hl.t32.data();
        L.fstart = hp.hl.fstart.data();
        L.f64 = hp.hl.f64.data();
        L.ft32 = hp.hl.ft32.data();
        RenderParams P = hp.P;
        P.nviews = ncams;
        P.xs = hp.xs.data();
        P.xsf = hp.xsf.data();
        bool vf = hp.volume_fast && !force_general;
        long total = rays ? nrays : (long)ncams * res * res;
        std::vector<unsigned long long> s0(nthreads, 0), s1(nthreads, 0);
        auto work = [&](int t) {
            for (long q = t; q < total; q += nthreads) {
                int v, i, j;
                if (rays) {
                    v = rays[3 * q];
                    i = rays[3 * q + 1];
                    j = rays[3 * q + 2];
                } else {
                    v = (int)(q / ((long)res * res));
                    i = (int)((q / res) % res);
                    j = (int)(q % res);
                }
                RayStats st{0, 0};
                float val;
                bool hier = integration == 1;
                if (trace) {
                    unsigned ev = 0;
                    if (S.affine)
                        val = hier ? trace_pixel<true, kMaxDepth, true, true>(S, L, P, views[v], i, j, ev)
                                   : trace_pixel<false, kMaxDepth, true, true>(S, L, P, views[v], i, j, ev);
                    else if (trace == 2)  // curved-ray certificates
                        val = hier ? trace_pixel<true, kMaxDepth, true, false, true>(S, L, P, views[v], i, j, ev)
                                   : trace_pixel<false, kMaxDepth, true, false, true>(S, L, P, views[v], i, j, ev);
                    else
                        val = hier ? trace_pixel<true, kMaxDepth, true, false>(S, L, P, views[v], i, j, ev)
                                   : trace_pixel<false, kMaxDepth, true, false>(S, L, P, views[v], i, j, ev);
                    st.samples = ev;
                } else if (hier)
                    val = vf ? render_pixel<true, true>(S, L, P, views[v], i, j, st)
                             : render_pixel<true, false>(S, L, P, views[v], i, j, st);
                else
                    val = vf ? render_pixel<false, true>(S, L, P, views[v], i, j, st)
                             : render_pixel<false, false>(S, L, P, views[v], i, j, st);
                out[q] = val;
                s0[t] += st.samples;
                s1[t] += st.fallbacks;
            }
        };
        std::vector<std::thread> th;
        for (int t = 1; t < nthreads; t++) th.emplace_back(work, t);
        work(0);
        for (auto& x : th) x.join();
        if (stats) {
            stats[0] = stats[1] = 0;
            for (int t = 0; t < nthreads; t++) {
                stats[0] += s0[t];
                stats[1] += s1[t];
            }
        }
        return 0;
    } catch (const std::exception& ex) {
        if (err && errlen > 0) {
            strncpy(err, ex.what(), errlen - 1);
            err[errlen - 1] = 0;
        }
        return 2;
    }
}

// Density (FP32 guarded; NaN when uncertain) and distance certificate
// (margin32, world units) at FP64 points rounded to FP32, for the soundness
// tests of the certificates; also the fused evaluator's pair, which must be
// identical, and with `dirs` (affine chains) the ray evaluator's density and
// ray bound along each direction.  R and fov enter the error analysis as for a
// render with those cameras.
extern "C" __attribute__((visibility("default"))) int hs_margin(
    const char* obj_json, const char* def_json, const double* pts, long n, double R, double fov,
    double ds, float* rho_out, float* m_out, float* rho2_out, float* m2_out, const double* dirs,
    float* rho3_out, float* t_out, int* affine_out, char* err, int errlen) {
    try {
        HostScene hs = load_scene(obj_json, def_json, {});
        HostPrepared hp = prepare_host(hs, 8, 0, ds, R, 0.0, 1.0, fov);
        SceneDev S = hp.S;
        S.nodes = hp.fs.nodes.data();
        S.nodes64 = hp.fs.nodes64.data();
        S.child = hp.fs.child.data();
        S.cells = hp.fs.cells.data();
        S.items = hp.fs.items.data();
        S.clear = hp.fs.clear.data();
        S.defs = hp.fs.defs.data();
        S.vols = hp.vols.data();
        for (long q = 0; q < n; q++) {
            float x = (float)pts[3 * q], y = (float)pts[3 * q + 1], z = (float)pts[3 * q + 2];
            rho_out[q] = density32<kMaxDepth, true>(S, x, y, z);
            m_out[q] = margin32<kMaxDepth, true>(S, x, y, z);
            rho2_out[q] = dens_margin32<kMaxDepth, true>(S, x, y, z, m2_out[q]);
            if (dirs && S.affine) {
                float d[3] = {(float)dirs[3 * q], (float)dirs[3 * q + 1], (float)dirs[3 * q + 2]};
                RayDir u = ray_dir32(S, d);
                rho3_out[q] = dens_ray32<kMaxDepth, true>(S, x, y, z, u, kFar, t_out[q]);
            }
        }
        if (affine_out) *affine_out = S.affine;
        return 0;
    } catch (const std::exception& ex) {
        if (err && errlen > 0) {
            strncpy(err, ex.what(), errlen - 1);
            err[errlen - 1] = 0;
        }
        return 2;
    }
}

// sqrt_lt_threshold for each of n radii.
extern "C" __attribute__((visibility("default"))) void hs_sqrt_threshold(const double* r, long n, double* out) {
    for (long q = 0; q < n; q++) out[q] = sqrt_lt_threshold(r[q]);
}

// The FP64 densities of the engine's two FP64 evaluators at FP64 points
// (density64: every primitive in FP64; density_hyb: the FP64 pass's, FP32
// decisions where they are certain), for the exactness test against the
// oracle.
extern "C" __attribute__((visibility("default"))) int hs_density64(
    const char* obj_json, const char* def_json, const double* pts, long n, double* d64_out, double* hyb_out,
    char* err, int errlen) {
    try {
        HostScene hs = load_scene(obj_json, def_json, {});
        HostPrepared hp = prepare_host(hs, 8, 0, 0.01, 4.0, 0.0, 1.0, 40.0);
        SceneDev S = hp.S;
        S.nodes = hp.fs.nodes.data();
        S.nodes64 = hp.fs.nodes64.data();
        S.child = hp.fs.child.data();
        S.cells = hp.fs.cells.data();
        S.items = hp.fs.items.data();
        S.clear = hp.fs.clear.data();
        S.defs = hp.fs.defs.data();
        S.vols = hp.vols.data();
        for (long q = 0; q < n; q++) {
            d64_out[q] = density64(S, pts[3 * q], pts[3 * q + 1], pts[3 * q + 2]);
            hyb_out[q] = density_hyb(S, pts[3 * q], pts[3 * q + 1], pts[3 * q + 2]);
        }
        return 0;
    } catch (const std::exception& ex) {
        if (err && errlen > 0) {
            strncpy(err, ex.what(), errlen - 1);
            err[errlen - 1] = 0;
        }
        return 2;
    }
}

// FP32 march rays of the listed pixels by the two setups (double-float FP32
// and FP64): out[q] = pc[3], d32[3] of each, for the equality test of the
// double-float arithmetic.
extern "C" __attribute__((visibility("default"))) int hs_ray_setup(const double* cams, int ncams, int res,
                                                                   double R, const int* rays, long n,
                                                                   float* out_df, float* out_64) {
    std::vector<ViewDev> views(ncams);
    for (int c = 0; c < ncams; c++) {
        const double* p = cams + 20 * c;
        view_from_camera(p, p + 3, p[19], views[c]);
    }
    HostLattice hl = build_lattice(R, 0.01, false);
    std::vector<double> xs = pixel_table(res);
    std::vector<float> xsf(2 * xs.size());
    for (size_t q = 0; q < xs.size(); q++) {
        xsf[2 * q] = (float)xs[q];
        xsf[2 * q + 1] = (float)(xs[q] - (double)xsf[2 * q]);
    }
    for (long q = 0; q < n; q++) {
        const ViewDev& V = views[rays[3 * q]];
        int i = rays[3 * q + 1], j = rays[3 * q + 2];
        Ray a, b;
        setup_ray32_df(V, xsf.data(), i, j, hl.hdr.s_c2, a);
        Ray64 r64;
        setup_ray64_fast(V, xs.data(), i, j, r64);
        setup_ray32(r64, hl.hdr.s_c, b);
        for (int k = 0; k < 3; k++) {
            out_df[6 * q + k] = a.pc[k];
            out_df[6 * q + 3 + k] = a.d32[k];
            out_64[6 * q + k] = b.pc[k];
            out_64[6 * q + 3 + k] = b.d32[k];
        }
    }
    return 0;
}

// Curved-ray certificates at FP64 points along FP64 world directions (CPU
// build): the density and the curve bound t, for the soundness tests.
extern "C" __attribute__((visibility("default"))) int hs_curve(const char* obj_json, const char* def_json,
                                                               const double* pts, const double* dirs, long n,
                                                               double R, double fov, double ds, float* rho_out,
                                                               float* t_out, char* err, int errlen) {
    try {
        HostScene hs = load_scene(obj_json, def_json, {});
        HostPrepared hp = prepare_host(hs, 8, 0, ds, R, 0.0, 1.0, fov);
        SceneDev S = hp.S;
        S.nodes = hp.fs.nodes.data();
        S.nodes64 = hp.fs.nodes64.data();
        S.child = hp.fs.child.data();
        S.cells = hp.fs.cells.data();
        S.items = hp.fs.items.data();
        S.clear = hp.fs.clear.data();
        S.defs = hp.fs.defs.data();
        S.vols = hp.vols.data();
        for (long q = 0; q < n; q++) {
            float d[3] = {(float)dirs[3 * q], (float)dirs[3 * q + 1], (float)dirs[3 * q + 2]};
            rho_out[q] = dens_curve32<kMaxDepth, true>(S, (float)pts[3 * q], (float)pts[3 * q + 1],
                                                       (float)pts[3 * q + 2], d, t_out[q]);
        }
        return 0;
    } catch (const std::exception& ex) {
        if (err && errlen > 0) {
            strncpy(err, ex.what(), errlen - 1);
            err[errlen - 1] = 0;
        }
        return 2;
    }
}
