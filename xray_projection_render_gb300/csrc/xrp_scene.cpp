// xrp_scene.cpp -- scene loading, flattening and error analysis (host).
#include "xrp_scene.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>

// cells per axis of candidate lists, per cube root of the children (build
// knobs): XRP_LIST_GRID by default, XRP_LIST_GRID_FINE where the caller asks
// for fine lists, XRP_LIST_GRID_TRACE for uniform collections rendered by
// certificate tracing
#ifndef XRP_LIST_GRID
#define XRP_LIST_GRID 1.6
#endif
#ifndef XRP_LIST_GRID_FINE
#define XRP_LIST_GRID_FINE 4.8
#endif
#ifndef XRP_LIST_GRID_TRACE
#define XRP_LIST_GRID_TRACE 1.2
#endif

namespace xrp {

static const double kU = 5.9604644775390625e-08;  // 2^-24, FP32 unit roundoff
static const double kSafety = 2.0;

// The smallest s whose correctly rounded square root reaches r (sqrt is
// monotonic, so sqrt(s) < r exactly when s < it).
double sqrt_lt_threshold(double r) {
    if (std::isnan(r) || std::isinf(r)) return r;
    if (!(r > 0.0)) return 0.0;  // sqrt(s) < r never holds for s >= 0
    double s = r * r;
    if (std::isinf(s)) s = std::numeric_limits<double>::max();
    while (s > 0.0 && std::sqrt(s) >= r) s = std::nextafter(s, 0.0);
    while (std::sqrt(s) < r) s = std::nextafter(s, std::numeric_limits<double>::infinity());
    return s;
}
static const double kInf = std::numeric_limits<double>::infinity();

// ---------------------------------------------------------------------------
// loading (objects/objects.go FromMap methods, deformations.go)
// ---------------------------------------------------------------------------

namespace {

const JValue* need(const JValue& m, const char* key) { return m.get(key); }

double to_float(const JValue* v, const std::string& err) {  // ToFloat64, objects.go:261-270
    if (!v || !v->is_num()) throw SchemaError(err);
    return v->num;
}

// ToVec (objects.go:272-282): numeric elements are copied, others skipped.
void to_vec(const JValue* v, double out[3], const std::string& err) {
    if (!v || v->kind != JValue::Array) throw SchemaError(err);
    if (v->arr.size() > 3) throw SchemaError(err + " (more than 3 elements)");
    for (size_t i = 0; i < v->arr.size(); i++)
        if (v->arr[i].is_num()) out[i] = v->arr[i].num;
}

// Vec3 parsed element by element with ToFloat64 (Sphere, Gyroid).
void to_vec_strict(const JValue* v, double out[3], const char* key) {
    if (!v || v->kind != JValue::Array) throw SchemaError(std::string(key) + " is not a Vec3");
    if (v->arr.size() > 3) throw SchemaError(std::string(key) + " is not a Vec3");
    for (size_t i = 0; i < v->arr.size(); i++) {
        if (!v->arr[i].is_num())
            throw SchemaError(std::string(key) + "[" + std::to_string(i) + "] is not a float64");
        out[i] = v->arr[i].num;
    }
}

struct Loader {
    HostScene& hs;
    const std::vector<HVolume>& ext;

    int add(HNode&& n) {
        hs.nodes.push_back(std::move(n));
        return (int)hs.nodes.size() - 1;
    }

    int object(const JValue& m, bool top) {
        if (m.kind != JValue::Object) throw SchemaError("object is not a map");
        const JValue* tv = m.get("type");
        std::string t = (tv && tv->kind == JValue::String) ? tv->str : std::string();
        HNode n;
        if (t == "sphere") {  // objects.go:42-61
            n.type = N_SPHERE;
            to_vec_strict(need(m, "center"), n.d, "center");
            n.d[3] = to_float(need(m, "radius"), "radius is not a float64");
            n.d[4] = to_float(need(m, "rho"), "rho is not a float64");
        } else if (t == "cube") {  // objects.go:100-117
            n.type = N_BOX;
            to_vec_strict(need(m, "center"), n.d, "center");
            double s = to_float(need(m, "side"), "side is not a float64");
            n.d[3] = n.d[4] = n.d[5] = s;
            n.d[6] = to_float(need(m, "rho"), "rho is not a float64");
        } else if (t == "box") {  // objects.go:148-169
            n.type = N_BOX;
            to_vec(need(m, "center"), n.d, "center is not a Vec3");
            to_vec(need(m, "sides"), n.d + 3, "sides is not a Vec3");
            n.d[6] = to_float(need(m, "rho"), "rho is not a float64");
        } else if (t == "cylinder") {  // objects.go:306-332
            n.type = N_CYL;
            to_vec(need(m, "p0"), n.d, "p0 is not a Vec3");
            to_vec(need(m, "p1"), n.d + 3, "p0 is not a Vec3");
            n.d[6] = to_float(need(m, "radius"), "radius is not a float64");
            n.d[7] = m.get("rho") ? to_float(m.get("rho"), "rho is not a float64") : 1.0;
        } else if (t == "parallelepiped") {  // objects.go:209-245
            n.type = N_PPD;
            double o[3] = {0}, v0[3] = {0}, v1[3] = {0}, v2[3] = {0};
            to_vec(need(m, "origin"), o, "origin is not a Vec3");
            to_vec(need(m, "v0"), v0, "v0 is not a Vec3");
            to_vec(need(m, "v1"), v1, "v1 is not a Vec3");
            to_vec(need(m, "v2"), v2, "v2 is not a Vec3");
            n.d[12] = to_float(need(m, "rho"), "rho is not a float64");
            for (int i = 0; i < 3; i++) n.d[i] = o[i];
            inv3_cols(v0, v1, v2, n.d + 3);
            // edge lengths (Vec3.Len) for MinFeatureSize (objects.go:257-259)
            n.d[13] = std::sqrt(v0[0] * v0[0] + v0[1] * v0[1] + v0[2] * v0[2]);
            n.d[14] = std::sqrt(v1[0] * v1[0] + v1[1] * v1[1] + v1[2] * v1[2]);
            n.d[15] = std::sqrt(v2[0] * v2[0] + v2[1] * v2[1] + v2[2] * v2[2]);
        } else if (t == "gyroid") {  // objects.go:983-1012
            n.type = N_GYROID;
            to_vec_strict(need(m, "center"), n.d, "center");
            n.d[3] = to_float(need(m, "scale"), "scale is not a float64");
            n.d[4] = to_float(need(m, "thickness"), "thickness is not a float64");
            n.d[5] = to_float(need(m, "rho"), "rho is not a float64");
        } else if (t == "object_collection" && top) {  // objects.go:381-420
            return collection(m, false);
        } else if (t == "tessellated_obj_coll") {  // objects.go:536-566
            const JValue* uc = m.get("uc");
            if (!uc || uc->kind != JValue::Object) throw SchemaError("uc is not a map");
            const JValue* objs = uc->get("objects");
            if (!objs || objs->kind != JValue::Object) throw SchemaError("objects is not a map");
            int coll = collection(*objs, true);  // UnitCell forces GreedyDensEval (objects.go:487)
            n.type = N_TESS;
            static const char* names[6] = {"xmin", "xmax", "ymin", "ymax", "zmin", "zmax"};
            for (int i = 0; i < 6; i++)
                n.d[6 + i] = to_float(uc->get(names[i]), std::string(names[i]) + " is not a float64");
            for (int i = 0; i < 6; i++)
                n.d[i] = to_float(m.get(names[i]), std::string(names[i]) + " is not a float64");
            n.sub = coll;
        } else if (t == "voxel_grid") {  // objects.go:715-787
            n.type = N_VOXEL;
            n.vol = voxel(m);
        } else {
            throw SchemaError(top ? "unknown object type `" + t + "`" : std::string("unknown object type"));
        }
        return add(std::move(n));
    }

    int collection(const JValue& m, bool force_greedy) {
        HNode c;
        c.type = N_COLL;
        c.clip = true;
        const JValue* g = m.get("greedy_dens_eval");
        c.greedy = force_greedy || (g && g->kind == JValue::Bool && g->b);
        const JValue* objs = m.get("objects");
        if (!objs || objs->kind != JValue::Array) throw SchemaError("objects is not a list");
        static const char* ok[] = {"sphere", "cube", "box", "cylinder", "parallelepiped", "gyroid",
                                   "tessellated_obj_coll", "voxel_grid"};
        for (auto& o : objs->arr) {
            const JValue* tv = o.kind == JValue::Object ? o.get("type") : nullptr;
            bool known = false;
            if (tv && tv->kind == JValue::String)
                for (auto* k : ok) known |= (tv->str == k);
            if (!known) throw SchemaError("unknown object type");
            c.kids.push_back(object(o, false));
        }
        return add(std::move(c));
    }

    // VoxelGrid.FromMap / VoxelGridFromRaw (objects.go:715-787, 892-958),
    // plus the in-memory extension {"volume": k}.
    int voxel(const JValue& m) {
        const JValue* vi = m.get("volume");
        if (vi && vi->is_num()) {
            int k = (int)vi->num;
            if (k < 0 || k >= (int)ext.size()) throw SchemaError("volume index out of range");
            hs.vols.push_back(ext[k]);
            return (int)hs.vols.size() - 1;
        }
        const JValue* path = m.get("path");
        if (!path || path->kind != JValue::String) throw SchemaError("nx is not an int");
        std::string p = path->str;
        size_t dot = p.find_last_of('.');
        std::string ext_s = dot == std::string::npos ? p : p.substr(dot + 1);
        for (auto& ch : ext_s) ch = (char)tolower(ch);
        if (ext_s != "raw") throw SchemaError("only raw files are supported");
        const JValue* res = m.get("resolution");
        if (!res || res->kind != JValue::Array)
            throw SchemaError("resolution must be provided for raw files as a list of 3 integers");
        if (res->arr.size() != 3) throw SchemaError("resolution must be a list of 3 integers");
        int r[3];
        for (int i = 0; i < 3; i++) {
            if (!res->arr[i].is_num())
                throw SchemaError("resolution[" + std::to_string(i) + "] has unsupported type");
            r[i] = (int)res->arr[i].num;
        }
        std::string dtype = "uint8";
        const JValue* dt = m.get("dtype");
        if (dt && dt->kind == JValue::String) dtype = dt->str;
        int bpe;
        if (dtype == "uint8") bpe = 1;
        else if (dtype == "uint16") bpe = 2;
        else if (dtype == "uint32" || dtype == "float32") bpe = 4;
        else if (dtype == "float64") bpe = 8;
        else throw SchemaError("unsupported data type: " + dtype);
        FILE* fp = fopen(p.c_str(), "rb");
        if (!fp) throw SchemaError("error reading file: " + p);
        std::vector<unsigned char> buf;
        unsigned char tmp[1 << 16];
        size_t got;
        while ((got = fread(tmp, 1, sizeof(tmp), fp)) > 0) buf.insert(buf.end(), tmp, tmp + got);
        fclose(fp);
        size_t n = (size_t)r[0] * r[1] * r[2];
        if (r[0] <= 0 || r[1] <= 0 || r[2] <= 0 || buf.size() != n * (size_t)bpe)
            throw SchemaError("file size (" + std::to_string(buf.size()) +
                              ") does not match expected size (" + std::to_string(n * bpe) +
                              ") for type " + dtype);
        HVolume v;
        v.nx = r[0];
        v.ny = r[1];
        v.nz = r[2];
        v.data.resize(n);
        v.data64.resize(n);
        bool exact32 = true;
        for (size_t i = 0; i < n; i++) {
            const unsigned char* b = &buf[i * bpe];
            double val;
            if (dtype == "uint8") {
                val = (double)b[0] / 255.0;
            } else if (dtype == "uint16") {
                unsigned u = (unsigned)b[0] | ((unsigned)b[1] << 8);
                val = (double)u / 65535.0;
            } else if (dtype == "uint32") {
                uint32_t u = (uint32_t)b[0] | ((uint32_t)b[1] << 8) | ((uint32_t)b[2] << 16) |
                             ((uint32_t)b[3] << 24);
                val = (double)u / 4294967295.0;
            } else if (dtype == "float32") {
                uint32_t u = (uint32_t)b[0] | ((uint32_t)b[1] << 8) | ((uint32_t)b[2] << 16) |
                             ((uint32_t)b[3] << 24);
                float f;
                memcpy(&f, &u, 4);
                val = (double)f;
            } else {
                uint64_t u = 0;
                for (int k = 7; k >= 0; k--) u = (u << 8) | b[k];
                memcpy(&val, &u, 8);
            }
            v.data64[i] = val;
            v.data[i] = (float)val;
            if ((double)v.data[i] != val) exact32 = false;
        }
        if (exact32) v.data64.clear();
        hs.vols.push_back(std::move(v));
        return (int)hs.vols.size() - 1;
    }

    // Mat3FromCols(v0, v1, v2).Inv() by the adjugate, column-major out;
    // a singular matrix gives zeros (as the FloatEqual(det, 0) branch).
    static void inv3_cols(const double* v0, const double* v1, const double* v2, double* out) {
        double m[9] = {v0[0], v0[1], v0[2], v1[0], v1[1], v1[2], v2[0], v2[1], v2[2]};
        double c00 = m[4] * m[8] - m[7] * m[5];
        double c01 = m[7] * m[2] - m[1] * m[8];
        double c02 = m[1] * m[5] - m[4] * m[2];
        double det = m[0] * c00 + m[3] * c01 + m[6] * c02;
        if (det == 0.0 || std::fabs(det) < 1e-300) {
            for (int i = 0; i < 9; i++) out[i] = 0.0;
            return;
        }
        double inv[9];
        inv[0] = c00;
        inv[1] = m[5] * m[6] - m[3] * m[8];
        inv[2] = m[3] * m[7] - m[6] * m[4];
        inv[3] = c01;
        inv[4] = m[0] * m[8] - m[6] * m[2];
        inv[5] = m[6] * m[1] - m[0] * m[7];
        inv[6] = c02;
        inv[7] = m[3] * m[2] - m[0] * m[5];
        inv[8] = m[0] * m[4] - m[3] * m[1];
        double s = 1.0 / det;
        for (int i = 0; i < 9; i++) out[i] = inv[i] * s;
    }
};

void deformation(const JValue& m, std::vector<HDef>& out) {  // deformations.go:308-343
    if (m.kind != JValue::Object) throw SchemaError("deformation is not a map");
    const JValue* tv = m.get("type");
    if (!tv || tv->kind == JValue::Null) throw SchemaError("deformation type is nil");
    std::string t = tv->kind == JValue::String ? tv->str : std::string("?");
    auto list = [&](const char* key, size_t need_n, double* dst, const char* err) {
        const JValue* v = m.get(key);
        if (!v || v->kind != JValue::Array) throw SchemaError(err);
        if (v->arr.size() < need_n) throw SchemaError(std::string(key) + " has too few elements");
        for (size_t i = 0; i < need_n; i++) {
            if (!v->arr[i].is_num()) throw SchemaError(err);
            dst[i] = v->arr[i].num;
        }
    };
    HDef d;
    if (t == "gaussian") {
        d.type = D_GAUSSIAN;
        list("amplitudes", 3, d.d, "amplitudes must be a list");
        list("sigmas", 3, d.d + 3, "sigmas must be a list");
        list("centers", 3, d.d + 6, "centers must be a list");
    } else if (t == "linear") {
        d.type = D_LINEAR;
        list("strains", 6, d.d, "strains must be a list");
    } else if (t == "rigid") {
        d.type = D_RIGID;
        list("displacements", 3, d.d, "displacements must be a list");
    } else if (t == "sigmoid") {
        d.type = D_SIGMOID;
        d.d[0] = to_float(m.get("amplitude"), "amplitude must be a float");
        d.d[1] = to_float(m.get("center"), "center must be a float");
        d.d[2] = to_float(m.get("lengthscale"), "lengthscale must be a float");
        const JValue* dir = m.get("direction");
        if (!dir || dir->kind != JValue::String) throw SchemaError("direction must be a string");
        if (dir->str == "x") d.axis = 0;
        else if (dir->str == "y") d.axis = 1;
        else if (dir->str == "z") d.axis = 2;
        else throw SchemaError("Invalid direction");  // deformations.go:218-219 (fatal at Apply)
    } else if (t == "affine") {
        d.type = D_AFFINE;
        const JValue* mat = m.get("matrix");
        if (!mat || mat->kind != JValue::Array) throw SchemaError("matrix must be a list");
        if (mat->arr.size() != 3) throw SchemaError("matrix must have 3 rows");
        for (int i = 0; i < 3; i++) {
            const JValue& row = mat->arr[i];
            if (row.kind != JValue::Array) throw SchemaError("matrix row must be a list");
            if (row.arr.size() != 3) throw SchemaError("matrix row must have 3 elements");
            for (int j = 0; j < 3; j++) {
                if (!row.arr[j].is_num()) throw SchemaError("matrix element must be a float");
                d.d[3 * i + j] = row.arr[j].num;
            }
        }
    } else if (t == "composed") {
        const JValue* ds = m.get("deformations");
        if (!ds || ds->kind != JValue::Array) throw SchemaError("deformations must be a list");
        for (auto& sub : ds->arr) deformation(sub, out);
        return;
    } else {
        throw SchemaError("unknown deformation type " + t);
    }
    out.push_back(d);
}

}  // namespace

HostScene load_scene(const char* object_json, const char* deformation_json,
                     const std::vector<HVolume>& ext_vols) {
    HostScene hs;
    if (!object_json) throw SchemaError("object JSON is null");
    JValue obj = parse_json(object_json);
    Loader L{hs, ext_vols};
    hs.root = L.object(obj, true);
    if (deformation_json && deformation_json[0]) {
        JValue dj = parse_json(deformation_json);
        if (!(dj.kind == JValue::Object && dj.obj.empty())) deformation(dj, hs.defs);
    }
    return hs;
}

// MinFeatureSize of a node (objects.go:74-76, 123-125, 181-183, 257-259,
// 352-354, 440-446, 584-586, 857-860, 1034-1037): the length the reference's
// automatic step divides by five (main.go:350-353).
static double min_feature(const HostScene& hs, int id) {
    const HNode& n = hs.nodes[id];
    const double* d = n.d;
    switch (n.type) {
    case N_SPHERE: return d[3];
    case N_BOX: return 0.1 * std::min(d[3], std::min(d[4], d[5]));
    case N_CYL: return d[6];
    case N_PPD: return 0.2 * std::min(d[13], std::min(d[14], d[15]));
    case N_GYROID: return d[3] * d[4] * 0.1;
    case N_COLL: {
        double out = INFINITY;
        for (int k : n.kids) out = std::min(out, min_feature(hs, k));
        return out;
    }
    case N_TESS: return min_feature(hs, n.sub);
    case N_VOXEL: {
        const HVolume& v = hs.vols[n.vol];
        return 2.0 / (double)std::max(v.nx, std::max(v.ny, v.nz));
    }
    default: return INFINITY;
    }
}

double min_feature_size(const HostScene& hs) { return hs.root < 0 ? INFINITY : min_feature(hs, hs.root); }

HostScene volume_scene(const float* data_dev, int nx, int ny, int nz) {
    HostScene hs;
    HVolume v;
    v.ext = data_dev;
    v.nx = nx;
    v.ny = ny;
    v.nz = nz;
    hs.vols.push_back(v);
    HNode n;
    n.type = N_VOXEL;
    n.vol = 0;
    hs.nodes.push_back(n);
    hs.root = 0;
    return hs;
}

// ---------------------------------------------------------------------------
// bounds
// ---------------------------------------------------------------------------

struct Box3 {
    double lo[3] = {kInf, kInf, kInf};
    double hi[3] = {-kInf, -kInf, -kInf};
    bool empty() const { return !(lo[0] <= hi[0] && lo[1] <= hi[1] && lo[2] <= hi[2]); }
    void add(const double p[3]) {
        for (int a = 0; a < 3; a++) {
            lo[a] = std::min(lo[a], p[a]);
            hi[a] = std::max(hi[a], p[a]);
        }
    }
    void unite(const Box3& b) {
        for (int a = 0; a < 3; a++) {
            lo[a] = std::min(lo[a], b.lo[a]);
            hi[a] = std::max(hi[a], b.hi[a]);
        }
    }
    void dilate(double e) {
        for (int a = 0; a < 3; a++) {
            lo[a] -= e;
            hi[a] += e;
        }
    }
    bool bounded() const {
        for (int a = 0; a < 3; a++)
            if (!std::isfinite(lo[a]) || !std::isfinite(hi[a])) return false;
        return true;
    }
    double maxabs() const {
        double m = 0;
        for (int a = 0; a < 3; a++) m = std::max(m, std::max(std::fabs(lo[a]), std::fabs(hi[a])));
        return m;
    }
    static Box3 all() {
        Box3 b;
        for (int a = 0; a < 3; a++) {
            b.lo[a] = -kInf;
            b.hi[a] = kInf;
        }
        return b;
    }
};

// Inverse of a column-major 3x3 given as rows for the ppd: the edge vectors
// are the columns of inv(M).
static bool inv3_rowmajor(const double a[9], double out[9]) {
    double c00 = a[4] * a[8] - a[5] * a[7];
    double c01 = a[5] * a[6] - a[3] * a[8];
    double c02 = a[3] * a[7] - a[4] * a[6];
    double det = a[0] * c00 + a[1] * c01 + a[2] * c02;
    if (!(std::fabs(det) > 1e-300)) return false;
    double id = 1.0 / det;
    out[0] = c00 * id;
    out[1] = (a[2] * a[7] - a[1] * a[8]) * id;
    out[2] = (a[1] * a[5] - a[2] * a[4]) * id;
    out[3] = c01 * id;
    out[4] = (a[0] * a[8] - a[2] * a[6]) * id;
    out[5] = (a[2] * a[3] - a[0] * a[5]) * id;
    out[6] = c02 * id;
    out[7] = (a[1] * a[6] - a[0] * a[7]) * id;
    out[8] = (a[0] * a[4] - a[1] * a[3]) * id;
    return true;
}

// Edge matrix E (row-major, columns v0 v1 v2) of a parallelepiped from its
// stored inverse.
static bool ppd_edges(const HNode& n, double E[9]) {
    // stored inverse is column-major: Minv(row r, col c) = d[3 + c*3 + r]
    double Mi[9];
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) Mi[r * 3 + c] = n.d[3 + c * 3 + r];
    return inv3_rowmajor(Mi, E);
}

// Box where the exact density of a leaf can be non-zero, dilated by `e`.
static Box3 leaf_box(const HNode& n, double e) {
    Box3 b;
    const double* d = n.d;
    switch (n.type) {
    case N_SPHERE:
        for (int a = 0; a < 3; a++) {
            b.lo[a] = d[a] - std::fabs(d[3]) - e;
            b.hi[a] = d[a] + std::fabs(d[3]) + e;
        }
        break;
    case N_BOX:
        for (int a = 0; a < 3; a++) {
            double h = 0.5 * std::fabs(d[3 + a]);
            b.lo[a] = d[a] - h - e;
            b.hi[a] = d[a] + h + e;
        }
        break;
    case N_CYL:
        for (int a = 0; a < 3; a++) {
            b.lo[a] = std::min(d[a], d[3 + a]) - std::fabs(d[6]) - e;
            b.hi[a] = std::max(d[a], d[3 + a]) + std::fabs(d[6]) + e;
        }
        break;
    case N_PPD: {
        double E[9];
        if (!ppd_edges(n, E)) return Box3();  // singular: density is 0 everywhere
        for (int corner = 0; corner < 8; corner++) {
            double p[3];
            for (int a = 0; a < 3; a++) {
                p[a] = d[a];
                for (int c = 0; c < 3; c++)
                    if (corner & (1 << c)) p[a] += E[a * 3 + c];
            }
            b.add(p);
        }
        b.dilate(e);
        break;
    }
    case N_GYROID:
        return Box3::all();
    default:
        return Box3::all();
    }
    return b;
}

// ---------------------------------------------------------------------------
// flattening with guard bands
// ---------------------------------------------------------------------------

namespace {

struct Flattener {
    const HostScene& hs;
    FlatScene& fs;
    bool hier;
    bool tracing;  // certificate tracing renders this scene
    bool fine;     // fine candidate lists (flattening time traded for march time)
    std::vector<int> map;  // host node -> flat node

    static int32_t i_of_f(float f) {
        int32_t i;
        memcpy(&i, &f, 4);
        return i;
    }
    static float f_of_i(int32_t i) {
        float f;
        memcpy(&f, &i, 4);
        return f;
    }

    // Is v a multiple of 2^-12 with |v| < 4096 (then FP32 sums are exact)?
    static bool dyadic(double v) {
        if (!(std::fabs(v) < 4096.0)) return false;
        double s = v * 4096.0;
        return s == std::floor(s) && (double)(float)v == v;
    }

    struct Info {
        bool dyadic = false;   // every output value is dyadic (see above)
        double maxabs = 0.0;   // max |output|
        Box3 box;              // where FP32 may report non-zero or uncertain
        bool can_be_positive = false;
        Box3 pos_box;          // where the exact output may be positive
        // spheres and cylinders: `box` is also contained in the capsule of
        // radius reff around the segment p0-p1 (p0 == p1 for a sphere); a
        // tighter test for the per-cell candidate lists than the box
        bool capsule = false;
        double p0[3] = {0, 0, 0}, p1[3] = {0, 0, 0};
        double reff = 0.0;
    };

    // Lower bound on the distance from box [lo, hi] (bounds may be
    // infinite) to the capsule of `in` (0 when they may touch).  The
    // distance from the box to the point p0 + t (p1 - p0) is convex in t:
    // golden-section search, then minus the Lipschitz constant |p1 - p0|
    // times the final bracket.
    static double capsule_gap(const Info& in, const double lo[3], const double hi[3]) {
        double v[3], L2 = 0;
        for (int a = 0; a < 3; a++) {
            v[a] = in.p1[a] - in.p0[a];
            L2 += v[a] * v[a];
        }
        auto dist = [&](double t) {
            double d2 = 0;
            for (int a = 0; a < 3; a++) {
                double p = in.p0[a] + v[a] * t;
                double g = std::max(0.0, std::max(lo[a] - p, p - hi[a]));
                d2 += g * g;
            }
            return std::sqrt(d2);
        };
        double a = 0.0, b = 1.0, best;
        if (L2 > 0) {
            const double q = 0.6180339887498949;
            double x1 = b - q * (b - a), x2 = a + q * (b - a);
            double f1 = dist(x1), f2 = dist(x2);
            for (int it = 0; it < 40; it++) {
                if (f1 < f2) {
                    b = x2; x2 = x1; f2 = f1;
                    x1 = b - q * (b - a); f1 = dist(x1);
                } else {
                    a = x1; x1 = x2; f1 = f2;
                    x2 = a + q * (b - a); f2 = dist(x2);
                }
            }
            best = std::min(f1, f2) - std::sqrt(L2) * (b - a) * 1.01;
        } else {
            best = dist(0.0);
        }
        best = best * (1.0 - 1e-9) - 1e-12 - in.reff;
        return std::isfinite(best) ? std::max(best, 0.0) : 0.0;
    }

    int emit(const Node& n, const Node64& n64) {
        fs.nodes.push_back(n);
        fs.nodes64.push_back(n64);
        return (int)fs.nodes.size() - 1;
    }

    // E: per-axis position error bound at this point of the evaluation;
    // P: bound on |coordinates|.
    int leaf(const HNode& h, double E, double P, Info& info) {
        Node n;
        memset(&n, 0, sizeof(n));
        Node64 n64;
        memset(&n64, 0, sizeof(n64));
        for (int i = 0; i < 16; i++) n64.d[i] = h.d[i];
        const double* d = h.d;
        n.type = h.type;
        double rho = 0;
        switch (h.type) {
        case N_SPHERE: {
            double r = std::fabs(d[3]);
            double cm = std::max(std::fabs(d[0]), std::max(std::fabs(d[1]), std::fabs(d[2])));
            double dist = std::sqrt(3.0) * (E + kU * (P + cm) * 2);
            double band = 2 * r * dist + dist * dist + 8 * kU * (r + dist) * (r + dist) + 2 * kU * r * r;
            for (int a = 0; a < 3; a++) n.f[a] = (float)d[a];
            n.f[3] = (float)(d[3] * d[3]);
            n.f[4] = (float)r;  // certificate radii
            n.f[F_BAND] = (float)(kSafety * band);
            rho = d[4];
            double reff = std::sqrt(r * r + kSafety * band) + E;
            for (int a = 0; a < 3; a++) {
                info.box.lo[a] = d[a] - reff;
                info.box.hi[a] = d[a] + reff;
                info.p0[a] = info.p1[a] = d[a];
            }
            info.capsule = true;
            info.reff = reff;
            break;
        }
        case N_BOX: {
            double band = 0;
            for (int a = 0; a < 3; a++) {
                double h2 = 0.5 * std::fabs(d[3 + a]);
                band = std::max(band, E + kU * (P + std::fabs(d[a])) * 2 + kU * h2 * 2);
                n.f[a] = (float)d[a];
                n.f[3 + a] = (float)(0.5 * d[3 + a]);
            }
            n.f[F_BAND] = (float)(kSafety * band);
            rho = d[6];
            info.box = leaf_box(h, kSafety * band + E);
            break;
        }
        case N_CYL: {
            double v[3] = {d[3] - d[0], d[4] - d[1], d[5] - d[2]};
            double vv = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
            double vl = std::sqrt(vv);
            double r = std::fabs(d[6]);
            rho = d[7];
            if (!(vv > 0.0) || !std::isfinite(vv)) {
                // zero-length segment: the reference's c is NaN and the
                // density is 0 everywhere; encode a box that never contains
                n.type = N_BOX;
                n.f[3] = n.f[4] = n.f[5] = -1.0f;
                n.f[F_BAND] = 0.0f;
                n.f[F_RHO] = 0.0f;
                memset(&n64, 0, sizeof(n64));
                n64.d[3] = n64.d[4] = n64.d[5] = -2.0;  // |x - c| < -1 never holds
                info.box = Box3();
                emit_leaf_finish(n, n64, 0.0, info);
                return emit(n, n64);
            }
            double pm = std::max(std::fabs(d[0]), std::max(std::fabs(d[1]), std::fabs(d[2])));
            double dw = E + kU * (P + pm) * 2;
            double band_c = std::sqrt(3.0) * dw / vl + 8 * kU * (1 + r / vl);
            double dd = std::sqrt(3.0) * dw + 6 * kU * (vl + r) * std::sqrt(3.0);
            double band_d = 2 * (r + dd) * dd + 8 * kU * (r * r + dd * dd);
            for (int a = 0; a < 3; a++) {
                n.f[a] = (float)d[a];
                n.f[3 + a] = (float)v[a];
            }
            n.f[6] = (float)(1.0 / vv);
            n.f[7] = (float)(r * r);
            // the FP64 test's per-cylinder terms, formed as the device would
            // form them (same operations, no contraction): the axis, its
            // squared length, and the threshold of its radius test
            for (int a = 0; a < 3; a++) n64.d[8 + a] = d[3 + a] - d[a];
            n64.d[11] = (n64.d[8] * n64.d[8] + n64.d[9] * n64.d[9]) + n64.d[10] * n64.d[10];
            n64.d[12] = sqrt_lt_threshold(d[6]);
            n.f[8] = (float)r;   // certificate radii: radius and axis length
            n.f[9] = (float)vl;
            n.f[F_BAND2] = (float)(kSafety * band_c);
            n.f[F_BAND] = (float)(kSafety * band_d);
            double reff = std::sqrt(r * r + kSafety * band_d) + vl * kSafety * band_c + E;
            info.box = leaf_box(h, 0.0);
            for (int a = 0; a < 3; a++) {
                info.box.lo[a] = std::min(d[a], d[3 + a]) - reff;
                info.box.hi[a] = std::max(d[a], d[3 + a]) + reff;
                info.p0[a] = d[a];
                info.p1[a] = d[3 + a];
            }
            info.capsule = true;
            info.reff = reff;
            break;
        }
        case N_PPD: {
            // row-major M for q = M (p - o): M(r,c) = d[3 + c*3 + r]
            double M[9];
            for (int r2 = 0; r2 < 3; r2++)
                for (int c = 0; c < 3; c++) M[r2 * 3 + c] = d[3 + c * 3 + r2];
            double E3[9];
            bool ok = ppd_edges(h, E3);
            double W = 0;
            if (ok)
                for (int a = 0; a < 3; a++)
                    W += std::sqrt(E3[a] * E3[a] + E3[3 + a] * E3[3 + a] + E3[6 + a] * E3[6 + a]);
            double om = std::max(std::fabs(d[0]), std::max(std::fabs(d[1]), std::fabs(d[2])));
            double dw = E + kU * (P + om) * 2;
            double band = 0;
            for (int r2 = 0; r2 < 3; r2++) {
                double row = std::fabs(M[r2 * 3]) + std::fabs(M[r2 * 3 + 1]) + std::fabs(M[r2 * 3 + 2]);
                band = std::max(band, row * (dw + 6 * kU * (W + 1e-30)) + 4 * kU);
            }
            for (int a = 0; a < 3; a++) n.f[a] = (float)d[a];
            for (int i = 0; i < 9; i++) n.f[3 + i] = (float)M[i];
            // row norms (ray certificates: world distance -> q units)
            for (int r2 = 0; r2 < 3; r2++)
                n.f[12 + r2] = (float)(std::sqrt(M[r2 * 3] * M[r2 * 3] + M[r2 * 3 + 1] * M[r2 * 3 + 1] +
                                                 M[r2 * 3 + 2] * M[r2 * 3 + 2]) * (1.0 + 1e-6));
            n.f[F_BAND] = (float)(kSafety * band);
            rho = d[12];
            if (!ok) {
                // singular edges: the inverse is the zero matrix and q == 0,
                // so the strict test 0 < q never holds: density 0 everywhere
                n.type = N_BOX;
                memset(n.f, 0, sizeof(n.f));
                n.f[3] = n.f[4] = n.f[5] = -1.0f;
                memset(&n64, 0, sizeof(n64));
                n64.d[3] = n64.d[4] = n64.d[5] = -2.0;
                info.box = Box3();
                emit_leaf_finish(n, n64, 0.0, info);
                return emit(n, n64);
            } else {
                double b = kSafety * band;
                Box3 bx;
                for (int corner = 0; corner < 8; corner++) {
                    double p[3];
                    for (int a = 0; a < 3; a++) {
                        p[a] = d[a];
                        for (int c = 0; c < 3; c++) {
                            double q = (corner & (1 << c)) ? 1.0 + b : -b;
                            p[a] += E3[a * 3 + c] * q;
                        }
                    }
                    bx.add(p);
                }
                bx.dilate(E);
                info.box = bx;
            }
            break;
        }
        case N_GYROID: {
            double is = 1.0 / d[3];
            double cm = std::max(std::fabs(d[0]), std::max(std::fabs(d[1]), std::fabs(d[2])));
            double X = (P + cm) * std::fabs(is);
            double dX = (E + kU * (P + cm) * 2) * std::fabs(is) + 4 * kU * X;
            double darg = dX + 4 * kU * X + 1e-15 * X;
            double trig = 4.0e-7;  // SFU sin/cos absolute error after reduction
            double band = 3 * 2 * (darg + trig) + 16 * kU + kU * std::fabs(d[4]);
            for (int a = 0; a < 3; a++) n.f[a] = (float)d[a];
            n.f[3] = (float)is;
            n.f[4] = (float)d[4];
            n.f[F_BAND] = (float)(kSafety * band);
            rho = d[5];
            info.box = Box3::all();
            if (!(d[4] > 0.0)) info.box = Box3();  // |g| < t <= 0 never holds
            break;
        }
        }
        emit_leaf_finish(n, n64, rho, info);
        return emit(n, n64);
    }

    void emit_leaf_finish(Node& n, const Node64&, double rho, Info& info) {
        n.f[F_RHO] = (float)rho;
        info.dyadic = dyadic(rho);
        info.maxabs = std::fabs(rho);
        info.can_be_positive = rho > 0.0 && !info.box.empty();
        info.pos_box = info.can_be_positive ? info.box : Box3();
    }

    int voxel(const HNode& h, double E, double P, Info& info) {
        (void)P;
        Node n;
        memset(&n, 0, sizeof(n));
        Node64 n64;
        memset(&n64, 0, sizeof(n64));
        n.type = N_VOXEL;
        n.a = h.vol;
        const HVolume& v = hs.vols[h.vol];
        double sc = std::max({(v.nx - 1) / 2.0, (v.ny - 1) / 2.0, (v.nz - 1) / 2.0, 1.0});
        n.f[0] = (float)(kSafety * (2 * E * sc + 32 * kU + 2 * kU * sc));  // zero-test band
        info.dyadic = false;
        info.maxabs = kInf;
        info.box = Box3();
        double bw = kSafety * (E + 4 * kU) + E;
        for (int a = 0; a < 3; a++) {
            info.box.lo[a] = -1 - bw;
            info.box.hi[a] = 1 + bw;
        }
        info.can_be_positive = true;
        info.pos_box = info.box;
        vol_band = std::max(vol_band, kSafety * (E + 4 * kU));
        return emit(n, n64);
    }

    int node(int hid, double E, double P, int depth, Info& info) {
        const HNode& h = hs.nodes[hid];
        if (h.type <= N_GYROID) return leaf(h, E, P, info);
        if (h.type == N_VOXEL) return voxel(h, E, P, info);
        if (h.type == N_COLL) return coll(h, E, P, depth, info);
        if (h.type == N_TESS) return tess(h, E, P, depth, info);
        throw SchemaError("internal: bad node type");
    }

    int max_depth = 0;

    int tess(const HNode& h, double E, double P, int depth, Info& info) {
        if (depth >= kMaxDepth) throw SchemaError("tessellations nested deeper than supported (3)");
        max_depth = std::max(max_depth, depth + 1);
        const double* o = h.d;
        const double* u = h.d + 6;
        Node n;
        memset(&n, 0, sizeof(n));
        Node64 n64;
        memset(&n64, 0, sizeof(n64));
        for (int i = 0; i < 12; i++) n64.d[i] = h.d[i];
        n.type = N_TESS;
        double bm = 0, um = 0;
        for (int i = 0; i < 6; i++) {
            bm = std::max(bm, std::fabs(o[i]));
            um = std::max(um, std::fabs(u[i]));
            n.f[i] = (float)o[i];
            n.f[7 + i] = (float)u[i];
        }
        n.f[6] = (float)(kSafety * (E + kU * (P + bm) * 2));
        double Qmax = 0, band_q = 0;
        double dmax = 0;
        for (int a = 0; a < 3; a++) {
            double dx = u[2 * a + 1] - u[2 * a];
            double idx = 1.0 / dx;
            n.f[14 + a] = (float)dx;
            n.f[17 + a] = (float)idx;
            n.f[20 + a] = (float)u[2 * a];
            double q = (std::min(P, bm) + um) * std::fabs(idx);
            Qmax = std::max(Qmax, q + 1);
            band_q = std::max(band_q, (E + kU * (P + um) * 2) * std::fabs(idx) + 6 * kU * q);
            dmax = std::max(dmax, std::fabs(dx));
        }
        n.f[23] = (float)(kSafety * band_q);
        // folded position: E' covers the rounding of dx, of the product and
        // of the subtraction
        double E2 = E + 3 * kU * (std::min(P, bm) + dmax * (Qmax + 1));
        double P2 = um + dmax + E2;
        n.f[13] = (float)(kSafety * (E2 + kU * (P2 + um) * 2));
        Info sub;
        n.a = -1;
        int me = emit(n, n64);
        int sc = coll(hs.nodes[h.sub], E2, P2, depth + 1, sub);
        fs.nodes[me].a = sc;
        // outputs: 0 outside the outer bounds, else the unit-cell collection
        info.dyadic = sub.dyadic;
        info.maxabs = sub.maxabs;
        Box3 ob;
        double b = n.f[6];
        for (int a = 0; a < 3; a++) {
            ob.lo[a] = o[2 * a] - b - E;
            ob.hi[a] = o[2 * a + 1] + b + E;
        }
        bool sub_any = !sub.box.empty();
        info.box = sub_any ? ob : Box3();
        info.can_be_positive = sub.can_be_positive;
        info.pos_box = sub.can_be_positive ? ob : Box3();
        return me;
    }

    int coll(const HNode& h, double E, double P, int depth, Info& info) {
        Node n;
        memset(&n, 0, sizeof(n));
        Node64 n64;
        memset(&n64, 0, sizeof(n64));
        n.type = N_COLL;
        int me = emit(n, n64);
        std::vector<int> kids;
        std::vector<Info> infos(h.kids.size());
        for (size_t k = 0; k < h.kids.size(); k++) kids.push_back(node(h.kids[k], E, P, depth, infos[k]));
        Node& c = fs.nodes[me];
        c.a = (int)fs.child.size();
        c.b = (int)kids.size();
        for (int k : kids) fs.child.push_back(k);
        int flags = C_CLIP | (h.greedy ? C_GREEDY : 0);
        bool dy = true;
        double sabs = 0;
        int homo = kids.empty() ? 0 : fs.nodes[kids[0]].type;
        for (size_t k = 0; k < kids.size(); k++) {
            dy = dy && infos[k].dyadic;
            sabs += infos[k].maxabs;
            if (fs.nodes[kids[k]].type != homo) homo = 0;
        }
        if (dy && sabs < 4096.0) flags |= C_EXACT_SUM;
        if (homo != N_CYL && homo != N_SPHERE) homo = 0;
        c.f[7] = (float)(2 * kSafety * ((double)kids.size() + 2) * kU);
        // per-cell candidate lists
        Box3 all;
        bool bounded = true;
        for (auto& in : infos) {
            if (in.box.empty()) continue;
            if (!in.box.bounded()) bounded = false;
            all.unite(in.box);
        }
        // uniform greedy collection: every child a leaf of one density > 0
        // (C_UNIFORM below); the lattices' unit cells
        bool uniform = h.greedy && !kids.empty();
        for (int k : kids) {
            const Node& kn = fs.nodes[k];
            uniform = uniform && kn.type <= N_GYROID && kn.f[F_RHO] == fs.nodes[kids[0]].f[F_RHO] &&
                      kn.f[F_RHO] > 0.0f;
        }
        if (kids.size() >= 6 && bounded && !all.empty()) {
            // cells per axis ~1.6 cbrt(children), ~4.8 cbrt with fine lists
            // (at most 16); tracing a uniform collection uses ~1.2 cbrt:
            // inside a cell the tracer stops at the cell's faces, and fewer,
            // fuller cells cost it less (deformed lattice, 16 struts: 3 cells
            // per axis 464 Mrays/s, 4 cells 424; with the FP64 pass
            // overlapped, 3 cells 523, 2 cells 396, one 241: coarser cells
            // cut the evaluations only 7-14 % while each evaluation reads
            // more struts), while the plain march pays per candidate (lattice,
            // 4 cells per axis 171 Mrays/s, 8: 176, 10: 184, 12: 194; 64
            // random scenes in one batch, plain 809 -> 1155, traced 4974 ->
            // 5237) and flattening pays per cell (the lattice 0.1 ms at 4
            // cells per axis, 3.9 ms at 12)
            const double gs = (tracing && uniform) ? XRP_LIST_GRID_TRACE
                                                   : (fine ? XRP_LIST_GRID_FINE : XRP_LIST_GRID);
            int G = (int)std::lround(std::cbrt((double)kids.size()) * gs);
            G = std::max(2, std::min(G, 16));
            double ext = 0;
            for (int a = 0; a < 3; a++) ext = std::max(ext, all.hi[a] - all.lo[a]);
            if (ext <= 0) ext = 1e-6;
            double h3[3];
            for (int a = 0; a < 3; a++) {
                double w = all.hi[a] - all.lo[a];
                if (w <= 0) w = ext * 1e-3;
                h3[a] = w / G;
                c.f[a] = (float)all.lo[a];
                c.f[3 + a] = (float)(1.0 / h3[a]);
                c.f[8 + a] = (float)h3[a];  // cell size (ray certificates)
            }
            double margin = 4 * E + 16 * kU * (P + all.maxabs() + ext) * (G + 1) + 1e-12;
            int cell_base = (int)fs.cells.size();
            c.f[6] = f_of_i(cell_base);
            // (dilated) cell bounds along each axis; the first/last cells also
            // hold points beyond the grid
            auto cell_lo = [&](int a, int i) { return i == 0 ? -kInf : all.lo[a] + i * h3[a] - margin; };
            auto cell_hi = [&](int a, int i) { return i == G - 1 ? kInf : all.lo[a] + (i + 1) * h3[a] + margin; };
            // squared gap of every child's box to each slab of cells, per axis
            // (0 where they overlap); a cell's squared box distance adds its
            // three slabs' terms in the order x, y, z
            const size_t nk = kids.size();
            std::vector<double> sq[3];
            for (int a = 0; a < 3; a++) {
                sq[a].assign((size_t)G * nk, 0.0);
                for (int i = 0; i < G; i++) {
                    const double l = cell_lo(a, i), u = cell_hi(a, i);
                    for (size_t k = 0; k < nk; k++) {
                        const Box3& b = infos[k].box;
                        if (b.empty()) continue;
                        double gap = std::max(b.lo[a] - u, l - b.hi[a]);
                        if (gap > 0) sq[a][(size_t)i * nk + k] = gap * gap;
                    }
                }
            }
            for (int iz = 0; iz < G; iz++)
                for (int iy = 0; iy < G; iy++)
                    for (int ix = 0; ix < G; ix++) {
                        fs.cells.push_back((int32_t)fs.items.size());
                        const double lo[3] = {cell_lo(0, ix), cell_lo(1, iy), cell_lo(2, iz)};
                        const double hi[3] = {cell_hi(0, ix), cell_hi(1, iy), cell_hi(2, iz)};
                        const double* sx = sq[0].data() + (size_t)ix * nk;
                        const double* sy = sq[1].data() + (size_t)iy * nk;
                        const double* sz = sq[2].data() + (size_t)iz * nk;
                        // clearance: distance from the (dilated) cell to the
                        // nearest child that is not listed (certificate radii)
                        double clear2 = kInf;
                        for (size_t k = 0; k < nk; k++) {
                            if (infos[k].box.empty()) continue;
                            double d2 = (sx[k] + sy[k]) + sz[k];
                            // spheres and cylinders: the distance to the capsule
                            // (a box hit may still miss the capsule, e.g. a
                            // diagonal strut and a corner cell)
                            if (d2 == 0 && infos[k].capsule) {
                                double g = capsule_gap(infos[k], lo, hi);
                                d2 = g * g;
                            }
                            if (d2 == 0) {
                                fs.items.push_back((int32_t)kids[k]);  // node index
                            } else {
                                clear2 = std::min(clear2, d2);
                            }
                        }
                        fs.clear.push_back(clear2 >= kInf ? 3.0e38f : (float)(std::sqrt(clear2) * (1.0 - 1e-6)));
                    }
            fs.cells.push_back((int32_t)fs.items.size());
            fs.clear.push_back(0.0f);
            flags |= C_ACCEL | (G << 16);
        }
        flags |= homo << 8;
        if (uniform) flags |= C_UNIFORM;
        fs.nodes[me].flags = flags;
        // outputs of the collection
        info.dyadic = (flags & C_EXACT_SUM) != 0;
        info.maxabs = h.greedy ? std::max(1.0, [&] {
            double m = 0;
            for (auto& in : infos) m = std::max(m, in.maxabs);
            return m;
        }()) : 1.0;
        info.box = Box3();
        info.pos_box = Box3();
        info.can_be_positive = false;
        for (auto& in : infos) {
            if (!in.box.empty()) info.box.unite(in.box);
            if (in.can_be_positive) {
                info.can_be_positive = true;
                info.pos_box.unite(in.pos_box);
            }
        }
        return me;
    }

    double vol_band = 0;
};

// Position-error growth through one deformation step (per axis).
double def_error(const HDef& d, double E, double P) {
    const double* a = d.d;
    switch (d.type) {
    case D_GAUSSIAN: {
        double lip = 1.0;
        double am = 0;
        for (int i = 0; i < 3; i++) {
            lip += std::fabs(a[i]) / std::fabs(a[3 + i]) * 0.61 * std::sqrt(3.0);
            am = std::max(am, std::fabs(a[i]));
        }
        return E * lip + kU * (2 * P + 2 * am) + 16 * kU * am + 4 * kU * am;
    }
    case D_LINEAR: {
        double row = 0;
        for (int r = 0; r < 3; r++) {
            int idx[3][3] = {{0, 5, 4}, {5, 1, 3}, {4, 3, 2}};
            double s = 1.0;
            for (int c = 0; c < 3; c++) s += std::fabs(a[idx[r][c]]);
            row = std::max(row, s);
        }
        return E * row + 6 * kU * P * row;
    }
    case D_RIGID: {
        double m = std::max(std::fabs(a[0]), std::max(std::fabs(a[1]), std::fabs(a[2])));
        return E + 2 * kU * (P + m);
    }
    case D_SIGMOID: {
        double A = std::fabs(a[0]), L = std::fabs(a[2]);
        return E * (1 + A / (4 * L)) + 2 * kU * (P + A) + 24 * kU * A;
    }
    case D_AFFINE: {
        double row = 0;
        for (int r = 0; r < 3; r++)
            row = std::max(row, std::fabs(a[3 * r]) + std::fabs(a[3 * r + 1]) + std::fabs(a[3 * r + 2]));
        return E * row + 6 * kU * P * row;
    }
    }
    return E;
}

// Lipschitz bound (Euclidean) of one deformation step, for the distance
// certificates: |def(p) - def(q)| <= lip * |p - q|.
double def_lip(const HDef& d) {
    const double* a = d.d;
    switch (d.type) {
    case D_GAUSSIAN: {
        // row i of the Jacobian minus I has norm |a_i| 2 s_i r exp(-s_i r^2)
        // <= |a_i| / sigma_i * exp(-1/2)
        double f2 = 0;
        for (int i = 0; i < 3; i++) {
            double n = std::fabs(a[i]) / std::fabs(a[3 + i]) * std::exp(-0.5);
            f2 += n * n;
        }
        return 1.0 + std::sqrt(f2);
    }
    case D_LINEAR: {
        double f2 = a[0] * a[0] + a[1] * a[1] + a[2] * a[2] + 2 * (a[3] * a[3] + a[4] * a[4] + a[5] * a[5]);
        return 1.0 + std::sqrt(f2);
    }
    case D_RIGID: return 1.0;
    case D_SIGMOID: return 1.0 + std::fabs(a[0]) / (4 * std::fabs(a[2]));
    case D_AFFINE: {
        double f2 = 0;
        for (int i = 0; i < 9; i++) f2 += a[i] * a[i];
        return std::sqrt(f2);
    }
    }
    return 1.0;
}

double def_mag(const HDef& d, double P) {
    const double* a = d.d;
    switch (d.type) {
    case D_GAUSSIAN: return P + std::max(std::fabs(a[0]), std::max(std::fabs(a[1]), std::fabs(a[2])));
    case D_LINEAR: {
        double m = 0;
        for (int i = 0; i < 6; i++) m = std::max(m, std::fabs(a[i]));
        return P * (1 + 3 * m);
    }
    case D_RIGID: return P + std::max(std::fabs(a[0]), std::max(std::fabs(a[1]), std::fabs(a[2])));
    case D_SIGMOID: return P + std::fabs(a[0]);
    case D_AFFINE: {
        double m = 0;
        for (int i = 0; i < 9; i++) m = std::max(m, std::fabs(a[i]));
        return P * 3 * m;
    }
    }
    return P;
}

// Preimage box of `b` under one deformation step.
Box3 def_preimage(const HDef& d, const Box3& b) {
    if (b.empty()) return b;
    if (!b.bounded()) return Box3::all();
    const double* a = d.d;
    Box3 out;
    switch (d.type) {
    case D_RIGID:
        for (int i = 0; i < 3; i++) {
            out.lo[i] = b.lo[i] - a[i];
            out.hi[i] = b.hi[i] - a[i];
        }
        return out;
    case D_GAUSSIAN:
        for (int i = 0; i < 3; i++) {
            out.lo[i] = b.lo[i] - std::max(0.0, a[i]);
            out.hi[i] = b.hi[i] - std::min(0.0, a[i]);
        }
        return out;
    case D_SIGMOID:
        out = b;
        out.lo[d.axis] = b.lo[d.axis] - std::max(0.0, a[0]);
        out.hi[d.axis] = b.hi[d.axis] - std::min(0.0, a[0]);
        return out;
    case D_LINEAR:
    case D_AFFINE: {
        double M[9];
        if (d.type == D_LINEAR) {
            double S[9] = {1 + a[0], a[5], a[4], a[5], 1 + a[1], a[3], a[4], a[3], 1 + a[2]};
            memcpy(M, S, sizeof(S));
        } else {
            memcpy(M, a, 9 * sizeof(double));
        }
        double Mi[9];
        if (!inv3_rowmajor(M, Mi)) return Box3::all();
        for (int corner = 0; corner < 8; corner++) {
            double p[3] = {(corner & 1) ? b.hi[0] : b.lo[0], (corner & 2) ? b.hi[1] : b.lo[1],
                           (corner & 4) ? b.hi[2] : b.lo[2]};
            double q[3];
            for (int r = 0; r < 3; r++) q[r] = Mi[3 * r] * p[0] + Mi[3 * r + 1] * p[1] + Mi[3 * r + 2] * p[2];
            out.add(q);
        }
        return out;
    }
    }
    return Box3::all();
}

}  // namespace

FlatScene flatten(const HostScene& hs, const RenderGeometry& g, bool hierarchical, bool tracing,
                  bool fine_lists) {
    FlatScene fs;
    // position error of the FP32 sample points (per axis), see xrp_device.h
    double half = std::tan(g.fov_deg * 0.5 * M_PI / 180.0);
    if (!std::isfinite(half) || half < 0) half = 1e3;
    double Pc = std::fabs(g.R) * std::min(half, 1e3) * 1.5 + 1e-3;
    double T = g.half_span + 1e-3;
    // magnitude of sample points: the support box if bounded, else the span
    double Pspan = std::fabs(g.R) + T + Pc;
    // rounding of p_c, of the direction (times |t|), of the offset t (three
    // roundings, lattice_t) and of the final fma
    double E0 = kSafety * kU * (Pc + 4 * T + Pspan) + 1e-11;  // + FP32 ray setup (~1e-12)
    double E = E0, P = Pspan, lip = 1.0;
    for (auto& d : hs.defs) {
        E = def_error(d, E, P);
        P = def_mag(d, P);
        lip *= def_lip(d);
    }
    fs.def_lip = lip * (1.0 + 1e-3);
    // a certificate radius is computed in FP32 from deformed coordinates of
    // magnitude P carrying the per-axis error E
    fs.margin_slack = 4.0 * (std::sqrt(3.0) * E + 64 * kU * (P + 1.0));
    // ray certificates: an affine, invertible chain maps the ray to a line.
    // The object-space direction is formed in FP32 from the FP32 direction
    // (relative error ~(ndefs + 2) kU of lip per step); over the sampled span
    // 2T that displaces the line by at most the term below, and the FP32
    // crossing arithmetic adds a relative error of the same order.
    {
        double J[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
        bool affine = true;
        for (auto& d : hs.defs) {
            const double* a = d.d;
            double A[9];
            if (d.type == D_LINEAR) {
                double L[9] = {1 + a[0], a[5], a[4], a[5], 1 + a[1], a[3], a[4], a[3], 1 + a[2]};
                std::memcpy(A, L, sizeof(A));
            } else if (d.type == D_AFFINE) {
                std::memcpy(A, a, sizeof(A));
            } else if (d.type == D_RIGID) {
                continue;
            } else {
                affine = false;
                break;
            }
            double N[9];
            for (int r = 0; r < 3; r++)
                for (int c = 0; c < 3; c++)
                    N[3 * r + c] = A[3 * r] * J[c] + A[3 * r + 1] * J[3 + c] + A[3 * r + 2] * J[6 + c];
            std::memcpy(J, N, sizeof(J));
        }
        double det = J[0] * (J[4] * J[8] - J[5] * J[7]) - J[1] * (J[3] * J[8] - J[5] * J[6]) +
                     J[2] * (J[3] * J[7] - J[4] * J[6]);
        // smallest singular value >= |det| / lip^2: keep 1/|u| finite and modest
        fs.affine = affine && std::isfinite(det) && std::fabs(det) > 1e-6 * lip * lip;
        double span = 2.0 * T + 1.0;
        fs.ray_slack = fs.margin_slack + 4.0 * (8.0 * (double)(hs.defs.size() + 2) + 32.0) * kU * lip * span;
    }
    // curved-ray certificates: the deformed point q(s) of a unit-speed ray
    // moves at most lip per unit s; its acceleration, step by step (chain
    // rule: q'' = J p'' + H[p', p']), with V the speed bound into the step
    {
        double acc = 0.0, V = 1.0;
        for (auto& d : hs.defs) {
            const double* a = d.d;
            const double l = def_lip(d);
            switch (d.type) {
            case D_SIGMOID: {  // q_k = p_k + A sigma((p_k - c)/L): |sigma'| <= 1/4, |sigma''| <= 0.0962
                const double A = std::fabs(a[0]), L = std::fabs(a[2]);
                acc = acc * (1.0 + A / (4.0 * L)) + A * 0.0963 * V * V / (L * L);
                break;
            }
            case D_GAUSSIAN: {  // Hessian of a e^{-s r^2}: norm <= 4 s |a| e^{-1/2}, s = 1/(2 sigma^2)
                double h2 = 0.0;
                for (int i = 0; i < 3; i++) {
                    const double s2 = 1.0 / (2.0 * a[3 + i] * a[3 + i]);
                    const double h = 4.0 * s2 * std::fabs(a[i]) * std::exp(-0.5);
                    h2 += h * h;
                }
                acc = acc * l + std::sqrt(h2) * V * V;
                break;
            }
            default: acc = acc * l; break;  // affine steps bend nothing
            }
            V *= l;
        }
        fs.curve_acc = acc * 1.01 + 1e-12;
    }
    Flattener F{hs, fs, hierarchical, tracing, fine_lists, {}};
    Flattener::Info info;
    fs.root = F.node(hs.root, E, P, 0, info);
    // support box: where density may be non-zero
    const HNode& r = hs.nodes[hs.root];
    Box3 sup;
    if (r.type <= N_GYROID) sup = info.box;  // a single primitive is not clipped
    else if (r.type == N_VOXEL) sup = info.box;
    else sup = info.can_be_positive ? info.pos_box : Box3();
    for (int i = (int)hs.defs.size() - 1; i >= 0; i--) sup = def_preimage(hs.defs[i], sup);
    fs.bounded = sup.bounded();
    for (int a = 0; a < 3; a++) {
        fs.sup_lo[a] = sup.lo[a];
        fs.sup_hi[a] = sup.hi[a];
        if (sup.empty()) {
            fs.sup32_lo[a] = 1.0f;
            fs.sup32_hi[a] = -1.0f;
        } else if (!fs.bounded) {
            fs.sup32_lo[a] = -3.0e38f;
            fs.sup32_hi[a] = 3.0e38f;
        } else {
            double w = sup.hi[a] - sup.lo[a];
            double m = 1e-4 + 1e-5 * (w + std::fabs(sup.lo[a]) + std::fabs(sup.hi[a]));
            fs.sup32_lo[a] = (float)(sup.lo[a] - m);
            fs.sup32_hi[a] = (float)(sup.hi[a] + m);
        }
    }
    // deformation steps
    for (auto& d : hs.defs) {
        DefStep s;
        memset(&s, 0, sizeof(s));
        s.type = d.type;
        s.axis = d.axis;
        for (int i = 0; i < 12; i++) s.d[i] = d.d[i];
        const double* a = d.d;
        switch (d.type) {
        case D_GAUSSIAN:
            for (int i = 0; i < 3; i++) {
                s.f[i] = (float)a[i];
                s.f[3 + i] = (float)(1.0 / (2 * a[3 + i] * a[3 + i]));
                s.f[6 + i] = (float)a[6 + i];
            }
            break;
        case D_LINEAR:
            for (int i = 0; i < 6; i++) s.f[i] = (float)a[i];
            break;
        case D_RIGID:
            for (int i = 0; i < 3; i++) s.f[i] = (float)a[i];
            break;
        case D_SIGMOID:
            s.f[0] = (float)a[0];
            s.f[1] = (float)a[1];
            s.f[2] = (float)(1.0 / a[2]);
            break;
        case D_AFFINE:
            for (int i = 0; i < 9; i++) s.f[i] = (float)a[i];
            break;
        }
        fs.defs.push_back(s);
    }
    fs.volume_root = (r.type == N_VOXEL) && hs.defs.empty();
    fs.depth = F.max_depth;
    // world-space band of the inclusive [-1,1] voxel-grid test: the position
    // error plus the rounding of grid coordinates (|u| <= N-1) seen in world
    // units (the fast path forms u = (p+1)(N-1)/2 directly)
    fs.vol_band_w = std::max(F.vol_band, kSafety * (E + 16 * kU * (1.0 + E)));
    return fs;
}

// ---------------------------------------------------------------------------
// camera (main.go:224-239 with mathgl restated) and lattices
// ---------------------------------------------------------------------------

static void normalize3(double v[3]) {
    double l = 1.0 / std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    v[0] = v[0] * l;
    v[1] = v[1] * l;
    v[2] = v[2] * l;
}

static void cross3(const double* a, const double* b, double* o) {
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
}

static void mat4_mul(const double* a, const double* b, double* out) {
    double r[16];
    for (int col = 0; col < 4; col++)
        for (int row = 0; row < 4; row++)
            r[col * 4 + row] = a[0 * 4 + row] * b[col * 4 + 0] + a[1 * 4 + row] * b[col * 4 + 1] +
                               a[2 * 4 + row] * b[col * 4 + 2] + a[3 * 4 + row] * b[col * 4 + 3];
    memcpy(out, r, sizeof(r));
}

// General inverse by cofactors (2x2 sub-determinants of the top and bottom
// row pairs); zero determinant -> zero matrix, NaN -> NaN, like mathgl.
static void mat4_inv(const double* m, double* out) {
#define M(r, c) m[(c) * 4 + (r)]
    double s0 = M(0, 0) * M(1, 1) - M(1, 0) * M(0, 1);
    double s1 = M(0, 0) * M(1, 2) - M(1, 0) * M(0, 2);
    double s2 = M(0, 0) * M(1, 3) - M(1, 0) * M(0, 3);
    double s3 = M(0, 1) * M(1, 2) - M(1, 1) * M(0, 2);
    double s4 = M(0, 1) * M(1, 3) - M(1, 1) * M(0, 3);
    double s5 = M(0, 2) * M(1, 3) - M(1, 2) * M(0, 3);
    double c5 = M(2, 2) * M(3, 3) - M(3, 2) * M(2, 3);
    double c4 = M(2, 1) * M(3, 3) - M(3, 1) * M(2, 3);
    double c3 = M(2, 1) * M(3, 2) - M(3, 1) * M(2, 2);
    double c2 = M(2, 0) * M(3, 3) - M(3, 0) * M(2, 3);
    double c1 = M(2, 0) * M(3, 2) - M(3, 0) * M(2, 2);
    double c0 = M(2, 0) * M(3, 1) - M(3, 0) * M(2, 1);
    double det = s0 * c5 - s1 * c4 + s2 * c3 + s3 * c2 - s4 * c1 + s5 * c0;
    if (det == 0.0 || !(std::fabs(det) > 1e-300)) {
        for (int i = 0; i < 16; i++) out[i] = (det != det) ? det : 0.0;
        return;
    }
    double r[16];
#define R(rr, cc) r[(cc) * 4 + (rr)]
    R(0, 0) = M(1, 1) * c5 - M(1, 2) * c4 + M(1, 3) * c3;
    R(0, 1) = -M(0, 1) * c5 + M(0, 2) * c4 - M(0, 3) * c3;
    R(0, 2) = M(3, 1) * s5 - M(3, 2) * s4 + M(3, 3) * s3;
    R(0, 3) = -M(2, 1) * s5 + M(2, 2) * s4 - M(2, 3) * s3;
    R(1, 0) = -M(1, 0) * c5 + M(1, 2) * c2 - M(1, 3) * c1;
    R(1, 1) = M(0, 0) * c5 - M(0, 2) * c2 + M(0, 3) * c1;
    R(1, 2) = -M(3, 0) * s5 + M(3, 2) * s2 - M(3, 3) * s1;
    R(1, 3) = M(2, 0) * s5 - M(2, 2) * s2 + M(2, 3) * s1;
    R(2, 0) = M(1, 0) * c4 - M(1, 1) * c2 + M(1, 3) * c0;
    R(2, 1) = -M(0, 0) * c4 + M(0, 1) * c2 - M(0, 3) * c0;
    R(2, 2) = M(3, 0) * s4 - M(3, 1) * s2 + M(3, 3) * s0;
    R(2, 3) = -M(2, 0) * s4 + M(2, 1) * s2 - M(2, 3) * s0;
    R(3, 0) = -M(1, 0) * c3 + M(1, 1) * c1 - M(1, 2) * c0;
    R(3, 1) = M(0, 0) * c3 - M(0, 1) * c1 + M(0, 2) * c0;
    R(3, 2) = -M(3, 0) * s3 + M(3, 1) * s1 - M(3, 2) * s0;
    R(3, 3) = M(2, 0) * s3 - M(2, 1) * s1 + M(2, 2) * s0;
#undef R
#undef M
    double inv = 1.0 / det;
    for (int i = 0; i < 16; i++) out[i] = r[i] * inv;
}

void camera_from_angles(double az_deg, double polar_deg, double R, double eye[3], double m[16]) {
    double th = az_deg * M_PI / 180;
    double phi = polar_deg * M_PI / 180;
    eye[0] = R * std::cos(th) * std::sin(phi);
    eye[1] = R * std::sin(th) * std::sin(phi);
    eye[2] = std::cos(phi) * R;
    double f[3] = {0.0 - eye[0], 0.0 - eye[1], 0.0 - eye[2]};
    normalize3(f);
    double up[3] = {0, 0, 1};
    normalize3(up);
    double s[3], u[3];
    cross3(f, up, s);
    normalize3(s);
    cross3(s, f, u);
    double Mv[16] = {s[0], u[0], -f[0], 0, s[1], u[1], -f[1], 0, s[2], u[2], -f[2], 0, 0, 0, 0, 1};
    double Tr[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, -eye[0], -eye[1], -eye[2], 1};
    double V[16];
    mat4_mul(Mv, Tr, V);
    mat4_inv(V, m);
}

void view_from_camera(const double eye[3], const double m[16], double fov_deg, ViewDev& v) {
    memset(&v, 0, sizeof(v));
    for (int i = 0; i < 3; i++) v.eye[i] = eye[i];
    for (int i = 0; i < 16; i++) v.m[i] = m[i];
    v.f = 1 / std::tan(fov_deg / 2 * M_PI / 180);
    // TransformCoordinate divides by w = m3*x + m7*y + m11*z + m15; with an
    // exactly zero last row the per-pixel w is m15 for every finite pixel
    if (m[3] == 0.0 && m[7] == 0.0 && m[11] == 0.0) {
        v.general_w = 0;
        v.inv_w = 1 / (m[15] * 1.0);
    } else {
        v.general_w = 1;
    }
    // double-float camera of the FP32 march (setup_ray32_df): the unnormalised
    // direction (M (x_i, x_j, -f, 1)) w - eye = c0 x_i + c1 x_j + k
    if (!v.general_w) {
        auto split = [](double x, float* out) {
            out[0] = (float)x;
            out[1] = (float)(x - (double)out[0]);
        };
        const double w = v.inv_w;
        for (int a = 0; a < 3; a++) {
            split(m[a] * w, v.c0 + 2 * a);
            split(m[4 + a] * w, v.c1 + 2 * a);
            split(std::fma(m[8 + a], -v.f, m[12 + a]) * w - eye[a], v.k + 2 * a);
            split(eye[a], v.eye2 + 2 * a);
        }
    }
}

HostLattice build_lattice(double R, double ds, bool hierarchical) {
    HostLattice L;
    const double half = 1.74;  // main.go:46
    double smin = R - half, smax = R + half;
    double s_c = R;
    memset(&L.hdr, 0, sizeof(L.hdr));
    if (!hierarchical) {
        for (double s = smin; s < smax; s += ds) {  // main.go:147
            L.s64.push_back(s);
            L.t32.push_back((float)(s - s_c));
            if (L.s64.size() > (size_t)200000000) break;
        }
        L.hdr.ds = ds;
        L.hdr.ds32 = (float)ds;
    } else {
        double DS = ds;
        double right = smin + DS, left = smin, dsf = DS / 10.0;  // main.go:171-173
        L.fstart.push_back(0);
        while (right <= smax) {
            L.s64.push_back(right);
            L.t32.push_back((float)(right - s_c));
            double l = left + dsf;
            while (l < right) {  // main.go:182-189
                L.f64.push_back(l);
                L.ft32.push_back((float)(l - s_c));
                l += dsf;
            }
            L.fstart.push_back((int32_t)L.f64.size());
            left = right;
            right += DS;
            if (L.s64.size() > (size_t)50000000) break;
        }
        L.hdr.ds = DS;
        L.hdr.ds_fine = dsf;
        L.hdr.ds32 = (float)DS;
        L.hdr.dsf32 = (float)dsf;
    }
    L.hdr.K = (int32_t)L.s64.size();
    L.hdr.hierarchical = hierarchical ? 1 : 0;
    L.hdr.s_c = s_c;
    L.hdr.s_c2[0] = (float)s_c;
    L.hdr.s_c2[1] = (float)(s_c - (double)L.hdr.s_c2[0]);
    L.hdr.smin = smin;
    L.hdr.t_first = L.t32.empty() ? 0.0f : L.t32[0];
    L.hdr.inv_ds = (float)(1.0 / ds);
    L.hdr.ds_hi = (float)ds;
    L.hdr.ds_lo = (float)(ds - (double)L.hdr.ds_hi);
    return L;
}

HostPrepared prepare_host(const HostScene& hs, int res, int integration, double ds, double R,
                          double flat_field, double density_multiplier, double fov_max, bool tracing,
                          bool fine_lists) {
    HostPrepared hp;
    bool hier = integration == 1;
    RenderGeometry g;
    g.R = R;
    g.fov_deg = fov_max;
    hp.fs = flatten(hs, g, hier, tracing, fine_lists);
    hp.hl = build_lattice(R, ds, hier);
    if (hp.hl.s64.empty()) {  // keep the tables non-empty; K = 0 means "no samples"
        hp.hl.s64.push_back(0.0);
        hp.hl.t32.push_back(0.0f);
    }
    if (hp.hl.fstart.size() < 2) hp.hl.fstart.resize(2, 0);
    if (hp.hl.f64.empty()) {
        hp.hl.f64.push_back(0.0);
        hp.hl.ft32.push_back(0.0f);
    }
    hp.xs = pixel_table(res);
    hp.xsf.resize(2 * hp.xs.size());
    for (size_t q = 0; q < hp.xs.size(); q++) {
        hp.xsf[2 * q] = (float)hp.xs[q];
        hp.xsf[2 * q + 1] = (float)(hp.xs[q] - (double)hp.xsf[2 * q]);
    }
    hp.vols.resize(hs.vols.size());
    for (size_t k = 0; k < hs.vols.size(); k++) {
        const HVolume& hv = hs.vols[k];
        Volume& v = hp.vols[k];
        memset(&v, 0, sizeof(v));
        v.nx = hv.nx;
        v.ny = hv.ny;
        v.nz = hv.nz;
        v.scale[0] = (float)((hv.nx - 1) / 2.0);
        v.scale[1] = (float)((hv.ny - 1) / 2.0);
        v.scale[2] = (float)((hv.nz - 1) / 2.0);
        v.band_w = (float)hp.fs.vol_band_w;
    }
    SceneDev& S = hp.S;
    memset(&S, 0, sizeof(S));
    S.root = hp.fs.root;
    S.ndefs = (int32_t)hp.fs.defs.size();
    S.hier_zero_guard = hier ? 1 : 0;
    for (int a = 0; a < 3; a++) {
        S.sup_lo[a] = hp.fs.sup32_lo[a];
        S.sup_hi[a] = hp.fs.sup32_hi[a];
    }
    S.inv_lip = (float)(1.0 / hp.fs.def_lip) * (1.0f - 1e-6f);
    S.m_slack = (float)hp.fs.margin_slack;
    S.affine = hp.fs.affine ? 1 : 0;
    S.ray_slack = (float)hp.fs.ray_slack;
    S.curve_vmax = (float)hp.fs.def_lip * (1.0f + 1e-6f);
    S.curve_acc = (float)hp.fs.curve_acc * (1.0f + 1e-6f);
    memset(&hp.P, 0, sizeof(hp.P));
    hp.P.res = res;
    hp.P.flat_field = (float)flat_field;
    hp.P.density_multiplier = (float)density_multiplier;
    hp.volume_fast = hp.fs.volume_root && hs.vols.size() == 1 && hs.vols[0].nx >= 2 &&
                     hs.vols[0].ny >= 2 && hs.vols[0].nz >= 2;
    return hp;
}

std::vector<double> pixel_table(int res) {
    std::vector<double> xs(res);
    double res_f = (double)res;
    for (int i = 0; i < res; i++) xs[i] = (double)i / (res_f / 2) - 1;  // main.go:463
    return xs;
}

}  // namespace xrp
