/*
 * xrp_oracle.c -- FP64 CPU oracle for the X-ray projection line integral.
 *
 * TEST INFRASTRUCTURE ONLY.  This file restates, in plain C and in double
 * precision, the CPU algorithm of igrega348/xray_projection_render so that the
 * GPU engine can be checked against it.  Only tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline leg load it.  The product library never links,
 * loads or calls it.
 *
 * Every function names the reference file:line it follows.  The object tree is
 * walked through per-node function pointers, like the reference's Go
 * interface dispatch (objects/objects.go:13-19), and the integrators keep the
 * reference loop structure (`s += ds` accumulated in FP64).  Floating-point
 * contraction is disabled at build time (-ffp-contract=off) so every product
 * and sum is rounded separately, as Go does on amd64.
 *
 * Third-party arithmetic: the camera uses github.com/go-gl/mathgl v1.1.0
 * (go.mod:6): LookAtV, Mat4.Inv, TransformCoordinate, Vec3.Normalize/Len,
 * Mat3FromCols(..).Inv(), Mul3x1.  That module is not vendored in the
 * reference tree.  Its published algorithms are restated here from the
 * mathematics: the OpenGL look-at matrix, the adjugate inverse, a homogeneous
 * multiply followed by a divide by w, and normalisation by the reciprocal
 * length.  Summation order inside those helpers is this file's choice, so the
 * camera matrix agrees with mathgl to rounding, not bit for bit (it is pinned
 * by the eye-position tests of main_test.go:90-195 only).
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORC_EXPORT __attribute__((visibility("default")))

/* ------------------------------------------------------------------------ */
/* Object tree (objects/objects.go)                                          */
/* ------------------------------------------------------------------------ */

enum {
    ORC_SPHERE = 1,
    ORC_BOX = 2,
    ORC_CYLINDER = 3,
    ORC_PARALLELEPIPED = 4,
    ORC_GYROID = 5,
    ORC_COLLECTION = 6,
    ORC_UNIT_CELL = 7,
    ORC_TESSELLATED = 8,
    ORC_VOXEL = 9,
};

typedef struct orc_node orc_node;
typedef double (*orc_density_fn)(const orc_node*, double, double, double);

struct orc_node {
    int type;
    orc_density_fn density; /* per-node dispatch, as the Go interface call */
    double a[16];           /* parameters, meaning depends on type */
    int greedy;             /* collections */
    int nchild;
    int* child;             /* node ids */
    int sub;                /* unit cell: collection id; tessellated: unit-cell id */
    double* rho;            /* voxel values (FP64, [z][x][y]) */
    int nx, ny, nz;
};

static orc_node* g_nodes = NULL;
static int g_nnodes = 0, g_cap = 0;

static int orc_new_node(int type, orc_density_fn fn) {
    if (g_nnodes == g_cap) {
        int cap = g_cap ? 2 * g_cap : 64;
        orc_node* n = (orc_node*)realloc(g_nodes, (size_t)cap * sizeof(orc_node));
        if (!n) return -1;
        g_nodes = n;
        g_cap = cap;
    }
    orc_node* n = &g_nodes[g_nnodes];
    memset(n, 0, sizeof(*n));
    n->type = type;
    n->density = fn;
    n->sub = -1;
    return g_nnodes++;
}

static inline double node_density(int id, double x, double y, double z) {
    const orc_node* n = &g_nodes[id];
    return n->density(n, x, y, z);
}

/* Sphere.Density, objects.go:63-72 */
static double sphere_density(const orc_node* s, double x, double y, double z) {
    x = x - s->a[0];
    y = y - s->a[1];
    z = z - s->a[2];
    double r_2 = x * x + y * y + z * z;
    if (r_2 < s->a[3] * s->a[3]) return s->a[4];
    return 0.0;
}

/* Box.Density, objects.go:171-179 (Cube delegates here, objects.go:119-121) */
static double box_density(const orc_node* b, double x, double y, double z) {
    x = fabs(x - b->a[0]);
    y = fabs(y - b->a[1]);
    z = fabs(z - b->a[2]);
    if (x < 0.5 * b->a[3] && y < 0.5 * b->a[4] && z < 0.5 * b->a[5]) return b->a[6];
    return 0.0;
}

/* Parallelepiped.Density, objects.go:247-255.  a[0..2] origin, a[3..11] the
 * inverse of [v0 v1 v2] stored column-major (mathgl Mat3 layout), a[12] rho. */
static double ppd_density(const orc_node* p, double x, double y, double z) {
    double wx = x - p->a[0], wy = y - p->a[1], wz = z - p->a[2];
    const double* m = &p->a[3];
    double qx = m[0] * wx + m[3] * wy + m[6] * wz;
    double qy = m[1] * wx + m[4] * wy + m[7] * wz;
    double qz = m[2] * wx + m[5] * wy + m[8] * wz;
    if (qx > 0.0 && qx < 1.0 && qy > 0.0 && qy < 1.0 && qz > 0.0 && qz < 1.0) return p->a[12];
    return 0.0;
}

/* Cylinder.Density, objects.go:334-350.  a[0..2] p0, a[3..5] p1, a[6] r, a[7] rho */
static double cylinder_density(const orc_node* c, double x, double y, double z) {
    double vx = c->a[3] - c->a[0], vy = c->a[4] - c->a[1], vz = c->a[5] - c->a[2];
    double wx = x - c->a[0], wy = y - c->a[1], wz = z - c->a[2];
    double cc = (wx * vx + wy * vy + wz * vz) / (vx * vx + vy * vy + vz * vz);
    if (cc < 0.0 || cc > 1.0) return 0.0;
    double dx = wx - vx * cc, dy = wy - vy * cc, dz = wz - vz * cc;
    double d = sqrt(dx * dx + dy * dy + dz * dz);
    if (d < c->a[6]) return c->a[7];
    return 0.0;
}

/* Gyroid.Density, objects.go:1014-1032.  a[0..2] centre, a[3] scale,
 * a[4] thickness, a[5] rho.  Coordinates are DIVIDED by scale. */
static double gyroid_density(const orc_node* g, double x, double y, double z) {
    x = (x - g->a[0]) / g->a[3];
    y = (y - g->a[1]) / g->a[3];
    z = (z - g->a[2]) / g->a[3];
    double v = sin(x) * cos(y) + sin(y) * cos(z) + sin(z) * cos(x);
    if (fabs(v) < g->a[4]) return g->a[5];
    return 0.0;
}

/* ObjectCollection.Density, objects.go:422-438 */
static double collection_density(const orc_node* c, double x, double y, double z) {
    double density = 0.0;
    for (int i = 0; i < c->nchild; i++) {
        double rho = node_density(c->child[i], x, y, z);
        if (c->greedy && rho > 0.0) return rho;
        density += rho;
    }
    if (density < 0.0)
        density = 0.0;
    else if (density > 1.0)
        density = 1.0;
    return density;
}

/* UnitCell.Density, objects.go:458-464.  a[0..5] = xmin,xmax,ymin,ymax,zmin,zmax */
static double unit_cell_density(const orc_node* u, double x, double y, double z) {
    if (x < u->a[0] || x > u->a[1] || y < u->a[2] || y > u->a[3] || z < u->a[4] || z > u->a[5])
        return 0.0;
    return node_density(u->sub, x, y, z);
}

/* TessellatedObjColl.Density, objects.go:568-582 */
static double tessellated_density(const orc_node* t, double x, double y, double z) {
    if (x < t->a[0] || x > t->a[1] || y < t->a[2] || y > t->a[3] || z < t->a[4] || z > t->a[5])
        return 0.0;
    const orc_node* uc = &g_nodes[t->sub];
    double dx = uc->a[1] - uc->a[0];
    x = x - dx * floor((x - uc->a[0]) / dx);
    double dy = uc->a[3] - uc->a[2];
    y = y - dy * floor((y - uc->a[2]) / dy);
    double dz = uc->a[5] - uc->a[4];
    z = z - dz * floor((z - uc->a[4]) / dz);
    return uc->density(uc, x, y, z);
}

/* VoxelGrid.Density, objects.go:789-855 ((N-1) scaling, [z][x][y] layout) */
static double voxel_density(const orc_node* v, double x, double y, double z) {
    if (x < -1 || x > 1 || y < -1 || y > 1 || z < -1 || z > 1) return 0.0;
    x = (x + 1) / 2;
    y = (y + 1) / 2;
    z = (z + 1) / 2;
    x = x * (double)(v->nx - 1);
    y = y * (double)(v->ny - 1);
    z = z * (double)(v->nz - 1);
    int x0 = (int)floor(x), y0 = (int)floor(y), z0 = (int)floor(z);
    int x1 = x0 + 1, y1 = y0 + 1, z1 = z0 + 1;
    if (x0 < 0) x0 = 0;
    if (y0 < 0) y0 = 0;
    if (z0 < 0) z0 = 0;
    if (x1 >= v->nx) x1 = v->nx - 1;
    if (y1 >= v->ny) y1 = v->ny - 1;
    if (z1 >= v->nz) z1 = v->nz - 1;
    double wx = x - (double)x0, wy = y - (double)y0, wz = z - (double)z0;
    long NXY = (long)v->nx * v->ny, NY = v->ny;
    const double* r = v->rho;
    double v000 = r[z0 * NXY + x0 * NY + y0];
    double v001 = r[z1 * NXY + x0 * NY + y0];
    double v010 = r[z0 * NXY + x0 * NY + y1];
    double v011 = r[z1 * NXY + x0 * NY + y1];
    double v100 = r[z0 * NXY + x1 * NY + y0];
    double v101 = r[z1 * NXY + x1 * NY + y0];
    double v110 = r[z0 * NXY + x1 * NY + y1];
    double v111 = r[z1 * NXY + x1 * NY + y1];
    double v00 = v000 * (1 - wz) + v001 * wz;
    double v01 = v010 * (1 - wz) + v011 * wz;
    double v10 = v100 * (1 - wz) + v101 * wz;
    double v11 = v110 * (1 - wz) + v111 * wz;
    double v0 = v00 * (1 - wy) + v01 * wy;
    double v1 = v10 * (1 - wy) + v11 * wy;
    return v0 * (1 - wx) + v1 * wx;
}

/* ---- node constructors (the FromMap/NewObject factory is done by the
 * Python side, which walks the reference JSON schema and calls these) ---- */

ORC_EXPORT void orc_reset(void) {
    for (int i = 0; i < g_nnodes; i++) {
        free(g_nodes[i].child);
        free(g_nodes[i].rho);
    }
    g_nnodes = 0;
}

ORC_EXPORT int orc_sphere(double cx, double cy, double cz, double r, double rho) {
    int id = orc_new_node(ORC_SPHERE, sphere_density);
    if (id < 0) return id;
    double* a = g_nodes[id].a;
    a[0] = cx; a[1] = cy; a[2] = cz; a[3] = r; a[4] = rho;
    return id;
}

ORC_EXPORT int orc_box(double cx, double cy, double cz, double sx, double sy, double sz, double rho) {
    int id = orc_new_node(ORC_BOX, box_density);
    if (id < 0) return id;
    double* a = g_nodes[id].a;
    a[0] = cx; a[1] = cy; a[2] = cz; a[3] = sx; a[4] = sy; a[5] = sz; a[6] = rho;
    return id;
}

ORC_EXPORT int orc_cylinder(double x0, double y0, double z0, double x1, double y1, double z1,
                            double r, double rho) {
    int id = orc_new_node(ORC_CYLINDER, cylinder_density);
    if (id < 0) return id;
    double* a = g_nodes[id].a;
    a[0] = x0; a[1] = y0; a[2] = z0; a[3] = x1; a[4] = y1; a[5] = z1; a[6] = r; a[7] = rho;
    return id;
}

/* Inverse of the 3x3 matrix with columns v0, v1, v2 (objects.go:243,
 * mgl64.Mat3FromCols(...).Inv()), by the adjugate; a singular matrix gives the
 * zero matrix, as mathgl does.  Output is column-major. */
static void orc_inv3_cols(const double* v0, const double* v1, const double* v2, double* out) {
    /* column-major m[col*3+row] */
    double m[9] = {v0[0], v0[1], v0[2], v1[0], v1[1], v1[2], v2[0], v2[1], v2[2]};
    double c00 = m[4] * m[8] - m[7] * m[5];
    double c01 = m[7] * m[2] - m[1] * m[8];
    double c02 = m[1] * m[5] - m[4] * m[2];
    double det = m[0] * c00 + m[3] * c01 + m[6] * c02;
    if (det == 0.0 || fabs(det) < 1e-300) {
        memset(out, 0, 9 * sizeof(double));
        return;
    }
    double inv[9];
    /* inverse = adj / det; adj[row][col] = cofactor[col][row] */
    inv[0] = c00;                          /* (0,0) */
    inv[1] = m[5] * m[6] - m[3] * m[8];    /* (1,0) */
    inv[2] = m[3] * m[7] - m[6] * m[4];    /* (2,0) */
    inv[3] = c01;                          /* (0,1) */
    inv[4] = m[0] * m[8] - m[6] * m[2];    /* (1,1) */
    inv[5] = m[6] * m[1] - m[0] * m[7];    /* (2,1) */
    inv[6] = c02;                          /* (0,2) */
    inv[7] = m[3] * m[2] - m[0] * m[5];    /* (1,2) */
    inv[8] = m[0] * m[4] - m[3] * m[1];    /* (2,2) */
    double s = 1.0 / det;
    for (int i = 0; i < 9; i++) out[i] = inv[i] * s;
}

ORC_EXPORT int orc_parallelepiped(const double* origin, const double* v0, const double* v1,
                                  const double* v2, double rho) {
    int id = orc_new_node(ORC_PARALLELEPIPED, ppd_density);
    if (id < 0) return id;
    double* a = g_nodes[id].a;
    a[0] = origin[0]; a[1] = origin[1]; a[2] = origin[2];
    orc_inv3_cols(v0, v1, v2, &a[3]);
    a[12] = rho;
    /* edge lengths for MinFeatureSize (objects.go:257-259) */
    a[13] = sqrt(v0[0] * v0[0] + v0[1] * v0[1] + v0[2] * v0[2]);
    a[14] = sqrt(v1[0] * v1[0] + v1[1] * v1[1] + v1[2] * v1[2]);
    a[15] = sqrt(v2[0] * v2[0] + v2[1] * v2[1] + v2[2] * v2[2]);
    return id;
}

ORC_EXPORT int orc_gyroid(double cx, double cy, double cz, double scale, double thickness, double rho) {
    int id = orc_new_node(ORC_GYROID, gyroid_density);
    if (id < 0) return id;
    double* a = g_nodes[id].a;
    a[0] = cx; a[1] = cy; a[2] = cz; a[3] = scale; a[4] = thickness; a[5] = rho;
    return id;
}

ORC_EXPORT int orc_collection(const int* children, int n, int greedy) {
    int id = orc_new_node(ORC_COLLECTION, collection_density);
    if (id < 0) return id;
    orc_node* c = &g_nodes[id];
    c->greedy = greedy;
    c->nchild = n;
    c->child = (int*)malloc((size_t)(n > 0 ? n : 1) * sizeof(int));
    if (n > 0) memcpy(c->child, children, (size_t)n * sizeof(int));
    return id;
}

/* UnitCell.FromMap forces GreedyDensEval on its collection (objects.go:487);
 * the caller passes a collection built with greedy=1. */
ORC_EXPORT int orc_unit_cell(int coll, const double* bounds6) {
    int id = orc_new_node(ORC_UNIT_CELL, unit_cell_density);
    if (id < 0) return id;
    memcpy(g_nodes[id].a, bounds6, 6 * sizeof(double));
    g_nodes[id].sub = coll;
    return id;
}

ORC_EXPORT int orc_tessellated(int unit_cell, const double* bounds6) {
    int id = orc_new_node(ORC_TESSELLATED, tessellated_density);
    if (id < 0) return id;
    memcpy(g_nodes[id].a, bounds6, 6 * sizeof(double));
    g_nodes[id].sub = unit_cell;
    return id;
}

/* VoxelGrid with values already in FP64 ([z][x][y], objects.go:837). */
ORC_EXPORT int orc_voxel_f64(const double* rho, int nx, int ny, int nz) {
    int id = orc_new_node(ORC_VOXEL, voxel_density);
    if (id < 0) return id;
    size_t n = (size_t)nx * ny * nz;
    orc_node* v = &g_nodes[id];
    v->rho = (double*)malloc(n * sizeof(double));
    if (!v->rho) return -1;
    memcpy(v->rho, rho, n * sizeof(double));
    v->nx = nx; v->ny = ny; v->nz = nz;
    return id;
}

/* VoxelGrid from FP32 values widened to FP64 (the volume a float32 raw file
 * or the GPU ABI carries, objects.go:938-941). */
ORC_EXPORT int orc_voxel_f32(const float* rho, int nx, int ny, int nz) {
    int id = orc_new_node(ORC_VOXEL, voxel_density);
    if (id < 0) return id;
    size_t n = (size_t)nx * ny * nz;
    orc_node* v = &g_nodes[id];
    v->rho = (double*)malloc(n * sizeof(double));
    if (!v->rho) return -1;
    for (size_t i = 0; i < n; i++) v->rho[i] = (double)rho[i];
    v->nx = nx; v->ny = ny; v->nz = nz;
    return id;
}

ORC_EXPORT double orc_density(int node, double x, double y, double z) {
    return node_density(node, x, y, z);
}

/* ------------------------------------------------------------------------ */
/* Deformations (deformations/deformations.go)                               */
/* ------------------------------------------------------------------------ */

enum { ORC_DEF_GAUSSIAN = 1, ORC_DEF_LINEAR, ORC_DEF_RIGID, ORC_DEF_SIGMOID, ORC_DEF_AFFINE, ORC_DEF_COMPOSED };

typedef struct {
    int type;
    double a[12];
    int axis;     /* sigmoid: 0,1,2 */
    int n;        /* composed */
    int* sub;
} orc_def;

static orc_def* g_defs = NULL;
static int g_ndefs = 0, g_defcap = 0;

static int orc_new_def(int type) {
    if (g_ndefs == g_defcap) {
        int cap = g_defcap ? 2 * g_defcap : 16;
        orc_def* d = (orc_def*)realloc(g_defs, (size_t)cap * sizeof(orc_def));
        if (!d) return -1;
        g_defs = d;
        g_defcap = cap;
    }
    memset(&g_defs[g_ndefs], 0, sizeof(orc_def));
    g_defs[g_ndefs].type = type;
    return g_ndefs++;
}

ORC_EXPORT void orc_reset_deformations(void) {
    for (int i = 0; i < g_ndefs; i++) free(g_defs[i].sub);
    g_ndefs = 0;
}

/* amplitudes, sigmas, centers: 3 each (deformations.go:29-38) */
ORC_EXPORT int orc_def_gaussian(const double* amp, const double* sig, const double* cen) {
    int id = orc_new_def(ORC_DEF_GAUSSIAN);
    if (id < 0) return id;
    double* a = g_defs[id].a;
    for (int i = 0; i < 3; i++) { a[i] = amp[i]; a[3 + i] = sig[i]; a[6 + i] = cen[i]; }
    return id;
}

/* Voigt strains [xx,yy,zz,yz,xz,xy] (deformations.go:136-141) */
ORC_EXPORT int orc_def_linear(const double* strains6) {
    int id = orc_new_def(ORC_DEF_LINEAR);
    if (id < 0) return id;
    memcpy(g_defs[id].a, strains6, 6 * sizeof(double));
    return id;
}

ORC_EXPORT int orc_def_rigid(const double* disp3) {
    int id = orc_new_def(ORC_DEF_RIGID);
    if (id < 0) return id;
    memcpy(g_defs[id].a, disp3, 3 * sizeof(double));
    return id;
}

ORC_EXPORT int orc_def_sigmoid(double amplitude, double center, double lengthscale, int axis) {
    int id = orc_new_def(ORC_DEF_SIGMOID);
    if (id < 0) return id;
    g_defs[id].a[0] = amplitude; g_defs[id].a[1] = center; g_defs[id].a[2] = lengthscale;
    g_defs[id].axis = axis;
    return id;
}

/* row-major 3x3 (deformations.go:87-92) */
ORC_EXPORT int orc_def_affine(const double* m9) {
    int id = orc_new_def(ORC_DEF_AFFINE);
    if (id < 0) return id;
    memcpy(g_defs[id].a, m9, 9 * sizeof(double));
    return id;
}

ORC_EXPORT int orc_def_composed(const int* subs, int n) {
    int id = orc_new_def(ORC_DEF_COMPOSED);
    if (id < 0) return id;
    g_defs[id].n = n;
    g_defs[id].sub = (int*)malloc((size_t)(n > 0 ? n : 1) * sizeof(int));
    if (n > 0) memcpy(g_defs[id].sub, subs, (size_t)n * sizeof(int));
    return id;
}

static void def_apply(int id, double* px, double* py, double* pz) {
    const orc_def* d = &g_defs[id];
    double x = *px, y = *py, z = *pz;
    const double* a = d->a;
    switch (d->type) {
    case ORC_DEF_GAUSSIAN: { /* deformations.go:29-38 */
        double x0 = x - a[6], y0 = y - a[7], z0 = z - a[8];
        double r2 = x0 * x0 + y0 * y0 + z0 * z0;
        double dx = a[0] * exp(-r2 / (2 * a[3] * a[3]));
        double dy = a[1] * exp(-r2 / (2 * a[4] * a[4]));
        double dz = a[2] * exp(-r2 / (2 * a[5] * a[5]));
        x = x + dx; y = y + dy; z = z + dz;
        break;
    }
    case ORC_DEF_LINEAR: { /* deformations.go:136-141 */
        double nx = x + a[0] * x + a[5] * y + a[4] * z;
        double ny = y + a[5] * x + a[1] * y + a[3] * z;
        double nz = z + a[4] * x + a[3] * y + a[2] * z;
        x = nx; y = ny; z = nz;
        break;
    }
    case ORC_DEF_RIGID: /* deformations.go:173-175 */
        x = x + a[0]; y = y + a[1]; z = z + a[2];
        break;
    case ORC_DEF_SIGMOID: /* deformations.go:210-222 */
        if (d->axis == 0)
            x = x + a[0] / (1 + exp(-(x - a[1]) / a[2]));
        else if (d->axis == 1)
            y = y + a[0] / (1 + exp(-(y - a[1]) / a[2]));
        else
            z = z + a[0] / (1 + exp(-(z - a[1]) / a[2]));
        break;
    case ORC_DEF_AFFINE: { /* deformations.go:87-92 */
        double nx = a[0] * x + a[1] * y + a[2] * z;
        double ny = a[3] * x + a[4] * y + a[5] * z;
        double nz = a[6] * x + a[7] * y + a[8] * z;
        x = nx; y = ny; z = nz;
        break;
    }
    case ORC_DEF_COMPOSED: /* deformations.go:269-274 */
        for (int i = 0; i < d->n; i++) def_apply(d->sub[i], &x, &y, &z);
        break;
    default:
        break;
    }
    *px = x; *py = y; *pz = z;
}

ORC_EXPORT void orc_def_apply(int id, double* xyz) { def_apply(id, &xyz[0], &xyz[1], &xyz[2]); }

/* ------------------------------------------------------------------------ */
/* Scene context: the reference's package globals lat[0], df, flat_field,    */
/* density_multiplier (main.go:37-41), passed explicitly here.               */
/* ------------------------------------------------------------------------ */

typedef struct {
    int root;       /* node id */
    int deform;     /* deformation id or -1 */
    double density_multiplier;
    double flat_field;
} orc_ctx;

/* density(), main.go:137-140 (deform first, main.go:123-133) */
static inline double ctx_density(const orc_ctx* c, double x, double y, double z) {
    if (c->deform >= 0) def_apply(c->deform, &x, &y, &z);
    return node_density(c->root, x, y, z) * c->density_multiplier;
}

/* mgl64 Vec3.Normalize: multiply by the reciprocal of the length */
static inline void normalize3(double* v) {
    double l = 1.0 / sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    v[0] = v[0] * l; v[1] = v[1] * l; v[2] = v[2] * l;
}

/* integrate_along_ray, main.go:144-154.  Returns exp(-T); optionally the
 * optical depth T and the number of samples. */
static double integrate_simple(const orc_ctx* c, const double* o, const double* dir_in, double ds,
                               double smin, double smax, double* T_out) {
    double d[3] = {dir_in[0], dir_in[1], dir_in[2]};
    normalize3(d);
    double T = c->flat_field;
    for (double s = smin; s < smax; s += ds) {
        double x = o[0] + d[0] * s;
        double y = o[1] + d[1] * s;
        double z = o[2] + d[2] * s;
        T += ctx_density(c, x, y, z) * ds;
    }
    if (T_out) *T_out = T;
    return exp(-T);
}

/* integrate_hierarchical, main.go:159-199 (the clipping warnings of
 * main.go:162-169 only log and do not change the result; they are omitted). */
static double integrate_hier(const orc_ctx* c, const double* o, const double* dir_in, double DS,
                             double smin, double smax, double* T_out) {
    double d[3] = {dir_in[0], dir_in[1], dir_in[2]};
    normalize3(d);
    double right = smin + DS;
    double left = smin;
    double ds = DS / 10.0;
    double prev_rho = 0.0;
    double T = c->flat_field;
    while (right <= smax) {
        double x = o[0] + d[0] * right;
        double y = o[1] + d[1] * right;
        double z = o[2] + d[2] * right;
        double rho = ctx_density(c, x, y, z);
        if ((rho == 0) != (prev_rho == 0)) {
            left += ds;
            while (left < right) {
                double lx = o[0] + d[0] * left;
                double ly = o[1] + d[1] * left;
                double lz = o[2] + d[2] * left;
                T += ctx_density(c, lx, ly, lz) * ds;
                left += ds;
            }
            T += rho * ds;
        } else {
            T += rho * DS;
        }
        prev_rho = rho;
        left = right;
        right += DS;
    }
    if (T_out) *T_out = T;
    return exp(-T);
}

ORC_EXPORT double orc_integrate(int root, int deform, double dm, double ff, int hierarchical,
                                const double* origin, const double* dir, double ds, double smin,
                                double smax, double* T_out) {
    orc_ctx c = {root, deform, dm, ff};
    if (hierarchical) return integrate_hier(&c, origin, dir, ds, smin, smax, T_out);
    return integrate_simple(&c, origin, dir, ds, smin, smax, T_out);
}

/* ------------------------------------------------------------------------ */
/* Camera (main.go:224-239, 455-465) with mathgl restated                    */
/* ------------------------------------------------------------------------ */

static inline double deg2rad(double a) { return a * M_PI / 180; }

/* 4x4 product, column-major m[col*4+row] (mathgl Mat4 layout) */
static void mat4_mul(const double* a, const double* b, double* out) {
    double r[16];
    for (int col = 0; col < 4; col++)
        for (int row = 0; row < 4; row++)
            r[col * 4 + row] = a[0 * 4 + row] * b[col * 4 + 0] + a[1 * 4 + row] * b[col * 4 + 1] +
                               a[2 * 4 + row] * b[col * 4 + 2] + a[3 * 4 + row] * b[col * 4 + 3];
    memcpy(out, r, sizeof(r));
}

/* General 4x4 inverse by cofactor expansion (column-major in and out).  A
 * zero determinant gives the zero matrix, as mathgl's Inv does. */
static void mat4_inv(const double* m, double* out) {
    /* element (row r, col c) = m[c*4+r] */
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
    if (det == 0.0 || !(fabs(det) > 1e-300)) {
        if (det != det) { /* NaN propagates, as in mathgl */
            for (int i = 0; i < 16; i++) out[i] = det;
        } else {
            memset(out, 0, 16 * sizeof(double));
        }
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

static void cross3(const double* a, const double* b, double* o) {
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
}

/* computeCameraFromAngles, main.go:226-239: eye and camera = LookAtV(eye, 0,
 * +z).Inv(); matrix returned column-major (mathgl layout). */
ORC_EXPORT void orc_camera_from_angles(double az_deg, double polar_deg, double R, double* eye,
                                       double* cam) {
    double th = deg2rad(az_deg);
    double phi = deg2rad(polar_deg);
    eye[0] = R * cos(th) * sin(phi);
    eye[1] = R * sin(th) * sin(phi);
    eye[2] = cos(phi) * R;
    /* LookAtV(eye, center=0, up=(0,0,1)) */
    double f[3] = {0.0 - eye[0], 0.0 - eye[1], 0.0 - eye[2]};
    normalize3(f);
    double up[3] = {0, 0, 1};
    normalize3(up);
    double s[3];
    cross3(f, up, s);
    normalize3(s);
    double u[3];
    cross3(s, f, u);
    double M[16] = {s[0], u[0], -f[0], 0, s[1], u[1], -f[1], 0, s[2], u[2], -f[2], 0, 0, 0, 0, 1};
    double Tr[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, -eye[0], -eye[1], -eye[2], 1};
    double V[16];
    mat4_mul(M, Tr, V);
    mat4_inv(V, cam);
}

/* mgl64.TransformCoordinate: homogeneous multiply then divide by w */
static void transform_coordinate(const double* v, const double* m, double* out) {
    double t0 = m[0] * v[0] + m[4] * v[1] + m[8] * v[2] + m[12] * 1.0;
    double t1 = m[1] * v[0] + m[5] * v[1] + m[9] * v[2] + m[13] * 1.0;
    double t2 = m[2] * v[0] + m[6] * v[1] + m[10] * v[2] + m[14] * 1.0;
    double t3 = m[3] * v[0] + m[7] * v[1] + m[11] * v[2] + m[15] * 1.0;
    double iw = 1 / t3;
    out[0] = t0 * iw;
    out[1] = t1 * iw;
    out[2] = t2 * iw;
}

ORC_EXPORT void orc_transform_coordinate(const double* v, const double* m, double* out) {
    transform_coordinate(v, m, out);
}

/* Per-pixel ray of main.go:457-465: origin = eye, direction = vx - eye (not
 * yet normalised; the integrators normalise). */
static void pixel_ray(const double* eye, const double* cam, double f, int res, int i, int j,
                      double* dir) {
    double res_f = (double)res;
    double v[3] = {(double)i / (res_f / 2) - 1, (double)j / (res_f / 2) - 1, -f};
    double vx[3];
    transform_coordinate(v, cam, vx);
    dir[0] = vx[0] - eye[0];
    dir[1] = vx[1] - eye[1];
    dir[2] = vx[2] - eye[2];
}

ORC_EXPORT void orc_pixel_ray(const double* eye, const double* cam, double fov_deg, int res, int i,
                              int j, double* dir) {
    double f = 1 / tan(deg2rad(fov_deg / 2));
    pixel_ray(eye, cam, f, res, i, j, dir);
}

/* ------------------------------------------------------------------------ */
/* Rendering over views and pixels, threaded over pixel rows                 */
/* ------------------------------------------------------------------------ */

#define CUBE_HALF_DIAGONAL 1.74 /* main.go:46 */

typedef struct {
    orc_ctx ctx;
    int hierarchical;
    double ds, R, f;
    int res;
    int nviews;
    const double* eyes;  /* 3 per view */
    const double* cams;  /* 16 per view, column-major */
    /* either a full image set or a ray list */
    const int* rays;     /* (view, i, j) triples, or NULL for all pixels */
    long nrays;
    double* out;         /* transmittance */
    double* out_T;       /* optical depth (optional) */
    long next;           /* work counter (rows or ray chunks) */
    pthread_mutex_t lock;
} orc_job;

static void run_ray(orc_job* J, int v, int i, int j, long slot) {
    double dir[3];
    const double* eye = &J->eyes[3 * v];
    pixel_ray(eye, &J->cams[16 * v], J->f, J->res, i, j, dir);
    double smin = J->R - CUBE_HALF_DIAGONAL, smax = J->R + CUBE_HALF_DIAGONAL;
    double T;
    double val = J->hierarchical ? integrate_hier(&J->ctx, eye, dir, J->ds, smin, smax, &T)
                                 : integrate_simple(&J->ctx, eye, dir, J->ds, smin, smax, &T);
    J->out[slot] = val;
    if (J->out_T) J->out_T[slot] = T;
}

static void* worker(void* arg) {
    orc_job* J = (orc_job*)arg;
    const long chunk = 64;
    for (;;) {
        pthread_mutex_lock(&J->lock);
        long start = J->next;
        J->next += J->rays ? chunk : 1;
        pthread_mutex_unlock(&J->lock);
        if (J->rays) {
            if (start >= J->nrays) break;
            long end = start + chunk < J->nrays ? start + chunk : J->nrays;
            for (long r = start; r < end; r++)
                run_ray(J, J->rays[3 * r], J->rays[3 * r + 1], J->rays[3 * r + 2], r);
        } else {
            long total_rows = (long)J->nviews * J->res;
            if (start >= total_rows) break;
            int v = (int)(start / J->res), i = (int)(start % J->res);
            for (int j = 0; j < J->res; j++)
                run_ray(J, v, i, j, ((long)v * J->res + i) * J->res + j);
        }
    }
    return NULL;
}

static void run_job(orc_job* J, int nthreads) {
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    pthread_mutex_init(&J->lock, NULL);
    J->next = 0;
    pthread_t th[256];
    for (int t = 1; t < nthreads; t++) pthread_create(&th[t], NULL, worker, J);
    worker(J);
    for (int t = 1; t < nthreads; t++) pthread_join(th[t], NULL);
    pthread_mutex_destroy(&J->lock);
}

/* Full render (main.go:429-471): views given by explicit FP64 eye and camera
 * matrices (column-major); out is [view][i][j] transmittance. */
ORC_EXPORT int orc_render(int root, int deform, double dm, double ff, int hierarchical, double ds,
                          double R, double fov_deg, int res, const double* eyes, const double* cams,
                          int nviews, const int* rays, long nrays, double* out, double* out_T,
                          int nthreads) {
    if (root < 0 || root >= g_nnodes || res <= 0 || nviews <= 0 || !(ds > 0)) return 2;
    orc_job J;
    memset(&J, 0, sizeof(J));
    J.ctx.root = root;
    J.ctx.deform = deform;
    J.ctx.density_multiplier = dm;
    J.ctx.flat_field = ff;
    J.hierarchical = hierarchical;
    J.ds = ds;
    J.R = R;
    J.f = 1 / tan(deg2rad(fov_deg / 2));
    J.res = res;
    J.nviews = nviews;
    J.eyes = eyes;
    J.cams = cams;
    J.rays = rays;
    J.nrays = nrays;
    J.out = out;
    J.out_T = out_T;
    run_job(&J, nthreads);
    return 0;
}

/* The CPU semantics applied to the inputs of the reference GPU ABI
 * (cuda_backend.h:78-112): FP32 eye, row-major FP32 camera-to-world matrix,
 * FP32 fov, R, ds and flat field, widened to FP64, and the simple integrator
 * over VoxelGrid.Density. */
ORC_EXPORT int orc_render_f32cams(int vox, const float* cams21, int ncams, int res, float ds,
                                  float ff, double* out, double* out_T, const int* rays, long nrays,
                                  int nthreads);

ORC_EXPORT int orc_render_volume_abi(const float* volume, int nx, int ny, int nz,
                                     const float* cams21, int ncams, int res, float ds, float ff,
                                     double* out, double* out_T, const int* rays, long nrays,
                                     int nthreads) {
    int vox = orc_voxel_f32(volume, nx, ny, nz);
    if (vox < 0) return 3;
    return orc_render_f32cams(vox, cams21, ncams, res, ds, ff, out, out_T, rays, nrays, nthreads);
}

/* The same with an already built root node (voxel grid). */
ORC_EXPORT int orc_render_f32cams(int vox, const float* cams21, int ncams, int res, float ds,
                                  float ff, double* out, double* out_T, const int* rays, long nrays,
                                  int nthreads) {
    double* eyes = (double*)malloc((size_t)ncams * 3 * sizeof(double));
    double* cams = (double*)malloc((size_t)ncams * 16 * sizeof(double));
    if (!eyes || !cams) { free(eyes); free(cams); return 3; }
    /* all cameras must share R and fov: the reference uses one value per run */
    double R = cams21[20], fov = cams21[19];
    for (int c = 0; c < ncams; c++) {
        const float* p = &cams21[21 * c];
        for (int k = 0; k < 3; k++) eyes[3 * c + k] = (double)p[k];
        for (int r = 0; r < 4; r++)
            for (int k = 0; k < 4; k++) cams[16 * c + k * 4 + r] = (double)p[3 + r * 4 + k];
    }
    int rc = orc_render(vox, -1, 1.0, (double)ff, 0, (double)ds, R, fov, res, eyes, cams, ncams,
                        rays, nrays, out, out_T, nthreads);
    free(eyes);
    free(cams);
    return rc;
}

/* Reference sample positions s_k of the uniform integrator: the FP64
 * sequence smin, smin+ds, ... while s < smax (main.go:147).  Returns K. */
ORC_EXPORT long orc_sample_table(double smin, double smax, double ds, double* out, long cap) {
    long k = 0;
    for (double s = smin; s < smax; s += ds) {
        if (out && k < cap) out[k] = s;
        k++;
    }
    return k;
}

/* Auto step (main.go:350-353): MinFeatureSize()/5, per object type
 * (objects.go:74-76,123-125,181-183,257-259,352-354,440-446,584-586,857-860,1034-1037). */
static double min_feature(int id) {
    const orc_node* n = &g_nodes[id];
    switch (n->type) {
    case ORC_SPHERE: return n->a[3];
    case ORC_BOX: {
        double m = n->a[4] < n->a[5] ? n->a[4] : n->a[5];
        m = n->a[3] < m ? n->a[3] : m;
        return 0.1 * m;
    }
    case ORC_CYLINDER: return n->a[6];
    case ORC_PARALLELEPIPED: {
        double m = n->a[14] < n->a[15] ? n->a[14] : n->a[15];
        m = n->a[13] < m ? n->a[13] : m;
        return 0.2 * m;
    }
    case ORC_GYROID: return n->a[3] * n->a[4] * 0.1;
    case ORC_COLLECTION: {
        double out = INFINITY;
        for (int i = 0; i < n->nchild; i++) {
            double m = min_feature(n->child[i]);
            out = m < out ? m : out;
        }
        return out;
    }
    case ORC_UNIT_CELL: return min_feature(n->sub);
    case ORC_TESSELLATED: return min_feature(g_nodes[n->sub].sub);
    case ORC_VOXEL: {
        int m = n->nx > n->ny ? n->nx : n->ny;
        m = m > n->nz ? m : n->nz;
        return 2.0 / (double)m;
    }
    default: return INFINITY;
    }
}

ORC_EXPORT double orc_min_feature_size(int id) { return min_feature(id); }
