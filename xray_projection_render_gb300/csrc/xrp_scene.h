// xrp_scene.h -- host side of the engine: the reference object schema is
// read, validated and flattened into the structure-of-arrays scene image of
// xrp_device.h, together with the guard bands that let the FP32 evaluator
// decide the reference's predicates, the per-cell candidate lists of large
// collections and the support box used to clip rays.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include "xrp_device.h"
#include "xrp_json.h"

namespace xrp {

// One node of the object tree as loaded (before flattening).
struct HNode {
    int type = 0;            // NodeType
    double d[16] = {0};      // exact reference parameters (Node64 layout)
    bool greedy = false;     // COLL
    bool clip = true;        // COLL
    std::vector<int> kids;   // COLL
    int sub = -1;            // TESS: unit-cell collection node
    int vol = -1;            // VOXEL: volume index
};

struct HVolume {
    std::vector<float> data;     // host copy ([z][x][y]); empty if external
    std::vector<double> data64;  // exact values when FP32 cannot hold them
    const float* ext = nullptr;  // caller-owned device data (no copy)
    int nx = 0, ny = 0, nz = 0;
};

struct HDef {
    int type = 0;  // DefType
    int axis = 0;
    double d[12] = {0};
};

struct HostScene {
    std::vector<HNode> nodes;
    int root = -1;
    std::vector<HDef> defs;      // composed deformations flattened in order
    std::vector<HVolume> vols;
};

class SchemaError : public std::runtime_error {
  public:
    using std::runtime_error::runtime_error;
};

// Builds the tree from the reference JSON schema (objects.NewObject,
// objects.go:658-689, and the FromMap methods).  External volumes (the
// "volume": k extension) are taken from `ext_vols`.
HostScene load_scene(const char* object_json, const char* deformation_json,
                     const std::vector<HVolume>& ext_vols);

// A scene made of one voxel grid (the RenderVolumeProjectionsCUDA path).
HostScene volume_scene(const float* data_dev, int nx, int ny, int nz);

// MinFeatureSize of the root object (the Object interface, objects.go:17).
double min_feature_size(const HostScene& hs);

// T such that, for every double s, sqrt(s) < r exactly when s < T, with
// sqrt correctly rounded (as the host's std::sqrt and the device's
// __dsqrt_rn are): the FP64 cylinder test compares with T instead of taking
// the square root.
double sqrt_lt_threshold(double r);

// Inputs of the error analysis that are fixed per render call.
struct RenderGeometry {
    double R = 4.0;        // camera distance
    double fov_deg = 40.0;
    double half_span = 1.74;  // smax - s_c
};

// Flattened, device-ready arrays (host copies) plus the scene header.
struct FlatScene {
    std::vector<Node> nodes;
    std::vector<Node64> nodes64;
    std::vector<int32_t> child;
    std::vector<int32_t> cells;
    std::vector<int32_t> items;
    std::vector<float> clear;  // per cell of `cells`: distance to the nearest unlisted child
    std::vector<DefStep> defs;
    int root = 0;
    bool bounded = true;
    double sup_lo[3], sup_hi[3];  // support box (world, FP64, undilated)
    float sup32_lo[3], sup32_hi[3];
    bool volume_root = false;     // root is a voxel grid and there is no deformation
    double vol_band_w = 0.0;      // world-space guard band of the voxel bounds test
    int depth = 0;                // deepest tessellation nesting (0: none)
    double def_lip = 1.0;         // Lipschitz bound of the deformation chain
    double margin_slack = 0.0;    // error allowance of certificate radii (deformed units)
    bool affine = true;           // deformation chain affine and invertible (ray certificates)
    double ray_slack = 0.0;       // capsule radius of ray certificates (deformed units)
    double curve_acc = 0.0;       // bound on |d^2 q/ds^2| of the deformed point along a unit ray
};

// `tracing`: the scene is rendered by certificate tracing (coarser candidate
// lists for uniform collections, see Flattener::coll).  `fine_lists`: finer
// candidate-list grids, which shorten the lists the march reads per sample
// but take longer to build (for large calls and for batches, which flatten
// once and replay).
FlatScene flatten(const HostScene& hs, const RenderGeometry& g, bool hierarchical, bool tracing = false,
                  bool fine_lists = false);

// mathgl restatement for the host-side camera (main.go:226-239).
void camera_from_angles(double az_deg, double polar_deg, double R, double eye[3], double m[16]);
void view_from_camera(const double eye[3], const double m[16], double fov_deg, ViewDev& v);

// Sample lattices (main.go:147 and main.go:171-197).
struct HostLattice {
    std::vector<double> s64;
    std::vector<float> t32;
    std::vector<int32_t> fstart;
    std::vector<double> f64;
    std::vector<float> ft32;
    Lattice hdr;  // pointers filled in after upload
};
HostLattice build_lattice(double R, double ds, bool hierarchical);

std::vector<double> pixel_table(int res);

// Host half of a render call: the flattened scene, the sample lattice, the
// pixel table and the volume descriptors, with every device pointer left
// null for the caller to fill in after the upload.
struct HostPrepared {
    FlatScene fs;
    HostLattice hl;
    std::vector<double> xs;
    std::vector<float> xsf;  // xs as (hi, lo) float pairs
    std::vector<Volume> vols;
    SceneDev S;       // pointers null
    RenderParams P;   // xs null
    bool volume_fast = false;
};
HostPrepared prepare_host(const HostScene& hs, int res, int integration, double ds, double R,
                          double flat_field, double density_multiplier, double fov_max, bool tracing = false,
                          bool fine_lists = false);

}  // namespace xrp
