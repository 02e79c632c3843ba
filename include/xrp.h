/*
 * xrp.h -- C ABI of libcuda_render.so, the GB300 (sm_103a) projection engine.
 *
 * The library is a drop-in for the dlopen'd native library of
 * igrega348/xray_projection_render: the Go loader (cuda_backend.go:27-43)
 * resolves exactly three symbols, declared first below with the signatures of
 * the reference header (cuda_backend.h).  The remaining entry points are
 * additions that give the same loader access to every object type,
 * deformation and integrator of the reference's CPU path.
 *
 * Conventions shared by every entry point:
 *   - return 0 on success and a positive code on failure; the codes of the
 *     reference functions keep their meaning (1 null pointer, 2 bad sizes,
 *     3-8 device allocation / copy / launch failures), and xrp_last_error()
 *     returns a message for the calling thread;
 *   - calls are synchronous unless they take a stream; host buffers belong to
 *     the caller; the library never frees caller memory;
 *   - transmittance images are float32, laid out [view][i][j] with i the
 *     horizontal and j the vertical pixel index, exactly as the reference's
 *     img[i][j] (main.go:460-470) and out_images (cuda_backend.h:96-97).
 */
#ifndef XRP_H
#define XRP_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define XRP_API __attribute__((visibility("default")))
#else
#define XRP_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------------- */
/* Reference ABI (cuda_backend.h), exported verbatim                         */
/* ------------------------------------------------------------------------- */

/* cuda_backend.h:22-27 */
typedef struct {
    float p0[3];
    float p1[3];
    float radius;
    float rho;
} CylinderParams;

/* cuda_backend.h:78-83: eye, row-major camera-to-world matrix, fov, R. */
typedef struct {
    float eye[3];
    float view[16];
    float fov_y;
    float R;
} XRayCameraParams;

/*
 * Replaces RenderVolumeProjectionsCUDA (cuda_backend.h:101-112,
 * cuda_backend.cu:82-203).  Renders num_cameras projections of a voxel grid
 * stored [z][x][y] (idx = k*nx*ny + i*ny + j).  Unlike the reference GPU
 * kernel, the result follows the reference CPU semantics exactly
 * (VoxelGrid.Density with the (N-1) lattice, objects.go:789-855, and
 * integrate_along_ray, main.go:144-154) evaluated on these FP32 inputs.
 * Codes: 1 null pointer; 2 bad sizes or ds <= 0 / not finite; 3 device
 * allocation; 4 volume upload; 5 table upload; 6 output allocation;
 * 7 kernel failure; 8 copy back.
 */
XRP_API int RenderVolumeProjectionsCUDA(const float* volume, int nx, int ny, int nz,
                                const XRayCameraParams* cameras, int num_cameras, int image_res,
                                float ds, float flat_field, float* out_images);

/*
 * Replaces AssembleVoxelGridCUDA (cuda_backend.h:33-39, cuda_backend.cu:208-292):
 * brute-force cylinder voxelizer, out[k*res*res + i*res + j].
 */
XRP_API int AssembleVoxelGridCUDA(const CylinderParams* cylinders, int num_cylinders, int res,
                          float density_multiplier, float* out_volume);

/*
 * Replaces AssembleVoxelGridSpatialCUDA (cuda_backend.h:58-68,
 * cuda_backend.cu:297-417): the same voxelizer with CSR cell lists.
 */
XRP_API int AssembleVoxelGridSpatialCUDA(const CylinderParams* cylinders, int num_cylinders, int res,
                                 float density_multiplier, int grid_dim, const int* cell_offsets,
                                 const int* cyl_indices, int num_cyl_indices, float* out_volume);

/* ------------------------------------------------------------------------- */
/* Additions                                                                 */
/* ------------------------------------------------------------------------- */

/* Message for the last failure on the calling thread ("" if none).  No
 * counterpart in the reference library; the Go shim keeps its own buffer
 * (cuda_backend.go:22-25). */
XRP_API const char* xrp_last_error(void);

/* Library version, 100*major + minor. */
XRP_API int xrp_version(void);

/* One camera, FP64, as computeCameraFromAngles returns it (main.go:226-239):
 * eye and the column-major (mathgl layout) camera-to-world matrix. */
typedef struct {
    double eye[3];
    double camera[16];
    double fov_deg;
} xrp_camera;

/* computeCameraFromAngles for n (azimuthal, polar) pairs in degrees
 * (main.go:226-239; the angle lists of main.go:242-257, 782-809). */
XRP_API int xrp_cameras_from_angles(const double* az_polar_deg, int n, double R, double fov_deg,
                            xrp_camera* out);

enum { XRP_INTEGRATE_SIMPLE = 0, XRP_INTEGRATE_HIERARCHICAL = 1 };
enum {
    XRP_FLAG_STATS = 1,        /* count evaluated and FP64-re-evaluated samples */
    XRP_FLAG_VOLUME_LOADS = 2, /* voxel-grid roots: per-tap loads instead of texture gathers */
    XRP_FLAG_NO_REFINE = 4,    /* proposal march: no certificate refinement of segments */
    XRP_FLAG_TRACE = 8,        /* per-ray certificate tracing (proposal march without network, batches) */
    XRP_FLAG_BALL = 16,        /* tracing: ball certificates only, even for affine deformation chains */
    XRP_FLAG_PLAIN_INPLACE = 32, /* plain integrator, general scene: FP64 re-evaluation inside the march */
    XRP_FLAG_PLAIN_LIST = 64     /* plain integrator, general scene: the FP64 list pass after the march;
                                    with neither flag the list serves calls of at least 2^22 rays */
};

/* Per-call options: the globals and flags of the reference CLI
 * (main.go:37-41, 683-707, 725-729). */
typedef struct {
    int resolution;            /* image side in pixels */
    int integration;           /* XRP_INTEGRATE_* (main.go:811-819) */
    double ds;                 /* step (> 0); DS for the hierarchical integrator */
    double R;                  /* camera distance; samples span [R-1.74, R+1.74] */
    double flat_field;         /* added to the optical depth (main.go:146) */
    double density_multiplier; /* main.go:139 */
    int flags;                 /* XRP_FLAG_* */
    int reserved;
} xrp_render_opts;

typedef struct xrp_scene xrp_scene;

/* A caller-provided voxel grid for {"type":"voxel_grid","volume":k} entries:
 * FP32 values [z][x][y]; `data` is a host pointer, or a device pointer when
 * `on_device` is 1 (then it must stay valid while the scene lives). */
typedef struct {
    const float* data;
    int nx, ny, nz;
    int on_device;
} xrp_volume_desc;

/*
 * Loads a scene from the reference's JSON object schema (objects.go:658-689:
 * sphere, cube, box, cylinder, parallelepiped, gyroid, object_collection,
 * tessellated_obj_coll, voxel_grid from a .raw path) and an optional
 * deformation map (deformations.go:308-343; NULL or "" for none).  The object
 * tree is flattened once and kept on the current device until
 * xrp_scene_destroy.  Codes: 1 null pointer, 2 schema error (see
 * xrp_last_error), 3 device allocation, 4 upload.
 */
XRP_API int xrp_scene_create(const char* object_json, const char* deformation_json,
                     const xrp_volume_desc* volumes, int num_volumes, xrp_scene** out);
XRP_API void xrp_scene_destroy(xrp_scene* scene);

/* Support box of the scene (where density may be non-zero), world units. */
XRP_API int xrp_scene_support(const xrp_scene* scene, double lo[3], double hi[3]);

/* MinFeatureSize() of the scene's object (objects.go:17, per type
 * objects.go:74-1037): the reference's automatic step is this / 5 when ds < 0
 * (main.go:350-353).  +inf for an empty collection. */
XRP_API int xrp_scene_min_feature_size(const xrp_scene* scene, double* out);

/*
 * Renders `num_views` cameras into host memory `out` (num_views*res*res
 * float32).  Same results as the reference CPU path (main.go:429-471) for the
 * same inputs; runs on the calling thread's current device and returns when
 * the images are in `out`.
 */
XRP_API int xrp_render(xrp_scene* scene, const xrp_camera* views, int num_views, const xrp_render_opts* opts,
               float* out);

/*
 * As xrp_render, but `out_device` is device memory and the work is queued on
 * `stream` (a cudaStream_t, NULL for the legacy default stream); returns
 * after queuing.  The scene and the cameras must not change until the stream
 * has passed this call.  Over a general scene (anything but a lone voxel
 * grid) a call of at least 2^22 rays leaves the samples FP32 cannot decide to
 * one FP64 pass over a list after the march (a ray with a sample that finds
 * the list full is marched again); smaller calls re-evaluate them inside the
 * march, in one launch.  XRP_FLAG_PLAIN_LIST / XRP_FLAG_PLAIN_INPLACE pick
 * one way for every call.
 */
XRP_API int xrp_render_device(xrp_scene* scene, const xrp_camera* views, int num_views,
                      const xrp_render_opts* opts, float* out_device, void* stream);

/* Counters of the last call on this thread that set XRP_FLAG_STATS:
 * samples evaluated and samples re-evaluated in FP64. */
XRP_API int xrp_last_stats(uint64_t* samples, uint64_t* fp64_samples);

/* Frees the device buffers the library caches between calls. */
XRP_API void xrp_release_cache(void);

/* Measured throughput of the texture gathers the voxel kernel issues
 * (tld4 on a layered texture resident in L1), gathers per second on the
 * current device: the peak the voxel kernel's binding unit can reach.  A
 * measurement hook for benchmarks; no counterpart in the reference. */
XRP_API int xrp_probe_gather_rate(double* gathers_per_s);

/*
 * Volume export of any scene (the CPU path of --export_volume,
 * main.go:549-635; the reference GPU voxelizer covers cylinders only):
 * density with the multiplier at x = i/res*2-1, y = j/res*2-1,
 * z = k/res*2-1, layout [k][i][j] (res^3 values).  out_f32: the densities
 * (FP32, equal to the reference's FP64 values rounded); out_u8: the
 * exported bytes byte(v / max * 255) (0 where v <= 0 or max is 0).  Either
 * may be NULL; host buffers; synchronous.
 */
XRP_API int xrp_voxelize_scene(xrp_scene* scene, int res, double density_multiplier, float* out_f32,
                               unsigned char* out_u8);

/*
 * Image finishing on the device (main.go:482-506, cuda_path.go:104-130), so
 * only 2 bytes per pixel cross to the host: for `num_views` images
 * (device, [view][i][j] float32) writes gray = uint16(val * 0xffff) at PNG
 * pixel (x = i, y = res-1-j) into d_gray ([view][y][x]), the alpha plane
 * (0xffff, or with transparency 0xffff where val < 1 and 0 elsewhere) into
 * d_alpha (may be NULL), and each image's (min, max) into d_minmax
 * (2 floats per view).  Device buffers; queued on `stream`.
 */
XRP_API int xrp_finish_images(const float* d_images, int num_views, int res, int transparency,
                              uint16_t* d_gray, uint16_t* d_alpha, float* d_minmax, void* stream);

/*
 * Batched rendering (no counterpart in the reference, which renders one
 * scene per process): many scenes, each with its own cameras and
 * resolution, in one persistent launch whose warps take 32-pixel tiles from
 * a global counter, so uneven items balance across the GPU.  xrp_batch_create
 * flattens and uploads every scene once, picks the tile shape and grid with
 * an autotuner (timed on a sample of the batch's tiles) and captures the
 * launch in a CUDA graph; xrp_batch_render replays the graph.  Results are
 * those of xrp_render for each item.  All items share the options (ds, R,
 * integration, flat field, multiplier; opts->resolution is ignored); with
 * XRP_FLAG_TRACE in opts->flags every ray is rendered by certificate
 * tracing (either integrator), which gives the same results (ray bounds
 * when every scene's deformation chain is affine, unless XRP_FLAG_BALL).
 */
typedef struct {
    xrp_scene* scene;
    const xrp_camera* views;
    int num_views;
    int resolution;
} xrp_batch_item;

typedef struct xrp_batch xrp_batch;

typedef struct {
    long long rays, tiles;
    int tile_w, tile_h;        /* chosen warp tile shape (tile_w * tile_h == 32) */
    int blocks_per_sm, num_sms;
    int tune_candidates;       /* autotuner: shapes x grids timed */
    float tune_ms[8];          /* their times on the sampled tiles */
    float build_ms;            /* flattening, upload, tuning, capture */
} xrp_batch_info;

/* autotune: 1 to time the candidates, 0 for 16x16 tiles at full occupancy. */
XRP_API int xrp_batch_create(const xrp_batch_item* items, int num_items, const xrp_render_opts* opts,
                             int autotune, xrp_batch** out);
/* Replays the captured launch on `stream` (NULL: legacy stream) into the
 * batch's device output; returns after queuing. */
XRP_API int xrp_batch_render(xrp_batch* batch, void* stream);
/* Device output: item k's images (num_views*res*res float32) start at
 * xrp_batch_item_offset(batch, k) floats. */
XRP_API const float* xrp_batch_output(const xrp_batch* batch);
XRP_API long long xrp_batch_item_offset(const xrp_batch* batch, int k);
/* Copies item k's images to host memory (synchronous; ordered after the
 * last xrp_batch_render, whatever its stream). */
XRP_API int xrp_batch_copy_item(const xrp_batch* batch, int k, float* out_host);
XRP_API int xrp_batch_get_info(const xrp_batch* batch, xrp_batch_info* out);
XRP_API void xrp_batch_destroy(xrp_batch* batch);

/*
 * Proposal march (no counterpart in the reference, whose integrators are
 * main.go:144-199).  The plain integrator's samples are cut into segments.
 * A segment whose end densities agree and whose end-point distance
 * certificates cover it is counted as constant.  The rest are either
 * refined (split at the middle sample, halves certified, recursively down to
 * 8 samples) or integrated sample by sample like the plain integrator; a
 * small network (64 positional features -> 3 x 64 ReLU -> 1 logit, BF16
 * weights, FP32 accumulation on tensor cores) proposes which of the two,
 * trained on the GPU on labels the plain integrator produces for the scene.
 * Every sample is either evaluated or covered by a certificate, so results
 * equal the plain integrator's (within FP32 summation order) whatever the
 * network predicts; it changes the speed only.  Analytic scenes and the
 * simple integrator only (code 2 otherwise).
 */
typedef struct xrp_proposal xrp_proposal;

typedef struct {
    int segment;       /* samples per segment, a multiple of 32 (0: 64) */
    int train_rays;    /* rays sampled for training rows (0: 65536) */
    int val_rays;      /* rays sampled for the threshold (0: 32768) */
    int steps;         /* Adam steps (0: 2000) */
    int batch;         /* rows per step (0: 4096) */
    float lr;          /* Adam learning rate (0: 2e-3) */
    float pos_weight;  /* loss weight of non-constant rows (0: 8) */
    float tau_margin;  /* routing threshold = log(pos_weight) + tau_margin */
    uint64_t seed;     /* ray sampling and initialisation */
    int reserved[4];
} xrp_proposal_opts;

typedef struct {
    float tau;           /* logits above tau route a candidate to dense integration */
    int segment;
    long long train_rows, train_pos;  /* candidate segments seen in training / non-constant */
    long long val_rows, val_pos;
    long long val_accepted;           /* validation candidates the network routes to refinement */
    float final_loss;    /* mean weighted BCE over the last 10% of steps */
    float train_ms;      /* wall time of data generation + training */
} xrp_proposal_info;

XRP_API int xrp_proposal_train(xrp_scene* scene, const xrp_camera* views, int num_views,
                               const xrp_render_opts* opts, const xrp_proposal_opts* popts,
                               xrp_proposal** out);
XRP_API int xrp_proposal_get_info(const xrp_proposal* p, xrp_proposal_info* out);
/* Copies the FP32 master parameters (xrp_mlp_param_count() floats; layout
 * W1[64][64], b1[64], W2, b2, W3, b3, w4[64], b4). */
XRP_API int xrp_proposal_params(const xrp_proposal* p, float* out, int n);
XRP_API int xrp_proposal_set_tau(xrp_proposal* p, float tau);
XRP_API void xrp_proposal_destroy(xrp_proposal* p);

/* Renders like xrp_render with the proposal march.  `proposal` NULL: every
 * candidate is refined (or, with XRP_FLAG_NO_REFINE, integrated densely);
 * segment: samples per segment, 0 for the proposal's own or 64.  With
 * XRP_FLAG_TRACE (proposal NULL; simple or hierarchical integrator) each ray
 * is traced on its own: at every evaluated sample the certificate radius
 * says how many following samples share its density, and the march jumps
 * past them (the hierarchical integrator still refines every coarse sample
 * whose zero-ness changes).  When the deformation chain is affine (linear,
 * affine, rigid or none) the certificate is a ray bound, the distance along
 * the ray to the next place where the density can change (the samples lie
 * on a line in object coordinates).  Otherwise the simple integrator uses a
 * curve bound (how far along the ray the curved path of the deformed samples
 * stays clear of every boundary) and the hierarchical one the radius of a
 * ball around the sample; XRP_FLAG_BALL forces balls.  A call of several
 * launch groups runs each group's FP64 pass on a side stream beside the next
 * group's march.  The device variant queues the work on `stream`
 * and then waits for it (it reads back whether the list of samples left to
 * FP64 overflowed, in which case the plain integrator renders the call). */
XRP_API int xrp_render_proposal(xrp_scene* scene, const xrp_proposal* proposal, int segment,
                                const xrp_camera* views, int num_views, const xrp_render_opts* opts,
                                float* out);
XRP_API int xrp_render_proposal_device(xrp_scene* scene, const xrp_proposal* proposal, int segment,
                                       const xrp_camera* views, int num_views,
                                       const xrp_render_opts* opts, float* out_device, void* stream);
/* Counters of the last xrp_render_proposal or xrp_render_proposal_device
 * call on this thread with XRP_FLAG_STATS: segments, segments certified, pieces certified in
 * refinement, pieces integrated densely, dense samples, certificate
 * evaluations, FP64 re-evaluations, network rounds, candidates routed to
 * dense integration, candidates refined, and 1 when the list of samples left
 * to FP64 overflowed (the call was then rendered by the plain integrator). */
XRP_API int xrp_proposal_last_stats(uint64_t out[11]);

/* The network's training step on the GPU, exposed for gradient checks:
 * for `rows` BF16 feature rows X (uint16 bit patterns, [rows][64]) and 0/1
 * labels y, writes the gradient of (1/rows) sum w_r BCE(logit_r, y_r)
 * (w_r = pos_weight for y_r = 1, else 1) with respect to `params` into
 * `grad`, the loss into *loss and the logits into `logits` (each may be
 * NULL).  Host buffers. */
XRP_API int xrp_mlp_param_count(void);
XRP_API int xrp_mlp_grad(const float* params, const uint16_t* X, const float* y, int rows,
                         float pos_weight, float* grad, float* loss, float* logits);

/*
 * RenderVolumeProjectionsCUDA for callers that cannot allocate device
 * memory: a host framework whose allocator owns the device memory, or a
 * service that runs under a fixed device-memory budget decided up front.
 * No counterpart in the reference library.  `d_volume` ([z][x][y], float32)
 * and `d_out` (num_cameras*res*res float32) are device buffers of the
 * caller; `cameras` stay on the host; the work is queued on `stream` (a
 * cudaStream_t, NULL for the legacy stream).  It calls no cudaMalloc,
 * cudaFree or other allocating routine: its tables go to one static 1 MiB
 * device array that every GPU loading the library holds until exit, copied
 * there from host memory before the call returns.  Limits: the tables of one
 * call (about 192 B per camera, 8 B per image row and 12 B per sample of
 * the lattice [R-1.74, R+1.74]) must fit in 1 MiB (code 2 otherwise), and
 * every camera of a call must share R.  The first call on each device looks
 * the array up (cudaGetSymbolAddress).  Calls share the array, so calls that
 * overlap on the GPU race: order them on one stream.  Results equal
 * RenderVolumeProjectionsCUDA's.
 */
XRP_API int xrp_render_volume_noalloc(const float* d_volume, int nx, int ny, int nz,
                                      const XRayCameraParams* cameras, int num_cameras,
                                      int image_res, float ds, float flat_field, float* d_out,
                                      void* stream);

#ifdef __cplusplus
}
#endif

#endif /* XRP_H */
