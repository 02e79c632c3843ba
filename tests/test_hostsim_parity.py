"""The engine's per-pixel code, built for the CPU (tests/hostsim), against
the FP64 oracle.

The same source runs in the CUDA kernels; on the CPU it checks, without a
GPU, the scene flattening, the guard bands that decide each predicate in
FP32, the FP64 re-evaluation of uncertain samples, the lattices and both
integrators.  Tolerance: 1e-5 relative on transmittance."""
import os
import sys

import numpy as np
import pytest

from oracle import oracle as O

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "hostsim"))
import hostsim  # noqa: E402

from xray_projection_render_gb300 import workloads as W  # noqa: E402

REL_TOL = 1e-5


def cams_of(w):
    eyes, cams = O.cameras(w.angles, w.R)
    return np.concatenate([eyes, cams, np.full((len(w.angles), 1), w.fov)], axis=1)


def check(w, integration="simple", nrays=2500, seed=0, **kw):
    rng = np.random.default_rng(seed)
    rays = np.stack([rng.integers(0, len(w.angles), nrays), rng.integers(0, w.res, nrays),
                     rng.integers(0, w.res, nrays)], 1).astype(np.int32)
    obj = {"type": "voxel_grid", "_voxels": w.volume} if w.volume is not None else w.obj
    ref = O.render(O.Scene(obj, w.deformation), w.angles, w.res, w.ds, R=w.R, fov=w.fov,
                   integration=integration, rays=rays,
                   density_multiplier=kw.get("density_multiplier", 1.0),
                   flat_field=kw.get("flat_field", 0.0))
    got, st = hostsim.render(w.obj, cams_of(w), w.res, w.ds, deformation=w.deformation,
                             volume=w.volume, R=w.R, integration=integration, rays=rays, **kw)
    rel = np.abs(got - ref) / ref
    assert rel.max() <= REL_TOL, f"{w.name}: max rel error {rel.max():.3g}"
    return st


@pytest.mark.parametrize("integration", ["simple", "hierarchical"])
def test_cube_minus_sphere_cylinder(integration):
    st = check(W.cube_minus_sphere_cylinder(256), integration)
    assert st[1] < 0.01 * st[0]


@pytest.mark.parametrize("integration", ["simple", "hierarchical"])
def test_deformed_lattice(integration):
    st = check(W.reduced(W.deformed_lattice(), 256, 6), integration)
    assert st[1] < 0.02 * st[0]


@pytest.mark.parametrize("integration", ["simple", "hierarchical"])
def test_fine_candidate_lists(integration):
    # the finer list grids of large calls and batches: 12 cells per axis in
    # the lattice's unit cell, up to 16 in the random scenes' collections
    check(W.reduced(W.deformed_lattice(), 256, 6), integration, nrays=4000, fine_lists=True)
    # a child left out of a cell's list has density 0 there, so the plain
    # march reads the same values with either grid: identical images
    w = W.reduced(W.deformed_lattice(), 96, 3)
    a, _ = hostsim.render(w.obj, cams_of(w), w.res, w.ds, deformation=w.deformation, R=w.R,
                          integration=integration)
    b, _ = hostsim.render(w.obj, cams_of(w), w.res, w.ds, deformation=w.deformation, R=w.R,
                          integration=integration, fine_lists=True)
    assert np.array_equal(a, b)
    for w in W.batched_scenes(6):
        check(W.reduced(w, 128, 3), integration, nrays=600, fine_lists=True)
        check(W.reduced(w, 128, 3), integration, nrays=600, fine_lists=True, trace=True)


@pytest.mark.parametrize("integration", ["simple", "hierarchical"])
@pytest.mark.parametrize("trace", [False, True])
def test_offset_unit_cell(integration, trace):
    # the ray certificates bound the fold cell and not the unit-cell box (the
    # fold cell is that box), which must leave the results exact for a box
    # away from the origin with non-dyadic extents
    w = W.offset_unit_cell()
    check(w, integration, nrays=6000, seed=5, trace=trace)


@pytest.mark.parametrize("integration", ["simple", "hierarchical"])
def test_gyroid_sigmoid(integration):
    check(W.reduced(W.gyroid_sigmoid(), 256, 6), integration)


@pytest.mark.parametrize("integration", ["simple", "hierarchical"])
@pytest.mark.parametrize("general", [False, True])
def test_voxel(integration, general):
    w = W.reduced(W.voxel_blobs(n=48), 192, 6)
    check(w, integration, force_general=general)


def test_batched_scenes():
    for w in W.batched_scenes(10):
        check(W.reduced(w, 128, 3), nrays=800)


def test_multiplier_and_flat_field():
    w = W.cube_minus_sphere_cylinder(128)
    check(w, density_multiplier=1.7, flat_field=0.4)
    check(w, "hierarchical", density_multiplier=1.7, flat_field=0.4)


def test_every_primitive_under_every_deformation():
    prims = [
        {"type": "sphere", "center": [0.1, -0.2, 0.05], "radius": 0.4, "rho": 0.7},
        {"type": "box", "center": [0.0, 0.2, 0.0], "sides": [0.5, 0.3, 0.9], "rho": 0.5},
        {"type": "cylinder", "p0": [-0.5, -0.5, -0.2], "p1": [0.5, 0.4, 0.3], "radius": 0.1},
        {"type": "parallelepiped", "origin": [0.0, 0.0, 0.0], "v0": [0.4, 0.1, 0.0],
         "v1": [0.0, 0.5, 0.1], "v2": [0.1, 0.0, 0.3], "rho": 0.9},
        {"type": "gyroid", "center": [0.0, 0.0, 0.0], "scale": 0.1, "thickness": 0.2, "rho": 1.0},
    ]
    defs = [None,
            {"type": "gaussian", "amplitudes": [0.1, -0.05, 0.02], "sigmas": [0.3, 0.3, 0.5],
             "centers": [0.0, 0.1, 0.0]},
            {"type": "linear", "strains": [0.02, -0.01, 0.05, 0.01, 0.0, 0.03]},
            {"type": "rigid", "displacements": [0.05, -0.1, 0.02]},
            {"type": "sigmoid", "amplitude": 0.2, "center": 0.0, "lengthscale": 0.2,
             "direction": "y"},
            {"type": "affine", "matrix": [[1.1, 0.0, 0.1], [0.0, 0.9, 0.0], [0.05, 0.0, 1.0]]}]
    for p in prims:
        for d in defs:
            check(W.Workload("p", p, d, [(10.0, 80.0), (200.0, 120.0)], 64, 0.01), nrays=600)
    coll = {"type": "object_collection", "objects": prims}
    for d in defs:
        w = W.Workload("c", coll, d, [(10.0, 80.0), (200.0, 120.0)], 64, 0.01)
        check(w, nrays=600)
        check(w, "hierarchical", nrays=600)


def test_greedy_sum_and_cancellation():
    # 0.7 + 0.3 - 1.0 is not exact in FP32: the cancellation guard must hand
    # such samples to FP64 so the hierarchical zero test agrees
    coll = {"type": "object_collection", "objects": [
        {"type": "sphere", "center": [0, 0, 0], "radius": 0.5, "rho": 0.7},
        {"type": "sphere", "center": [0.1, 0, 0], "radius": 0.5, "rho": 0.3},
        {"type": "sphere", "center": [0, 0.1, 0], "radius": 0.45, "rho": -1.0}]}
    for greedy in (False, True):
        c = dict(coll, greedy_dens_eval=greedy)
        w = W.Workload("g", c, None, [(0.0, 90.0), (70.0, 60.0)], 96, 0.004)
        check(w)
        check(w, "hierarchical")


@pytest.mark.parametrize("integration", ["simple", "hierarchical"])
@pytest.mark.parametrize("name", ["gyroid", "gyroid_fine", "lattice", "cube", "batched", "coll_defs", "coll_affine"])
def test_certificate_tracing(name, integration):
    """Certificate tracing (trace_pixel, the algorithm of k_trace and the
    tracing batch kernel), both integrators, against the FP64 oracle on the
    CPU build."""
    if name == "gyroid":
        w = W.reduced(W.gyroid_sigmoid(), 128, 4)
    elif name == "gyroid_fine":
        w = W.reduced(W.gyroid_fine_sigmoid(), 96, 2)
    elif name == "lattice":
        w = W.reduced(W.deformed_lattice(), 128, 3)
    elif name == "cube":
        w = W.cube_minus_sphere_cylinder(128)
    elif name == "batched":
        w = W.reduced(W.batched_scenes(3)[2], 128, 3)
    elif name == "coll_affine":
        # ray certificates of every primitive under a chain of affine steps
        coll = {"type": "object_collection", "objects": [
            {"type": "sphere", "center": [0.1, -0.2, 0.05], "radius": 0.4, "rho": 0.7},
            {"type": "box", "center": [0.0, 0.2, 0.0], "sides": [0.5, 0.3, 0.9], "rho": 0.5},
            {"type": "cylinder", "p0": [-0.5, -0.5, -0.2], "p1": [0.5, 0.4, 0.3], "radius": 0.1},
            {"type": "parallelepiped", "origin": [0.0, 0.0, 0.0], "v0": [0.4, 0.1, 0.0],
             "v1": [0.0, 0.5, 0.1], "v2": [0.1, 0.0, 0.3], "rho": 0.9},
            {"type": "gyroid", "center": [0.0, 0.0, 0.0], "scale": 0.1, "thickness": 0.2, "rho": 1.0}]}
        deform = {"type": "composed", "deformations": [
            {"type": "affine", "matrix": [[1.1, 0.0, 0.1], [0.0, 0.9, 0.0], [0.05, 0.0, 1.0]]},
            {"type": "rigid", "displacements": [0.05, -0.1, 0.02]},
            {"type": "linear", "strains": [0.02, -0.01, 0.05, 0.01, 0.0, 0.03]}]}
        w = W.Workload("c", coll, deform, [(10.0, 80.0), (200.0, 120.0), (95.0, 40.0)], 96, 0.004)
    else:
        coll = {"type": "object_collection", "objects": [
            {"type": "sphere", "center": [0.1, -0.2, 0.05], "radius": 0.4, "rho": 0.7},
            {"type": "cylinder", "p0": [-0.5, -0.5, -0.2], "p1": [0.5, 0.4, 0.3], "radius": 0.1},
            {"type": "gyroid", "center": [0.0, 0.0, 0.0], "scale": 0.1, "thickness": 0.2, "rho": 1.0}]}
        w = W.Workload("c", coll, {"type": "gaussian", "amplitudes": [0.1, -0.05, 0.02],
                                   "sigmas": [0.3, 0.3, 0.5], "centers": [0.0, 0.1, 0.0]},
                       [(10.0, 80.0), (200.0, 120.0)], 64, 0.01)
    st = check(w, integration, nrays=1500, trace=True)
    assert st[0] > 0


@pytest.mark.parametrize("res", [64, 96, 512, 1024])
def test_double_float_ray_setup_matches_fp64(res):
    """The FP32-only ray setup of the march (double-float camera, pixel table
    and s_c) gives the FP32 origin and direction of the FP64 setup: the same
    floats but for rare rounding ties."""
    import ctypes
    rng = np.random.default_rng(res)
    angles = [(float(a), float(p)) for a, p in zip(rng.uniform(0, 360, 24), rng.uniform(5, 175, 24))]
    w = W.Workload("r", {"type": "sphere", "center": [0, 0, 0], "radius": 0.5, "rho": 1.0}, None,
                   angles, res, 0.01)
    cams = np.ascontiguousarray(cams_of(w))
    n = 20000
    rays = np.stack([rng.integers(0, len(angles), n), rng.integers(0, res, n), rng.integers(0, res, n)],
                    1).astype(np.int32)
    a = np.zeros((n, 6), np.float32)
    b = np.zeros((n, 6), np.float32)
    L = hostsim.lib()
    L.hs_ray_setup.restype = ctypes.c_int
    L.hs_ray_setup.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                               ctypes.c_void_p, ctypes.c_long, ctypes.c_void_p, ctypes.c_void_p]
    assert L.hs_ray_setup(cams.ctypes.data, len(angles), res, w.R, rays.ctypes.data, n,
                          a.ctypes.data, b.ctypes.data) == 0
    same = a == b
    assert same.mean() > 0.999
    # one unit apart at most, or (origins near 0, where o + d s_c cancels)
    # within 1e-12, the absolute term of the position error bound
    ulp = np.spacing(np.abs(b).astype(np.float32))
    assert np.all(np.abs(a - b) <= np.maximum(ulp, 1e-12))


@pytest.mark.parametrize("integration", ["simple", "hierarchical"])
def test_tracing_far_narrow_camera(integration):
    """Ray and ball certificates with a distant, narrow camera (R 20, fov 12):
    larger position error bounds and capsule radius."""
    coll = {"type": "object_collection", "objects": [
        {"type": "sphere", "center": [0.1, -0.2, 0.05], "radius": 0.4, "rho": 0.7},
        {"type": "cylinder", "p0": [-0.5, -0.5, -0.2], "p1": [0.5, 0.4, 0.3], "radius": 0.1},
        {"type": "parallelepiped", "origin": [0.0, 0.0, 0.0], "v0": [0.4, 0.1, 0.0],
         "v1": [0.0, 0.5, 0.1], "v2": [0.1, 0.0, 0.3], "rho": 0.9}]}
    for deform in (None, {"type": "affine", "matrix": [[1.1, 0.0, 0.1], [0.0, 0.9, 0.0], [0.05, 0.0, 1.0]]},
                   {"type": "gaussian", "amplitudes": [0.1, -0.05, 0.02], "sigmas": [0.3, 0.3, 0.5],
                    "centers": [0.0, 0.1, 0.0]}):
        w = W.Workload("far", coll, deform, [(10.0, 80.0), (200.0, 120.0)], 64, 0.004, R=20.0, fov=12.0)
        check(w, integration, nrays=1200, trace=True)


def _nested_lattice(depth):
    """Tessellations nested `depth` deep; the innermost unit cell holds eight
    struts of density 1 (a uniform greedy collection with candidate lists),
    the middle one mixes densities (not uniform)."""
    a = 0.2
    struts = [{"type": "cylinder", "p0": [0.0, u, v], "p1": [a, u, v], "radius": 0.02, "rho": 1.0}
              for u in (0.0, a) for v in (0.0, a)]
    struts += [{"type": "cylinder", "p0": [u, 0.0, v], "p1": [u, a, v], "radius": 0.02, "rho": 1.0}
               for u in (0.0, a) for v in (0.0, a)]
    obj = {"type": "tessellated_obj_coll",
           "uc": {"objects": {"type": "object_collection", "objects": struts},
                  "xmin": 0, "xmax": a, "ymin": 0, "ymax": a, "zmin": 0, "zmax": a},
           "xmin": 0, "xmax": 0.4, "ymin": 0, "ymax": 0.4, "zmin": 0, "zmax": 0.4}
    if depth == 1:
        obj.update(xmin=-1, xmax=1, ymin=-1, ymax=1, zmin=-1, zmax=1)
    for level in range(1, depth):
        objs = [obj, {"type": "sphere", "center": [0.45, 0.45, 0.45], "radius": 0.04, "rho": 0.5}]
        size = 0.5 * (2 ** (level - 1)) if level < depth - 1 else 0.5
        hi = 1.0 if level == depth - 1 else 2 * size
        lo = -1.0 if level == depth - 1 else 0.0
        obj = {"type": "tessellated_obj_coll",
               "uc": {"objects": {"type": "object_collection", "objects": objs},
                      "xmin": 0, "xmax": 0.5, "ymin": 0, "ymax": 0.5, "zmin": 0, "zmax": 0.5},
               "xmin": lo, "xmax": hi, "ymin": lo, "ymax": hi, "zmin": lo, "zmax": hi}
    return obj


@pytest.mark.parametrize("integration", ["simple", "hierarchical"])
@pytest.mark.parametrize("name", ["gyroid", "gyroid_fine", "coll_defs", "lattice_gauss"])
def test_curved_ray_tracing(name, integration):
    """Curved-ray certificates (CPU build) for non-affine chains: the traced
    renders match the oracle, with fewer evaluations than ball certificates
    on the gyroid."""
    gauss = {"type": "gaussian", "amplitudes": [0.1, -0.05, 0.02], "sigmas": [0.3, 0.3, 0.5],
             "centers": [0.0, 0.1, 0.0]}
    if name == "gyroid":
        w = W.reduced(W.gyroid_sigmoid(), 128, 4)
    elif name == "gyroid_fine":
        w = W.reduced(W.gyroid_fine_sigmoid(), 96, 2)
    elif name == "lattice_gauss":
        base = W.reduced(W.deformed_lattice(), 96, 3)
        w = W.Workload("lattice_gauss", base.obj, gauss, base.angles, base.res, base.ds)
    else:
        coll = {"type": "object_collection", "objects": [
            {"type": "sphere", "center": [0.1, -0.2, 0.05], "radius": 0.4, "rho": 0.7},
            {"type": "cylinder", "p0": [-0.5, -0.5, -0.2], "p1": [0.5, 0.4, 0.3], "radius": 0.1},
            {"type": "gyroid", "center": [0.0, 0.0, 0.0], "scale": 0.1, "thickness": 0.2, "rho": 1.0}]}
        w = W.Workload("c", coll, gauss, [(10.0, 80.0), (200.0, 120.0)], 64, 0.01)
    st_curve = check(w, integration, nrays=1500, trace="curve")
    if name == "gyroid" and integration == "simple":
        st_ball = check(w, integration, nrays=1500, trace=True)
        assert 2 * st_curve[0] < st_ball[0]


@pytest.mark.parametrize("integration", ["simple", "hierarchical"])
@pytest.mark.parametrize("depth", [1, 2, 3])
def test_tracing_nested_tessellations(depth, integration):
    """Ray certificates through nested tessellations (folds at every level,
    uniform and mixed unit cells) under a linear strain, and ball
    certificates under a gaussian deformation."""
    obj = _nested_lattice(depth)
    for deform in ({"type": "linear", "strains": [0.01, 0.0, 0.05, 0.0, 0.02, 0.0]},
                   {"type": "gaussian", "amplitudes": [0.05, -0.03, 0.02], "sigmas": [0.4, 0.4, 0.5],
                    "centers": [0.0, 0.1, 0.0]}):
        w = W.Workload("nested", obj, deform, [(30.0, 75.0), (200.0, 110.0)], 64, 0.004)
        check(w, integration, nrays=1500, trace=True)
        if deform["type"] == "gaussian":
            check(w, integration, nrays=1500, trace="curve")


def test_fp64_evaluators_exact_at_cylinder_surfaces():
    """The FP64 evaluators (every primitive in FP64, and the FP64 pass's
    hybrid, which decides primitives in FP32 where that is certain and tests
    a cylinder's radius against a threshold precomputed on the host instead
    of taking the square root) equal the oracle exactly at points within
    1e-15 to 1e-6 of the deformed lattice's strut surfaces."""
    w = W.deformed_lattice()
    rng = np.random.default_rng(17)
    cell = W.lattice_unit_cell()
    struts = [o for o in cell["objects"]["objects"]] if "objects" in cell.get("objects", {}) else cell["objects"]
    pts = []
    for _ in range(3000):
        c = struts[rng.integers(len(struts))]
        p0, p1, r = np.array(c["p0"]), np.array(c["p1"]), c["radius"]
        v = p1 - p0
        t = rng.uniform(-0.05, 1.05)
        nrm = np.cross(v, rng.normal(size=3))
        nrm /= np.linalg.norm(nrm)
        off = rng.choice([-1, 1]) * 10.0 ** rng.uniform(-15, -6)
        q = p0 + t * v + (r + off) * nrm  # object space, near the strut's side
        q += 0.2 * rng.integers(-5, 5, size=3)  # some tessellation cell
        # back to world space through the linear strain (z scaled by 1.05)
        pts.append([q[0], q[1], q[2] / 1.05])
    pts = np.array(pts)
    d64, hyb = hostsim.density64(w.obj, pts, deformation=w.deformation)
    sc = O.Scene(w.obj, w.deformation)
    ref = np.array([sc.density(*p) for p in pts])
    assert np.array_equal(d64, ref)
    assert np.array_equal(hyb, ref)
    assert 0 < np.count_nonzero(ref) < len(ref)


def test_sqrt_threshold_is_exact():
    """The FP64 cylinder test compares the squared distance s with T instead
    of sqrt(s) with the radius r: T is the smallest double whose correctly
    rounded square root reaches r, so sqrt(s) < r exactly when s < T
    (checked at T and its neighbours, for radii over many decades and the
    special values)."""
    import ctypes as C
    rng = np.random.default_rng(5)
    r = np.concatenate([10.0 ** rng.uniform(-6, 3, 20000), [0.03, 0.1, 1.0, 2.0, 0.0, -1.0, np.inf]])
    T = np.zeros_like(r)
    L = hostsim.lib()
    L.hs_sqrt_threshold.restype = None
    L.hs_sqrt_threshold.argtypes = [C.c_void_p, C.c_long, C.c_void_p]
    L.hs_sqrt_threshold(r.ctypes.data, len(r), T.ctypes.data)
    fin = np.isfinite(r) & (r > 0)
    below = np.nextafter(T[fin], 0.0)
    assert np.all(np.sqrt(T[fin]) >= r[fin])
    assert np.all(np.sqrt(below) < r[fin])
    assert np.all(T[~fin][:2] == 0.0) and T[-1] == np.inf
    # and the equivalence on random squared distances near r^2
    s = (r[fin] ** 2)[:, None] * (1.0 + rng.uniform(-1e-12, 1e-12, (fin.sum(), 8)))
    assert np.array_equal(np.sqrt(s) < r[fin][:, None], s < T[fin][:, None])
