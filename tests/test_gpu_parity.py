"""GPU parity: the sm_103a engine against the FP64 oracle, through the C ABI.

Bar (from the engine's contract): transmittance within 1e-5 relative of the
oracle -- the reference CPU algorithm restated in FP64 -- on the same inputs.
Sizes are reduced so the oracle finishes in seconds; full-size runs are
checked on a seeded subset of rays.
"""
import json

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

REL_TOL = 1e-5


@pytest.fixture(scope="module")
def X():
    import torch
    torch.cuda.set_device(0)
    import __graft_entry__ as g
    g.build()
    import xray_projection_render_gb300 as X
    return X


def W():
    from xray_projection_render_gb300 import workloads
    return workloads


def _oracle_obj(w):
    return {"type": "voxel_grid", "_voxels": w.volume} if w.volume is not None else w.obj


def _compare(got, ref, tol=REL_TOL):
    rel = np.abs(got.astype(np.float64) - ref) / ref
    assert np.all(np.isfinite(got))
    assert rel.max() <= tol, f"max rel error {rel.max():.3g} (>{tol}) at {np.unravel_index(rel.argmax(), rel.shape)}"
    return rel.max()


def _render_both(X, w, integration="simple", stats=False, **kw):
    vols = [w.volume] if w.volume is not None else []
    with X.Scene(w.obj, w.deformation, vols) as s:
        r = X.render(s, w.angles, resolution=w.res, ds=w.ds, R=w.R, fov=w.fov,
                     integration=integration, stats=stats, **kw)
    ref = O.render(O.Scene(_oracle_obj(w), w.deformation), w.angles, w.res, w.ds, R=w.R,
                   fov=w.fov, integration=integration,
                   density_multiplier=kw.get("density_multiplier", 1.0),
                   flat_field=kw.get("flat_field", 0.0))
    return r, ref


@pytest.mark.parametrize("integration", ["simple", "hierarchical"])
def test_offset_unit_cell_traced(X, integration):
    """A tessellated unit cell away from the origin with non-dyadic extents:
    ray certificates bound the fold cell only (it is the unit cell's box)."""
    w = W().offset_unit_cell()
    kw = dict(resolution=w.res, ds=w.ds, R=w.R, fov=w.fov, integration=integration)
    with X.Scene(w.obj, w.deformation) as s:
        traced = X.render_proposal(s, None, w.angles, trace=True, **kw)
        plain = X.render(s, w.angles, **kw)
    ref = O.render(O.Scene(w.obj, w.deformation), w.angles, w.res, w.ds, R=w.R, fov=w.fov,
                   integration=integration)
    _compare(traced, ref)
    _compare(plain, ref)


@pytest.mark.parametrize("integration", ["simple", "hierarchical"])
def test_cube_minus_sphere_cylinder_full_size(X, integration):
    w = W().cube_minus_sphere_cylinder(512)
    (got, ns, nf), ref = _render_both(X, w, integration, stats=True)
    _compare(got, ref)
    assert nf < 0.01 * ns


@pytest.mark.parametrize("integration", ["simple", "hierarchical"])
def test_deformed_lattice_reduced(X, integration):
    w = W().reduced(W().deformed_lattice(), 128, 4)
    got, ref = _render_both(X, w, integration)
    _compare(got, ref)


@pytest.mark.parametrize("integration", ["simple", "hierarchical"])
def test_gyroid_sigmoid_reduced(X, integration):
    w = W().reduced(W().gyroid_sigmoid(), 128, 4)
    got, ref = _render_both(X, w, integration)
    _compare(got, ref)


@pytest.mark.parametrize("integration", ["simple", "hierarchical"])
@pytest.mark.parametrize("name", ["deformed_lattice", "gyroid_sigmoid", "cube_minus_sphere_cylinder"])
def test_plain_fp64_list_matches_inplace(X, name, integration):
    """The plain integrator's two FP64 passes: the list after the march
    (default) and the re-evaluation inside it.  The FP32 decisions are the
    same, so they count the same samples; the images agree to FP32 rounding
    (the list's values are added to the optical depth after the march), on
    the host path and the device path alike, and match the oracle."""
    import torch
    w = getattr(W(), name)()
    w = W().reduced(w, 96, 3)
    kw = dict(resolution=w.res, ds=w.ds, R=w.R, fov=w.fov, integration=integration)
    with X.Scene(w.obj, w.deformation) as s:
        a, na, fa = X.render(s, w.angles, stats=True, plain_fp64="list", **kw)
        b, nb, fb = X.render(s, w.angles, stats=True, plain_fp64="inplace", **kw)
        auto = X.render(s, w.angles, **kw)  # a small call: in place
        dev = torch.empty((len(w.angles), w.res, w.res), dtype=torch.float32, device="cuda")
        X.render(s, w.angles, out=dev, plain_fp64="list", **kw)
        torch.cuda.synchronize()
        d = dev.cpu().numpy()
    assert (na, fa) == (nb, fb)  # the same FP32 decisions
    assert np.array_equal(auto, b)
    if name == "deformed_lattice":
        assert fa > 0
    np.testing.assert_allclose(a, b, rtol=2e-6, atol=1e-7)
    np.testing.assert_allclose(d, a, rtol=2e-6, atol=1e-7)
    ref = O.render(O.Scene(w.obj, w.deformation), w.angles, w.res, w.ds, R=w.R, fov=w.fov,
                   integration=integration)
    _compare(a, ref)


@pytest.mark.parametrize("res", [97, 33])
def test_merged_fp64_on_partial_warps(X, res):
    """Odd image sizes leave lanes of the edge tiles outside the image: the
    warp-merged FP64 re-evaluations (hierarchical tracing, the traced batch)
    ballot over the lanes that march only.  Both match the oracle."""
    w = W().reduced(W().deformed_lattice(), res, 2)
    g = W().reduced(W().gyroid_sigmoid(), res, 2)
    kw = dict(resolution=res, ds=w.ds, R=w.R, fov=w.fov)
    with X.Scene(w.obj, w.deformation) as s, X.Scene(g.obj, g.deformation) as sg:
        hier = X.render_proposal(s, None, w.angles, trace=True, integration="hierarchical", **kw)
        hier_g = X.render_proposal(sg, None, g.angles, trace=True, integration="hierarchical",
                                   resolution=res, ds=g.ds, R=g.R, fov=g.fov)
        with X.Batch([(s, w.angles, res), (sg, g.angles, res)], ds=w.ds, trace=True) as b:
            b.render()
            batch_l, batch_g = b.item(0), b.item(1)
    _compare(hier, O.render(O.Scene(w.obj, w.deformation), w.angles, res, w.ds, R=w.R, fov=w.fov,
                            integration="hierarchical"))
    _compare(hier_g, O.render(O.Scene(g.obj, g.deformation), g.angles, res, g.ds, R=g.R, fov=g.fov,
                              integration="hierarchical"))
    _compare(batch_l, O.render(O.Scene(w.obj, w.deformation), w.angles, res, w.ds, R=w.R, fov=w.fov))
    _compare(batch_g, O.render(O.Scene(g.obj, g.deformation), g.angles, res, w.ds, R=g.R, fov=g.fov))


@pytest.mark.parametrize("integration", ["simple", "hierarchical"])
def test_fp64_list_overflow_paths(X, integration, monkeypatch):
    """A 16-entry FP64 list (the XRP_FALLBACK_LIST test hook) overflows on
    the lattice.  The plain mode marches the rays that lost a sample again
    (FP64 inside the march): the result equals the in-place re-evaluation to
    FP32 rounding.  Tracing renders the call again with the plain kernel and
    reports the overflow.  Both match the oracle."""
    w = W().reduced(W().deformed_lattice(), 96, 2)
    kw = dict(resolution=w.res, ds=w.ds, R=w.R, fov=w.fov, integration=integration)
    with X.Scene(w.obj, w.deformation) as s:
        inplace = X.render(s, w.angles, plain_fp64="inplace", **kw)
        monkeypatch.setenv("XRP_FALLBACK_LIST", "16")
        listed, ns, nf = X.render(s, w.angles, stats=True, plain_fp64="list", **kw)
        traced, st = X.render_proposal(s, None, w.angles, trace=True, stats=True, **kw)
    assert nf > 16 and st["fp64_list_overflow"] == 1
    np.testing.assert_allclose(listed, inplace, rtol=2e-6, atol=1e-7)
    ref = O.render(O.Scene(w.obj, w.deformation), w.angles, w.res, w.ds, R=w.R, fov=w.fov,
                   integration=integration)
    _compare(listed, ref)
    _compare(traced, ref)


@pytest.mark.parametrize("integration", ["simple", "hierarchical"])
@pytest.mark.parametrize("path", ["gather", "loads"])
def test_voxel_scene_reduced(X, integration, path):
    w = W().reduced(W().voxel_blobs(n=64), 128, 6)
    got, ref = _render_both(X, w, integration, volume_path=path)
    _compare(got, ref)


def test_voxel_gather_and_loads_agree_non_cubic(X):
    # non-cubic grid: catches any axis or component-order mix-up in the gathers
    vol = W().gaussian_blob_volume(40, 12, seed=9)[:24, :40, :31].copy()  # nz=24, nx=40, ny=31
    angles = [(0.0, 90.0), (63.0, 50.0), (250.0, 130.0)]
    with X.Scene({"type": "voxel_grid", "volume": 0}, None, [vol]) as s:
        a = X.render(s, angles, resolution=80, ds=0.01)
        b = X.render(s, angles, resolution=80, ds=0.01, volume_path="loads")
    ref = O.render(O.Scene({"type": "voxel_grid", "_voxels": vol}), angles, 80, 0.01)
    _compare(a, ref)
    _compare(b, ref)


def test_batched_random_scenes(X):
    for w in W().batched_scenes(8):
        w = W().reduced(w, 96, 3)
        got, ref = _render_both(X, w)
        _compare(got, ref)


def test_flat_field_and_multiplier(X):
    w = W().cube_minus_sphere_cylinder(96)
    got, ref = _render_both(X, w, flat_field=0.3, density_multiplier=2.5)
    _compare(got, ref)
    got, ref = _render_both(X, w, "hierarchical", flat_field=0.3, density_multiplier=2.5)
    _compare(got, ref)


def test_every_primitive_and_deformation(X):
    prims = [
        {"type": "sphere", "center": [0.1, -0.2, 0.05], "radius": 0.4, "rho": 0.7},
        {"type": "box", "center": [0.0, 0.2, 0.0], "sides": [0.5, 0.3, 0.9], "rho": 0.5},
        {"type": "cube", "center": [-0.3, 0.0, 0.1], "side": 0.35, "rho": 1.2},
        {"type": "cylinder", "p0": [-0.5, -0.5, -0.2], "p1": [0.5, 0.4, 0.3], "radius": 0.1},
        {"type": "parallelepiped", "origin": [0.0, 0.0, 0.0], "v0": [0.4, 0.1, 0.0],
         "v1": [0.0, 0.5, 0.1], "v2": [0.1, 0.0, 0.3], "rho": 0.9},
        {"type": "gyroid", "center": [0.0, 0.0, 0.0], "scale": 0.1, "thickness": 0.2,
         "rho": 1.0},
    ]
    defs = [None,
            {"type": "gaussian", "amplitudes": [0.1, -0.05, 0.02], "sigmas": [0.3, 0.3, 0.5],
             "centers": [0.0, 0.1, 0.0]},
            {"type": "linear", "strains": [0.02, -0.01, 0.05, 0.01, 0.0, 0.03]},
            {"type": "rigid", "displacements": [0.05, -0.1, 0.02]},
            {"type": "sigmoid", "amplitude": 0.2, "center": 0.0, "lengthscale": 0.2,
             "direction": "x"},
            {"type": "affine", "matrix": [[1.1, 0.0, 0.1], [0.0, 0.9, 0.0], [0.05, 0.0, 1.0]]},
            {"type": "composed", "deformations": [
                {"type": "rigid", "displacements": [0.0, 0.05, 0.0]},
                {"type": "linear", "strains": [0.0, 0.0, 0.1, 0.0, 0.0, 0.0]}]}]
    angles = [(10.0, 80.0), (200.0, 120.0)]
    for p in prims:
        for d in defs:
            w = W().Workload("prim", p, d, angles, 48, 0.01)
            got, ref = _render_both(X, w)
            _compare(got, ref)
    coll = {"type": "object_collection", "objects": prims}
    for d in defs:
        w = W().Workload("coll", coll, d, angles, 48, 0.01)
        got, ref = _render_both(X, w)
        _compare(got, ref)
        got, ref = _render_both(X, w, "hierarchical")
        _compare(got, ref)


def test_reference_example_scenes(X):
    examples = [
        {"objects": [{"center": [-0.5, -0.5, 0], "radius": 0.15, "rho": 1, "type": "sphere"},
                     {"center": [0.5, 0.5, 0], "radius": 0.15, "rho": 1, "type": "sphere"}],
         "type": "object_collection"},
        {"type": "object_collection", "objects": [
            {"type": "cube", "side": 1.5, "center": [0.0, 0.0, 0.0], "rho": 0.7},
            {"type": "sphere", "radius": 0.3, "center": [0.1, 0.2, 0.0], "rho": -1.0},
            {"type": "cylinder", "radius": 0.3, "p0": [0.1, 0.2, 0.0], "p1": [0.1, 0.2, 0.8],
             "rho": -1.0}]},
        {"uc": {"objects": {"objects": [{"p0": [0.25, 0.25, 0.75], "p1": [0.25, 0.25, -0.75],
                                          "radius": 0.1, "rho": 1, "type": "cylinder"}],
                            "type": "object_collection"},
                "type": "unit_cell", "xmax": 0.5, "xmin": 0.0, "ymax": 0.5, "ymin": 0.0,
                "zmax": 1.0, "zmin": -1.0},
         "type": "tessellated_obj_coll", "xmax": 1.0, "xmin": -1.0, "ymax": 1.0, "ymin": -1.0,
         "zmax": 1.0, "zmin": -1.0},
    ]
    for obj in examples:
        w = W().Workload("example", obj, None, [(0.0, 90.0), (45.0, 60.0)], 64, 0.005)
        got, ref = _render_both(X, w)
        _compare(got, ref)


def test_nested_tessellation_and_voxel_in_collection(X):
    inner = {"type": "tessellated_obj_coll",
             "uc": {"objects": {"type": "object_collection", "objects": [
                 {"type": "sphere", "center": [0.1, 0.1, 0.1], "radius": 0.08, "rho": 1.0}]},
                    "xmin": 0, "xmax": 0.2, "ymin": 0, "ymax": 0.2, "zmin": 0, "zmax": 0.2},
             "xmin": 0, "xmax": 0.4, "ymin": 0, "ymax": 0.4, "zmin": 0, "zmax": 0.4}
    outer = {"type": "tessellated_obj_coll",
             "uc": {"objects": {"type": "object_collection", "objects": [inner]},
                    "xmin": 0, "xmax": 0.5, "ymin": 0, "ymax": 0.5, "zmin": 0, "zmax": 0.5},
             "xmin": -1, "xmax": 1, "ymin": -1, "ymax": 1, "zmin": -1, "zmax": 1}
    w = W().Workload("nested", outer, None, [(30.0, 75.0)], 64, 0.005)
    got, ref = _render_both(X, w)
    _compare(got, ref)
    vol = W().gaussian_blob_volume(24, 6, seed=7)
    coll = {"type": "object_collection", "objects": [
        {"type": "voxel_grid", "volume": 0},
        {"type": "sphere", "center": [0.3, 0.0, 0.0], "radius": 0.3, "rho": -0.5}]}
    with X.Scene(coll, None, [vol]) as s:
        got = X.render(s, [(20.0, 90.0)], resolution=64, ds=0.01)
    ocoll = {"type": "object_collection", "objects": [
        {"type": "voxel_grid", "_voxels": vol},
        {"type": "sphere", "center": [0.3, 0.0, 0.0], "radius": 0.3, "rho": -0.5}]}
    ref = O.render(O.Scene(ocoll), [(20.0, 90.0)], 64, 0.01)
    _compare(got, ref)


def test_reference_gpu_tests_scenes_through_abi(X):
    """cuda_test.go:41-215 scenes (32^3 sphere, 24x32x16 box) through
    RenderVolumeProjectionsCUDA, now at the oracle's tolerance."""
    for (NX, NY, NZ), kind in [((32, 32, 32), "sphere"), ((24, 32, 16), "box")]:
        vol = np.zeros((NZ, NX, NY), dtype=np.float32)
        x = np.arange(NX) / NX * 2 - 1
        y = np.arange(NY) / NY * 2 - 1
        z = np.arange(NZ) / NZ * 2 - 1
        Z, Xg, Y = np.meshgrid(z, x, y, indexing="ij")
        if kind == "sphere":
            vol[Xg ** 2 + Y ** 2 + Z ** 2 < 0.09] = 1.0
        else:
            vol[(np.abs(Xg) < 0.4) & (np.abs(Y) < 0.2) & (np.abs(Z) < 0.3)] = 1.0
        ds = 2.0 / min(NX, NY, NZ) / 5.0
        cams = X.xray_camera_params([(0.0, 90.0)], 4.0, 40.0)
        got = X.render_volume_projections(vol, cams, 32, ds)
        ref = O.render_volume_abi(vol, cams, 32, np.float32(ds))
        _compare(got, ref)


def test_volume_abi_full_grid_subset(X):
    """The 256^3 grid of the voxel benchmark through the reference ABI at
    full 1024^2 resolution on two views, checked on a seeded ray subset."""
    vol = W().gaussian_blob_volume(256, 64, seed=2)
    angles = [(0.0, 90.0), (122.0, 90.0)]
    cams = X.xray_camera_params(angles, 4.0, 40.0)
    got = X.render_volume_projections(vol, cams, 1024, 2.0 / 256 * 0.5)
    rng = np.random.default_rng(11)
    rays = np.stack([rng.integers(0, 2, 4000), rng.integers(0, 1024, 4000),
                     rng.integers(0, 1024, 4000)], 1).astype(np.int32)
    ref = O.render_volume_abi(vol, cams, 1024, np.float32(2.0 / 256 * 0.5), rays=rays)
    _compare(got[rays[:, 0], rays[:, 1], rays[:, 2]], ref)


def test_probe_call_and_edge_sizes(X):
    """probeCUDA (cuda_test.go:15-29): 1x1x1 volume, one pixel."""
    cam = np.array([[4, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 40, 4]],
                   dtype=np.float32)
    got = X.render_volume_projections(np.zeros((1, 1, 1), np.float32), cam, 1, 0.1)
    assert got.shape == (1, 1, 1) and got[0, 0, 0] == 1.0
    # odd resolution, tiny images, single voxel planes
    vol = W().gaussian_blob_volume(8, 3, seed=5)[:, :, :1].copy()  # ny == 1
    cams = X.xray_camera_params([(15.0, 80.0)], 4.0, 40.0)
    for res in (1, 3, 17):
        got = X.render_volume_projections(vol, cams, res, 0.03)
        ref = O.render_volume_abi(vol, cams, res, np.float32(0.03))
        _compare(got, ref)


def test_error_codes(X):
    from xray_projection_render_gb300._lib import EngineError
    cams = X.xray_camera_params([(0.0, 90.0)])
    vol = np.ones((2, 2, 2), np.float32)
    with pytest.raises(EngineError) as e:
        X.render_volume_projections(vol, cams, 8, 0.0)
    assert e.value.code == 2
    with pytest.raises(EngineError) as e:
        X.Scene({"type": "torus"})
    assert e.value.code == 2 and "unknown object type" in str(e.value)
    with pytest.raises(EngineError):
        X.Scene({"type": "object_collection", "objects": [{"type": "object_collection",
                                                            "objects": []}]})


def test_empty_and_missing_scenes(X):
    # no positive density anywhere -> every pixel is exp(-flat_field)
    obj = {"type": "object_collection", "objects": [
        {"type": "sphere", "center": [0, 0, 0], "radius": 0.5, "rho": -1.0}]}
    with X.Scene(obj) as s:
        got = X.render(s, [(0.0, 90.0)], resolution=16, ds=0.01, flat_field=0.25)
    assert np.allclose(got, np.exp(-0.25), rtol=1e-6)
    # camera at the pole is degenerate in the reference (main_test.go:149)
    w = W().Workload("pole", {"type": "sphere", "center": [0, 0, 0], "radius": 0.5, "rho": 1.0},
                     None, [(0.0, 0.0)], 8, 0.01)
    got, ref = _render_both(X, w, flat_field=0.5)
    assert np.allclose(got, ref, rtol=1e-6)


def test_voxelizer_matches_reference_semantics(X):
    rng = np.random.default_rng(3)
    cyl = np.zeros((40, 8), np.float32)
    cyl[:, 0:6] = rng.uniform(-0.8, 0.8, (40, 6))
    cyl[:, 6] = rng.uniform(0.02, 0.1, 40)
    cyl[:, 7] = rng.choice([1.0, -1.0], 40)
    res = 24
    got = X.assemble_voxel_grid(cyl, res, 1.0)
    # FP32 restatement of cuda_backend.cu:208-252
    i = np.arange(res, dtype=np.float32)
    c = (i / np.float32(res) * np.float32(2) - np.float32(1)).astype(np.float32)
    K, I, J = np.meshgrid(c, c, c, indexing="ij")
    dens = np.zeros_like(K)
    for p in cyl:
        v = p[3:6] - p[0:3]
        vv = np.float32(v @ v)
        wx, wy, wz = I - p[0], J - p[1], K - p[2]
        t = (wx * v[0] + wy * v[1] + wz * v[2]) / vv
        dx, dy, dz = wx - v[0] * t, wy - v[1] * t, wz - v[2] * t
        inside = (t >= 0) & (t <= 1) & (dx * dx + dy * dy + dz * dz < p[6] * p[6])
        dens += np.where(inside, p[7], 0).astype(np.float32)
    dens = np.clip(dens, 0, 1)
    assert np.mean(got != dens) < 1e-3  # FP32 boundary ties only
