"""Soundness of the distance certificates (margin32) the proposal march uses
to count segments without sampling them.

The engine's FP32 code runs on the CPU (tests/hostsim).  For sample points
of several scenes it returns the density and a radius m; every point within
m of the sample must then have the same FP64 density (oracle) as the sample
itself.  Points are drawn inside the ball and on its surface, where a
too-large radius would show first."""
import os
import sys

import numpy as np
import pytest

from oracle import oracle as O

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "hostsim"))
import hostsim  # noqa: E402

from xray_projection_render_gb300 import workloads as W  # noqa: E402


def check_scene(obj, deformation=None, n=1500, per=6, seed=0, lo=-1.1, hi=1.1, ds=0.002):
    rng = np.random.default_rng(seed)
    P = rng.uniform(lo, hi, (n, 3))
    rho, m, rho2, m2 = hostsim.margin(obj, P, deformation=deformation, ds=ds, fused=True)
    # the fused evaluator (certificate tracing) decides and bounds identically
    assert np.array_equal(np.isnan(rho), np.isnan(rho2))
    ok = ~np.isnan(rho)
    assert np.array_equal(rho[ok], rho2[ok])
    assert np.array_equal(m[ok], m2[ok])
    sc = O.Scene(obj, deformation)
    certified = 0
    for k in range(n):
        if not (m[k] > 0) or np.isnan(rho[k]):
            continue
        r0 = sc.density(*P[k])
        assert np.float32(r0) == rho[k], (k, P[k], r0, rho[k])
        u = rng.normal(size=(per, 3))
        u /= np.linalg.norm(u, axis=1, keepdims=True)
        rad = m[k] * np.concatenate([np.full(per // 2, 0.999), rng.uniform(0, 1, per - per // 2)])
        for q in P[k] + u * rad[:, None]:
            assert sc.density(*q) == r0, (k, P[k], q, float(m[k]))
        certified += 1
    return certified, n


def test_cube_minus_sphere_cylinder_collection():
    c, n = check_scene(W.cube_minus_sphere_cylinder(8).obj)
    assert c > n // 2


def test_deformed_lattice():
    w = W.deformed_lattice()
    c, n = check_scene(w.obj, w.deformation, n=800)
    assert c > n // 5


def test_gyroid_sigmoid():
    w = W.gyroid_sigmoid()
    c, n = check_scene(w.obj, w.deformation)
    assert c > n // 2


def test_fine_gyroid():
    obj = {"type": "gyroid", "center": [0.0, 0.0, 0.0], "scale": 0.1, "thickness": 0.3, "rho": 1.0}
    c, n = check_scene(obj, n=800)
    assert c > n // 4


@pytest.mark.parametrize("k", [0, 3, 7])
def test_batched_scene_with_candidate_lists(k):
    w = W.batched_scenes(8)[k]
    check_scene(w.obj, n=800, seed=k)


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
            check_scene(p, d, n=200, per=4)
    coll = {"type": "object_collection", "objects": prims}
    for d in defs:
        check_scene(coll, d, n=300, per=4)


# ---------------------------------------------------------------------------
# Ray certificates (affine chains): along a direction D the density must
# stay that of the point for every ray parameter in [0, t].
# ---------------------------------------------------------------------------

def check_ray(obj, deformation=None, n=1200, per=8, seed=0, lo=-1.1, hi=1.1, ds=0.002, span=4.0):
    rng = np.random.default_rng(seed)
    P = rng.uniform(lo, hi, (n, 3))
    D = rng.normal(size=(n, 3))
    D /= np.linalg.norm(D, axis=1, keepdims=True)
    rho, t, affine = hostsim.ray_bound(obj, P, D, deformation=deformation, ds=ds)
    assert affine
    # the ray evaluator decides exactly as the point evaluators
    rho_pt, _ = hostsim.margin(obj, P, deformation=deformation, ds=ds)
    assert np.array_equal(np.isnan(rho), np.isnan(rho_pt))
    ok = ~np.isnan(rho)
    assert np.array_equal(rho[ok], rho_pt[ok])
    sc = O.Scene(obj, deformation)
    certified, far = 0, 0
    for k in range(n):
        if not (t[k] > 0) or np.isnan(rho[k]):
            continue
        r0 = sc.density(*P[k])
        assert np.float32(r0) == rho[k], (k, P[k], r0, rho[k])
        tk = min(float(t[k]), span)
        far += t[k] > span
        taus = np.concatenate([[tk, 0.999 * tk, 0.5 * tk], rng.uniform(0, tk, per - 3)])
        for tau in taus:
            q = P[k] + D[k] * tau
            assert sc.density(*q) == r0, (k, P[k], D[k], float(t[k]), tau)
        certified += 1
    return certified, far, n


def test_ray_cube_minus_sphere_cylinder():
    c, far, n = check_ray(W.cube_minus_sphere_cylinder(8).obj)
    assert c > n // 2


def test_ray_deformed_lattice():
    w = W.deformed_lattice()
    c, far, n = check_ray(w.obj, w.deformation, n=800)
    assert c > n // 3


@pytest.mark.parametrize("k", [0, 3, 7])
def test_ray_batched_scene_with_candidate_lists(k):
    w = W.batched_scenes(8)[k]
    check_ray(w.obj, n=800, seed=k)


def test_ray_every_primitive_under_affine_deformations():
    prims = [
        {"type": "sphere", "center": [0.1, -0.2, 0.05], "radius": 0.4, "rho": 0.7},
        {"type": "box", "center": [0.0, 0.2, 0.0], "sides": [0.5, 0.3, 0.9], "rho": 0.5},
        {"type": "cylinder", "p0": [-0.5, -0.5, -0.2], "p1": [0.5, 0.4, 0.3], "radius": 0.1},
        {"type": "cylinder", "p0": [0.0, 0.0, -0.6], "p1": [0.0, 0.0, 0.6], "radius": 0.3},
        {"type": "parallelepiped", "origin": [0.0, 0.0, 0.0], "v0": [0.4, 0.1, 0.0],
         "v1": [0.0, 0.5, 0.1], "v2": [0.1, 0.0, 0.3], "rho": 0.9},
        {"type": "gyroid", "center": [0.0, 0.0, 0.0], "scale": 0.1, "thickness": 0.2, "rho": 1.0},
    ]
    defs = [None,
            {"type": "linear", "strains": [0.02, -0.01, 0.05, 0.01, 0.0, 0.03]},
            {"type": "rigid", "displacements": [0.05, -0.1, 0.02]},
            {"type": "affine", "matrix": [[1.1, 0.0, 0.1], [0.0, 0.9, 0.0], [0.05, 0.0, 1.0]]}]
    for p in prims:
        for d in defs:
            check_ray(p, d, n=250, per=6)
    coll = {"type": "object_collection", "objects": prims}
    for d in defs:
        check_ray(coll, d, n=300, per=6)


def test_ray_axis_aligned_directions():
    # directions along the axes and along a cylinder axis: zero components,
    # rays parallel to faces and to the axis
    obj = {"type": "object_collection", "objects": [
        {"type": "box", "center": [0.0, 0.0, 0.0], "sides": [0.6, 0.6, 0.6], "rho": 0.5},
        {"type": "cylinder", "p0": [0.0, 0.0, -0.8], "p1": [0.0, 0.0, 0.8], "radius": 0.2}]}
    rng = np.random.default_rng(5)
    P = rng.uniform(-1, 1, (600, 3))
    axes = np.eye(3)[rng.integers(0, 3, 600)] * rng.choice([-1.0, 1.0], (600, 1))
    rho, t, _ = hostsim.ray_bound(obj, P, axes)
    sc = O.Scene(obj)
    for k in range(600):
        if not (t[k] > 0) or np.isnan(rho[k]):
            continue
        r0 = sc.density(*P[k])
        for tau in np.linspace(0, min(float(t[k]), 4.0), 9):
            assert sc.density(*(P[k] + axes[k] * tau)) == r0


def test_non_affine_chain_has_no_ray_certificates():
    w = W.gyroid_sigmoid()
    _, _, affine = hostsim.ray_bound(w.obj, np.zeros((1, 3)), np.array([[1.0, 0, 0]]),
                                     deformation=w.deformation)
    assert not affine


def test_ray_far_camera_and_offset_scene():
    # a distant, narrow camera (R 60, fov 8) and a scene offset from the
    # origin: larger position errors, larger capsule radius
    obj = {"type": "object_collection", "objects": [
        {"type": "sphere", "center": [3.1, -2.2, 1.05], "radius": 0.4, "rho": 0.7},
        {"type": "cylinder", "p0": [2.5, -2.5, 0.8], "p1": [3.5, -1.6, 1.3], "radius": 0.1},
        {"type": "box", "center": [3.0, -2.0, 1.0], "sides": [0.5, 0.3, 0.9], "rho": 0.5}]}
    rng = np.random.default_rng(11)
    n = 600
    P = np.array([3.0, -2.0, 1.0]) + rng.uniform(-0.7, 0.7, (n, 3))
    D = rng.normal(size=(n, 3))
    D /= np.linalg.norm(D, axis=1, keepdims=True)
    d = {"type": "linear", "strains": [0.02, -0.01, 0.05, 0.01, 0.0, 0.03]}
    rho, t, affine = hostsim.ray_bound(obj, P, D, deformation=d, R=60.0, fov=8.0)
    assert affine
    sc = O.Scene(obj, d)
    checked = 0
    for k in range(n):
        if not (t[k] > 0) or np.isnan(rho[k]):
            continue
        r0 = sc.density(*P[k])
        assert np.float32(r0) == rho[k]
        for tau in np.concatenate([[0.999 * min(float(t[k]), 4.0)], rng.uniform(0, min(float(t[k]), 4.0), 5)]):
            assert sc.density(*(P[k] + D[k] * tau)) == r0
        checked += 1
    assert checked > n // 2


# ---------------------------------------------------------------------------
# Curved-ray certificates (smooth non-affine chains, CPU build): along a
# world direction D the density must stay that of the point for every ray
# parameter in [0, t], the deformed path being curved.
# ---------------------------------------------------------------------------

def check_curve(obj, deformation, n=800, per=8, seed=0, span=4.0):
    rng = np.random.default_rng(seed)
    P = rng.uniform(-1.1, 1.1, (n, 3))
    D = rng.normal(size=(n, 3))
    D /= np.linalg.norm(D, axis=1, keepdims=True)
    rho, t = hostsim.curve_bound(obj, P, D, deformation=deformation)
    rho_pt, _ = hostsim.margin(obj, P, deformation=deformation)
    assert np.array_equal(np.isnan(rho), np.isnan(rho_pt))
    ok = ~np.isnan(rho)
    assert np.array_equal(rho[ok], rho_pt[ok])
    sc = O.Scene(obj, deformation)
    certified = 0
    for k in range(n):
        if not (t[k] > 0) or np.isnan(rho[k]):
            continue
        r0 = sc.density(*P[k])
        assert np.float32(r0) == rho[k]
        tk = min(float(t[k]), span)
        for tau in np.concatenate([[tk, 0.999 * tk, 0.5 * tk], rng.uniform(0, tk, per - 3)]):
            assert sc.density(*(P[k] + D[k] * tau)) == r0, (k, P[k], D[k], float(t[k]), tau)
        certified += 1
    return certified, n


GAUSS = {"type": "gaussian", "amplitudes": [0.1, -0.05, 0.02], "sigmas": [0.3, 0.3, 0.5],
         "centers": [0.0, 0.1, 0.0]}
SIGMOID = {"type": "sigmoid", "amplitude": 0.2, "center": 0.0, "lengthscale": 0.2, "direction": "y"}


def test_curve_gyroid_sigmoid():
    w = W.gyroid_sigmoid()
    c, n = check_curve(w.obj, w.deformation)
    assert c > n // 2


def test_curve_every_primitive_and_collection():
    prims = [
        {"type": "sphere", "center": [0.1, -0.2, 0.05], "radius": 0.4, "rho": 0.7},
        {"type": "box", "center": [0.0, 0.2, 0.0], "sides": [0.5, 0.3, 0.9], "rho": 0.5},
        {"type": "cylinder", "p0": [-0.5, -0.5, -0.2], "p1": [0.5, 0.4, 0.3], "radius": 0.1},
        {"type": "parallelepiped", "origin": [0.0, 0.0, 0.0], "v0": [0.4, 0.1, 0.0],
         "v1": [0.0, 0.5, 0.1], "v2": [0.1, 0.0, 0.3], "rho": 0.9},
        {"type": "gyroid", "center": [0.0, 0.0, 0.0], "scale": 0.1, "thickness": 0.2, "rho": 1.0},
    ]
    chain = {"type": "composed", "deformations": [
        GAUSS, {"type": "linear", "strains": [0.02, -0.01, 0.05, 0.01, 0.0, 0.03]}, SIGMOID]}
    # None: a scene without deformation traced with curve bounds, as in a
    # batch whose other scenes have non-affine chains
    for d in (GAUSS, SIGMOID, chain, None):
        for p in prims:
            check_curve(p, d, n=250, per=6)
        check_curve({"type": "object_collection", "objects": prims}, d, n=300, per=6)


def test_curve_tessellated_lattice_under_gaussian():
    w = W.deformed_lattice()
    c, n = check_curve(w.obj, GAUSS, n=600)
    assert c > n // 3


def test_curve_near_faces_moving_away_under_strong_bending():
    # points just outside a box's faces, moving away, under a sharp sigmoid:
    # the curve can turn back, and the bound must see it (the root of the
    # gap equation without cancellation)
    obj = {"type": "box", "center": [0.0, 0.0, 0.0], "sides": [0.8, 0.8, 0.8], "rho": 1.0}
    d = {"type": "sigmoid", "amplitude": 0.3, "center": 0.05, "lengthscale": 0.05, "direction": "x"}
    rng = np.random.default_rng(3)
    n = 600
    face = rng.integers(0, 3, n)
    side = rng.choice([-1.0, 1.0], n)
    P = rng.uniform(-0.35, 0.35, (n, 3))
    P[np.arange(n), face] = side * (0.4 + rng.uniform(1e-4, 3e-3, n))
    D = rng.normal(size=(n, 3))
    D[np.arange(n), face] = side * np.abs(D[np.arange(n), face])  # away from the face
    D /= np.linalg.norm(D, axis=1, keepdims=True)
    rho, t = hostsim.curve_bound(obj, P, D, deformation=d)
    sc = O.Scene(obj, d)
    for k in range(n):
        if not (t[k] > 0) or np.isnan(rho[k]):
            continue
        r0 = sc.density(*P[k])
        for tau in np.linspace(0.0, min(float(t[k]), 4.0), 17):
            assert sc.density(*(P[k] + D[k] * tau)) == r0, (k, P[k], D[k], float(t[k]), tau)
