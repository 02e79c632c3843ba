"""Pins the FP64 oracle to the reference's own known-answer tests.

Each test restates one Go test of igrega348/xray_projection_render, with the
same inputs, expected values and tolerances:
main_test.go:90-522, objects/objects_test.go:14-461,
deformations/deformations_test.go:11-56.
"""
import math

import numpy as np
import pytest

from oracle import oracle as O


def sphere(c, r, rho):
    return {"type": "sphere", "center": list(c), "radius": r, "rho": rho}


def box(c, sides, rho):
    return {"type": "box", "center": list(c), "sides": list(sides), "rho": rho}


def cyl(p0, p1, r, rho=1.0):
    return {"type": "cylinder", "p0": list(p0), "p1": list(p1), "radius": r, "rho": rho}


# ---- camera (main_test.go:90-195) ----------------------------------------

@pytest.mark.parametrize("az,polar,R,expected", [
    (0, 90, 4.0, (4.0, 0, 0)),
    (90, 90, 4.0, (0, 4.0, 0)),
    (0, 0, 4.0, (0, 0, 4.0)),
])
def test_camera_eye_positions(az, polar, R, expected):
    eye, cam = O.camera_from_angles(az, polar, R)
    assert np.linalg.norm(eye - np.array(expected)) <= 1e-6
    if polar != 0:
        assert np.any(np.abs(cam) > 1e-10)


def test_camera_distance_check():
    eye, _ = O.camera_from_angles(45, 60, 5.0)
    assert abs(np.linalg.norm(eye) - 5.0) <= 1e-6


def test_camera_matrix_is_rigid_and_centre_ray_hits_origin():
    # Self-checks of the restated LookAtV(...).Inv() (mathgl is not vendored).
    for az, pol in [(0, 90), (37.5, 61), (200, 120), (359.5, 90)]:
        eye, cam = O.camera_from_angles(az, pol, 4.0)
        M = cam.reshape(4, 4).T  # row-major view
        Rm = M[:3, :3]
        assert np.allclose(Rm.T @ Rm, np.eye(3), atol=1e-14)
        assert np.allclose(M[:3, 3], eye, atol=1e-14)
        assert np.allclose(M[3], [0, 0, 0, 1], atol=1e-15)
        # pixel (res/2, res/2) is the optical axis: its ray passes through 0
        d = O.pixel_ray(eye, cam, 40.0, 64, 32, 32)
        d = d / np.linalg.norm(d)
        closest = eye - np.dot(eye, d) * d
        assert np.linalg.norm(closest) < 1e-12


def test_polar_zero_is_degenerate_like_reference():
    # main_test.go:149-150: the matrix may be degenerate at the pole.  The
    # oracle then renders every pixel as exp(-flat_field).
    s = O.Scene(sphere((0, 0, 0), 0.5, 1.0))
    img = O.render(s, [(0, 0)], 4, 0.01, flat_field=0.5)
    assert np.allclose(img, math.exp(-0.5))


# ---- camera angle generation (main_test.go:197-283) ----------------------

def test_generate_camera_angles_equispaced():
    a = O.generate_camera_angles(4, 0, 1, 90.0)
    assert [x[0] for x in a] == pytest.approx([90.0, 180.0, 270.0, 360.0])
    assert all(abs(p - 90.0) < 1e-6 for _, p in a)


def test_generate_camera_angles_custom_polar():
    a = O.generate_camera_angles(2, 0, 1, 45.0)
    assert len(a) == 2 and all(abs(p - 45.0) < 1e-6 for _, p in a)


def test_generate_camera_angles_jobs_modulo():
    a = O.generate_camera_angles(8, 1, 2, 90.0)
    assert [x[0] for x in a] == pytest.approx([135.0, 225.0, 315.0, 405.0])


# ---- integrators (main_test.go:326-522) ------------------------------------

ORIGIN = [0, 0, -5]
DIR = [0, 0, 1]


def test_simple_sphere_center_ray():
    s = O.Scene(sphere((0, 0, 0), 0.5, 1.0))
    got = O.integrate(s, ORIGIN, DIR, 0.001, 4.5, 5.5)
    assert abs(got - math.exp(-1.0)) <= 2 * 0.001


def test_simple_slab_attenuation():
    s = O.Scene(box((0, 0, 0), (10, 10, 1), 2.0))
    got = O.integrate(s, ORIGIN, DIR, 0.001, 0, 10)
    assert abs(got - math.exp(-2.0)) <= 2 * 0.001 * 2.0


def test_hierarchical_sphere_center_ray():
    s = O.Scene(sphere((0, 0, 0), 0.5, 1.0))
    got = O.integrate(s, ORIGIN, DIR, 0.05, 4.5, 5.5, integration="hierarchical")
    assert abs(got - math.exp(-1.0)) <= 0.05


def test_simple_vs_hierarchical_agreement():
    s = O.Scene(sphere((0, 0, 0), 0.5, 1.0))
    simple = O.integrate(s, ORIGIN, DIR, 0.001, 4.5, 5.5)
    hier = O.integrate(s, ORIGIN, DIR, 0.05, 4.5, 5.5, integration="hierarchical")
    assert abs(simple - hier) <= 0.01


@pytest.mark.parametrize("integration", ["simple", "hierarchical"])
def test_flat_field_applied_once(integration):
    s = O.Scene(sphere((0, 0, 10), 0.01, 1.0))
    got = O.integrate(s, ORIGIN, DIR, 0.01, 0, 1, integration=integration, flat_field=1.0)
    assert abs(got - math.exp(-1.0)) <= 1e-9


def test_density_multiplier_applied():
    s = O.Scene(sphere((0, 0, 0), 0.5, 1.0))
    got = O.integrate(s, ORIGIN, DIR, 0.001, 4.5, 5.5, density_multiplier=2.0)
    assert abs(got - math.exp(-2.0)) <= 2 * 0.001 * 2.0


@pytest.mark.parametrize("ds,tol", [(0.01, 5e-2), (0.001, 5e-3), (0.0001, 5e-4)])
def test_simple_ds_convergence(ds, tol):
    s = O.Scene(sphere((0, 0, 0), 0.5, 1.0))
    got = O.integrate(s, ORIGIN, DIR, ds, 4.5, 5.5)
    assert abs(got - math.exp(-1.0)) <= tol


@pytest.mark.parametrize("DS", [0.1, 0.05, 0.02])
def test_hierarchical_boundary_accuracy(DS):
    s = O.Scene(sphere((0, 0, 0), 0.5, 1.0))
    ref = O.integrate(s, ORIGIN, DIR, 0.0001, 4.5, 5.5)
    got = O.integrate(s, ORIGIN, DIR, DS, 4.5, 5.5, integration="hierarchical")
    assert abs(got - ref) <= DS


def test_hierarchical_off_center_rays():
    s = O.Scene(sphere((0, 0, 0), 0.5, 1.0))
    d = 0.3
    want = math.exp(-2 * math.sqrt(0.25 - d * d))
    ref = O.integrate(s, [d, 0, -5], DIR, 0.0001, 4.5, 5.5)
    got = O.integrate(s, [d, 0, -5], DIR, 0.05, 4.5, 5.5, integration="hierarchical")
    assert abs(ref - want) <= 1e-3
    assert abs(got - ref) <= 0.05


# ---- geometry (objects_test.go:14-112) ----------------------------------------

@pytest.mark.parametrize("p,want", [
    ((0, 0, 0), 2.0), ((0, 0, 0.4), 2.0), ((0, 0, 0.5), 0.0), ((0, 0, 0.6), 0.0)])
def test_sphere_geometry(p, want):
    assert O.density_of(sphere((0, 0, 0), 0.5, 2.0), *p) == want


def test_sphere_off_origin():
    s = sphere((1, 2, 3), 0.3, 5.0)
    assert O.density_of(s, 1, 2, 3) == 5.0
    assert O.density_of(s, 1, 2, 3.31) == 0.0


@pytest.mark.parametrize("p,want", [
    ((0, 0, 0), 1.0), ((0.9, 0, 0), 1.0), ((1.0, 0, 0), 0.0), ((0, 0.4, 0), 1.0),
    ((0, 0.5, 0), 0.0), ((0, 0, 0.24), 1.0), ((0, 0, 0.25), 0.0)])
def test_box_geometry(p, want):
    assert O.density_of(box((0, 0, 0), (2, 1, 0.5), 1.0), *p) == want


@pytest.mark.parametrize("p,want", [
    ((0, 0, 0), 1.0), ((0.4, 0, 0), 1.0), ((0.5, 0, 0), 0.0), ((0, 0, -1.0), 1.0),
    ((0, 0, 1.0), 1.0), ((0, 0, -1.001), 0.0), ((0, 0, 1.001), 0.0), ((0.4, 0, 1.0), 1.0)])
def test_cylinder_geometry(p, want):
    assert O.density_of(cyl((0, 0, -1), (0, 0, 1), 0.5, 1.0), *p) == want


def test_cylinder_rho_defaults_to_one():
    c = {"type": "cylinder", "p0": [0, 0, -1], "p1": [0, 0, 1], "radius": 0.5}
    assert O.density_of(c, 0, 0, 0) == 1.0


def test_object_collection_clamping_and_greedy():
    coll = {"type": "object_collection",
            "objects": [sphere((0, 0, 0), 0.5, 0.8), sphere((0, 0, 0), 0.5, 0.8)]}
    assert O.density_of(coll, 0, 0, 0) == 1.0
    coll["greedy_dens_eval"] = True
    assert O.density_of(coll, 0, 0, 0) == 0.8


def test_parallelepiped_strict_bounds():
    p = {"type": "parallelepiped", "origin": [0, 0, 0], "v0": [1, 0, 0], "v1": [0, 2, 0],
         "v2": [0.5, 0, 1], "rho": 0.7}
    assert O.density_of(p, 0.75, 1.0, 0.5) == 0.7
    assert O.density_of(p, 0.0, 1.0, 0.5) == 0.0     # q_x = -0.25
    assert O.density_of(p, 0.5, 1.0, 0.0) == 0.0     # q_z = 0 (strict)
    assert O.density_of(p, 0.5, 2.0, 0.5) == 0.0     # q_y = 1 (strict)


def test_gyroid_divides_by_scale():
    g = {"type": "gyroid", "center": [0, 0, 0], "scale": 8.0, "thickness": 0.1, "rho": 1.0}
    # q = p/8; value ~ (x+y+z)/8 near the origin
    assert O.density_of(g, 0.1, 0.1, 0.1) == 1.0
    assert O.density_of(g, 0.5, 0.5, 0.5) == 0.0


# ---- voxel grid (objects_test.go:119-349) -----------------------------------

def voxel(vol):
    return {"type": "voxel_grid", "_voxels": np.asarray(vol, dtype=np.float64)}


def test_voxel_coordinate_layout():
    N = 3
    rho = np.zeros((N, N, N))
    rho[0, 2, 0] = 1.0  # [z][x][y]
    v = voxel(rho)
    assert abs(O.density_of(v, 1.0, -1.0, -1.0) - 1.0) <= 1e-9
    assert O.density_of(v, -1.0, 1.0, -1.0) <= 1e-9
    rho2 = np.zeros((N, N, N))
    rho2[1, 0, 0] = 1.0
    v2 = voxel(rho2)
    assert abs(O.density_of(v2, -1.0, -1.0, 0.0) - 1.0) <= 1e-9
    assert O.density_of(v2, -1.0, 0.0, -1.0) <= 1e-9


def test_voxel_round_trip_uint8():
    # objects_test.go:157-205 (ExportToRaw + VoxelGridFromRaw), with the
    # uint8 quantisation of ExportToRaw restated (objects.go:862-890, 925-927).
    res = 64
    i = np.arange(res)
    c = i / res * 2.0 - 1.0
    X, Y, Z = np.meshgrid(c, c, c, indexing="ij")  # X->i, Y->j, Z->k
    d = ((X - 0.5) ** 2 + Y ** 2 + Z ** 2 < 0.15 ** 2).astype(float)
    d += (X ** 2 + (Y - 0.3) ** 2 + Z ** 2 < 0.08 ** 2).astype(float)
    d = np.minimum(d, 1.0)
    vol = np.transpose(d, (2, 0, 1))  # [k][i][j]
    # ExportToRaw samples the grid through Density() at i/res*2-1 and writes uint8.
    # The export samples each voxel at its own lattice point, so the exported
    # values are the grid values; the uint8 quantisation is what round-trips.
    q = np.floor(vol / vol.max() * 255).astype(np.uint8)
    back = voxel(q.astype(np.float64) / 255.0)
    assert O.density_of(back, 0.5, 0.0, 0.0) >= 0.5
    assert O.density_of(back, 0.0, 0.5, 0.0) <= 0.1
    assert O.density_of(back, 0.0, 0.3, 0.0) >= 0.5
    assert O.density_of(back, 0.3, 0.0, 0.0) <= 0.1


def test_voxel_outside_bounds_and_corners():
    v = voxel(np.ones((2, 2, 2)))
    for p in [(1.001, 0, 0), (-1.001, 0, 0), (0, 1.001, 0), (0, -1.001, 0), (0, 0, 1.001),
              (0, 0, -1.001), (2, 2, 2)]:
        assert O.density_of(v, *p) == 0.0
    assert O.density_of(v, 1.0, 1.0, 1.0) == 1.0
    assert O.density_of(v, -1.0, -1.0, -1.0) == 1.0


def test_voxel_trilinear_known_values():
    v = voxel(np.ones((2, 2, 2)))
    for p in [(0, 0, 0), (0.5, -0.5, 0.3), (1, 1, 1), (-1, -1, -1)]:
        assert abs(O.density_of(v, *p) - 1.0) <= 1e-9
    r = np.zeros((2, 2, 2))
    r[0, 0, 0] = 1.0
    v2 = voxel(r)
    assert abs(O.density_of(v2, -1.0, -1.0, -1.0) - 1.0) <= 1e-9
    assert abs(O.density_of(v2, 0.0, -1.0, -1.0) - 0.5) <= 1e-9


def test_voxel_uint8_precision():
    raw = np.array([255, 128, 0], dtype=np.uint8)
    vals = raw.astype(np.float64) / 255.0  # objects.go:925-927
    assert np.allclose(vals, [1.0, 128.0 / 255.0, 0.0], atol=1e-10)


def test_voxel_non_cubic():
    nx, ny, nz = 2, 4, 3
    rho = np.zeros((nz, nx, ny))
    rho[2, 1, 3] = 1.0
    v = voxel(rho)
    assert abs(O.density_of(v, 1.0, 1.0, 1.0) - 1.0) <= 1e-9
    assert O.density_of(v, -1.0, 1.0, 1.0) <= 1e-9
    assert O.density_of(v, 1.0, -1.0, 1.0) <= 1e-9
    rho2 = np.zeros((nz, nx, ny))
    rho2[0, 0, 1] = 1.0
    v2 = voxel(rho2)
    wy = 1 / (ny - 1) * 2.0 - 1.0
    assert abs(O.density_of(v2, -1.0, wy, -1.0) - 1.0) <= 1e-9
    assert O.density_of(v2, wy, -1.0, -1.0) <= 1e-9


def test_voxel_non_cubic_axis_separation():
    nx, ny, nz = 16, 32, 16
    xs = np.arange(nx) / (nx - 1) * 2 - 1
    ys = np.arange(ny) / (ny - 1) * 2 - 1
    zs = np.arange(nz) / (nz - 1) * 2 - 1
    Z, X, Y = np.meshgrid(zs, xs, ys, indexing="ij")
    rho = (((X - 0.5) ** 2 + Y ** 2 + Z ** 2) < 0.09).astype(np.float64)
    v = voxel(rho)
    assert O.density_of(v, 0.5, 0.0, 0.0) >= 0.8
    assert O.density_of(v, 0.0, 0.5, 0.0) <= 0.1


# ---- tessellation seams (objects_test.go:356-428) ------------------------------

def kelvin(rad, scale=1.0):
    """MakeKelvin (objects.go:588-637): the 36-strut Kelvin cell."""
    s = [((0.25, 0.00, 0.50), (0.50, 0.00, 0.75)), ((0.25, 1.00, 0.50), (0.50, 1.00, 0.75)),
         ((0.25, 0.00, 0.50), (0.50, 0.00, 0.25)), ((0.25, 1.00, 0.50), (0.50, 1.00, 0.25)),
         ((0.25, 0.00, 0.50), (0.00, 0.25, 0.50)), ((0.50, 0.00, 0.75), (0.75, 0.00, 0.50)),
         ((0.50, 1.00, 0.75), (0.75, 1.00, 0.50)), ((0.50, 0.00, 0.75), (0.50, 0.25, 1.00)),
         ((0.75, 0.00, 0.50), (0.50, 0.00, 0.25)), ((0.75, 1.00, 0.50), (0.50, 1.00, 0.25)),
         ((0.75, 0.00, 0.50), (1.00, 0.25, 0.50)), ((0.50, 0.00, 0.25), (0.50, 0.25, 0.00)),
         ((1.00, 0.50, 0.75), (0.75, 0.50, 1.00)), ((1.00, 0.75, 0.50), (0.75, 1.00, 0.50)),
         ((1.00, 0.50, 0.25), (0.75, 0.50, 0.00)), ((0.25, 1.00, 0.50), (0.00, 0.75, 0.50)),
         ((0.50, 1.00, 0.75), (0.50, 0.75, 1.00)), ((0.50, 1.00, 0.25), (0.50, 0.75, 0.00)),
         ((0.00, 0.25, 0.50), (0.00, 0.50, 0.75)), ((1.00, 0.25, 0.50), (1.00, 0.50, 0.75)),
         ((0.00, 0.25, 0.50), (0.00, 0.50, 0.25)), ((1.00, 0.25, 0.50), (1.00, 0.50, 0.25)),
         ((0.00, 0.50, 0.75), (0.25, 0.50, 1.00)), ((0.00, 0.50, 0.75), (0.00, 0.75, 0.50)),
         ((1.00, 0.50, 0.75), (1.00, 0.75, 0.50)), ((0.00, 0.75, 0.50), (0.00, 0.50, 0.25)),
         ((1.00, 0.75, 0.50), (1.00, 0.50, 0.25)), ((0.00, 0.50, 0.25), (0.25, 0.50, 0.00)),
         ((0.25, 0.50, 0.00), (0.50, 0.75, 0.00)), ((0.25, 0.50, 1.00), (0.50, 0.75, 1.00)),
         ((0.25, 0.50, 0.00), (0.50, 0.25, 0.00)), ((0.25, 0.50, 1.00), (0.50, 0.25, 1.00)),
         ((0.50, 0.75, 0.00), (0.75, 0.50, 0.00)), ((0.50, 0.75, 1.00), (0.75, 0.50, 1.00)),
         ((0.75, 0.50, 0.00), (0.50, 0.25, 0.00)), ((0.75, 0.50, 1.00), (0.50, 0.25, 1.00))]
    objs = [cyl([scale * a for a in p0], [scale * a for a in p1], rad, 1.0) for p0, p1 in s]
    return {"objects": {"type": "object_collection", "objects": objs},
            "xmin": 0.0, "xmax": scale, "ymin": 0.0, "ymax": scale, "zmin": 0.0, "zmax": scale}


def tess(uc, lo, hi):
    return {"type": "tessellated_obj_coll", "uc": uc, "xmin": lo, "xmax": hi, "ymin": lo,
            "ymax": hi, "zmin": lo, "zmax": hi}


def test_tessellated_x_axis_cylinder_seams():
    uc = {"objects": {"type": "object_collection",
                      "objects": [cyl((0, 0.5, 0.5), (1, 0.5, 0.5), 0.1, 1.0)]},
          "xmin": 0, "xmax": 1, "ymin": 0, "ymax": 1, "zmin": 0, "zmax": 1}
    s = O.Scene(tess(uc, -2, 2))
    for x in [-1.9, -1.5, -1.0, -0.5, 0.0, 0.5, 1.0, 1.5, 1.9]:
        assert s.density(x, 0.5, 0.5) != 0
    assert s.density(1.0 - 1e-9, 0.5, 0.5) != 0 and s.density(1.0 + 1e-9, 0.5, 0.5) != 0


def test_tessellated_kelvin_z_boundary():
    s = O.Scene(tess(kelvin(0.1), -2, 2))
    a = s.density(0.5, 0.1875, 0.9375)
    b = s.density(0.5, 0.1875, 1.0625)
    assert a != 0 and b != 0 and abs(a - b) <= 1e-9


def test_tessellated_kelvin_y_face_struts():
    s = O.Scene(tess(kelvin(0.1), -2, 2))
    assert s.density(0.375, 0.01, 0.625) != 0
    assert s.density(0.375, -0.01, 0.625) != 0


# ---- deformations (deformations_test.go:11-56) ------------------------------------

def _apply(d, p):
    s = O.Scene(sphere((0, 0, 0), 0.0, 0.0), d)
    xyz = np.array(p, dtype=np.float64)
    O.lib().orc_def_apply(s.deform, xyz.ctypes.data_as(__import__("ctypes").c_void_p))
    return xyz


def test_affine_is_linear_map():
    assert list(_apply({"type": "affine", "matrix": [[1, 0, 0], [0, 1, 0], [0, 0, 1]]},
                       (3, 4, 5))) == [3, 4, 5]
    assert list(_apply({"type": "affine", "matrix": [[2, 0, 0], [0, 1, 0], [0, 0, 1]]},
                       (3, 4, 5))) == [6, 4, 5]


def test_gaussian_is_displacement_field():
    g = {"type": "gaussian", "amplitudes": [0.5, 0, 0], "sigmas": [1.0, 1.0, 1.0],
         "centers": [0, 0, 0]}
    x = _apply(g, (0, 0, 0))
    assert abs(x[0] - 0.5) <= 1e-9 and x[1] == 0 and x[2] == 0
    g0 = dict(g, amplitudes=[0, 0, 0])
    assert list(_apply(g0, (3, 4, 5))) == [3, 4, 5]


def test_linear_rigid_sigmoid_composed():
    lin = {"type": "linear", "strains": [0.0, 0.0, 0.05, 0.0, 0.0, 0.0]}
    assert np.allclose(_apply(lin, (1, 1, 1)), [1, 1, 1.05])
    rig = {"type": "rigid", "displacements": [0.1, -0.2, 0.3]}
    assert np.allclose(_apply(rig, (0, 0, 0)), [0.1, -0.2, 0.3])
    sig = {"type": "sigmoid", "amplitude": 0.1, "center": 0.0, "lengthscale": 0.2,
           "direction": "z"}
    assert np.allclose(_apply(sig, (0.3, 0.4, 0.0)), [0.3, 0.4, 0.05])
    comp = {"type": "composed", "deformations": [rig, lin]}
    assert np.allclose(_apply(comp, (0, 0, 0)), [0.1, -0.2, 0.315])


def test_min_feature_size_auto_ds():
    # main.go:350-353 with the MinFeatureSize rules of objects.go
    coll = {"type": "object_collection", "objects": [
        {"type": "cube", "side": 1.0, "center": [0, 0, 0], "rho": 1.0},
        sphere((0, 0, 0), 0.3, -1.0), cyl((0, 0, -0.6), (0, 0, 0.6), 0.2, -1.0)]}
    assert O.Scene(coll).min_feature_size() == pytest.approx(0.1)
    vg = voxel(np.zeros((4, 8, 16)))
    assert O.Scene(vg).min_feature_size() == pytest.approx(2.0 / 16)


def test_unknown_object_type_rejected():
    with pytest.raises(O.SchemaError):
        O.Scene({"type": "torus"})
    with pytest.raises(O.SchemaError):  # object_collection cannot nest directly
        O.Scene({"type": "object_collection", "objects": [
            {"type": "object_collection", "objects": []}]})


def test_sample_table_matches_accumulated_loop():
    t = O.sample_table(4 - 1.74, 4 + 1.74, 0.005)
    s, k = 4 - 1.74, 0
    while s < 4 + 1.74:
        assert t[k] == s
        s += 0.005
        k += 1
    # 3.48/0.005 = 696 steps; FP64 accumulation leaves s_696 just below smax
    assert len(t) == k == 697
