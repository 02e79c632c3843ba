"""Python loader for the FP64 CPU oracle (``xrp_oracle.c``).

TEST INFRASTRUCTURE ONLY.  The oracle restates the CPU algorithm of
igrega348/xray_projection_render in plain C and FP64; this module builds it
with gcc, loads it with ctypes and builds its object tree from the reference's
JSON/YAML object schema.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` import this module, as the checker; the
product library never does.

The tree builder follows the reference factories:
``objects.NewObject`` (objects/objects.go:658-689), the per-type ``FromMap``
methods (objects.go:42-61, 100-117, 148-169, 209-245, 306-332, 381-420,
479-510, 536-566, 715-787, 983-1012) and ``deformations.NewDeformation``
(deformations/deformations.go:308-343).
"""
from __future__ import annotations

import ctypes
import math
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SRC = os.path.join(_HERE, "xrp_oracle.c")
_BUILD_DIR = os.path.join(_HERE, "_build")
_LIB_PATH = os.path.join(_BUILD_DIR, "libxrp_oracle.so")

_lib = None
_lock = threading.Lock()

CUBE_HALF_DIAGONAL = 1.74  # main.go:46


def build(force: bool = False) -> str:
    """Compile the oracle shared library (gcc, FP contraction off)."""
    os.makedirs(_BUILD_DIR, exist_ok=True)
    if (not force and os.path.exists(_LIB_PATH)
            and os.path.getmtime(_LIB_PATH) >= os.path.getmtime(_SRC)):
        return _LIB_PATH
    tmp = _LIB_PATH + f".tmp{os.getpid()}"
    cmd = ["gcc", "-std=gnu11", "-O2", "-fPIC", "-shared", "-ffp-contract=off",
           "-fno-fast-math", "-pthread", _SRC, "-o", tmp, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, _LIB_PATH)
    return _LIB_PATH


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = ctypes.CDLL(_LIB_PATH)
            D, I, P, L_ = ctypes.c_double, ctypes.c_int, ctypes.c_void_p, ctypes.c_long
            sig = {
                "orc_reset": (None, []),
                "orc_reset_deformations": (None, []),
                "orc_sphere": (I, [D, D, D, D, D]),
                "orc_box": (I, [D, D, D, D, D, D, D]),
                "orc_cylinder": (I, [D, D, D, D, D, D, D, D]),
                "orc_parallelepiped": (I, [P, P, P, P, D]),
                "orc_gyroid": (I, [D, D, D, D, D, D]),
                "orc_collection": (I, [P, I, I]),
                "orc_unit_cell": (I, [I, P]),
                "orc_tessellated": (I, [I, P]),
                "orc_voxel_f64": (I, [P, I, I, I]),
                "orc_voxel_f32": (I, [P, I, I, I]),
                "orc_density": (D, [I, D, D, D]),
                "orc_def_gaussian": (I, [P, P, P]),
                "orc_def_linear": (I, [P]),
                "orc_def_rigid": (I, [P]),
                "orc_def_sigmoid": (I, [D, D, D, I]),
                "orc_def_affine": (I, [P]),
                "orc_def_composed": (I, [P, I]),
                "orc_def_apply": (None, [I, P]),
                "orc_integrate": (D, [I, I, D, D, I, P, P, D, D, D, P]),
                "orc_camera_from_angles": (None, [D, D, D, P, P]),
                "orc_transform_coordinate": (None, [P, P, P]),
                "orc_pixel_ray": (None, [P, P, D, I, I, I, P]),
                "orc_render": (I, [I, I, D, D, I, D, D, D, I, P, P, I, P, L_, P, P, I]),
                "orc_render_volume_abi": (I, [P, I, I, I, P, I, I, ctypes.c_float,
                                              ctypes.c_float, P, P, P, L_, I]),
                "orc_render_f32cams": (I, [I, P, I, I, ctypes.c_float, ctypes.c_float, P, P, P,
                                           L_, I]),
                "orc_sample_table": (L_, [D, D, D, P, L_]),
                "orc_min_feature_size": (D, [I]),
            }
            for name, (res, args) in sig.items():
                f = getattr(L, name)
                f.restype = res
                f.argtypes = args
            _lib = L
        return _lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def _f64(v, n=None):
    a = np.ascontiguousarray(np.asarray(v, dtype=np.float64))
    if n is not None and a.size != n:
        raise ValueError(f"expected {n} values, got {a.size}")
    return a


class SchemaError(ValueError):
    """The object or deformation map does not satisfy the reference schema."""


def _num(d, key, what):
    v = d.get(key)
    if isinstance(v, bool) or not isinstance(v, (int, float)):
        raise SchemaError(f"{key} is not a float64 ({what})")
    return float(v)


def _vec3(d, key, what):
    v = d.get(key)
    if not isinstance(v, (list, tuple)):
        raise SchemaError(f"{key} is not a Vec3 ({what})")
    out = [0.0, 0.0, 0.0]
    for i, x in enumerate(v[:3]):
        out[i] = float(x)
    return out


def _bounds(d, what):
    return [_num(d, k, what) for k in ("xmin", "xmax", "ymin", "ymax", "zmin", "zmax")]


_COLLECTION_CHILD_TYPES = ("sphere", "cube", "box", "cylinder", "parallelepiped", "gyroid",
                           "tessellated_obj_coll", "voxel_grid")


def _build_object(d, L, voxels, top_level):
    """objects.NewObject / ObjectCollection.FromMap dispatch."""
    if not isinstance(d, dict):
        raise SchemaError("object is not a map")
    t = d.get("type")
    if t == "sphere":  # objects.go:42-61
        c = _vec3(d, "center", t)
        return L.orc_sphere(c[0], c[1], c[2], _num(d, "radius", t), _num(d, "rho", t))
    if t in ("cube", "box"):  # objects.go:100-117, 148-169
        c = _vec3(d, "center", t)
        if t == "cube":
            s = _num(d, "side", t)
            sides = [s, s, s]
        else:
            sides = _vec3(d, "sides", t)
        return L.orc_box(c[0], c[1], c[2], sides[0], sides[1], sides[2], _num(d, "rho", t))
    if t == "cylinder":  # objects.go:306-332 (rho defaults to 1)
        p0, p1 = _vec3(d, "p0", t), _vec3(d, "p1", t)
        rho = _num(d, "rho", t) if "rho" in d else 1.0
        return L.orc_cylinder(*p0, *p1, _num(d, "radius", t), rho)
    if t == "parallelepiped":  # objects.go:209-245
        o = _f64(_vec3(d, "origin", t))
        v0, v1, v2 = (_f64(_vec3(d, k, t)) for k in ("v0", "v1", "v2"))
        return L.orc_parallelepiped(_ptr(o), _ptr(v0), _ptr(v1), _ptr(v2), _num(d, "rho", t))
    if t == "gyroid":  # objects.go:983-1012
        c = _vec3(d, "center", t)
        return L.orc_gyroid(c[0], c[1], c[2], _num(d, "scale", t), _num(d, "thickness", t),
                            _num(d, "rho", t))
    if t == "object_collection" and top_level:
        return _build_collection(d, L, voxels, bool(d.get("greedy_dens_eval", False)))
    if t == "tessellated_obj_coll":  # objects.go:536-566
        uc = d.get("uc")
        if not isinstance(uc, dict):
            raise SchemaError("uc is not a map")
        objs = uc.get("objects")
        if not isinstance(objs, dict):
            raise SchemaError("objects is not a map")
        coll = _build_collection(objs, L, voxels, True)  # objects.go:487
        ucid = L.orc_unit_cell(coll, _ptr(_f64(_bounds(uc, "unit_cell"))))
        return L.orc_tessellated(ucid, _ptr(_f64(_bounds(d, t))))
    if t == "voxel_grid":
        if d.get("_voxels") is None:
            raise SchemaError("voxel_grid needs its values (key '_voxels': array [nz][nx][ny])")
        vol = np.ascontiguousarray(d["_voxels"])
        nz, nx, ny = vol.shape
        voxels.append(vol)
        if vol.dtype == np.float32:
            return L.orc_voxel_f32(_ptr(vol), nx, ny, nz)
        vol64 = np.ascontiguousarray(vol, dtype=np.float64)
        voxels.append(vol64)
        return L.orc_voxel_f64(_ptr(vol64), nx, ny, nz)
    raise SchemaError(f"unknown object type `{t}`")


def _build_collection(d, L, voxels, greedy):
    """ObjectCollection.FromMap, objects.go:381-420."""
    if "greedy_dens_eval" in d and isinstance(d["greedy_dens_eval"], bool):
        greedy = greedy or d["greedy_dens_eval"]
    objs = d.get("objects")
    if not isinstance(objs, list):
        raise SchemaError("objects is not a list")
    ids = []
    for o in objs:
        if not isinstance(o, dict) or o.get("type") not in _COLLECTION_CHILD_TYPES:
            raise SchemaError("unknown object type")
        ids.append(_build_object(o, L, voxels, top_level=False))
    arr = np.asarray(ids if ids else [0], dtype=np.int32)
    return L.orc_collection(_ptr(arr), len(ids), 1 if greedy else 0)


_AXES = {"x": 0, "y": 1, "z": 2}


def _build_deformation(d, L):
    """deformations.NewDeformation, deformations.go:308-343."""
    t = d.get("type")
    if t == "gaussian":
        return L.orc_def_gaussian(_ptr(_f64(d["amplitudes"], 3)), _ptr(_f64(d["sigmas"], 3)),
                                  _ptr(_f64(d["centers"], 3)))
    if t == "linear":
        return L.orc_def_linear(_ptr(_f64(d["strains"], 6)))
    if t == "rigid":
        return L.orc_def_rigid(_ptr(_f64(d["displacements"], 3)))
    if t == "sigmoid":
        if d.get("direction") not in _AXES:
            raise SchemaError("Invalid direction")
        return L.orc_def_sigmoid(float(d["amplitude"]), float(d["center"]),
                                 float(d["lengthscale"]), _AXES[d["direction"]])
    if t == "affine":
        m = _f64(d["matrix"], 9)
        return L.orc_def_affine(_ptr(m))
    if t == "composed":
        subs = [_build_deformation(x, L) for x in d["deformations"]]
        arr = np.asarray(subs if subs else [0], dtype=np.int32)
        return L.orc_def_composed(_ptr(arr), len(subs))
    raise SchemaError(f"unknown deformation type {t}")


class Scene:
    """One loaded object (the reference's ``lat[0]``) plus an optional
    deformation (``df[0]``), main.go:37-38."""

    def __init__(self, obj: dict, deformation: dict | None = None):
        L = lib()
        L.orc_reset()
        L.orc_reset_deformations()
        self._keep = []
        self.root = _build_object(obj, L, self._keep, top_level=True)
        if self.root < 0:
            raise MemoryError("oracle node allocation failed")
        self.deform = _build_deformation(deformation, L) if deformation else -1

    def density(self, x, y, z, density_multiplier=1.0):
        p = np.array([x, y, z], dtype=np.float64)
        if self.deform >= 0:
            lib().orc_def_apply(self.deform, _ptr(p))
        return lib().orc_density(self.root, p[0], p[1], p[2]) * density_multiplier

    def min_feature_size(self):
        return lib().orc_min_feature_size(self.root)


def density_of(obj: dict, x, y, z):
    return Scene(obj).density(x, y, z)


def camera_from_angles(az_deg, polar_deg, R):
    """computeCameraFromAngles, main.go:226-239 -> (eye[3], cam[16] column-major)."""
    eye = np.zeros(3)
    cam = np.zeros(16)
    lib().orc_camera_from_angles(float(az_deg), float(polar_deg), float(R), _ptr(eye), _ptr(cam))
    return eye, cam


def pixel_ray(eye, cam, fov_deg, res, i, j):
    d = np.zeros(3)
    e = _f64(eye, 3)
    c = _f64(cam, 16)
    lib().orc_pixel_ray(_ptr(e), _ptr(c), float(fov_deg), int(res), int(i), int(j), _ptr(d))
    return d


def integrate(scene: Scene, origin, direction, ds, smin, smax, *, integration="simple",
              density_multiplier=1.0, flat_field=0.0, return_T=False):
    """integrate_along_ray / integrate_hierarchical, main.go:144-199."""
    o, d = _f64(origin, 3), _f64(direction, 3)
    T = ctypes.c_double()
    v = lib().orc_integrate(scene.root, scene.deform, float(density_multiplier), float(flat_field),
                            1 if integration == "hierarchical" else 0, _ptr(o), _ptr(d),
                            float(ds), float(smin), float(smax), ctypes.byref(T))
    return (v, T.value) if return_T else v


def generate_camera_angles(num_images, job_num=0, jobs_modulo=1, polar_angle=90.0):
    """generateCameraAngles, main.go:242-257 (in-plane mode)."""
    out = []
    for i in range(job_num, num_images, jobs_modulo):
        dth = 360.0 / float(num_images)
        out.append((float(i) * dth + 90.0, float(polar_angle)))
    return out


def cameras(angles, R):
    eyes = np.zeros((len(angles), 3))
    cams = np.zeros((len(angles), 16))
    for k, (az, pol) in enumerate(angles):
        eyes[k], cams[k] = camera_from_angles(az, pol, R)
    return eyes, cams


def default_threads():
    return os.cpu_count() or 1


def render(scene: Scene, angles, res, ds, *, R=4.0, fov=40.0, density_multiplier=1.0,
           flat_field=0.0, integration="simple", rays=None, nthreads=None, return_T=False):
    """Render views (main.go:429-471).  ``angles`` is a list of (azimuth,
    polar) degrees.  With ``rays`` (int array of (view, i, j) rows) only those
    pixels are computed and a flat array is returned; otherwise the result is
    [view][i][j]."""
    eyes, cams = cameras(angles, R)
    return render_cams(scene, eyes, cams, res, ds, R=R, fov=fov,
                       density_multiplier=density_multiplier, flat_field=flat_field,
                       integration=integration, rays=rays, nthreads=nthreads, return_T=return_T)


def render_cams(scene: Scene, eyes, cams, res, ds, *, R=4.0, fov=40.0, density_multiplier=1.0,
                flat_field=0.0, integration="simple", rays=None, nthreads=None, return_T=False):
    eyes = np.ascontiguousarray(eyes, dtype=np.float64)
    cams = np.ascontiguousarray(cams, dtype=np.float64)
    nv = eyes.shape[0]
    if rays is not None:
        rays = np.ascontiguousarray(rays, dtype=np.int32).reshape(-1, 3)
        n = rays.shape[0]
        out = np.zeros(n)
        outT = np.zeros(n)
        rp, nr = _ptr(rays), n
    else:
        out = np.zeros((nv, res, res))
        outT = np.zeros((nv, res, res))
        rp, nr = None, 0
    rc = lib().orc_render(scene.root, scene.deform, float(density_multiplier), float(flat_field),
                          1 if integration == "hierarchical" else 0, float(ds), float(R),
                          float(fov), int(res), _ptr(eyes), _ptr(cams), nv, rp, nr, _ptr(out),
                          _ptr(outT), int(nthreads or default_threads()))
    if rc != 0:
        raise ValueError(f"oracle render failed with code {rc}")
    return (out, outT) if return_T else out


def render_volume_abi(volume, cams21, res, ds, flat_field=0.0, *, rays=None, nthreads=None,
                      return_T=False):
    """CPU semantics on the inputs of RenderVolumeProjectionsCUDA
    (cuda_backend.h:101-112): ``volume`` float32 [nz][nx][ny], ``cams21``
    float32 [ncams][21] laid out as XRayCameraParams."""
    vol = np.ascontiguousarray(volume, dtype=np.float32)
    nz, nx, ny = vol.shape
    c = np.ascontiguousarray(cams21, dtype=np.float32).reshape(-1, 21)
    nc = c.shape[0]
    L = lib()
    L.orc_reset()
    if rays is not None:
        rays = np.ascontiguousarray(rays, dtype=np.int32).reshape(-1, 3)
        out = np.zeros(rays.shape[0])
        outT = np.zeros(rays.shape[0])
        rp, nr = _ptr(rays), rays.shape[0]
    else:
        out = np.zeros((nc, res, res))
        outT = np.zeros((nc, res, res))
        rp, nr = None, 0
    rc = L.orc_render_volume_abi(_ptr(vol), nx, ny, nz, _ptr(c), nc, int(res),
                                 ctypes.c_float(ds), ctypes.c_float(flat_field), _ptr(out),
                                 _ptr(outT), rp, nr, int(nthreads or default_threads()))
    if rc != 0:
        raise ValueError(f"oracle volume render failed with code {rc}")
    return (out, outT) if return_T else out


class VolumeABIScene:
    """A voxel grid loaded once for repeated RenderVolumeProjectionsCUDA-
    semantics renders (the CPU-baseline timing loop)."""

    def __init__(self, volume):
        self.vol = np.ascontiguousarray(volume, dtype=np.float32)
        nz, nx, ny = self.vol.shape
        L = lib()
        L.orc_reset()
        self.root = L.orc_voxel_f32(_ptr(self.vol), nx, ny, nz)
        if self.root < 0:
            raise MemoryError("oracle voxel allocation failed")

    def render_rays(self, cams21, res, ds, rays, flat_field=0.0, nthreads=None):
        c = np.ascontiguousarray(cams21, dtype=np.float32).reshape(-1, 21)
        rays = np.ascontiguousarray(rays, dtype=np.int32).reshape(-1, 3)
        out = np.zeros(rays.shape[0])
        rc = lib().orc_render_f32cams(self.root, _ptr(c), c.shape[0], int(res), ctypes.c_float(ds),
                                      ctypes.c_float(flat_field), _ptr(out), None, _ptr(rays),
                                      rays.shape[0], int(nthreads or default_threads()))
        if rc != 0:
            raise ValueError(f"oracle volume render failed with code {rc}")
        return out


def sample_table(smin, smax, ds):
    n = lib().orc_sample_table(float(smin), float(smax), float(ds), None, 0)
    out = np.zeros(n)
    lib().orc_sample_table(float(smin), float(smax), float(ds), _ptr(out), n)
    return out


def xray_camera_params(angles, R, fov):
    """The float32 XRayCameraParams rows the reference Go glue builds
    (cuda_path.go:61-77): eye, row-major camera-to-world matrix, fov, R."""
    rows = np.zeros((len(angles), 21), dtype=np.float32)
    for k, (az, pol) in enumerate(angles):
        eye, cam = camera_from_angles(az, pol, R)
        rows[k, 0:3] = eye
        m = cam.reshape(4, 4).T  # row-major view of the column-major matrix
        rows[k, 3:19] = m.reshape(16)
        rows[k, 19] = fov
        rows[k, 20] = R
    return rows


__all__ = ["build", "lib", "Scene", "SchemaError", "density_of", "camera_from_angles",
           "pixel_ray", "integrate", "generate_camera_angles", "cameras", "render",
           "render_cams", "render_volume_abi", "sample_table", "xray_camera_params",
           "CUBE_HALF_DIAGONAL", "math"]
