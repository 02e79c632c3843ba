"""Loader for the CPU build of the engine's per-pixel code (test harness only).

The engine's device code (xray_projection_render_gb300/csrc/xrp_device.h) is
host+device; compiled here with g++ it lets the tests check the guard-band
decisions, the flattened scene and the lattices against the FP64 oracle on a
machine without a GPU.  The product never loads this library.
"""
import ctypes
import json
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
CSRC = os.path.join(ROOT, "xray_projection_render_gb300", "csrc")
LIB = os.path.join(HERE, "_build", "libxrp_hostsim.so")
# AddressSanitizer + UndefinedBehaviorSanitizer build (a process that loads it
# needs the ASan runtime preloaded); XRP_HOSTSIM_SANITIZED=1 selects it
LIB_SAN = os.path.join(HERE, "_build", "libxrp_hostsim_san.so")
SAN_FLAGS = ["-O1", "-g", "-fno-omit-frame-pointer", "-fsanitize=address,undefined",
             "-fno-sanitize-recover=undefined"]
_lib = None


def build(sanitize=False):
    out = LIB_SAN if sanitize else LIB
    srcs = [os.path.join(HERE, "xrp_hostsim.cpp"), os.path.join(CSRC, "xrp_scene.cpp")]
    deps = srcs + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".h")] + [__file__]
    if os.path.exists(out) and all(os.path.getmtime(out) >= os.path.getmtime(d) for d in deps):
        return out
    os.makedirs(os.path.dirname(out), exist_ok=True)
    tmp = out + f".tmp{os.getpid()}"
    subprocess.run(["g++", "-std=c++17", *(SAN_FLAGS if sanitize else ["-O2"]), "-fPIC", "-shared",
                    "-ffp-contract=off", "-fno-fast-math", "-pthread", "-I", os.path.join(ROOT, "include"),
                    *srcs, "-o", tmp], check=True)
    os.replace(tmp, out)
    return out


def lib():
    global _lib
    if _lib is None:
        L = ctypes.CDLL(build(sanitize=os.environ.get("XRP_HOSTSIM_SANITIZED") == "1"))
        P, I, D, L_ = ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_long
        L.hs_render.restype = I
        L.hs_render.argtypes = [ctypes.c_char_p, ctypes.c_char_p, P, I, I, I, P, I, I, I, D, D, D,
                                D, P, P, I, P, L_, I, I, I, ctypes.c_char_p, I]
        L.hs_margin.restype = I
        L.hs_margin.argtypes = [ctypes.c_char_p, ctypes.c_char_p, P, L_, D, D, D, P, P, P, P,
                                P, P, P, P, ctypes.c_char_p, I]
        _lib = L
    return _lib


def margin(obj, points, *, deformation=None, R=4.0, fov=40.0, ds=0.01, fused=False):
    """(density, certificate radius) of the engine's FP32 code at points [n,3];
    with ``fused`` also the fused evaluator's (density, radius)."""
    pts = np.ascontiguousarray(points, dtype=np.float64).reshape(-1, 3)
    n = pts.shape[0]
    rho, m, rho2, m2 = (np.zeros(n, np.float32) for _ in range(4))
    err = ctypes.create_string_buffer(512)
    rc = lib().hs_margin(json.dumps(obj).encode(),
                         json.dumps(deformation).encode() if deformation else None,
                         pts.ctypes.data, n, R, fov, ds, rho.ctypes.data, m.ctypes.data,
                         rho2.ctypes.data, m2.ctypes.data, None, None, None, None, err, 512)
    if rc != 0:
        raise ValueError(err.value.decode())
    return (rho, m, rho2, m2) if fused else (rho, m)


def density64(obj, points, *, deformation=None):
    """The engine's FP64 densities at FP64 points [n,3]: (every primitive in
    FP64, the FP64 pass's hybrid evaluator)."""
    import ctypes as C
    pts = np.ascontiguousarray(points, dtype=np.float64).reshape(-1, 3)
    n = pts.shape[0]
    a, b = np.zeros(n), np.zeros(n)
    L = lib()
    L.hs_density64.restype = C.c_int
    L.hs_density64.argtypes = [C.c_char_p, C.c_char_p, C.c_void_p, C.c_long, C.c_void_p, C.c_void_p,
                               C.c_char_p, C.c_int]
    err = C.create_string_buffer(512)
    rc = L.hs_density64(json.dumps(obj).encode(), json.dumps(deformation).encode() if deformation else None,
                        pts.ctypes.data, n, a.ctypes.data, b.ctypes.data, err, 512)
    if rc != 0:
        raise ValueError(err.value.decode())
    return a, b


def ray_bound(obj, points, dirs, *, deformation=None, R=4.0, fov=40.0, ds=0.01):
    """Ray evaluator at points [n,3] along world directions [n,3]: (density,
    ray bound t, affine).  Every sample at parameter s in [0, t] must have
    the density of the point; ``affine`` False means the chain is not affine
    (no ray certificates; density and t are then not computed)."""
    pts = np.ascontiguousarray(points, dtype=np.float64).reshape(-1, 3)
    d = np.ascontiguousarray(dirs, dtype=np.float64).reshape(-1, 3)
    n = pts.shape[0]
    rho, m, rho2, m2, rho3, t = (np.zeros(n, np.float32) for _ in range(6))
    aff = ctypes.c_int(0)
    err = ctypes.create_string_buffer(512)
    rc = lib().hs_margin(json.dumps(obj).encode(),
                         json.dumps(deformation).encode() if deformation else None,
                         pts.ctypes.data, n, R, fov, ds, rho.ctypes.data, m.ctypes.data,
                         rho2.ctypes.data, m2.ctypes.data, d.ctypes.data, rho3.ctypes.data,
                         t.ctypes.data, ctypes.byref(aff), err, 512)
    if rc != 0:
        raise ValueError(err.value.decode())
    return rho3, t, bool(aff.value)


def render(obj, cams, res, ds, *, deformation=None, volume=None, R=4.0, integration="simple",
           flat_field=0.0, density_multiplier=1.0, rays=None, nthreads=None, force_general=False,
           trace=False, fine_lists=False):
    """cams: array (n, 20) = eye(3), column-major camera(16), fov.  ``trace``:
    certificate tracing (stats[0] counts evaluations); "curve": curved-ray
    certificates for non-affine chains.  ``fine_lists``: the finer candidate-list
    grids of large calls and batches."""
    cams = np.ascontiguousarray(cams, dtype=np.float64).reshape(-1, 20)
    n = cams.shape[0]
    vol = None
    nx = ny = nz = 0
    if volume is not None:
        vol = np.ascontiguousarray(volume, dtype=np.float32)
        nz, nx, ny = vol.shape
    if rays is not None:
        rays = np.ascontiguousarray(rays, dtype=np.int32).reshape(-1, 3)
        out = np.zeros(rays.shape[0], dtype=np.float32)
    else:
        out = np.zeros((n, res, res), dtype=np.float32)
    stats = np.zeros(2, dtype=np.uint64)
    err = ctypes.create_string_buffer(512)
    rc = lib().hs_render(json.dumps(obj).encode(), json.dumps(deformation).encode()
                         if deformation else None,
                         vol.ctypes.data if vol is not None else None, nx, ny, nz,
                         cams.ctypes.data, n, res, 1 if integration == "hierarchical" else 0,
                         ds, R, flat_field, density_multiplier, out.ctypes.data, stats.ctypes.data,
                         nthreads or os.cpu_count() or 1,
                         rays.ctypes.data if rays is not None else None,
                         rays.shape[0] if rays is not None else 0, 1 if force_general else 0,
                         2 if trace == "curve" else (1 if trace else 0), 1 if fine_lists else 0, err, 512)
    if rc != 0:
        raise ValueError(err.value.decode())
    return out, stats


def curve_bound(obj, points, dirs, *, deformation=None, R=4.0, fov=40.0, ds=0.01):
    """Curved-ray certificates at points [n,3] along world directions [n,3]:
    (density, bound t).  Every sample at ray parameter s in [0, t] must have
    the density of the point."""
    pts = np.ascontiguousarray(points, dtype=np.float64).reshape(-1, 3)
    d = np.ascontiguousarray(dirs, dtype=np.float64).reshape(-1, 3)
    n = pts.shape[0]
    rho, t = np.zeros(n, np.float32), np.zeros(n, np.float32)
    err = ctypes.create_string_buffer(512)
    L = lib()
    L.hs_curve.restype = ctypes.c_int
    L.hs_curve.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_void_p, ctypes.c_void_p,
                           ctypes.c_long, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                           ctypes.c_void_p, ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int]
    rc = L.hs_curve(json.dumps(obj).encode(), json.dumps(deformation).encode() if deformation else None,
                    pts.ctypes.data, d.ctypes.data, n, R, fov, ds, rho.ctypes.data, t.ctypes.data, err, 512)
    if rc != 0:
        raise ValueError(err.value.decode())
    return rho, t
