"""Drop-in for the reference's Python API, rendering on the GB300 engine.

``XRayRenderer().render(params, camera_angles=None)`` takes the parameter
dictionary of the reference's ``XRayRenderer.render``
(xray_projection_render/xray_renderer.py:357-448) with the same defaults,
and does what the Go side behind it does (``RenderProjections``,
api.go:75-177, calling ``render``, main.go:310-549): it loads the object and
deformation files (JSON or YAML, chosen by the last four characters of the
name, main.go:63-76, 97-110), picks the automatic step for ``ds < 0``
(MinFeatureSize / 5, main.go:350-353), generates or takes the camera angles
(main.go:242-257), renders every view, writes one PNG per view
(main.go:482-516), ``transforms.json`` and ``object.json`` (main.go:518-547)
and, with ``export_volume``, ``volume.raw`` (main.go:549-635).  It returns
the reference's result dictionary (api.go:66-72): ``success``, ``error`` on
failure, ``num_images`` and ``output_dir``.

What differs: every view renders on the GPU (certificate tracing for
analytic scenes, the plain integrator for voxel grids; both equal the
reference CPU path within 1e-5 on transmittance), the per-pixel image
finishing runs on the device (``xrp_finish_images``), and YAML files are
read by a subset reader (``yaml_subset``).  The PNGs hold the same pixels as
the reference's (8-bit RGB, RGBA with ``transparency``); their compressed
bytes differ.
"""
from __future__ import annotations

import json
import math
import os
import re
import struct
import zlib
from decimal import Decimal

import numpy as np

from . import engine, yaml_subset
from . import _lib

# xray_renderer.py:415-437
DEFAULTS = {
    "input": None, "output_dir": "images", "fname_pattern": "image_%03d.png", "resolution": 512,
    "num_images": 1, "out_of_plane": False, "ds": -1.0, "R": 4.0, "fov": 40.0, "jobs_modulo": 1,
    "job_num": 0, "transforms_file": "transforms.json", "deformation_file": "", "time_label": 0.0,
    "transparency": False, "export_volume": False, "polar_angle": 90.0, "density_multiplier": 1.0,
    "flat_field": 0.0, "integration": "hierarchical", "log_level": "error",
}

CUBE_HALF_DIAGONAL = 1.74  # main.go:46


class XRayRenderer:
    """The reference's ``XRayRenderer`` (xray_renderer.py:63-448) on the GPU.

    ``library_path``: the engine library (default: the in-tree
    libcuda_render.so, or $XRAY_CUDA_LIB)."""

    def __init__(self, library_path: str | None = None):
        self.lib = _lib.load(library_path) if library_path else _lib.load()

    def render(self, params: dict, camera_angles: list | None = None) -> dict:
        p = dict(DEFAULTS)
        for k in DEFAULTS:
            if k in params:
                p[k] = params[k]
        p["camera_angles"] = []
        if camera_angles is not None:
            p["camera_angles"] = camera_angles
        elif "camera_angles" in params:
            p["camera_angles"] = params["camera_angles"]
        if not p["input"]:
            raise ValueError("'input' parameter is required")
        return render_projections(p)


def render_projections(p: dict) -> dict:
    """RenderProjections (api.go:75-177) on a complete parameter map."""
    if p.get("ds", 0) == 0:
        return {"success": False,
                "error": "ds is 0; use a negative value for automatic step-size selection"}
    if p.get("density_multiplier", 0) == 0:
        return {"success": False,
                "error": "density_multiplier is 0; all densities will be zero and the render will "
                         "produce a blank image"}
    try:
        _render(p)
    except Exception as ex:  # the reference recovers panics into the result
        return {"success": False, "error": f"render failed: {ex}"}
    return {"success": True, "num_images": int(p.get("num_images", 0)),
            "output_dir": p.get("output_dir", "")}


def load_map(path: str) -> dict:
    """An object or deformation file as a map, by the last four characters of
    its name (main.go:63-76, 97-110); other extensions give an empty map."""
    with open(path, "rb") as f:
        text = f.read().decode("utf-8")
    ext = path[-4:]
    if ext == "yaml":
        out = yaml_subset.loads(text)
    elif ext == "json":
        out = json.loads(text)
    else:
        out = {}
    return out if isinstance(out, dict) else {}


def generate_camera_angles(num_images, job_num, jobs_modulo, out_of_plane, polar_angle, rng=None):
    """generateCameraAngles (main.go:242-257): azimuth i*360/N + 90 for
    i = job_num, job_num + jobs_modulo, ...; polar fixed, or acos(U[-1,1])
    with out_of_plane (unseeded, as the reference's math/rand)."""
    rng = rng or np.random.default_rng()
    out = []
    i = int(job_num)
    step = int(jobs_modulo)
    if step <= 0:
        raise ValueError("jobs_modulo must be positive")
    while i < num_images:
        th = float(i) * (360.0 / float(num_images)) + 90.0
        phi = math.acos(rng.uniform() * 2 - 1) * 180.0 / math.pi if out_of_plane else float(polar_angle)
        out.append((th, phi))
        i += step
    return out


def _angle(a):
    """(azimuthal, polar) of a camera-angle entry; JSON keys match the Go
    struct's field names without regard to case (encoding/json)."""
    if isinstance(a, dict):
        low = {str(k).lower(): v for k, v in a.items()}
        return float(low.get("azimuthal", 0.0)), float(low.get("polar", 0.0))
    az, pol = a
    return float(az), float(pol)


def _has_voxels(obj) -> bool:
    if isinstance(obj, dict):
        return obj.get("type") == "voxel_grid" or any(_has_voxels(v) for v in obj.values())
    if isinstance(obj, list):
        return any(_has_voxels(v) for v in obj)
    return False


# --- files ----------------------------------------------------------------

def _go_dir(path: str) -> str:
    """filepath.Dir: all but the last element, cleaned; "." when empty."""
    d = os.path.dirname(path)
    return os.path.normpath(d) if d else "."


def _go_join(*parts) -> str:
    return os.path.normpath(os.path.join(*parts))


def _go_base(path: str) -> str:
    """filepath.Base: the last element, trailing slashes dropped; "." when empty."""
    if path == "":
        return "."
    p = path.rstrip("/")
    return os.path.basename(p) if p else "/"


def write_png(path: str, rgb8: np.ndarray, alpha8: np.ndarray | None):
    """8-bit RGB (or RGBA) PNG: the pixels Go's png.Encode writes for the
    reference's image.RGBA (main.go:482-513): opaque images as RGB, others
    as RGBA with fully transparent pixels stored as (0, 0, 0, 0)."""
    h, w = rgb8.shape[:2]
    if alpha8 is None or np.all(alpha8 == 0xFF):
        px = np.repeat(rgb8[:, :, None], 3, axis=2)
        ctype, ch = 2, 3
    else:
        px = np.stack([rgb8, rgb8, rgb8, alpha8], axis=2)
        px[alpha8 == 0] = 0
        ctype, ch = 6, 4
    raw = np.empty((h, 1 + w * ch), dtype=np.uint8)
    raw[:, 0] = 0
    raw[:, 1:] = px.reshape(h, w * ch)

    def chunk(tag, data):
        return (struct.pack(">I", len(data)) + tag + data
                + struct.pack(">I", zlib.crc32(tag + data) & 0xFFFFFFFF))

    with open(path, "wb") as f:
        f.write(b"\x89PNG\r\n\x1a\n")
        f.write(chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, ctype, 0, 0, 0)))
        f.write(chunk(b"IDAT", zlib.compress(raw.tobytes(), 6)))
        f.write(chunk(b"IEND", b""))


def _go_float(v: float) -> str:
    """A float64 as Go's encoding/json writes it: the shortest digits, fixed
    notation for 1e-6 <= |v| < 1e21, else exponent notation with at least
    one exponent digit ("1e-7")."""
    if not math.isfinite(v):
        raise ValueError("json: unsupported value")
    r = repr(float(v))
    a = abs(v)
    if a != 0 and (a < 1e-6 or a >= 1e21):
        m = re.match(r"^(-?[0-9.]+)e([-+])0*([0-9]+)$", r)
        if m is None:  # repr chose fixed notation: go through Decimal
            mant, e = format(Decimal(r), "e").split("e")
            sign, ex = ("-" if e.startswith("-") else "+"), e.lstrip("+-").lstrip("0") or "0"
            mant = mant.rstrip("0").rstrip(".") if "." in mant else mant
            return f"{mant}e{sign}{ex if sign == '-' else ex.zfill(2)}"
        ex = m.group(3)
        return f"{m.group(1)}e{m.group(2)}{ex if m.group(2) == '-' else ex.zfill(2)}"
    s = format(Decimal(r), "f")
    if "." in s:
        s = s.rstrip("0").rstrip(".")
    return s


def _go_json(v, ind="") -> str:
    """json.MarshalIndent(v, "", "  ") for maps (keys as given), lists,
    strings, bools, ints and floats."""
    nxt = ind + "  "
    if isinstance(v, dict):
        if not v:
            return "{}"
        items = [f'{nxt}{json.dumps(str(k))}: {_go_json(x, nxt)}' for k, x in v.items()]
        return "{\n" + ",\n".join(items) + "\n" + ind + "}"
    if isinstance(v, (list, tuple)):
        if not v:
            return "[]"
        return "[\n" + ",\n".join(nxt + _go_json(x, nxt) for x in v) + "\n" + ind + "]"
    if isinstance(v, bool):
        return "true" if v else "false"
    if isinstance(v, int):
        return str(v)
    if isinstance(v, float):
        return _go_float(v)
    if v is None:
        return "null"
    return json.dumps(str(v))


def _vec(m, key):
    return [float(x) for x in m.get(key, [0.0, 0.0, 0.0])]


def to_map(m: dict) -> dict:
    """The object as the reference's ToMap methods re-serialise it
    (objects.go:33-40, 91-98, 139-146, 198-207, 296-304, 370-379, 466-477,
    523-534, 704-713, 973-981); Go writes map keys sorted."""
    t = m.get("type")
    if t == "sphere":
        out = {"center": _vec(m, "center"), "radius": float(m["radius"]), "rho": float(m["rho"]),
               "type": "sphere"}
    elif t == "cube":
        out = {"center": _vec(m, "center"), "rho": float(m["rho"]), "side": float(m["side"]),
               "type": "cube"}
    elif t == "box":
        out = {"center": _vec(m, "center"), "rho": float(m["rho"]), "sides": _vec(m, "sides"),
               "type": "box"}
    elif t == "parallelepiped":
        out = {"origin": _vec(m, "origin"), "rho": float(m["rho"]), "type": "parallelepiped",
               "v0": _vec(m, "v0"), "v1": _vec(m, "v1"), "v2": _vec(m, "v2")}
    elif t == "cylinder":
        out = {"p0": _vec(m, "p0"), "p1": _vec(m, "p1"), "radius": float(m["radius"]),
               "rho": float(m.get("rho", 1.0)), "type": "cylinder"}
    elif t == "gyroid":
        out = {"center": _vec(m, "center"), "rho": float(m["rho"]), "scale": float(m["scale"]),
               "thickness": float(m["thickness"]), "type": "gyroid"}
    elif t == "object_collection":
        out = {"objects": [to_map(o) for o in m.get("objects", [])], "type": "object_collection"}
    elif t == "tessellated_obj_coll":
        uc = m["uc"]
        ucm = {"objects": to_map(dict(uc["objects"], type="object_collection")), "type": "unit_cell"}
        ucm.update({k: float(uc[k]) for k in ("xmax", "xmin", "ymax", "ymin", "zmax", "zmin")})
        out = {"type": "tessellated_obj_coll", "uc": dict(sorted(ucm.items()))}
        out.update({k: float(m[k]) for k in ("xmax", "xmin", "ymax", "ymin", "zmax", "zmin")})
    elif t == "voxel_grid":
        out = {"dtype": "float64", "nx": int(m.get("nx", 0)), "ny": int(m.get("ny", 0)),
               "nz": int(m.get("nz", 0)), "path": m.get("path", ""), "type": "voxel_grid"}
    else:
        out = dict(m)
    return dict(sorted(out.items()))


# --- the render -----------------------------------------------------------

def _render(p: dict):
    import torch

    obj = load_map(p["input"])
    deformation = load_map(p["deformation_file"]) if p.get("deformation_file") else None
    out_dir = p["output_dir"]
    os.makedirs(out_dir, exist_ok=True)
    res = int(p["resolution"])
    R, fov = float(p["R"]), float(p["fov"])
    integration = "simple" if p.get("integration") == "simple" else "hierarchical"
    angles = [_angle(a) for a in (p.get("camera_angles") or [])]
    if not angles:
        angles = generate_camera_angles(int(p["num_images"]), int(p["job_num"]),
                                        int(p["jobs_modulo"]), bool(p["out_of_plane"]),
                                        float(p["polar_angle"]))
    transparency = bool(p["transparency"])
    flat_field = float(p["flat_field"])
    dm = float(p["density_multiplier"])
    tp = {"flat_field": math.exp(-flat_field), "camera_angle_x": fov * math.pi / 180.0, "fl_x": 0.0,
          "fl_y": 0.0, "w": res, "h": res, "cx": res / 2.0, "cy": res / 2.0, "frames": []}
    with engine.Scene(obj, deformation) as scene:
        ds = float(p["ds"])
        if ds < 0:
            mfs = _lib_min_feature(scene)
            ds = mfs / 5.0
        if angles:
            f = 1.0 / math.tan(fov / 2.0 * math.pi / 180.0)
            tp["fl_x"] = tp["fl_y"] = f * res / 2.0
        traced = not _has_voxels(obj)
        dev = torch.device("cuda", torch.cuda.current_device())
        per = max(1, (1 << 28) // (res * res))  # at most 1 GiB of images per pass
        eyes_cams = engine.camera_arrays(angles, R, fov) if angles else (None, None)
        kw = dict(resolution=res, ds=ds, R=R, fov=fov, flat_field=flat_field, density_multiplier=dm,
                  integration=integration)
        for v0 in range(0, len(angles), per):
            chunk = angles[v0:v0 + per]
            img = torch.empty((len(chunk), res, res), device=dev, dtype=torch.float32)
            if traced:
                engine.render_proposal(scene, None, chunk, trace=True, out=img, **kw)
            else:
                engine.render(scene, chunk, out=img, **kw)
            gray, alpha, _ = engine.finish_images(img, transparency=transparency)
            gray8 = (gray.view(torch.int16).cpu().numpy().view(np.uint16) >> 8).astype(np.uint8)
            alpha8 = (alpha.cpu().numpy().view(np.uint16) >> 8).astype(np.uint8)
            for k in range(len(chunk)):
                i_img = v0 + k
                filename = _go_join(out_dir, p["fname_pattern"] % i_img)
                write_png(filename, gray8[k], alpha8[k])
                dname, fname = os.path.split(filename)
                rel = _go_join(_go_base(dname), fname)
                cam = eyes_cams[1][i_img]
                tm = [[float(cam[j * 4 + i]) for j in range(4)] for i in range(4)]
                tp["frames"].append({"file_path": rel.replace(os.sep, "/"),
                                     "time": float(p["time_label"]), "transform_matrix": tm})
        with open(p["transforms_file"], "w") as fh:
            fh.write(_go_json(tp))
        with open(_go_join(_go_dir(out_dir), "object.json"), "w") as fh:
            fh.write(_go_json(to_map(obj)))
        if p.get("export_volume"):
            _, u8 = engine.voxelize_scene(scene, res, density_multiplier=dm)
            u8.tofile(_go_join(_go_dir(out_dir), "volume.raw"))


def _lib_min_feature(scene) -> float:
    import ctypes
    v = ctypes.c_double()
    _lib.check(_lib.load().xrp_scene_min_feature_size(scene.handle, ctypes.byref(v)),
               "xrp_scene_min_feature_size")
    return v.value


__all__ = ["XRayRenderer", "render_projections", "load_map", "generate_camera_angles", "write_png",
           "to_map", "DEFAULTS", "CUBE_HALF_DIAGONAL"]
