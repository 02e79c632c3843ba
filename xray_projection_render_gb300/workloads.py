"""Seeded synthetic workloads (the five configurations the engine is measured on).

No public dataset is involved: every input is generated here from
``numpy.random.default_rng(seed)`` with the shapes, sizes and value
distributions of the benchmark definitions.  Each function returns a
``Workload`` holding the reference-schema object map, an optional deformation
map, the camera angles, and the render settings; ``scale`` shrinks the view
count and resolution for tests while keeping the scene identical.

Common camera: R = 4, fov = 40 degrees (main.go:688-697 defaults), flat field
0, density multiplier 1, uniform-step integrator.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np


@dataclasses.dataclass
class Workload:
    name: str
    obj: dict
    deformation: dict | None
    angles: list            # (azimuthal, polar) degrees
    res: int
    ds: float
    R: float = 4.0
    fov: float = 40.0
    volume: np.ndarray | None = None   # float32 [z][x][y] for voxel scenes

    @property
    def rays(self) -> int:
        return len(self.angles) * self.res * self.res


def cube_minus_sphere_cylinder(res=512) -> Workload:
    """Cube (side 1, rho 1) minus a sphere (r 0.3) and a cylinder
    (r 0.2, z from -0.6 to 0.6); one view at azimuth 0, polar 90; ds 0.005."""
    obj = {"type": "object_collection", "objects": [
        {"type": "cube", "side": 1.0, "center": [0.0, 0.0, 0.0], "rho": 1.0},
        {"type": "sphere", "center": [0.0, 0.0, 0.0], "radius": 0.3, "rho": -1.0},
        {"type": "cylinder", "p0": [0.0, 0.0, -0.6], "p1": [0.0, 0.0, 0.6], "radius": 0.2,
         "rho": -1.0}]}
    return Workload("cube_minus_sphere_cylinder_512", obj, None, [(0.0, 90.0)], res, 0.005)


def gaussian_blob_volume(n=256, blobs=64, seed=2) -> np.ndarray:
    """Sum of isotropic Gaussians sampled on the (N-1) lattice x_i = i/(N-1)*2-1
    (objects.go:800-802), stored [z][x][y] as float32."""
    rng = np.random.default_rng(seed)
    c = rng.uniform(-0.8, 0.8, size=(blobs, 3))
    sig = rng.uniform(0.02, 0.1, size=blobs)
    amp = rng.uniform(0.0, 1.0, size=blobs)
    x = np.arange(n, dtype=np.float64) / (n - 1) * 2.0 - 1.0
    # exp(-|x-c|^2/(2 s^2)) factorises over the axes
    g = [np.exp(-((x[None, :] - c[:, a, None]) ** 2) / (2.0 * sig[:, None] ** 2)) for a in range(3)]
    gx, gy, gz = g
    # vol[k, i, j] = sum_m amp_m gz[m,k] gx[m,i] gy[m,j]
    gxy = (gx[:, :, None] * gy[:, None, :]).reshape(blobs, n * n)
    vol = ((amp[:, None] * gz).T @ gxy).reshape(n, n, n)
    return np.ascontiguousarray(vol, dtype=np.float32)


def voxel_blobs(res=1024, views=180, n=256, seed=2) -> Workload:
    """Voxel grid: 256^3 FP32 grid of 64 Gaussians, 180 views evenly spaced in
    azimuth (0, 2, ..., 358) at polar 90, 1024^2, ds = half a voxel."""
    vol = gaussian_blob_volume(n, 64, seed)
    angles = [(360.0 * k / views, 90.0) for k in range(views)]
    obj = {"type": "voxel_grid", "volume": 0}
    return Workload(f"voxel_{n}^3_gaussians_{views}x{res}^2", obj, None, angles, res,
                    0.5 * 2.0 / n, volume=vol)


def lattice_unit_cell(a=0.2, r=0.03):
    """Unit cell [0,a]^3: 12 edge cylinders and 4 body diagonals."""
    cyl = []
    for u in (0.0, a):
        for v in (0.0, a):
            cyl.append(([0.0, u, v], [a, u, v]))   # along x
            cyl.append(([u, 0.0, v], [u, a, v]))   # along y
            cyl.append(([u, v, 0.0], [u, v, a]))   # along z
    cyl += [([0, 0, 0], [a, a, a]), ([a, 0, 0], [0, a, a]), ([0, a, 0], [a, 0, a]),
            ([0, 0, a], [a, a, 0])]
    objs = [{"type": "cylinder", "p0": [float(t) for t in p0], "p1": [float(t) for t in p1],
             "radius": r, "rho": 1.0} for p0, p1 in cyl]
    return {"objects": {"type": "object_collection", "objects": objs},
            "xmin": 0.0, "xmax": a, "ymin": 0.0, "ymax": a, "zmin": 0.0, "zmax": a}


def offset_unit_cell(res=256) -> Workload:
    """Tessellation of a unit cell whose box does not start at the origin and
    whose extents are not dyadic (a sphere, an axial and a diagonal strut
    reaching its faces), under an affine chain; three views, ds 0.003."""
    lo, hi = [0.05, -0.13, 0.2], [0.31, 0.11, 0.37]
    c = [(a + b) / 2 for a, b in zip(lo, hi)]
    objs = [{"type": "sphere", "center": c, "radius": 0.06, "rho": 1.0},
            {"type": "cylinder", "p0": [lo[0], c[1], c[2]], "p1": [hi[0], c[1], c[2]],
             "radius": 0.025, "rho": 1.0},
            {"type": "cylinder", "p0": lo, "p1": hi, "radius": 0.02, "rho": 1.0}]
    uc = {"objects": {"type": "object_collection", "objects": objs},
          "xmin": lo[0], "xmax": hi[0], "ymin": lo[1], "ymax": hi[1], "zmin": lo[2], "zmax": hi[2]}
    obj = {"type": "tessellated_obj_coll", "uc": uc,
           "xmin": -0.9, "xmax": 0.85, "ymin": -0.8, "ymax": 0.95, "zmin": -0.7, "zmax": 0.9}
    deform = {"type": "affine", "matrix": [[1.02, 0.03, 0.0], [0.0, 0.97, 0.04], [0.02, 0.0, 1.05]]}
    return Workload(f"offset_unit_cell_3x{res}^2", obj, deform,
                    [(17.0, 70.0), (133.0, 95.0), (251.0, 120.0)], res, 0.003)


def deformed_lattice(res=1024, views=360, seed=3) -> Workload:
    """Deformed lattice: 16-cylinder cell tessellated 10x10x10 over [-1,1]^3 with 5 %
    axial (zz) strain; seeded random azimuth U[0,360) and polar U[30,150]."""
    rng = np.random.default_rng(seed)
    az = rng.uniform(0.0, 360.0, size=views)
    pol = rng.uniform(30.0, 150.0, size=views)
    obj = {"type": "tessellated_obj_coll", "uc": lattice_unit_cell(),
           "xmin": -1.0, "xmax": 1.0, "ymin": -1.0, "ymax": 1.0, "zmin": -1.0, "zmax": 1.0}
    deform = {"type": "linear", "strains": [0.0, 0.0, 0.05, 0.0, 0.0, 0.0]}
    return Workload(f"deformed_lattice_{views}x{res}^2", obj, deform,
                    [(float(a), float(p)) for a, p in zip(az, pol)], res, 0.002)


def _random_unit(rng):
    v = rng.normal(size=3)
    return v / np.linalg.norm(v)


def random_scene(rng) -> dict:
    n = int(rng.integers(1, 201))
    objs = []
    for _ in range(n):
        kind = ["sphere", "box", "cylinder", "parallelepiped"][int(rng.integers(0, 4))]
        c = rng.uniform(-0.8, 0.8, size=3)
        s = float(rng.uniform(0.02, 0.2))
        rho = 1.0 if rng.uniform() < 0.7 else -1.0
        if kind == "sphere":
            objs.append({"type": "sphere", "center": c.tolist(), "radius": s, "rho": rho})
        elif kind == "box":
            objs.append({"type": "box", "center": c.tolist(),
                         "sides": rng.uniform(0.02, 0.2, size=3).tolist(), "rho": rho})
        elif kind == "cylinder":
            L = s * float(rng.uniform(2.0, 5.0))
            u = _random_unit(rng)
            objs.append({"type": "cylinder", "p0": (c - 0.5 * L * u).tolist(),
                         "p1": (c + 0.5 * L * u).tolist(), "radius": s / 2, "rho": rho})
        else:
            e = [(_random_unit(rng) * rng.uniform(0.02, 0.2)).tolist() for _ in range(3)]
            objs.append({"type": "parallelepiped", "origin": c.tolist(), "v0": e[0], "v1": e[1],
                         "v2": e[2], "rho": rho})
    return {"type": "object_collection", "objects": objs}


def batched_scenes(count=64, seed=4) -> list:
    """Batch: 64 collections of 1-200 random primitives with uneven
    resolutions {256, 512, 1024} and 8-128 evenly spaced views each; ds 0.005."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(count):
        obj = random_scene(rng)
        res = int(rng.choice([256, 512, 1024]))
        nv = int(rng.integers(8, 129))
        angles = [(360.0 * v / nv, 90.0) for v in range(nv)]
        out.append(Workload(f"batched_scene_{k}", obj, None, angles, res, 0.005))
    return out


def gyroid_sigmoid(res=2048, views=720) -> Workload:
    """Gyroid (scale 8, thickness 0.1) tessellated with outer and
    unit-cell bounds [-1,1]^3, sigmoid deformation (A 0.1, L 0.2, along z);
    720 views evenly spaced in azimuth; 2048^2; ds 0.001."""
    obj = {"type": "tessellated_obj_coll",
           "uc": {"objects": {"type": "object_collection", "objects": [
               {"type": "gyroid", "center": [0.0, 0.0, 0.0], "scale": 8.0, "thickness": 0.1,
                "rho": 1.0}]},
                  "xmin": -1.0, "xmax": 1.0, "ymin": -1.0, "ymax": 1.0, "zmin": -1.0, "zmax": 1.0},
           "xmin": -1.0, "xmax": 1.0, "ymin": -1.0, "ymax": 1.0, "zmin": -1.0, "zmax": 1.0}
    deform = {"type": "sigmoid", "amplitude": 0.1, "center": 0.0, "lengthscale": 0.2,
              "direction": "z"}
    angles = [(0.5 * k, 90.0) for k in range(views)]
    return Workload(f"gyroid_sigmoid_{views}x{res}^2", obj, deform, angles, res, 0.001)


def gyroid_fine_sigmoid(res=2048, views=64) -> Workload:
    """The gyroid of the reference's example scene (scale 0.1, thickness 0.2:
    a period of about 0.63, a lattice of sheets, where scale 8 gives one
    smooth band) tessellated with unit-cell bounds [-1,1]^3 and outer bounds
    [-0.8,0.8]^3, under the sigmoid deformation of the scale-8 workload
    (A 0.1, L 0.2, along z); `views` of its 720 cameras, evenly strided;
    2048^2; ds 0.001."""
    obj = {"type": "tessellated_obj_coll",
           "uc": {"objects": {"type": "object_collection", "objects": [
               {"type": "gyroid", "center": [0.0, 0.0, 0.0], "scale": 0.1, "thickness": 0.2,
                "rho": 1.0}]},
                  "xmin": -1.0, "xmax": 1.0, "ymin": -1.0, "ymax": 1.0, "zmin": -1.0, "zmax": 1.0},
           "xmin": -0.8, "xmax": 0.8, "ymin": -0.8, "ymax": 0.8, "zmin": -0.8, "zmax": 0.8}
    deform = {"type": "sigmoid", "amplitude": 0.1, "center": 0.0, "lengthscale": 0.2,
              "direction": "z"}
    angles = [(0.5 * k, 90.0) for k in range(0, 720, max(1, 720 // views))][:views]
    return Workload(f"gyroid_fine_sigmoid_{views}x{res}^2", obj, deform, angles, res, 0.001)


def reduced(w: Workload, res: int, views: int | None = None) -> Workload:
    """The same scene at another resolution and/or on an evenly strided
    subset of its views (parity tests, profiling).  The name says so: the
    full workload's name with ``_subset<views>x<res>^2`` appended."""
    ang = w.angles if views is None else w.angles[:: max(1, len(w.angles) // views)][:views]
    if res == w.res and len(ang) == len(w.angles):
        return w
    return dataclasses.replace(w, res=res, angles=list(ang),
                               name=f"{w.name}_subset{len(ang)}x{res}^2")


WORKLOADS = {
    "cube_minus_sphere_cylinder": cube_minus_sphere_cylinder,
    "voxel_blobs": voxel_blobs,
    "deformed_lattice": deformed_lattice,
    "gyroid_sigmoid": gyroid_sigmoid,
    "gyroid_fine_sigmoid": gyroid_fine_sigmoid,
}

__all__ = ["Workload", "cube_minus_sphere_cylinder", "gaussian_blob_volume", "voxel_blobs",
           "lattice_unit_cell", "deformed_lattice", "random_scene", "batched_scenes",
           "gyroid_sigmoid", "gyroid_fine_sigmoid", "reduced", "WORKLOADS", "math"]
