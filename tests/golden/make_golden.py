"""Generates the golden fixtures of tests/golden from the FP64 oracle.

    python tests/golden/make_golden.py

Each fixture is a small render (reduced resolution and view count) of one of
the five benchmark scenes, or of the reference's own GPU test scenes
(cuda_test.go:41-215), stored with its inputs.  The oracle is pinned to the
reference's known-answer tests (tests/test_oracle_kat.py); these fixtures pin
the engine and the oracle on the same bytes wherever they run.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import oracle as O  # noqa: E402
from xray_projection_render_gb300 import workloads as W  # noqa: E402


def scene_cases():
    out = {
        "scene_cube_minus_sphere_cylinder": W.cube_minus_sphere_cylinder(48),
        "scene_deformed_lattice": W.reduced(W.deformed_lattice(), 40, 2),
        "scene_gyroid_sigmoid": W.reduced(W.gyroid_sigmoid(), 40, 2),
        "scene_batched_scene0": W.reduced(W.batched_scenes(1)[0], 40, 2),
    }
    return out


def cuda_test_volumes():
    """TestCPUvsCUDA (32^3 sphere) and TestCPUvsCUDA_NonCubic (24x32x16 box)."""
    vols = {}
    for (NX, NY, NZ), kind in [((32, 32, 32), "sphere"), ((24, 32, 16), "box")]:
        vol = np.zeros((NZ, NX, NY), dtype=np.float32)
        x = np.arange(NX) / NX * 2 - 1
        y = np.arange(NY) / NY * 2 - 1
        z = np.arange(NZ) / NZ * 2 - 1
        Z, X, Y = np.meshgrid(z, x, y, indexing="ij")
        if kind == "sphere":
            vol[X ** 2 + Y ** 2 + Z ** 2 < 0.09] = 1.0
        else:
            vol[(np.abs(X) < 0.4) & (np.abs(Y) < 0.2) & (np.abs(Z) < 0.3)] = 1.0
        vols[f"cuda_test_{kind}"] = (vol, 2.0 / min(NX, NY, NZ) / 5.0)
    return vols


def main():
    import json
    for name, w in scene_cases().items():
        for integ in ("simple", "hierarchical"):
            img = O.render(O.Scene(w.obj, w.deformation), w.angles, w.res, w.ds, R=w.R, fov=w.fov,
                           integration=integ)
            np.savez_compressed(os.path.join(HERE, f"{name}_{integ}.npz"), image=img,
                                obj=json.dumps(w.obj),
                                deformation=json.dumps(w.deformation) if w.deformation else "",
                                angles=np.asarray(w.angles), res=w.res, ds=w.ds, R=w.R, fov=w.fov,
                                integration=integ)
    vol = W.gaussian_blob_volume(24, 8, seed=2)
    for name, (v, ds) in dict(cuda_test_volumes(), voxel_blobs=(vol, 2.0 / 24 / 2)).items():
        angles = [(0.0, 90.0), (75.0, 90.0)]
        cams = O.xray_camera_params(angles, 4.0, 40.0)
        img = O.render_volume_abi(v, cams, 32, np.float32(ds))
        np.savez_compressed(os.path.join(HERE, f"{name}_abi.npz"), image=img, volume=v,
                            cams21=cams, res=32, ds=np.float32(ds))
    print("fixtures written to", HERE)


if __name__ == "__main__":
    main()
