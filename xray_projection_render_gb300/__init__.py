"""GB300-native (sm_103a) engine for the per-pixel X-ray projection line
integral of igrega348/xray_projection_render.

The engine is the C-ABI library ``libcuda_render.so`` (include/xrp.h), a
drop-in for the reference's dlopen'd GPU library; this package holds its
CUDA/C++ sources (``csrc/``), its build recipe (``build.py``), a ctypes
front end (``engine.py``) and the seeded synthetic workloads
(``workloads.py``) and ``XRayRenderer``, the drop-in for the reference's
Python API (``renderer.py``).
"""
from .engine import (Batch, Proposal, Scene, assemble_voxel_grid, camera_arrays, cameras_from_angles,
                     mlp_grad, release_cache, render, render_proposal, render_volume_projections,
                     finish_images, voxelize_scene, xray_camera_params)
from .renderer import XRayRenderer

__all__ = ["Scene", "render", "render_volume_projections", "assemble_voxel_grid",
           "cameras_from_angles", "camera_arrays", "xray_camera_params", "release_cache",
           "Proposal", "render_proposal", "mlp_grad", "Batch", "voxelize_scene", "finish_images",
           "XRayRenderer"]
