"""ctypes binding of libcuda_render.so (the C ABI declared in include/xrp.h).

The library is built in-tree by ``build.py``; loading fails loudly when it is
missing -- there is no CPU fallback of the engine.
"""
from __future__ import annotations

import ctypes
import os
import threading

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libcuda_render.so")

c_int, c_float, c_double, c_void_p = ctypes.c_int, ctypes.c_float, ctypes.c_double, ctypes.c_void_p


class CylinderParams(ctypes.Structure):  # cuda_backend.h:22-27
    _fields_ = [("p0", c_float * 3), ("p1", c_float * 3), ("radius", c_float), ("rho", c_float)]


class XRayCameraParams(ctypes.Structure):  # cuda_backend.h:78-83
    _fields_ = [("eye", c_float * 3), ("view", c_float * 16), ("fov_y", c_float), ("R", c_float)]


class XrpCamera(ctypes.Structure):
    _fields_ = [("eye", c_double * 3), ("camera", c_double * 16), ("fov_deg", c_double)]


class XrpRenderOpts(ctypes.Structure):
    _fields_ = [("resolution", c_int), ("integration", c_int), ("ds", c_double), ("R", c_double),
                ("flat_field", c_double), ("density_multiplier", c_double), ("flags", c_int),
                ("reserved", c_int)]


class XrpVolumeDesc(ctypes.Structure):
    _fields_ = [("data", c_void_p), ("nx", c_int), ("ny", c_int), ("nz", c_int),
                ("on_device", c_int)]


class XrpProposalOpts(ctypes.Structure):
    _fields_ = [("segment", c_int), ("train_rays", c_int), ("val_rays", c_int), ("steps", c_int),
                ("batch", c_int), ("lr", c_float), ("pos_weight", c_float), ("tau_margin", c_float),
                ("seed", ctypes.c_uint64), ("reserved", c_int * 4)]


class XrpProposalInfo(ctypes.Structure):
    _fields_ = [("tau", c_float), ("segment", c_int), ("train_rows", ctypes.c_longlong),
                ("train_pos", ctypes.c_longlong), ("val_rows", ctypes.c_longlong),
                ("val_pos", ctypes.c_longlong), ("val_accepted", ctypes.c_longlong),
                ("final_loss", c_float), ("train_ms", c_float)]


class XrpBatchItem(ctypes.Structure):
    _fields_ = [("scene", c_void_p), ("views", c_void_p), ("num_views", c_int), ("resolution", c_int)]


class XrpBatchInfo(ctypes.Structure):
    _fields_ = [("rays", ctypes.c_longlong), ("tiles", ctypes.c_longlong), ("tile_w", c_int),
                ("tile_h", c_int), ("blocks_per_sm", c_int), ("num_sms", c_int),
                ("tune_candidates", c_int), ("tune_ms", c_float * 8), ("build_ms", c_float)]


XRP_INTEGRATE_SIMPLE = 0
XRP_INTEGRATE_HIERARCHICAL = 1
XRP_FLAG_STATS = 1
XRP_FLAG_VOLUME_LOADS = 2
XRP_FLAG_NO_REFINE = 4
XRP_FLAG_TRACE = 8
XRP_FLAG_BALL = 16
XRP_FLAG_PLAIN_INPLACE = 32
XRP_FLAG_PLAIN_LIST = 64

# Every symbol include/xrp.h declares, with (restype, argtypes).
SIGNATURES = {
    "RenderVolumeProjectionsCUDA": (c_int, [c_void_p, c_int, c_int, c_int, c_void_p, c_int, c_int,
                                            c_float, c_float, c_void_p]),
    "AssembleVoxelGridCUDA": (c_int, [c_void_p, c_int, c_int, c_float, c_void_p]),
    "AssembleVoxelGridSpatialCUDA": (c_int, [c_void_p, c_int, c_int, c_float, c_int, c_void_p,
                                             c_void_p, c_int, c_void_p]),
    "xrp_last_error": (ctypes.c_char_p, []),
    "xrp_version": (c_int, []),
    "xrp_cameras_from_angles": (c_int, [c_void_p, c_int, c_double, c_double, c_void_p]),
    "xrp_scene_create": (c_int, [ctypes.c_char_p, ctypes.c_char_p, c_void_p, c_int, c_void_p]),
    "xrp_scene_destroy": (None, [c_void_p]),
    "xrp_scene_support": (c_int, [c_void_p, c_void_p, c_void_p]),
    "xrp_scene_min_feature_size": (c_int, [c_void_p, c_void_p]),
    "xrp_render": (c_int, [c_void_p, c_void_p, c_int, c_void_p, c_void_p]),
    "xrp_render_device": (c_int, [c_void_p, c_void_p, c_int, c_void_p, c_void_p, c_void_p]),
    "xrp_last_stats": (c_int, [c_void_p, c_void_p]),
    "xrp_release_cache": (None, []),
    "xrp_render_volume_noalloc": (c_int, [c_void_p, c_int, c_int, c_int, c_void_p, c_int, c_int,
                                          c_float, c_float, c_void_p, c_void_p]),
    "xrp_probe_gather_rate": (c_int, [c_void_p]),
    "xrp_voxelize_scene": (c_int, [c_void_p, c_int, c_double, c_void_p, c_void_p]),
    "xrp_finish_images": (c_int, [c_void_p, c_int, c_int, c_int, c_void_p, c_void_p, c_void_p,
                                  c_void_p]),
    "xrp_batch_create": (c_int, [c_void_p, c_int, c_void_p, c_int, c_void_p]),
    "xrp_batch_render": (c_int, [c_void_p, c_void_p]),
    "xrp_batch_output": (c_void_p, [c_void_p]),
    "xrp_batch_item_offset": (ctypes.c_longlong, [c_void_p, c_int]),
    "xrp_batch_copy_item": (c_int, [c_void_p, c_int, c_void_p]),
    "xrp_batch_get_info": (c_int, [c_void_p, c_void_p]),
    "xrp_batch_destroy": (None, [c_void_p]),
    "xrp_proposal_train": (c_int, [c_void_p, c_void_p, c_int, c_void_p, c_void_p, c_void_p]),
    "xrp_proposal_get_info": (c_int, [c_void_p, c_void_p]),
    "xrp_proposal_params": (c_int, [c_void_p, c_void_p, c_int]),
    "xrp_proposal_set_tau": (c_int, [c_void_p, c_float]),
    "xrp_proposal_destroy": (None, [c_void_p]),
    "xrp_render_proposal": (c_int, [c_void_p, c_void_p, c_int, c_void_p, c_int, c_void_p, c_void_p]),
    "xrp_render_proposal_device": (c_int, [c_void_p, c_void_p, c_int, c_void_p, c_int, c_void_p,
                                           c_void_p, c_void_p]),
    "xrp_proposal_last_stats": (c_int, [c_void_p]),
    "xrp_mlp_param_count": (c_int, []),
    "xrp_mlp_grad": (c_int, [c_void_p, c_void_p, c_void_p, c_int, c_float, c_void_p, c_void_p,
                             c_void_p]),
}

_lib = None
_lock = threading.Lock()


class EngineError(RuntimeError):
    def __init__(self, code: int, func: str, msg: str):
        super().__init__(f"{func} failed with code {code}: {msg}")
        self.code = code


def load(path: str | None = None):
    """Load libcuda_render.so (RTLD_LOCAL, like the Go loader) and bind it."""
    global _lib
    with _lock:
        if _lib is not None and path is None:
            return _lib
        p = path or os.environ.get("XRAY_CUDA_LIB") or LIB_PATH
        if not os.path.exists(p):
            raise FileNotFoundError(
                f"libcuda_render.so not found at {p}; build it with "
                "`python -m xray_projection_render_gb300.build`")
        L = ctypes.CDLL(p, mode=os.RTLD_LAZY | os.RTLD_LOCAL)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        if path is None:
            _lib = L
        return L


def check(code: int, func: str):
    if code != 0:
        msg = load().xrp_last_error()
        raise EngineError(code, func, msg.decode() if msg else "")
