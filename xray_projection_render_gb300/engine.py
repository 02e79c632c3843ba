"""Python front end of the GB300 projection engine (libcuda_render.so).

Mirrors the reference's render interface (main.go:310-471 / api.go:40-64):
an object map in the reference JSON/YAML schema, an optional deformation
map, camera angles and the CLI options (resolution, ds, R, fov, flat_field,
density_multiplier, integration).  Every call goes through the C ABI of
include/xrp.h; the images are float32 transmittance [view][i][j].
"""
from __future__ import annotations

import ctypes
import json

import numpy as np

from . import _lib
from ._lib import XrpCamera, XrpRenderOpts, XrpVolumeDesc, check


def _json(x) -> bytes | None:
    if x is None:
        return None
    if isinstance(x, (bytes, bytearray)):
        return bytes(x)
    if isinstance(x, str):
        return x.encode()
    return json.dumps(x).encode()


def _is_torch_cuda(t) -> bool:
    return type(t).__module__.startswith("torch") and getattr(t, "is_cuda", False)


class Scene:
    """A scene resident on the current CUDA device (xrp_scene_create).

    ``volumes`` lists the grids referenced by ``{"type": "voxel_grid",
    "volume": k}`` entries: float32 numpy arrays [z][x][y] (copied to the
    device) or CUDA tensors (used in place; keep them alive)."""

    def __init__(self, obj, deformation=None, volumes=()):
        L = _lib.load()
        self._keep = []
        descs = (XrpVolumeDesc * max(1, len(volumes)))()
        for k, v in enumerate(volumes):
            if _is_torch_cuda(v):
                if v.dtype.__repr__() != "torch.float32" or not v.is_contiguous():
                    raise ValueError("device volumes must be contiguous float32")
                nz, nx, ny = v.shape
                descs[k] = XrpVolumeDesc(v.data_ptr(), nx, ny, nz, 1)
            else:
                a = np.ascontiguousarray(v, dtype=np.float32)
                nz, nx, ny = a.shape
                descs[k] = XrpVolumeDesc(a.ctypes.data, nx, ny, nz, 0)
            self._keep.append(v)
        h = ctypes.c_void_p()
        check(L.xrp_scene_create(_json(obj), _json(deformation), descs, len(volumes),
                                 ctypes.byref(h)), "xrp_scene_create")
        self._h = h

    @property
    def handle(self):
        return self._h

    def support(self):
        lo = (ctypes.c_double * 3)()
        hi = (ctypes.c_double * 3)()
        check(_lib.load().xrp_scene_support(self._h, lo, hi), "xrp_scene_support")
        return list(lo), list(hi)

    def close(self):
        if getattr(self, "_h", None):
            _lib.load().xrp_scene_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def cameras_from_angles(angles, R=4.0, fov=40.0):
    """computeCameraFromAngles (main.go:226-239) for a list of (azimuthal,
    polar) degrees, as an array of XrpCamera."""
    a = np.ascontiguousarray(np.asarray(angles, dtype=np.float64).reshape(-1, 2))
    cams = (XrpCamera * max(1, a.shape[0]))()
    check(_lib.load().xrp_cameras_from_angles(a.ctypes.data, a.shape[0], float(R), float(fov),
                                              cams), "xrp_cameras_from_angles")
    return cams, a.shape[0]


def camera_arrays(angles, R=4.0, fov=40.0):
    """(eyes [n,3], column-major cameras [n,16]) from the engine's camera code."""
    cams, n = cameras_from_angles(angles, R, fov)
    eyes = np.array([list(cams[k].eye) for k in range(n)])
    mats = np.array([list(cams[k].camera) for k in range(n)])
    return eyes, mats


def _opts(resolution, ds, R, flat_field, density_multiplier, integration, stats,
          volume_path="gather", plain_fp64="auto"):
    if integration not in ("simple", "hierarchical"):
        raise ValueError(f"Unknown integration method: {integration}")
    if volume_path not in ("gather", "loads"):
        raise ValueError(f"Unknown volume path: {volume_path}")
    if plain_fp64 not in ("auto", "list", "inplace"):
        raise ValueError(f"Unknown FP64 pass: {plain_fp64}")
    flags = (_lib.XRP_FLAG_STATS if stats else 0) | \
        (_lib.XRP_FLAG_VOLUME_LOADS if volume_path == "loads" else 0) | \
        (_lib.XRP_FLAG_PLAIN_INPLACE if plain_fp64 == "inplace" else 0) | \
        (_lib.XRP_FLAG_PLAIN_LIST if plain_fp64 == "list" else 0)
    return XrpRenderOpts(int(resolution),
                         _lib.XRP_INTEGRATE_HIERARCHICAL if integration == "hierarchical"
                         else _lib.XRP_INTEGRATE_SIMPLE,
                         float(ds), float(R), float(flat_field), float(density_multiplier),
                         flags, 0)


def render(scene: Scene, angles, *, resolution, ds, R=4.0, fov=40.0, flat_field=0.0,
           density_multiplier=1.0, integration="simple", out=None, stream=None, stats=False,
           volume_path="gather", plain_fp64="auto"):
    """Render the views given by ``angles`` ((azimuthal, polar) degrees).

    Host path (default): returns a float32 numpy array [views, res, res];
    ``out`` may be a preallocated (ideally pinned) host array.  Device path:
    pass ``out`` as a contiguous float32 CUDA tensor; the work is queued on
    ``stream`` (default: torch's current stream) and the call returns once it
    is queued.
    With ``stats`` (host path) returns (images, samples, fp64_samples).
    ``volume_path`` picks how a voxel-grid root is read: texture gathers
    (default) or per-tap loads; both give the same results.  ``plain_fp64``
    (general scenes): "list" leaves the samples FP32 cannot decide to one FP64
    pass after the march; "inplace" re-evaluates them inside the march;
    "auto" takes the list for calls of at least 2^22 rays.  Both agree to FP32
    rounding."""
    L = _lib.load()
    cams, n = cameras_from_angles(angles, R, fov)
    o = _opts(resolution, ds, R, flat_field, density_multiplier, integration, stats, volume_path,
              plain_fp64)
    if out is not None and _is_torch_cuda(out):
        import torch
        if out.dtype != torch.float32 or not out.is_contiguous() or out.numel() < n * resolution ** 2:
            raise ValueError("out must be a contiguous float32 CUDA tensor of views*res*res")
        st = stream if stream is not None else torch.cuda.current_stream(out.device)
        check(L.xrp_render_device(scene.handle, cams, n, ctypes.byref(o),
                                  ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(st.cuda_stream)),
              "xrp_render_device")
        return out
    if out is None:
        out = np.empty((n, resolution, resolution), dtype=np.float32)
    ptr = out.data_ptr() if hasattr(out, "data_ptr") else out.ctypes.data
    check(L.xrp_render(scene.handle, cams, n, ctypes.byref(o), ctypes.c_void_p(ptr)), "xrp_render")
    if stats:
        s = ctypes.c_uint64()
        f = ctypes.c_uint64()
        L.xrp_last_stats(ctypes.byref(s), ctypes.byref(f))
        return out, s.value, f.value
    return out


def voxelize_scene(scene: Scene, res, density_multiplier=1.0):
    """Volume export of a scene (xrp_voxelize_scene): (float32 densities
    [res][res][res] in [k][i][j] order, uint8 export bytes)."""
    L = _lib.load()
    f = np.empty((res, res, res), dtype=np.float32)
    u = np.empty((res, res, res), dtype=np.uint8)
    check(L.xrp_voxelize_scene(scene.handle, int(res), float(density_multiplier), f.ctypes.data,
                               u.ctypes.data), "xrp_voxelize_scene")
    return f, u


def finish_images(images, transparency=False, stream=None):
    """Device-side image finishing (xrp_finish_images) of a float32 CUDA
    tensor [views, res, res]: returns (gray uint16-as-int16 tensor
    [views, res, res] in PNG order, alpha, minmax [views, 2])."""
    import torch
    if not _is_torch_cuda(images) or images.dtype != torch.float32 or not images.is_contiguous():
        raise ValueError("images must be a contiguous float32 CUDA tensor [views, res, res]")
    n, res = images.shape[0], images.shape[-1]
    gray = torch.empty((n, res, res), dtype=torch.int16, device=images.device)
    alpha = torch.empty((n, res, res), dtype=torch.int16, device=images.device)
    mm = torch.empty((n, 2), dtype=torch.float32, device=images.device)
    st = stream if stream is not None else torch.cuda.current_stream(images.device)
    check(_lib.load().xrp_finish_images(ctypes.c_void_p(images.data_ptr()), n, res,
                                        1 if transparency else 0, ctypes.c_void_p(gray.data_ptr()),
                                        ctypes.c_void_p(alpha.data_ptr()), ctypes.c_void_p(mm.data_ptr()),
                                        ctypes.c_void_p(st.cuda_stream)), "xrp_finish_images")
    return gray, alpha, mm


class Batch:
    """Many scenes rendered in one persistent, autotuned launch captured in a
    CUDA graph (xrp_batch_create).  ``items``: (scene, angles, resolution)
    triples; every item shares ds, R, fov and the other options.  ``trace``:
    True for certificate tracing (ray bounds when every scene's chain is
    affine), "ball" for ball certificates only."""

    def __init__(self, items, *, ds, R=4.0, fov=40.0, flat_field=0.0, density_multiplier=1.0,
                 integration="simple", autotune=True, trace=False):
        L = _lib.load()
        self._keep = []
        arr = (_lib.XrpBatchItem * len(items))()
        self.shapes = []
        for k, (scene, angles, res) in enumerate(items):
            cams, n = cameras_from_angles(angles, R, fov)
            self._keep.append((scene, cams))
            arr[k] = _lib.XrpBatchItem(scene.handle, ctypes.cast(cams, ctypes.c_void_p), n, int(res))
            self.shapes.append((n, int(res), int(res)))
        o = _opts(items[0][2], ds, R, flat_field, density_multiplier, integration, False)
        if trace:
            o.flags |= _lib.XRP_FLAG_TRACE
            if trace == "ball":
                o.flags |= _lib.XRP_FLAG_BALL
        h = ctypes.c_void_p()
        check(L.xrp_batch_create(arr, len(items), ctypes.byref(o), 1 if autotune else 0,
                                 ctypes.byref(h)), "xrp_batch_create")
        self._h = h

    def render(self, stream=None):
        """Queue one replay of the captured launch (torch stream or None)."""
        st = ctypes.c_void_p(stream.cuda_stream) if stream is not None else None
        check(_lib.load().xrp_batch_render(self._h, st), "xrp_batch_render")

    def item(self, k) -> np.ndarray:
        out = np.empty(self.shapes[k], dtype=np.float32)
        check(_lib.load().xrp_batch_copy_item(self._h, k, out.ctypes.data), "xrp_batch_copy_item")
        return out

    def info(self) -> dict:
        i = _lib.XrpBatchInfo()
        check(_lib.load().xrp_batch_get_info(self._h, ctypes.byref(i)), "xrp_batch_get_info")
        d = {k: getattr(i, k) for k, _ in i._fields_}
        d["tune_ms"] = list(i.tune_ms)[: i.tune_candidates]
        return d

    def close(self):
        if getattr(self, "_h", None):
            _lib.load().xrp_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


PROPOSAL_STATS = ("segments", "certified", "refined", "dense", "dense_samples", "evaluations",
                  "fp64_samples", "mlp_rounds", "routed_dense", "subdivided", "fp64_list_overflow")


class Proposal:
    """The learned proposal of a scene, trained on the GPU (xrp_proposal_train)
    on the cameras given by ``angles`` and the render options."""

    def __init__(self, scene: Scene, angles, *, resolution, ds, R=4.0, fov=40.0, segment=64,
                 train_rays=65536, val_rays=32768, steps=2000, batch=4096, lr=2e-3,
                 pos_weight=8.0, tau_margin=0.0, seed=0):
        L = _lib.load()
        cams, n = cameras_from_angles(angles, R, fov)
        o = _opts(resolution, ds, R, 0.0, 1.0, "simple", False)
        po = _lib.XrpProposalOpts(int(segment), int(train_rays), int(val_rays), int(steps),
                                  int(batch), float(lr), float(pos_weight), float(tau_margin),
                                  int(seed))
        h = ctypes.c_void_p()
        check(L.xrp_proposal_train(scene.handle, cams, n, ctypes.byref(o), ctypes.byref(po),
                                   ctypes.byref(h)), "xrp_proposal_train")
        self._h = h

    @property
    def handle(self):
        return self._h

    def info(self) -> dict:
        i = _lib.XrpProposalInfo()
        check(_lib.load().xrp_proposal_get_info(self._h, ctypes.byref(i)), "xrp_proposal_get_info")
        return {k: getattr(i, k) for k, _ in i._fields_}

    def params(self) -> np.ndarray:
        L = _lib.load()
        n = L.xrp_mlp_param_count()
        out = np.empty(n, dtype=np.float32)
        check(L.xrp_proposal_params(self._h, out.ctypes.data, n), "xrp_proposal_params")
        return out

    def set_tau(self, tau: float):
        check(_lib.load().xrp_proposal_set_tau(self._h, float(tau)), "xrp_proposal_set_tau")

    def close(self):
        if getattr(self, "_h", None):
            _lib.load().xrp_proposal_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def render_proposal(scene: Scene, proposal: Proposal | None, angles, *, resolution, ds, R=4.0,
                    fov=40.0, flat_field=0.0, density_multiplier=1.0, segment=0, refine=True,
                    trace=False, integration="simple", out=None, stream=None, stats=False):
    """Render with the proposal march (xrp_render_proposal).  ``proposal``
    None: no network (every candidate refined, or integrated densely with
    ``refine=False``; ``trace=True``: per-ray certificate tracing, either
    ``integration``, with ray bounds where the deformation chain is affine
    (``trace="ball"``: ball certificates only); the segment march needs
    "simple").  Host path
    returns a float32 array [views, res, res]; a contiguous float32 CUDA
    tensor as ``out`` selects the device path (the call then waits for the
    stream).  With ``stats`` either path returns (images, dict)."""
    L = _lib.load()
    cams, n = cameras_from_angles(angles, R, fov)
    o = _opts(resolution, ds, R, flat_field, density_multiplier, integration, stats)
    if not refine:
        o.flags |= _lib.XRP_FLAG_NO_REFINE
    if trace:
        o.flags |= _lib.XRP_FLAG_TRACE
        if trace == "ball":
            o.flags |= _lib.XRP_FLAG_BALL
    ph = proposal.handle if proposal is not None else None
    if out is not None and _is_torch_cuda(out):
        import torch
        if out.dtype != torch.float32 or not out.is_contiguous() or out.numel() < n * resolution ** 2:
            raise ValueError("out must be a contiguous float32 CUDA tensor of views*res*res")
        st = stream if stream is not None else torch.cuda.current_stream(out.device)
        check(L.xrp_render_proposal_device(scene.handle, ph, int(segment), cams, n, ctypes.byref(o),
                                           ctypes.c_void_p(out.data_ptr()),
                                           ctypes.c_void_p(st.cuda_stream)),
              "xrp_render_proposal_device")
        if stats:
            c = (ctypes.c_uint64 * 11)()
            L.xrp_proposal_last_stats(c)
            return out, dict(zip(PROPOSAL_STATS, list(c)))
        return out
    if out is None:
        out = np.empty((n, resolution, resolution), dtype=np.float32)
    ptr = out.data_ptr() if hasattr(out, "data_ptr") else out.ctypes.data
    check(L.xrp_render_proposal(scene.handle, ph, int(segment), cams, n, ctypes.byref(o),
                                ctypes.c_void_p(ptr)), "xrp_render_proposal")
    if stats:
        c = (ctypes.c_uint64 * 11)()
        L.xrp_proposal_last_stats(c)
        return out, dict(zip(PROPOSAL_STATS, list(c)))
    return out


def mlp_grad(params, X_bf16_bits, y, pos_weight=1.0):
    """The GPU training step's gradient (xrp_mlp_grad): returns
    (grad [N] float32, loss, logits [rows])."""
    L = _lib.load()
    params = np.ascontiguousarray(params, dtype=np.float32)
    X = np.ascontiguousarray(X_bf16_bits, dtype=np.uint16)
    y = np.ascontiguousarray(y, dtype=np.float32)
    rows = X.shape[0]
    grad = np.zeros_like(params)
    loss = ctypes.c_float()
    logits = np.zeros(rows, dtype=np.float32)
    check(L.xrp_mlp_grad(params.ctypes.data, X.ctypes.data, y.ctypes.data, rows, float(pos_weight),
                         grad.ctypes.data, ctypes.byref(loss), logits.ctypes.data), "xrp_mlp_grad")
    return grad, float(loss.value), logits


def xray_camera_params(angles, R=4.0, fov=40.0) -> np.ndarray:
    """The float32 XRayCameraParams rows the reference Go glue builds
    (cuda_path.go:61-77): eye, row-major camera-to-world, fov, R; shape [n,21]."""
    eyes, mats = camera_arrays(angles, R, fov)
    rows = np.zeros((len(eyes), 21), dtype=np.float32)
    rows[:, 0:3] = eyes
    rows[:, 3:19] = mats.reshape(-1, 4, 4).transpose(0, 2, 1).reshape(-1, 16)
    rows[:, 19] = fov
    rows[:, 20] = R
    return rows


def render_volume_projections(volume, cams21, image_res, ds, flat_field=0.0, out=None):
    """RenderVolumeProjectionsCUDA (cuda_backend.h:101-112) on host buffers:
    ``volume`` float32 [nz][nx][ny], ``cams21`` float32 [n,21]."""
    L = _lib.load()
    vol = np.ascontiguousarray(volume, dtype=np.float32)
    nz, nx, ny = vol.shape
    c = np.ascontiguousarray(cams21, dtype=np.float32).reshape(-1, 21)
    n = c.shape[0]
    if out is None:
        out = np.empty((n, image_res, image_res), dtype=np.float32)
    ptr = out.data_ptr() if hasattr(out, "data_ptr") else out.ctypes.data
    check(L.RenderVolumeProjectionsCUDA(vol.ctypes.data, nx, ny, nz, c.ctypes.data, n,
                                        int(image_res), ctypes.c_float(ds),
                                        ctypes.c_float(flat_field), ctypes.c_void_p(ptr)),
          "RenderVolumeProjectionsCUDA")
    return out


def assemble_voxel_grid(cylinders, res, density_multiplier=1.0):
    """AssembleVoxelGridCUDA (cuda_backend.h:33-39); cylinders: float32 [n, 8]
    rows (p0, p1, radius, rho).  Returns float32 [res, res, res] ([k][i][j])."""
    L = _lib.load()
    c = np.ascontiguousarray(cylinders, dtype=np.float32).reshape(-1, 8)
    out = np.empty((res, res, res), dtype=np.float32)
    check(L.AssembleVoxelGridCUDA(c.ctypes.data, c.shape[0], int(res),
                                  ctypes.c_float(density_multiplier), out.ctypes.data),
          "AssembleVoxelGridCUDA")
    return out


def release_cache():
    _lib.load().xrp_release_cache()
