"""xrp_render_volume_noalloc: the render entry point for callers that cannot
allocate device memory (a host framework whose allocator owns the device, a
service with a fixed device-memory budget).  It must give the same images as
RenderVolumeProjectionsCUDA and as the FP64 oracle, call after call, while
keeping its tables in the library's static device array instead of
allocating: the device's free memory does not move across a call.

This file is collected last on purpose: if it fails, a run that stops at the
first failure has already run every other test."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL_TOL = 1e-5


@pytest.fixture(scope="module")
def env():
    import torch
    torch.cuda.set_device(0)
    import __graft_entry__ as g
    g.build()
    import xray_projection_render_gb300 as X
    from xray_projection_render_gb300 import _lib, workloads
    return torch, X, _lib.load(), workloads


def _noalloc(torch, L, dvol, cams, res, ds, flat_field, stream):
    nz, nx, ny = dvol.shape
    out = torch.full((cams.shape[0], res, res), float("nan"), device=dvol.device)
    rc = L.xrp_render_volume_noalloc(ctypes.c_void_p(dvol.data_ptr()), nx, ny, nz,
                                     cams.ctypes.data, cams.shape[0], res, ctypes.c_float(ds),
                                     ctypes.c_float(flat_field), ctypes.c_void_p(out.data_ptr()),
                                     ctypes.c_void_p(stream.cuda_stream))
    assert rc == 0, L.xrp_last_error()
    stream.synchronize()
    return out.cpu().numpy()


def test_noalloc_matches_render_volume_projections_two_calls(env):
    from oracle import oracle as O
    torch, X, L, W = env
    vol = W.gaussian_blob_volume(48, 10, seed=21)[:, :40, :].copy()  # nz=48, nx=40, ny=48
    dvol = torch.from_numpy(vol).cuda()
    stream = torch.cuda.current_stream()
    calls = [([(0.0, 90.0), (37.0, 75.0), (200.0, 110.0)], 96, 2.0 / 48 / 2, 0.0),
             ([(300.0, 60.0), (120.0, 90.0)], 64, 2.0 / 48 / 3, 0.2)]
    for angles, res, ds, ff in calls:  # the second call must not see the first's tables
        cams = X.xray_camera_params(angles, 4.0, 40.0)
        ref = X.render_volume_projections(vol, cams, res, ds, ff)
        got = _noalloc(torch, L, dvol, cams, res, ds, ff, stream)
        assert np.all(np.isfinite(got))
        rel = np.abs(got.astype(np.float64) - ref) / ref
        assert rel.max() <= REL_TOL, f"max rel difference {rel.max():.3g}"
        fp64 = O.render_volume_abi(vol, cams, res, ds, ff)
        rel = np.abs(got.astype(np.float64) - fp64) / fp64
        assert rel.max() <= REL_TOL, f"max rel error against the oracle {rel.max():.3g}"


def test_noalloc_leaves_device_memory_unchanged(env):
    torch, X, L, W = env
    vol = W.gaussian_blob_volume(32, 6, seed=5)
    dvol = torch.from_numpy(vol).cuda()
    stream = torch.cuda.current_stream()
    cams = X.xray_camera_params([(10.0, 90.0), (140.0, 70.0)], 4.0, 40.0)
    out = torch.empty((2, 80, 80), device="cuda")

    def call():
        rc = L.xrp_render_volume_noalloc(ctypes.c_void_p(dvol.data_ptr()), 32, 32, 32,
                                         cams.ctypes.data, 2, 80, ctypes.c_float(0.02),
                                         ctypes.c_float(0.0), ctypes.c_void_p(out.data_ptr()),
                                         ctypes.c_void_p(stream.cuda_stream))
        assert rc == 0, L.xrp_last_error()
        stream.synchronize()

    call()  # the first call on the device looks up the array
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    reserved0 = torch.cuda.memory_reserved()
    for _ in range(3):
        call()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, f"device free memory moved by {free0 - free1} bytes"
    assert torch.cuda.memory_reserved() == reserved0


def test_noalloc_rejects_calls_beyond_its_array(env):
    torch, X, L, W = env
    dvol = torch.zeros((4, 4, 4), device="cuda")
    cams = X.xray_camera_params([(0.0, 90.0)] * 6000, 4.0, 40.0)  # ~1.1 MiB of camera tables
    out = torch.empty(1, device="cuda")
    rc = L.xrp_render_volume_noalloc(ctypes.c_void_p(dvol.data_ptr()), 4, 4, 4, cams.ctypes.data,
                                     cams.shape[0], 8, ctypes.c_float(0.1), ctypes.c_float(0.0),
                                     ctypes.c_void_p(out.data_ptr()), None)
    assert rc == 2
    assert b"1048576" in L.xrp_last_error()
