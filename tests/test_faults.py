"""Error paths of the reference ABI, driven by host-side fault injection.

RenderVolumeProjectionsCUDA keeps the reference's return codes
(cuda_backend.cu:95-201): 3 device allocation, 4 volume upload, 5 table
upload, 6 output allocation, 7 kernel launch, 8 copy back.  XRP_FAULT makes
the named site report the CUDA error it would see, on the host, before any
device work is queued there -- no GPU operation actually fails -- and the
engine must return the code, name the site in xrp_last_error(), leave no
partial state behind and render correctly on the next call."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

SITES = [("alloc", 3, b"volume allocation"), ("upload", 4, b"volume upload"),
         ("tables", 5, b"table upload"), ("output", 6, b"image buffer allocation"),
         ("launch", 7, b"kernel launch"), ("copy", 8, b"image copy")]


@pytest.fixture(scope="module")
def env():
    import torch
    torch.cuda.set_device(0)
    import __graft_entry__ as g
    g.build()
    import xray_projection_render_gb300 as X
    from xray_projection_render_gb300 import _lib, workloads
    vol = workloads.gaussian_blob_volume(24, 5, seed=7)
    cams = X.xray_camera_params([(0.0, 90.0), (50.0, 70.0)], 4.0, 40.0)
    ref = O.render_volume_abi(vol, cams, 32, 0.02)
    return X, _lib, vol, cams, ref


@pytest.mark.parametrize("site,code,msg", SITES, ids=[s[0] for s in SITES])
def test_injected_fault_returns_the_reference_code(env, monkeypatch, site, code, msg):
    X, L, vol, cams, ref = env
    monkeypatch.setenv("XRP_FAULT", site)
    with pytest.raises(L.EngineError) as ei:
        X.render_volume_projections(vol, cams, 32, 0.02)
    assert ei.value.code == code
    assert msg in L.load().xrp_last_error()
    monkeypatch.delenv("XRP_FAULT")
    got = X.render_volume_projections(vol, cams, 32, 0.02)  # the engine is still usable
    assert np.max(np.abs(got - ref) / ref) <= 1e-5


def test_fault_list_and_scene_path(env, monkeypatch):
    X, L, vol, cams, ref = env
    monkeypatch.setenv("XRP_FAULT", "upload,launch")
    with pytest.raises(L.EngineError) as ei:
        X.render_volume_projections(vol, cams, 32, 0.02)
    assert ei.value.code == 4
    # the scene entry points share the render path: a launch fault is code 7
    with X.Scene({"type": "sphere", "center": [0.0, 0.0, 0.0], "radius": 0.5, "rho": 1.0}) as s:
        with pytest.raises(L.EngineError) as ei:
            X.render(s, [(0.0, 90.0)], resolution=16, ds=0.01)
        assert ei.value.code == 7
        monkeypatch.setenv("XRP_FAULT", "")
        img = X.render(s, [(0.0, 90.0)], resolution=16, ds=0.01)
    assert np.all(np.isfinite(img)) and img.min() < 1.0
