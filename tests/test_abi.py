"""C-ABI boundary checks that need no GPU: the library loads, exports every
symbol include/xrp.h declares, satisfies the reference Go loader's dlopen/dlsym
sequence (cuda_backend.go:27-43), rejects bad arguments before touching the
device, and computes the same FP64 cameras as the oracle."""
import ctypes
import os
import re

import numpy as np
import pytest

from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    from xray_projection_render_gb300 import build, _lib
    build.build()
    return _lib.load()


def header_symbols():
    text = open(os.path.join(ROOT, "include", "xrp.h")).read()
    return re.findall(r"XRP_API\s+[\w\s\*]+?\b(\w+)\s*\(", text)


def test_header_symbols_all_exported(lib):
    syms = header_symbols()
    assert "RenderVolumeProjectionsCUDA" in syms and len(syms) >= 13
    for s in syms:
        assert hasattr(lib, s), f"{s} not exported"


def test_go_loader_sequence():
    """dlopen(RTLD_LAZY|RTLD_LOCAL) then dlsym of the three reference symbols."""
    from xray_projection_render_gb300 import _lib
    h = ctypes.CDLL(_lib.LIB_PATH, mode=os.RTLD_LAZY | os.RTLD_LOCAL)
    libdl = ctypes.CDLL(None)
    libdl.dlsym.restype = ctypes.c_void_p
    libdl.dlsym.argtypes = [ctypes.c_void_p, ctypes.c_char_p]
    for name in (b"AssembleVoxelGridCUDA", b"AssembleVoxelGridSpatialCUDA",
                 b"RenderVolumeProjectionsCUDA"):
        assert libdl.dlsym(h._handle, name), name
    assert not libdl.dlsym(h._handle, b"render_kernel")  # internals stay hidden


def test_argument_errors_before_device(lib):
    cams = np.zeros((1, 21), np.float32)
    vol = np.zeros((2, 2, 2), np.float32)
    out = np.zeros((1, 4, 4), np.float32)
    f = lib.RenderVolumeProjectionsCUDA
    assert f(None, 2, 2, 2, cams.ctypes.data, 1, 4, ctypes.c_float(0.1), ctypes.c_float(0), out.ctypes.data) == 1
    assert f(vol.ctypes.data, 0, 2, 2, cams.ctypes.data, 1, 4, ctypes.c_float(0.1), ctypes.c_float(0), out.ctypes.data) == 2
    assert f(vol.ctypes.data, 2, 2, 2, cams.ctypes.data, 0, 4, ctypes.c_float(0.1), ctypes.c_float(0), out.ctypes.data) == 2
    assert f(vol.ctypes.data, 2, 2, 2, cams.ctypes.data, 1, 4, ctypes.c_float(-1), ctypes.c_float(0), out.ctypes.data) == 2
    assert f(vol.ctypes.data, 2, 2, 2, cams.ctypes.data, 1, 4, ctypes.c_float(float("nan")), ctypes.c_float(0), out.ctypes.data) == 2
    assert b"ds" in lib.xrp_last_error()
    cyl = np.zeros((1, 8), np.float32)
    assert lib.AssembleVoxelGridCUDA(None, 1, 4, ctypes.c_float(1), out.ctypes.data) == 1
    assert lib.AssembleVoxelGridCUDA(cyl.ctypes.data, 0, 4, ctypes.c_float(1), out.ctypes.data) == 1
    off = np.array([0, 5], np.int32)
    idx = np.array([0], np.int32)
    big = np.zeros(64, np.float32)
    # offsets beyond the index list are rejected on the host
    assert lib.AssembleVoxelGridSpatialCUDA(cyl.ctypes.data, 1, 4, ctypes.c_float(1), 1,
                                            off.ctypes.data, idx.ctypes.data, 1, big.ctypes.data) == 2
    idx_bad = np.array([3], np.int32)
    off_ok = np.array([0, 1], np.int32)
    assert lib.AssembleVoxelGridSpatialCUDA(cyl.ctypes.data, 1, 4, ctypes.c_float(1), 1,
                                            off_ok.ctypes.data, idx_bad.ctypes.data, 1, big.ctypes.data) == 2


def test_cameras_bitwise_equal_to_oracle(lib):
    from xray_projection_render_gb300 import engine
    angles = [(0, 90), (90, 90), (37.25, 61.5), (200, 120), (359.5, 90), (123.4, 30.1)]
    eyes, mats = engine.camera_arrays(angles, 4.0, 40.0)
    for k, (az, pol) in enumerate(angles):
        e, m = O.camera_from_angles(az, pol, 4.0)
        assert np.array_equal(eyes[k], e)
        assert np.array_equal(mats[k], m)


def test_version(lib):
    assert lib.xrp_version() >= 100


def test_python_flag_constants_match_header():
    """The bindings' XRP_FLAG_* / XRP_INTEGRATE_* values are the header's."""
    from xray_projection_render_gb300 import _lib
    hdr = open(os.path.join(ROOT, "include", "xrp.h")).read()
    found = dict(re.findall(r"\b(XRP_(?:FLAG|INTEGRATE)_[A-Z_]+)\s*=\s*(\d+)", hdr))
    assert "XRP_FLAG_BALL" in found and "XRP_FLAG_TRACE" in found
    for name, value in found.items():
        assert getattr(_lib, name) == int(value), name
