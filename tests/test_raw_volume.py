"""Voxel grids loaded from .raw files inside the library (VoxelGridFromRaw,
objects/objects.go:892-958, and the voxel_grid map, objects.go:715-760):
every data type, the (N-1) lattice and [z][x][y] layout, and the loader's
errors, against the FP64 oracle."""
import json

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

NX, NY, NZ = 12, 10, 9
SCALE = {"uint8": 255.0, "uint16": 65535.0, "uint32": 4294967295.0}


@pytest.fixture(scope="module")
def X():
    import torch
    torch.cuda.set_device(0)
    import __graft_entry__ as g
    g.build()
    import xray_projection_render_gb300 as X
    return X


def _values(dtype, rng):
    if dtype in SCALE:
        top = {"uint8": 255, "uint16": 65535, "uint32": 4294967295}[dtype]
        raw = rng.integers(0, top, NX * NY * NZ, dtype=np.uint64, endpoint=True).astype(dtype)
        return raw, raw.astype(np.float64) / SCALE[dtype]
    raw = rng.uniform(0.0, 1.5, NX * NY * NZ).astype(dtype)
    return raw, raw.astype(np.float64)


@pytest.mark.parametrize("dtype", ["uint8", "uint16", "uint32", "float32", "float64"])
def test_raw_grid_matches_oracle(X, tmp_path, dtype):
    rng = np.random.default_rng(3)
    raw, vals = _values(dtype, rng)
    path = tmp_path / f"grid_{dtype}.raw"
    raw.astype("<" + raw.dtype.str[1:]).tofile(path)
    obj = {"type": "voxel_grid", "path": str(path), "resolution": [NX, NY, NZ], "dtype": dtype}
    angles = [(0.0, 90.0), (33.0, 70.0), (200.0, 120.0)]
    with X.Scene(json.dumps(obj)) as s:
        got = X.render(s, angles, resolution=40, ds=0.01)
    vol = vals.reshape(NZ, NX, NY)  # [z][x][y] (objects.go:837)
    ref = O.render(O.Scene({"type": "voxel_grid", "_voxels": vol}), angles, 40, 0.01)
    assert np.max(np.abs(got - ref) / ref) <= 1e-5


def test_raw_default_dtype_is_uint8(X, tmp_path):
    raw = np.arange(NX * NY * NZ, dtype=np.uint64).astype(np.uint8)
    path = tmp_path / "g.raw"
    raw.tofile(path)
    with X.Scene({"type": "voxel_grid", "path": str(path), "resolution": [NX, NY, NZ]}) as s:
        got = X.render(s, [(10.0, 80.0)], resolution=24, ds=0.01)
    vol = (raw.astype(np.float64) / 255.0).reshape(NZ, NX, NY)
    ref = O.render(O.Scene({"type": "voxel_grid", "_voxels": vol}), [(10.0, 80.0)], 24, 0.01)
    assert np.max(np.abs(got - ref) / ref) <= 1e-5


@pytest.mark.parametrize("obj,msg", [
    ({"path": "g.raw", "resolution": [NX, NY, NZ + 1]}, b"does not match expected size"),
    ({"path": "g.bin", "resolution": [NX, NY, NZ]}, b"only raw files are supported"),
    ({"path": "g.raw"}, b"resolution must be provided"),
    ({"path": "g.raw", "resolution": [NX, NY]}, b"resolution must be a list of 3 integers"),
    ({"path": "g.raw", "resolution": [NX, NY, NZ], "dtype": "int8"}, b"unsupported data type"),
    ({"path": "missing.raw", "resolution": [NX, NY, NZ]}, b"error reading file"),
])
def test_raw_loader_errors(X, tmp_path, obj, msg):
    from xray_projection_render_gb300 import _lib
    np.zeros(NX * NY * NZ, dtype=np.uint8).tofile(tmp_path / "g.raw")
    np.zeros(NX * NY * NZ, dtype=np.uint8).tofile(tmp_path / "g.bin")
    o = dict(obj, type="voxel_grid", path=str(tmp_path / obj["path"]))
    with pytest.raises(_lib.EngineError) as ei:
        X.Scene(o)
    assert ei.value.code == 2
    assert msg in _lib.load().xrp_last_error()
