"""Volume export of any scene (xrp_voxelize_scene, main.go:549-635) and the
device-side image finishing (xrp_finish_images, main.go:482-506) against
their definitions evaluated on the CPU (FP64 oracle densities; the Go
conversions restated in numpy)."""
import numpy as np
import pytest

from oracle import oracle as O
from xray_projection_render_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def X():
    import __graft_entry__ as g
    g.build()
    import xray_projection_render_gb300 as X
    return X


def _oracle_volume(obj, deformation, res, dm):
    sc = O.Scene(obj, deformation)
    v = np.empty((res, res, res))
    g = np.arange(res) / res * 2.0 - 1.0
    for k in range(res):
        for i in range(res):
            for j in range(res):
                v[k, i, j] = sc.density(g[i], g[j], g[k], dm)
    return v


CASES = {
    "cube_minus_sphere_cylinder": lambda: W.cube_minus_sphere_cylinder(8),
    "deformed_lattice": W.deformed_lattice,
    "gyroid_sigmoid": W.gyroid_sigmoid,
    "batched_scene0": lambda: W.batched_scenes(1)[0],
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_voxelize_scene_matches_oracle(X, name):
    w = CASES[name]()
    res, dm = 20, 1.3
    ref = _oracle_volume(w.obj, w.deformation, res, dm)
    with X.Scene(w.obj, w.deformation) as s:
        f, u = X.voxelize_scene(s, res, dm)
    assert np.array_equal(f, ref.astype(np.float32))
    mx = ref.max()
    t = ref / mx * 255.0 if mx > 0 else np.zeros_like(ref)
    want = np.clip(np.floor(np.maximum(t, 0.0)), 0, 255).astype(np.uint8)
    assert np.array_equal(u, want)


@pytest.mark.parametrize("res,offset", [(45, 0), (100, 0), (64, 0), (64, 1)],
                         ids=["odd_side", "side_4k", "side_64", "misaligned"])
def test_finish_images(X, res, offset):
    """Odd sides and misaligned buffers take the scalar kernel, sides that
    are multiples of 4 with aligned buffers the vectorised one."""
    import torch
    rng = np.random.default_rng(3)
    n = 3
    img = rng.uniform(0.0, 1.0, (n, res, res)).astype(np.float32)
    img[0, 3, 4] = 1.0
    img[1, 0, 0] = 0.0
    img[2, res - 1, res - 1] = np.float32(1.0) - np.float32(2.0 ** -24)
    img[2, 5, res - 2] = np.float32(3.0) / np.float32(65535.0)  # near a whole quantum
    flat = torch.zeros(n * res * res + offset, device="cuda")
    flat[offset:] = torch.from_numpy(img.reshape(-1)).cuda()
    d = flat[offset:].view(n, res, res)
    for transparency in (False, True):
        gray, alpha, mm = X.finish_images(d, transparency=transparency)
        torch.cuda.synchronize()
        gray = gray.cpu().numpy().view(np.uint16)
        alpha = alpha.cpu().numpy().view(np.uint16)
        mm = mm.cpu().numpy()
        want = np.zeros((n, res, res), np.uint16)
        want_a = np.zeros((n, res, res), np.uint16)
        for v in range(n):
            for i in range(res):
                for j in range(res):
                    val = float(img[v, i, j])
                    want[v, res - j - 1, i] = int(val * 0xffff)
                    want_a[v, res - j - 1, i] = (0xffff if val < 1.0 else 0) if transparency else 0xffff
        assert np.array_equal(gray, want)
        assert np.array_equal(alpha, want_a)
        assert np.array_equal(mm[:, 0], img.reshape(n, -1).min(1))
        assert np.array_equal(mm[:, 1], img.reshape(n, -1).max(1))
