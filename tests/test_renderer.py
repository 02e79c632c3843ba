"""The drop-in front end for the reference's Python API (XRayRenderer.render,
xray_projection_render/xray_renderer.py:357-448, and RenderProjections,
api.go:75-177): the reference's own example files go in, PNGs,
transforms.json, object.json and volume.raw come out, and their pixels
match the FP64 oracle's transmittances.

CPU tests cover the file-format pieces (YAML subset, Go-style JSON, PNG
encoding, angle generation, argument errors); the GPU tests render."""
import json
import math
import os
import struct
import zlib

import numpy as np
import pytest

from oracle import oracle as O
from xray_projection_render_gb300 import renderer as RR
from xray_projection_render_gb300 import yaml_subset

EX = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "examples")


def read_png(path):
    """(pixels [h][w][channels] uint8) of an 8-bit PNG without filters."""
    data = open(path, "rb").read()
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, idat, hdr = 8, b"", None
    while pos < len(data):
        n = struct.unpack(">I", data[pos:pos + 4])[0]
        tag, body = data[pos + 4:pos + 8], data[pos + 8:pos + 8 + n]
        assert zlib.crc32(tag + body) & 0xFFFFFFFF == struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])[0]
        if tag == b"IHDR":
            hdr = struct.unpack(">IIBBBBB", body)
        elif tag == b"IDAT":
            idat += body
        pos += 12 + n
    w, h, depth, ctype = hdr[0], hdr[1], hdr[2], hdr[3]
    assert depth == 8
    ch = {2: 3, 6: 4}[ctype]
    raw = np.frombuffer(zlib.decompress(idat), dtype=np.uint8).reshape(h, 1 + w * ch)
    assert np.all(raw[:, 0] == 0)
    return raw[:, 1:].reshape(h, w, ch)


def expected_gray8(T):
    """main.go:482-501: uint16(val * 0xffff) stored in an 8-bit RGBA image
    (the high byte), pixel (i, res-1-j) -> row-major [y][x]."""
    g16 = np.floor(np.asarray(T, dtype=np.float64) * 65535.0).astype(np.uint16)
    g8 = (g16 >> 8).astype(np.uint8)  # [i][j]
    return g8.T[::-1, :]  # [y = res-1-j][x = i]


# --- CPU ------------------------------------------------------------------

def test_yaml_subset_reads_the_reference_examples():
    d = yaml_subset.loads(open(os.path.join(EX, "cube_w_hole.yaml")).read())
    assert d == {"type": "object_collection", "objects": [
        {"type": "cube", "side": 1.5, "center": [0.0, 0.0, 0.0], "rho": 0.7},
        {"type": "sphere", "radius": 0.3, "center": [0.1, 0.2, 0.0], "rho": -1.0},
        {"type": "cylinder", "radius": 0.3, "p0": [0.1, 0.2, 0.0], "p1": [0.1, 0.2, 0.8], "rho": -1.0}]}
    g = yaml_subset.loads(open(os.path.join(EX, "gyroid_example.yaml")).read())
    assert g["uc"]["objects"]["objects"][0]["scale"] == 0.1 and g["xmin"] == -0.8
    assert yaml_subset.loads(open(os.path.join(EX, "deformation_sigmoid.yaml")).read()) == {
        "amplitude": 0.2, "lengthscale": 0.2, "center": 0.0, "direction": "z", "type": "sigmoid"}
    # sequences at their key's indentation, nested sequences, comments, quotes
    t = "a:\n- 1\n- - 2\n  - 3\nb: {x: [1, 2], y: 'q # r'}  # c\nc: \"s\"\nd: ~\n"
    assert yaml_subset.loads(t) == {"a": [1, [2, 3]], "b": {"x": [1, 2], "y": "q # r"}, "c": "s",
                                    "d": None}
    with pytest.raises(ValueError):
        yaml_subset.loads("a: &anchor 1\n")


def test_go_json_floats_and_layout():
    assert [RR._go_float(v) for v in (4.0, 0.5, 1e-7, 1e-6, 3e-5, 1e21, -0.0)] == \
        ["4", "0.5", "1e-7", "0.000001", "0.00003", "1e+21", "-0"]
    assert RR._go_json({"a": [1.0, 2], "b": {}, "c": "x"}) == \
        '{\n  "a": [\n    1,\n    2\n  ],\n  "b": {},\n  "c": "x"\n}'


def test_png_round_trip(tmp_path):
    rng = np.random.default_rng(0)
    g = rng.integers(0, 256, (7, 9), dtype=np.uint8)
    RR.write_png(str(tmp_path / "a.png"), g, np.full_like(g, 0xFF))
    px = read_png(str(tmp_path / "a.png"))
    assert px.shape == (7, 9, 3) and np.array_equal(px[:, :, 1], g)
    a = np.where(g > 128, 0xFF, 0).astype(np.uint8)
    RR.write_png(str(tmp_path / "b.png"), g, a)
    px = read_png(str(tmp_path / "b.png"))
    assert px.shape == (7, 9, 4)
    assert np.array_equal(px[:, :, 3], a) and np.all(px[a == 0] == 0)
    assert np.array_equal(px[:, :, 0][a == 0xFF], g[a == 0xFF])


def test_camera_angles_follow_the_reference_rule():
    assert RR.generate_camera_angles(12, 1, 3, False, 70.0) == \
        [(a, 70.0) for a, _ in O.generate_camera_angles(12, 1, 3, 70.0)]
    out = RR.generate_camera_angles(50, 0, 1, True, 90.0, rng=np.random.default_rng(1))
    assert all(0.0 <= p <= 180.0 for _, p in out) and len({p for _, p in out}) == 50


def test_argument_errors_are_reported_like_the_reference(tmp_path):
    r = RR.render_projections(dict(RR.DEFAULTS, input="x.json", ds=0))
    assert r == {"success": False,
                 "error": "ds is 0; use a negative value for automatic step-size selection"}
    r = RR.render_projections(dict(RR.DEFAULTS, input="x.json", density_multiplier=0))
    assert not r["success"] and r["error"].startswith("density_multiplier is 0")
    with pytest.raises(ValueError):
        RR.XRayRenderer.render(object.__new__(RR.XRayRenderer), {})
    r = RR.render_projections(dict(RR.DEFAULTS, input=str(tmp_path / "missing.json")))
    assert not r["success"] and r["error"].startswith("render failed:")


def test_to_map_sorts_like_go():
    m = RR.to_map(json.load(open(os.path.join(EX, "pillar_array.json"))))
    assert list(m) == ["type", "uc", "xmax", "xmin", "ymax", "ymin", "zmax", "zmin"]
    assert list(m["uc"]) == ["objects", "type", "xmax", "xmin", "ymax", "ymin", "zmax", "zmin"]
    assert m["uc"]["objects"]["objects"][0] == {"p0": [0.25, 0.25, 0.75], "p1": [0.25, 0.25, -0.75],
                                               "radius": 0.1, "rho": 1.0, "type": "cylinder"}


# --- GPU ------------------------------------------------------------------

@pytest.fixture(scope="module")
def gpu():
    import torch
    torch.cuda.set_device(0)
    import __graft_entry__ as g
    g.build()
    return RR.XRayRenderer()


def _check_images(out_dir, obj, deform, angles, res, ds, integration, transparency=False, **kw):
    T = O.render(O.Scene(obj, deform), angles, res, ds, integration=integration, **kw)
    for k in range(len(angles)):
        px = read_png(os.path.join(out_dir, f"image_{k:03d}.png"))
        want = expected_gray8(T[k])
        got = px[:, :, 0]
        if transparency:
            alpha = (T[k].T[::-1, :] < 1.0)
            if px.shape[2] == 3:  # every pixel opaque: Go's encoder writes RGB
                assert np.all(alpha)
            else:
                assert np.array_equal(px[:, :, 3] == 0xFF, alpha)
            want = np.where(alpha, want, 0)
        d = np.abs(got.astype(int) - want.astype(int))
        # FP32 transmittance: the quantised byte may differ by one where
        # T * 0xffff lands within 1e-5 of a multiple of 256
        assert d.max() <= 1 and np.count_nonzero(d) <= max(2, d.size // 2000), (k, d.max())
    return T


@pytest.mark.gpu
@pytest.mark.parametrize("integration", ["simple", "hierarchical"])
def test_balls_json_through_the_front_end(gpu, tmp_path, integration):
    out_dir = str(tmp_path / "images")
    angles = [{"azimuthal": 0.0, "polar": 90.0}, {"azimuthal": 45.0, "polar": 60.0}]
    params = {"input": os.path.join(EX, "balls.json"), "output_dir": out_dir, "resolution": 64,
              "ds": 0.01, "integration": integration,
              "transforms_file": str(tmp_path / "transforms.json")}
    r = gpu.render(params, camera_angles=angles)
    assert r == {"success": True, "num_images": 1, "output_dir": out_dir}
    obj = json.load(open(os.path.join(EX, "balls.json")))
    _check_images(out_dir, obj, None, [(0.0, 90.0), (45.0, 60.0)], 64, 0.01, integration)
    tp = json.load(open(tmp_path / "transforms.json"))
    f = 1.0 / math.tan(math.radians(20.0))
    assert tp["w"] == tp["h"] == 64 and tp["cx"] == 32 and tp["flat_field"] == 1.0
    assert tp["fl_x"] == pytest.approx(f * 32, rel=1e-15) and tp["camera_angle_x"] == pytest.approx(
        40 * math.pi / 180, rel=1e-15)
    assert [fr["file_path"] for fr in tp["frames"]] == ["images/image_000.png", "images/image_001.png"]
    _, cam = O.camera_from_angles(45.0, 60.0, 4.0)
    assert np.array_equal(np.array(tp["frames"][1]["transform_matrix"]), cam.reshape(4, 4).T)
    assert json.load(open(tmp_path / "object.json"))["objects"][1]["center"] == [0.5, 0.5, 0.0]


@pytest.mark.gpu
def test_yaml_scene_deformation_auto_step_transparency_and_volume(gpu, tmp_path):
    out_dir = str(tmp_path / "out" / "images")
    params = {"input": os.path.join(EX, "cube_w_hole.yaml"),
              "deformation_file": os.path.join(EX, "deformation_sigmoid.yaml"),
              "output_dir": out_dir, "resolution": 48, "num_images": 3, "ds": -1.0,
              "transparency": True, "export_volume": True, "flat_field": 0.0,
              "density_multiplier": 1.5, "transforms_file": str(tmp_path / "t.json")}
    r = gpu.render(params)
    assert r["success"], r
    obj = yaml_subset.loads(open(os.path.join(EX, "cube_w_hole.yaml")).read())
    deform = yaml_subset.loads(open(os.path.join(EX, "deformation_sigmoid.yaml")).read())
    ds = O.Scene(obj).min_feature_size() / 5.0
    angles = O.generate_camera_angles(3)
    _check_images(out_dir, obj, deform, angles, 48, ds, "hierarchical", transparency=True,
                  density_multiplier=1.5)
    assert read_png(os.path.join(out_dir, "image_000.png")).shape[2] == 4  # T = 1 outside: RGBA
    vol = np.fromfile(str(tmp_path / "out" / "volume.raw"), dtype=np.uint8).reshape(48, 48, 48)
    sc = O.Scene(obj, deform)
    x = np.arange(48) / 48 * 2 - 1
    for (k, i, j) in [(24, 10, 30), (5, 40, 2), (30, 24, 24), (47, 0, 47)]:
        d = sc.density(x[i], x[j], x[k], 1.5)
        assert d == 0 or vol[k, i, j] > 0
    assert vol.max() == 255


@pytest.mark.gpu
def test_tessellated_json_and_failures(gpu, tmp_path):
    out_dir = str(tmp_path / "img")
    r = gpu.render({"input": os.path.join(EX, "pillar_array.json"), "output_dir": out_dir,
                    "resolution": 40, "ds": 0.01, "integration": "simple",
                    "transforms_file": str(tmp_path / "t.json"),
                    "camera_angles": [{"Azimuthal": 30.0, "Polar": 80.0}]})
    assert r["success"], r
    obj = json.load(open(os.path.join(EX, "pillar_array.json")))
    _check_images(out_dir, obj, None, [(30.0, 80.0)], 40, 0.01, "simple")
    bad = tmp_path / "bad.json"
    bad.write_text(json.dumps({"type": "torus"}))
    r = gpu.render({"input": str(bad), "output_dir": out_dir, "transforms_file": str(tmp_path / "u.json")})
    assert not r["success"] and "render failed" in r["error"]
