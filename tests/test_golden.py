"""Golden fixtures (tests/golden, made by make_golden.py from the FP64
oracle): the oracle reproduces them, and the engine -- its CPU build here,
the GPU kernels under the gpu marker -- matches them within 1e-5 relative."""
import glob
import json
import os
import sys

import numpy as np
import pytest

from oracle import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")
sys.path.insert(0, os.path.join(HERE, "hostsim"))

REL_TOL = 1e-5
SCENES = sorted(glob.glob(os.path.join(GOLD, "scene_*.npz")))
ABI = sorted(glob.glob(os.path.join(GOLD, "*_abi.npz")))


def _load(f):
    z = np.load(f, allow_pickle=False)
    d = {k: z[k] for k in z.files}
    d["obj"] = json.loads(str(d["obj"])) if "obj" in d else None
    dj = str(d.get("deformation", ""))
    d["deformation"] = json.loads(dj) if dj else None
    return d


def _rel(got, ref):
    return float(np.max(np.abs(np.asarray(got, np.float64) - ref) / ref))


def test_fixtures_present():
    assert len(SCENES) == 8 and len(ABI) == 3


@pytest.mark.parametrize("f", SCENES, ids=os.path.basename)
def test_oracle_reproduces_scene_fixture(f):
    d = _load(f)
    img = O.render(O.Scene(d["obj"], d["deformation"]), [tuple(a) for a in d["angles"]],
                   int(d["res"]), float(d["ds"]), R=float(d["R"]), fov=float(d["fov"]),
                   integration=str(d["integration"]))
    assert _rel(img, d["image"]) <= 1e-9


@pytest.mark.parametrize("f", ABI, ids=os.path.basename)
def test_oracle_reproduces_abi_fixture(f):
    d = _load(f)
    img = O.render_volume_abi(d["volume"], d["cams21"], int(d["res"]), d["ds"])
    assert _rel(img, d["image"]) <= 1e-9


@pytest.mark.parametrize("f", SCENES, ids=os.path.basename)
def test_engine_cpu_build_matches_scene_fixture(f):
    import hostsim
    d = _load(f)
    eyes, cams = O.cameras([tuple(a) for a in d["angles"]], float(d["R"]))
    C = np.concatenate([eyes, cams, np.full((len(eyes), 1), float(d["fov"]))], axis=1)
    img, _ = hostsim.render(d["obj"], C, int(d["res"]), float(d["ds"]),
                            deformation=d["deformation"], R=float(d["R"]),
                            integration=str(d["integration"]))
    assert _rel(img, d["image"]) <= REL_TOL


@pytest.mark.gpu
@pytest.mark.parametrize("f", SCENES, ids=os.path.basename)
def test_engine_gpu_matches_scene_fixture(f):
    import __graft_entry__ as g
    g.build()
    import xray_projection_render_gb300 as X
    d = _load(f)
    with X.Scene(d["obj"], d["deformation"]) as s:
        img = X.render(s, [tuple(a) for a in d["angles"]], resolution=int(d["res"]),
                       ds=float(d["ds"]), R=float(d["R"]), fov=float(d["fov"]),
                       integration=str(d["integration"]))
    assert _rel(img, d["image"]) <= REL_TOL


@pytest.mark.gpu
@pytest.mark.parametrize("f", ABI, ids=os.path.basename)
def test_engine_gpu_matches_abi_fixture(f):
    import __graft_entry__ as g
    g.build()
    import xray_projection_render_gb300 as X
    d = _load(f)
    img = X.render_volume_projections(d["volume"], d["cams21"], int(d["res"]), float(d["ds"]))
    assert _rel(img, d["image"]) <= REL_TOL
