"""The benchmark's JSON contract on the host: the reference arm's line (the
FP64 CPU restatement timed on the host cores) and the launch accounting the
engine arm reports.  No GPU: the reference arm loads the oracle only."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402  (numpy only at import)


def _run(args, env=None):
    e = dict(os.environ)
    e.update(env or {})
    p = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *args], capture_output=True,
                       text=True, timeout=300, env=e, cwd=ROOT)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [l for l in p.stdout.splitlines() if l.startswith("{")]
    return [json.loads(l) for l in lines]


def test_reference_arm_line():
    (line,) = _run(["--impl", "reference", "--workload", "cube", "--steps", "1", "--warmup", "0"])
    assert line["impl"] == "reference" and line["unit"] == "Mrays/s" and line["value"] > 0
    assert line["higher_is_better"] is True and line["n_gpus"] == 1 and line["steps"] == 1
    cfg = line["config"]
    assert cfg["workload"].startswith("cube") and cfg["res"] == 512 and cfg["ds"] == 0.005
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == line["value"] and cb["sample"]
    assert line["e2e"] == {"value": line["value"], "unit": "Mrays/s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}


def test_reference_arm_other_ranks_print_nothing():
    assert _run(["--impl", "reference", "--workload", "cube", "--steps", "1", "--warmup", "0"],
                env={"RANK": "1", "WORLD_SIZE": "2", "LOCAL_RANK": "1"}) == []


def test_reference_arm_unavailable_steps():
    (line,) = _run(["--impl", "reference", "--workload", "finish"])
    assert line["impl"] == "reference" and "unavailable" in line


def test_reference_and_engine_configs_agree():
    from xray_projection_render_gb300 import workloads as W
    w = bench.make_workload("lattice", W, 0, 0)
    a = bench.workload_config(w, "trace", 1, "lattice")
    b = bench.workload_config(w, bench.resolve_march(type("A", (), {"march": "auto"})(), w), 1, "lattice")
    assert a == b and a["views"] == 360 and a["res"] == 1024 and a["march"] == "trace"


@pytest.mark.parametrize("march,rays,voxel,integration,plain,probe,want", [
    ("trace", 360 * 1024 * 1024, False, "simple", "auto", False, 3 * 45),
    ("trace", 720 * 2048 * 2048, False, "simple", "auto", True, 3 * 360 + 6),
    ("trace", 8 * 2048 * 2048, False, "hierarchical", "auto", True, 3 * 16),
    ("plain", 36 * 1024 * 1024, False, "simple", "auto", False, 4 * 5),
    ("plain", 512 * 512, False, "simple", "auto", False, 1),
    ("plain", 512 * 512, False, "simple", "list", False, 4),
    ("plain", 36 * 1024 * 1024, False, "simple", "inplace", False, 1),
    ("plain", 180 * 1024 * 1024, True, "simple", "auto", False, 1),
])
def test_launch_accounting(march, rays, voxel, integration, plain, probe, want):
    assert bench.launches_per_step(march, rays, voxel, integration, plain, probe) == want


def test_non_affine_chains():
    assert not bench.non_affine(None)
    assert not bench.non_affine({"type": "linear", "strains": [0, 0, 0.05, 0, 0, 0]})
    assert bench.non_affine({"type": "sigmoid"})
    assert bench.non_affine({"type": "composed", "deformations": [{"type": "rigid"}, {"type": "gaussian"}]})
    assert not bench.non_affine({"type": "composed", "deformations": [{"type": "rigid"}, {"type": "affine"}]})
