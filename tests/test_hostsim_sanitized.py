"""The engine's per-pixel code (xrp_device.h, built for the CPU) and the
scene flattener under AddressSanitizer and UndefinedBehaviorSanitizer: out of
bounds reads of the node, cell, list and lattice tables, signed overflow in
index arithmetic and invalid shifts stop the child process with a report.
Small renders of every scene family, both integrators, plain and traced
(ray, ball and curve certificates), each also checked against the FP64
oracle.  CPU only; skipped where the compiler has no sanitizer runtime."""
import os
import subprocess
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)

CHILD = r"""
import os, sys
sys.path.insert(0, os.path.join(sys.argv[1], "tests", "hostsim"))
sys.path.insert(0, os.path.join(sys.argv[1], "tests"))
sys.path.insert(0, sys.argv[1])
from test_hostsim_parity import check
from xray_projection_render_gb300 import workloads as W
cases = [
    (W.reduced(W.deformed_lattice(), 96, 2), {}),
    (W.reduced(W.deformed_lattice(), 96, 2), {"trace": True}),
    (W.reduced(W.deformed_lattice(), 96, 2), {"fine_lists": True}),
    (W.offset_unit_cell(96), {"trace": True}),
    (W.reduced(W.gyroid_sigmoid(), 96, 2), {"trace": "curve"}),
    (W.reduced(W.gyroid_sigmoid(), 96, 2), {"trace": True}),
    (W.cube_minus_sphere_cylinder(96), {"trace": True}),
    (W.reduced(W.voxel_blobs(n=24), 64, 2), {}),
]
cases += [(W.reduced(w, 64, 2), {"trace": True}) for w in W.batched_scenes(4)]
# edge cases: nested tessellation, empty and degenerate children, a
# collection at the list-grid cap, a negative density
inner = {"type": "tessellated_obj_coll",
         "uc": {"objects": {"type": "object_collection", "objects": [
             {"type": "sphere", "center": [0.1, 0.1, 0.1], "radius": 0.08, "rho": 1.0}]},
                "xmin": 0, "xmax": 0.2, "ymin": 0, "ymax": 0.2, "zmin": 0, "zmax": 0.2},
         "xmin": 0, "xmax": 0.4, "ymin": 0, "ymax": 0.4, "zmin": 0, "zmax": 0.4}
nested = {"type": "tessellated_obj_coll",
          "uc": {"objects": {"type": "object_collection", "objects": [inner]},
                 "xmin": 0, "xmax": 0.5, "ymin": 0, "ymax": 0.5, "zmin": 0, "zmax": 0.5},
          "xmin": -1, "xmax": 1, "ymin": -1, "ymax": 1, "zmin": -1, "zmax": 1}
many = {"type": "object_collection", "objects": [
    {"type": "sphere", "center": [-0.9 + 0.12 * (k % 15), -0.9 + 0.12 * ((k // 15) % 15), -0.5 + 0.05 * (k // 225)],
     "radius": 0.05, "rho": 0.3} for k in range(300)]}
empty = {"type": "object_collection", "objects": []}
edge = {"type": "object_collection", "objects": [
    {"type": "cylinder", "p0": [0.1, 0.2, 0.3], "p1": [0.1, 0.2, 0.3], "radius": 0.2, "rho": 1.0},
    {"type": "sphere", "center": [0.0, 0.0, 0.0], "radius": 0.0, "rho": 1.0},
    {"type": "cube", "center": [0.2, -0.1, 0.0], "side": 0.5, "rho": 0.7},
    {"type": "sphere", "center": [0.2, -0.1, 0.0], "radius": 0.2, "rho": -0.4}]}
for name, obj in (("nested", nested), ("many", many), ("edge", edge), ("empty", empty)):
    w = W.Workload(name, obj, None, [(30.0, 75.0), (200.0, 110.0)], 64, 0.005)
    cases += [(w, {}), (w, {"trace": True}), (w, {"fine_lists": True, "trace": True})]
for w, kw in cases:
    for integration in ("simple", "hierarchical"):
        check(w, integration, nrays=1500, seed=1, nthreads=4, **kw)
import hostsim
for bad in ({"type": "sphere", "center": [0, 0]}, {"type": "no_such_object"},
            {"type": "object_collection", "objects": [{"type": "cylinder"}]}):
    try:
        hostsim.render(bad, check.__globals__["cams_of"](cases[0][0]), 16, 0.05)
    except ValueError:
        pass
    else:
        raise AssertionError("schema error not reported")
print("sanitized renders ok", len(cases))
"""


def _runtime(name):
    try:
        p = subprocess.run(["g++", f"-print-file-name={name}"], capture_output=True, text=True,
                           timeout=30)
    except (OSError, subprocess.TimeoutExpired):
        return None
    path = p.stdout.strip()
    return path if os.path.isabs(path) and os.path.exists(path) else None


def test_per_pixel_code_under_sanitizers():
    asan, cxx = _runtime("libasan.so"), _runtime("libstdc++.so")
    if asan is None or cxx is None:
        pytest.skip("no AddressSanitizer runtime")
    sys.path.insert(0, os.path.join(HERE, "hostsim"))
    import hostsim
    hostsim.build(sanitize=True)
    # the C++ runtime is preloaded too, so that ASan finds the real
    # __cxa_throw when the scene loader reports a schema error
    env = dict(os.environ, XRP_HOSTSIM_SANITIZED="1", LD_PRELOAD=f"{asan} {cxx}",
               ASAN_OPTIONS="detect_leaks=0:abort_on_error=0:exitcode=23",
               UBSAN_OPTIONS="halt_on_error=1:print_stacktrace=1:exitcode=24")
    p = subprocess.run([sys.executable, "-c", CHILD, ROOT], capture_output=True, text=True, env=env,
                       timeout=900, cwd=ROOT)
    report = p.stdout[-3000:] + p.stderr[-6000:]
    assert p.returncode == 0, report
    assert "runtime error" not in p.stderr and "AddressSanitizer" not in p.stderr, report
    assert "sanitized renders ok" in p.stdout
