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
for w, kw in cases:
    for integration in ("simple", "hierarchical"):
        check(w, integration, nrays=300, seed=1, nthreads=2, **kw)
print("sanitized renders ok", len(cases))
"""


def _asan_runtime():
    try:
        p = subprocess.run(["g++", "-print-file-name=libasan.so"], capture_output=True, text=True,
                           timeout=30)
    except (OSError, subprocess.TimeoutExpired):
        return None
    path = p.stdout.strip()
    return path if os.path.isabs(path) and os.path.exists(path) else None


def test_per_pixel_code_under_sanitizers():
    asan = _asan_runtime()
    if asan is None:
        pytest.skip("no AddressSanitizer runtime")
    sys.path.insert(0, os.path.join(HERE, "hostsim"))
    import hostsim
    hostsim.build(sanitize=True)
    env = dict(os.environ, XRP_HOSTSIM_SANITIZED="1", LD_PRELOAD=asan,
               ASAN_OPTIONS="detect_leaks=0:abort_on_error=0:exitcode=23",
               UBSAN_OPTIONS="halt_on_error=1:print_stacktrace=1:exitcode=24")
    p = subprocess.run([sys.executable, "-c", CHILD, ROOT], capture_output=True, text=True, env=env,
                       timeout=900, cwd=ROOT)
    report = p.stdout[-3000:] + p.stderr[-6000:]
    assert p.returncode == 0, report
    assert "runtime error" not in p.stderr and "AddressSanitizer" not in p.stderr, report
    assert "sanitized renders ok" in p.stdout
