"""The reference's GPU kernel as a measured bar.

TEST INFRASTRUCTURE (the benchmark's reference-GPU arm): nothing here is part
of the engine.  ``build()`` compiles the reference's unmodified
``cuda_backend.cu`` (from the reference tree, when present) to cubins for
sm_103a and for the sm_100 target the reference's Makefile ships
(Makefile:14-17), into ``oracle/_ref/``, and compiles the timing harness
``ref_gpu_harness.cu`` (this directory) next to them.  ``run()`` feeds the
harness a voxel grid and XRayCameraParams rows and returns its end-to-end
and kernel-only times and, optionally, its images.
"""
from __future__ import annotations

import json
import os
import shutil
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
REF_SRC = os.path.join("/root/reference", "cuda_backend.cu")
HARNESS_SRC = os.path.join(HERE, "ref_gpu_harness.cu")
HARNESS = os.path.join(OUT, "ref_gpu_harness")
CUBINS = {"sm_103a": os.path.join(OUT, "render_kernel_sm_103a.cubin"),
          "sm_100": os.path.join(OUT, "render_kernel_sm_100.cubin")}
GENCODE = {"sm_103a": "arch=compute_103a,code=sm_103a", "sm_100": "arch=compute_100,code=sm_100"}


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _stale(target, src):
    return not os.path.exists(target) or os.path.getmtime(target) < os.path.getmtime(src)


def build(force: bool = False) -> dict:
    """Cubins of the reference kernel (only where the reference tree is
    present) and the harness (wherever nvcc is).  Returns what exists."""
    os.makedirs(OUT, exist_ok=True)
    nvcc = _nvcc()
    if os.path.exists(REF_SRC):
        for arch, path in CUBINS.items():
            if force or _stale(path, REF_SRC):
                subprocess.run([nvcc, "-cubin", "-O2", "-gencode", GENCODE[arch], "-I",
                                os.path.dirname(REF_SRC), "-o", path, REF_SRC], check=True)
    if force or _stale(HARNESS, HARNESS_SRC):
        tmp = HARNESS + f".tmp{os.getpid()}"
        subprocess.run([nvcc, "-O2", "-std=c++17", "-o", tmp, HARNESS_SRC, "-lcuda"], check=True)
        os.replace(tmp, HARNESS)
    return {"harness": os.path.exists(HARNESS),
            "cubins": {a: p for a, p in CUBINS.items() if os.path.exists(p)}}


def run(volume, cams21, res, ds, flat_field=0.0, warmup=1, steps=3, arch="sm_103a", images=False):
    """Times the reference kernel on `volume` (float32 [z][x][y]) and the
    cameras (float32 [n, 21]); returns the harness's record (and the
    end-to-end images [n, res, res] with ``images``)."""
    cubin = CUBINS[arch]
    if not os.path.exists(cubin):
        raise FileNotFoundError(f"{cubin} is missing (built where the reference tree is present)")
    vol = np.ascontiguousarray(volume, dtype=np.float32)
    nz, nx, ny = vol.shape
    cams = np.ascontiguousarray(cams21, dtype=np.float32).reshape(-1, 21)
    with tempfile.TemporaryDirectory() as d:
        vp, cp, op = (os.path.join(d, n) for n in ("vol.f32", "cams.f32", "out.f32"))
        vol.tofile(vp)
        cams.tofile(cp)
        cmd = [HARNESS, cubin, vp, str(nx), str(ny), str(nz), cp, str(cams.shape[0]), str(res),
               repr(float(ds)), repr(float(flat_field)), str(warmup), str(steps)]
        if images:
            cmd.append(op)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"reference GPU harness failed ({r.returncode}): {r.stderr.strip()}")
        rec = json.loads(r.stdout.strip().splitlines()[-1])
        if images:
            rec["images"] = np.fromfile(op, dtype=np.float32).reshape(cams.shape[0], res, res)
    return rec


__all__ = ["build", "run", "CUBINS", "HARNESS"]
