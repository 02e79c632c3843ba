"""Build recipe for libcuda_render.so (sm_103a) -- no cmake.

    python -m xray_projection_render_gb300.build

compiles ``csrc/xrp_scene.cpp`` with g++ and the CUDA units (host code and
voxel kernels, general-scene kernels, proposal march, training) with nvcc for
``sm_103a``, all in parallel, then links ``libcuda_render.so`` next to this file (the
name the reference's Go loader looks for, cuda_backend.go:103-114).  Host
floating point is built with contraction off so the FP64 camera and scene
arithmetic rounds every operation, as the reference does.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libcuda_render.so")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# extra nvcc options, e.g. the occupancy knobs of xrp_launch.h
# (XRP_NVCC_FLAGS="-DXRP_CURVE_MIN_BLOCKS=3"; its -D options reach the host
# scene code too); they take part in the staleness check through the flags
# file below
EXTRA = os.environ.get("XRP_NVCC_FLAGS", "").split()


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _sources():
    return [os.path.join(CSRC, f) for f in sorted(os.listdir(CSRC))
            if f.endswith((".cu", ".cuh", ".cpp", ".h"))] + [os.path.join(INCLUDE, "xrp.h")]


FLAGS_FILE = os.path.join(BUILD, "nvcc_flags.txt")


def _stale(target):
    if not os.path.exists(target):
        return True
    try:
        with open(FLAGS_FILE) as f:
            if f.read() != " ".join(EXTRA):
                return True
    except OSError:
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in _sources() + [__file__])


def _run(cmd, verbose):
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if verbose and (r.stdout or r.stderr):
        print(r.stdout, r.stderr, flush=True)
    return r


CUDA_UNITS = ["xrp_engine.cu", "xrp_kern_scene.cu", "xrp_kern_batch.cu", "xrp_kern_batch_ball.cu",
              "xrp_kern_batch_ray.cu", "xrp_kern_batch_curve.cu", "xrp_kern_export.cu",
              "xrp_kern_trace.cu", "xrp_kern_trace_ray.cu", "xrp_kern_trace_curve.cu",
              "xrp_kern_trace_plain.cu",
              "xrp_kern_prop.cu", "xrp_kern_prop_net.cu", "xrp_kern_train.cu"]


def build(force: bool = False, verbose: bool = False, ptxas_info: bool = False) -> str:
    """Compile the engine for sm_103a and return the path of the shared library."""
    if not force and not ptxas_info and not _stale(LIB):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    common_host = ["-O2", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-fvisibility=hidden"]
    o_scene = os.path.join(BUILD, "xrp_scene.o")
    defines = [e for e in EXTRA if e.startswith("-D")]
    cmds = [["g++", "-std=c++17", *common_host, "-Wall", "-I", INCLUDE, *defines, "-c",
             os.path.join(CSRC, "xrp_scene.cpp"), "-o", o_scene]]
    objs = [o_scene]
    for unit in CUDA_UNITS:
        o = os.path.join(BUILD, unit.replace(".cu", ".o"))
        cmd = [nvcc, *ARCH, "-std=c++17", "-O3", "-lineinfo", "-Xcompiler", ",".join(common_host),
               "-I", INCLUDE, *EXTRA, "-c", os.path.join(CSRC, unit), "-o", o]
        if ptxas_info:
            cmd.insert(1, "-Xptxas=-v")
        cmds.append(cmd)
        objs.append(o)
    with ThreadPoolExecutor(len(cmds)) as ex:
        results = list(ex.map(lambda c: _run(c, verbose), cmds))
    tmp = LIB + f".tmp{os.getpid()}"
    _run([nvcc, *ARCH, "-shared", "-cudart", "static", "-o", tmp, *objs, "-lpthread"], verbose)
    os.replace(tmp, LIB)
    with open(FLAGS_FILE, "w") as f:
        f.write(" ".join(EXTRA))
    if ptxas_info:
        return "".join(r.stderr for r in results[1:])
    return LIB


if __name__ == "__main__":
    info = "--ptxas" in sys.argv
    out = build(force=True, verbose="-v" in sys.argv, ptxas_info=info)
    print(out)
