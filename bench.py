"""Benchmark: Mrays/s of the GB300 projection engine.

Default workload (the headline): the deformed lattice -- a unit cell of 12
edge and 4 body-diagonal cylinders (radius 0.03, rho 1) tessellated
10 x 10 x 10 over [-1,1]^3 under 5 % axial (zz) strain -- from 360 seeded
views (azimuth U[0,360), polar U[30,150], seed 3) at 1024 x 1024, ds 0.002,
R 4, fov 40: 377.5 M rays per step.

One step = one pass of the fastest exact path over every view: certificate
tracing with ray certificates (each evaluated sample certifies how many of
the following samples share its density; results equal the plain
integrator's).  The same record carries
  plain          : the uniform-step integrator (main.go:144-154), same views;
  speedup_vs_plain
  proposal       : the segment march routed by the trained 3 x 64 network, on
                   a view subset (its rate per ray does not depend on which
                   other views share a call);
  error_vs_fp64  : for every path, the max relative and absolute
                   transmittance error against the FP64 oracle on the CPU
                   baseline leg's seeded rays;
  gyroid         : the gyroid (scale 8, thickness 0.1) under the sigmoid
                   deformation (A 0.1, L 0.2, along z), 720 views x 2048^2,
                   ds 0.001, with the same fields.

value     : device throughput, scene resident in HBM, output to a device
            buffer, L2 flushed (256 MiB write) before every timed step, each
            step timed with CUDA events on the launching stream.
e2e       : the same metric through the C ABI with the scene created from
            its JSON map and the images copied into pinned host memory
            inside the timed region (RenderVolumeProjectionsCUDA for the
            voxel grid).
roofline  : FP32 issue for the analytic scenes (evaluations x FLOPs per
            evaluation against a CUDA-core SGEMM measured in this run); the
            voxel grid reports its texture gathers against the gather rate
            measured in this run.
cpu_baseline / --impl reference: the FP64 CPU restatement of the reference
            path (oracle/), on all host cores, on a seeded ray subset.

Multi-GPU: the path has no exchange step; N processes render disjoint view
subsets (view k on rank k mod N) with no collective ("scaling": "weak").
"""
from __future__ import annotations

import argparse
import dataclasses
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

HEADLINE_METRIC = ("Mrays/s on 1 GB300 at <=1e-4 error vs FP64: fastest exact path on the deformed "
                   "lattice, with the plain GPU integrator and the learned proposal in the same record")
VOXEL_METRIC = "Mrays/s on 1 GB300 (uniform-step integrator, voxel grid 256^3, 180 views x 1024^2)"

# the definitions of the workloads, printed in `config` by both arms
DEFINITIONS = {
    "lattice": {"cells": "10x10x10 over [-1,1]^3", "unit_cell": "12 edge + 4 body-diagonal cylinders",
                "strut_radius": 0.03, "deformation": "linear, strain zz 0.05",
                "cameras": "azimuth U[0,360), polar U[30,150], seed 3"},
    "gyroid_fine": {"gyroid": "scale 0.1, thickness 0.2, rho 1 (the reference's example scene), unit cell "
                              "[-1,1]^3, outer bounds [-0.8,0.8]^3",
                    "deformation": "sigmoid A 0.1, center 0, lengthscale 0.2, along z",
                    "cameras": "64 of azimuth 0, 0.5, ..., 359.5 (evenly strided), polar 90"},
    "gyroid": {"gyroid": "scale 8, thickness 0.1, rho 1, tessellated over [-1,1]^3",
               "deformation": "sigmoid A 0.1, center 0, lengthscale 0.2, along z",
               "cameras": "azimuth 0, 0.5, ..., 359.5, polar 90"},
    "voxel": {"grid": "256^3 FP32, 64 seeded Gaussians (seed 2)",
              "cameras": "azimuth 0, 2, ..., 358, polar 90"},
    "cube": {"scene": "cube side 1 minus sphere r 0.3 and cylinder r 0.2",
             "cameras": "azimuth 0, polar 90"},
}


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="engine", choices=["engine", "reference", "reference_gpu"],
                   help="engine (this library), reference (the reference's CPU algorithm on the "
                        "host cores) or reference_gpu (the reference's own GPU kernel, voxel grid only)")
    p.add_argument("--workload", default="lattice",
                   choices=["lattice", "gyroid", "gyroid_fine", "voxel", "cube", "batched", "finish",
                            "voxelize"],
                   help="lattice (default, the headline), the gyroid (scale 8), the example scene's "
                        "gyroid (scale 0.1, 64 views), the voxel grid, the cube minus "
                        "sphere and cylinder, the batch of 64 uneven scenes (one persistent launch "
                        "replayed from a CUDA graph), device-side image finishing of 64 images of "
                        "1024^2, or the volume export of the deformed lattice at 256^3")
    p.add_argument("--scenes", type=int, default=64, help="batched: number of scenes")
    p.add_argument("--march", default="auto",
                   choices=["auto", "plain", "trace", "ball", "certificate", "proposal"],
                   help="auto: certificate tracing for analytic scenes, the plain integrator for "
                        "the voxel grid; plain integrator, per-ray certificate tracing (ray bounds "
                        "for affine deformation chains), tracing with ball certificates only, "
                        "segment march with certificates and no network, or the trained proposal")
    p.add_argument("--integration", default="simple", choices=["simple", "hierarchical"],
                   help="integrator (main.go:144-199); the reference CLI's default is hierarchical")
    p.add_argument("--views", type=int, default=0, help="view count (0: the workload's)")
    p.add_argument("--res", type=int, default=0, help="resolution (0: the workload's)")
    p.add_argument("--cpu-seconds", type=float, default=12.0)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-e2e", action="store_true", help="skip the host-buffer ABI timing")
    p.add_argument("--no-compare", action="store_true",
                   help="skip the plain / proposal comparisons and the gyroid record")
    p.add_argument("--volume-path", default="gather", choices=["gather", "loads"],
                   help="voxel reads: texture gathers (default) or per-tap loads")
    p.add_argument("--plain-fp64", default="auto", choices=["auto", "list", "inplace"],
                   help="plain integrator over analytic scenes: undecided samples to one FP64 list "
                        "pass, or re-evaluated inside the march (auto: the list from 2^22 rays a call)")
    return p.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks during the timed region (the recipe's query)."""

    def __init__(self, index):
        self.index = index
        self.samples = []
        self.proc = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for s in self.samples:
            try:
                sm.append(float(s[1]))
                mx = float(s[2])
                for k, n in enumerate(names):
                    if s[5 + k].lower().startswith("active"):
                        reasons.add(n)
            except (ValueError, IndexError):
                continue
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except Exception:
        return {}


def fp32_peak_tflops(torch):
    """CUDA-core FP32 throughput via SGEMM with TF32 disabled (best of 5)."""
    torch.backends.cuda.matmul.allow_tf32 = False
    n = 8192
    a = torch.randn(n, n, device="cuda")
    b = torch.randn(n, n, device="cuda")
    for _ in range(2):
        torch.mm(a, b)
    best = 0.0
    for _ in range(5):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.mm(a, b)
        e1.record()
        torch.cuda.synchronize()
        best = max(best, 2 * n ** 3 / (e0.elapsed_time(e1) * 1e-3) / 1e12)
    del a, b
    return best


# ---------------------------------------------------------------------------
# the FP64 oracle: CPU baseline and error against FP64 (test infrastructure:
# it checks and times the reference algorithm, it never renders a result)
# ---------------------------------------------------------------------------

def draw_rays(rng, nviews, res, n):
    return np.stack([rng.integers(0, nviews, n), rng.integers(0, res, n),
                     rng.integers(0, res, n)], 1).astype(np.int32)


def oracle_rays(w, angles, rays, threads=None, integration="simple"):
    """FP64 transmittance of the (view, i, j) rays of `angles` (the oracle
    builds its own cameras; nothing here touches the engine library)."""
    from oracle import oracle as O
    obj = {"type": "voxel_grid", "_voxels": w.volume} if w.volume is not None else w.obj
    return O.render(O.Scene(obj, w.deformation), angles, w.res, w.ds, R=w.R, fov=w.fov,
                    integration=integration, rays=rays, nthreads=threads or os.cpu_count() or 1)


def cpu_baseline(w, seconds, threads=None, seed=1234, integration="simple"):
    """The oracle on all host cores on seeded random rays of `w` for about
    `seconds`: (cpu_baseline record, rays, FP64 transmittances)."""
    threads = threads or os.cpu_count() or 1
    rng = np.random.default_rng(seed)
    n = 2000
    t = time.perf_counter()
    oracle_rays(w, w.angles, draw_rays(rng, len(w.angles), w.res, n), threads, integration)
    dt = time.perf_counter() - t
    # batches sized from the probe, until the timed renders reach `seconds`
    batch = int(max(2000, min(20_000_000, 0.35 * n * seconds / max(dt, 1e-3))))
    all_rays, all_ref, spent = [], [], 0.0
    while spent < seconds and sum(len(r) for r in all_rays) < 60_000_000:
        rays = draw_rays(rng, len(w.angles), w.res, batch)
        t = time.perf_counter()
        all_ref.append(oracle_rays(w, w.angles, rays, threads, integration))
        spent += time.perf_counter() - t
        all_rays.append(rays)
    rays = np.concatenate(all_rays)
    ref = np.concatenate(all_ref)
    return ({"value": len(rays) / spent / 1e6, "unit": "Mrays/s", "cores": threads, "kind": "port",
             "sample": f"{len(rays)} seeded random rays of {w.name} ({spent:.1f} s)"}, rays, ref)


def error_vs_fp64(out, rays, ref, res):
    """Max relative / absolute error of a device image stack [view][i][j]
    at the given rays against their FP64 values."""
    import torch
    idx = (torch.from_numpy(rays[:, 0].astype(np.int64)) * res * res
           + torch.from_numpy(rays[:, 1].astype(np.int64)) * res
           + torch.from_numpy(rays[:, 2].astype(np.int64))).to(out.device)
    got = out.reshape(-1)[idx].cpu().numpy().astype(np.float64)
    if not np.all(np.isfinite(got)):
        return {"max_rel": None, "max_abs": None, "rays": int(len(rays)), "non_finite": True}
    d = np.abs(got - ref)
    return {"max_rel": float(np.max(d / ref)), "max_abs": float(np.max(d)), "rays": int(len(rays))}


def subset_views(angles, views):
    return list(angles[:: max(1, len(angles) // views)][:views])


def workload_config(w, march, world, name, integration="simple"):
    """`config` of a scene workload: the same dict in both arms."""
    cfg = {"workload": w.name, "views": len(w.angles), "res": w.res, "ds": w.ds,
           "integrator": integration, "R": w.R, "fov": w.fov, "march": march,
           "l2": "flushed before every timed step (256 MiB write)",
           "parallelism": f"views k mod {world}"}
    cfg.update(DEFINITIONS.get(name, {}))
    return cfg


def resolve_march(args, w):
    if args.march != "auto":
        return args.march
    return "plain" if w.volume is not None else "trace"


MARCH_PATHS = {
    "plain": "uniform-step integrator (main.go:144-154)",
    "trace": "certificate tracing (ray certificates for affine deformation chains, curve "
             "certificates for the others)",
    "ball": "certificate tracing with ball certificates",
    "certificate": "segment march with certificates, no network",
    "proposal": "segment march routed by the trained 3 x 64 network (BF16, FP32 accumulate)",
}


def run_reference(args):
    """The reference's CPU algorithm (the FP64 oracle port) on the host
    cores, on the engine arm's workload, metric and config; every timed step
    renders a seeded ray sample of at least 10 s."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from xray_projection_render_gb300 import workloads as W  # numpy only: no engine library
    if args.workload in ("finish", "voxelize"):
        print(json.dumps({"impl": "reference", "unavailable":
                          "the reference runs this step in Go on the host (PNG / raw writing); "
                          "no CPU arm is timed for it here"}), flush=True)
        return
    if args.workload == "batched":
        ws = W.batched_scenes(args.scenes)[:8]
        name = f"batched_scenes_{args.scenes}"
        cfg = batched_config(args.scenes, world, args.integration)

        def measure(sec):
            return cpu_baseline_multi(ws, sec, args.integration)
        metric = BATCH_METRIC
    else:
        w = make_workload(args.workload, W, args.views, args.res)
        name = w.name
        cfg = workload_config(w, resolve_march(args, w), world, args.workload, args.integration)

        def measure(sec):
            return cpu_baseline(w, sec, integration=args.integration)[0]
        metric = VOXEL_METRIC if args.workload == "voxel" else (
            HEADLINE_METRIC if args.workload == "lattice" else f"Mrays/s on 1 GB300 ({name})")
    vals = []
    for i in range(args.warmup + args.steps):
        cb = measure(2.0 if i < args.warmup else max(10.0, args.cpu_seconds))
        if i >= args.warmup:
            vals.append(cb["value"])
    v = float(np.median(vals))
    cb["value"] = v
    line = {"impl": "reference", "metric": metric, "value": v, "unit": "Mrays/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded)", "config": cfg, "cpu_baseline": cb,
            "e2e": {"value": v, "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_reference_gpu(args):
    """The reference's own GPU kernel (render_kernel, cuda_backend.cu:19-80,
    compiled from its unmodified source into oracle/_ref) on the voxel-grid
    workload, driven the way RenderVolumeProjectionsCUDA drives it
    (cuda_backend.cu:82-203): end to end (allocation, upload, per-camera
    launch, synchronisation and copy back) and kernel only (CUDA events
    around back-to-back launches, L2 flushed), with its error against FP64
    on seeded rays.  The reference GPU path supports voxel grids only."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from xray_projection_render_gb300 import workloads as W
    if args.workload != "voxel":
        print(json.dumps({"impl": "reference_gpu", "unavailable":
                          "the reference's GPU kernel renders voxel grids only (--workload voxel)"}),
              flush=True)
        return
    from oracle import oracle as O
    from oracle import ref_gpu
    try:
        ref_gpu.build()
    except Exception as ex:
        print(json.dumps({"impl": "reference_gpu", "unavailable": f"harness build failed: {ex}"}))
        return
    w = make_workload(args.workload, W, args.views, args.res)
    cams21 = O.xray_camera_params(w.angles, w.R, w.fov)
    rng = np.random.default_rng(4321)
    rays = draw_rays(rng, len(w.angles), w.res, 20000)
    ref = O.render_volume_abi(w.volume, cams21, w.res, np.float32(w.ds), rays=rays)
    line = {"impl": "reference_gpu", "metric": VOXEL_METRIC, "unit": "Mrays/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "dtype": "f32",
            "data": "synthetic (seeded)",
            "config": workload_config(w, "plain", 1, args.workload), "arch": {}}
    for arch in ("sm_103a", "sm_100"):
        if not os.path.exists(ref_gpu.CUBINS[arch]):
            line["arch"][arch] = {"unavailable": "cubin not built (the reference tree was absent)"}
            continue
        try:
            rec = ref_gpu.run(w.volume, cams21, w.res, w.ds, warmup=max(1, args.warmup),
                              steps=args.steps, arch=arch, images=True)
        except Exception as ex:
            line["arch"][arch] = {"unavailable": str(ex)[:300]}
            continue
        imgs = rec.pop("images")
        got = imgs[rays[:, 0], rays[:, 1], rays[:, 2]].astype(np.float64)
        d = np.abs(got - ref)
        k_s = float(np.mean(rec["kernel_ms"])) * 1e-3
        e_s = float(np.mean(rec["e2e_ms"])) * 1e-3
        line["arch"][arch] = {
            "value": rec["rays"] / k_s / 1e6, "ms_per_step": k_s * 1e3,
            "e2e": {"value": rec["rays"] / e_s / 1e6, "unit": "Mrays/s", "ms_per_step": e_s * 1e3},
            "error_vs_fp64": {"max_rel": float(np.max(d / ref)), "max_abs": float(np.max(d)),
                              "rays": int(len(rays))}}
    best = [a for a in line["arch"].values() if "value" in a]
    if best:
        line["value"] = best[0]["value"]
        line["e2e"] = best[0]["e2e"]
        line["error_vs_fp64"] = best[0]["error_vs_fp64"]
    print(json.dumps(line), flush=True)


# Algorithmic FP32 work per evaluated sample (FMA = 2), from the per-item
# table of the benchmark definitions: common 8 + object terms.
FLOPS = {
    "voxel": 58,     # 50 trilinear
    "cube": 54,      # sphere 9 + box 9 + cylinder 23 + collection 3 + clip 2
    "lattice": 437,  # linear deformation 18 + fold/bounds 27 + 16 cylinders x 23 + 16
    "gyroid": 53,    # gyroid 13 (+6 SFU) + sigmoid 5 (+2 SFU) + fold/bounds 27
    "gyroid_fine": 53,
}

# DRAM bytes (read + write) per view of the voxel render kernel: a constant
# from an ncu capture of 8 views (the grid streams through L2 once per view,
# so the traffic grows with the views).
TRAFFIC_PER_VIEW = {"voxel": (404.93e6 + 47.01e6) / 8}


def make_workload(name, W, views, res):
    if name == "voxel":
        w = W.voxel_blobs(1024, 180)
    elif name == "cube":
        w = W.cube_minus_sphere_cylinder(512)
    elif name == "lattice":
        w = W.deformed_lattice(1024, 360)
    elif name == "gyroid":
        w = W.gyroid_sigmoid(2048, 720)
    elif name == "gyroid_fine":
        w = W.gyroid_fine_sigmoid(2048, 64)
    else:
        raise ValueError(name)
    if views or res:
        w = W.reduced(w, res or w.res, views or None)
    return w


def _event_time(torch, step, steps, stream, flush):
    """Mean seconds of `steps` calls of step(), each bracketed by CUDA events
    on `stream` after an L2 flush."""
    times = []
    for _ in range(steps):
        flush.fill_(1.0)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        step()
        e1.record(stream)
        e1.synchronize()
        times.append(e0.elapsed_time(e1) * 1e-3)
    return float(np.mean(times))


def scene_step(X, scene, w, angles, march, out, stream, prop=None, volume_path="gather",
               integration="simple", plain_fp64="auto"):
    """One render of `angles` by `march` into the device buffer `out`."""
    kw = dict(resolution=w.res, ds=w.ds, R=w.R, fov=w.fov, integration=integration)
    if march == "plain":
        return lambda: X.render(scene, angles, out=out, stream=stream, volume_path=volume_path,
                                plain_fp64=plain_fp64, **kw)
    trace = {"trace": True, "ball": "ball"}.get(march, False)
    return lambda: X.render_proposal(scene, prop, angles, segment=64, refine=march == "proposal",
                                     trace=trace, out=out, stream=stream, **kw)


def non_affine(deformation):
    """Whether a deformation map has a step that is not affine."""
    if not deformation:
        return False
    steps = deformation.get("deformations", [deformation]) if deformation.get("type") == "composed" \
        else [deformation]
    return any(non_affine(d) if d.get("type") == "composed" else d.get("type") in ("gaussian", "sigmoid")
               for d in steps)


def launches_per_step(march, rays, voxel, integration="simple", plain_fp64="auto", probe=False):
    """Kernels one step launches: one render launch for a voxel-grid root
    and for the plain integrator re-evaluating in place (below 2^22 rays a
    call unless told otherwise); otherwise, per launch group of at most 8 M
    rays (2 M for the hierarchical integrator), the march, its FP64 pass and
    the exp pass, and for the plain integrator the re-march of rays that
    found the FP64 list full.  `probe`: tracing over a non-affine chain,
    whose calls of 2^22 rays or more first render two small probes (three
    launches each) to pick the certificate kind."""
    if voxel:
        return 1
    if march == "plain" and (plain_fp64 == "inplace" or (plain_fp64 == "auto" and rays < (1 << 22))):
        return 1
    group = 1 << (21 if integration == "hierarchical" else 23)
    n = (4 if march == "plain" else 3) * -(-rays // group)
    if probe and march == "trace" and integration == "simple" and rays >= (1 << 22):
        n += 6
    return n


def time_path(X, torch, scene, w, angles, march, stream, flush, steps, prop=None, err_rays=4000):
    """Rate and error vs FP64 of one march on `angles` (at the workload's
    resolution and step): one warm-up call, then `steps` timed calls."""
    out = torch.empty((len(angles), w.res, w.res), device="cuda", dtype=torch.float32)
    step = scene_step(X, scene, w, angles, march, out, stream, prop)
    step()
    torch.cuda.synchronize()
    t = _event_time(torch, step, steps, stream, flush)
    rec = {"value": len(angles) * w.res * w.res / t / 1e6, "unit": "Mrays/s", "views": len(angles),
           "res": w.res, "steps": steps, "ms_per_step": t * 1e3, "path": MARCH_PATHS[march],
           "gpu_launches_per_step": launches_per_step(march, len(angles) * w.res * w.res, False,
                                                      probe=non_affine(w.deformation))}
    rng = np.random.default_rng(4321)
    rays = draw_rays(rng, len(angles), w.res, err_rays)
    wa = dataclasses.replace(w, angles=angles)
    rec["error_vs_fp64"] = error_vs_fp64(out, rays, oracle_rays(wa, angles, rays), w.res)
    del out
    return rec


def compare_paths(X, torch, scene, w, value, stream, flush, args, full_plain=True):
    """The plain integrator and the learned proposal on the same scene, with
    their errors against FP64, and the speed-up of `value` over plain."""
    steps = max(1, min(args.steps, 2))
    rec = {}
    plain_angles = w.angles if full_plain else subset_views(w.angles, 24)
    rec["plain"] = time_path(X, torch, scene, w, plain_angles, "plain", stream, flush, steps)
    if not full_plain:
        rec["plain"]["note"] = "view subset (the per-ray cost does not depend on the other views)"
    rec["speedup_vs_plain"] = value / rec["plain"]["value"]
    pv = subset_views(w.angles, 16 if w.res <= 1024 else 8)
    t0 = time.perf_counter()
    with X.Proposal(scene, pv, resolution=w.res, ds=w.ds, R=w.R, fov=w.fov, segment=64) as P:
        train_s = time.perf_counter() - t0
        pr = time_path(X, torch, scene, w, pv, "proposal", stream, flush, steps, prop=P)
        _, st = X.render_proposal(scene, P, pv[:1], resolution=w.res, ds=w.ds, R=w.R, fov=w.fov,
                                  stats=True)
    pr["train_s"] = train_s
    pr["speedup_vs_plain"] = pr["value"] / rec["plain"]["value"]
    pr["counters_one_view"] = st
    pr["note"] = "view subset; the network routes segments between refinement and dense sampling"
    rec["proposal"] = pr
    return rec


def secondary_gyroid(X, torch, W, stream, flush, args):
    """The gyroid under the sigmoid deformation at full size (720 x 2048^2,
    ds 0.001): certificate tracing over every view, plain and proposal on
    view subsets, errors against FP64."""
    w = W.gyroid_sigmoid(2048, 720)
    steps = max(1, min(args.steps, 3))
    with X.Scene(w.obj, w.deformation) as s:
        rec = time_path(X, torch, s, w, w.angles, "trace", stream, flush, steps, err_rays=6000)
        rec.update({"workload": w.name, "ds": w.ds, "march": "trace"})
        _, st = X.render_proposal(s, None, w.angles[:1], resolution=w.res, ds=w.ds, R=w.R, fov=w.fov,
                                  trace=True, stats=True)
        rec["evaluations_per_ray"] = st["evaluations"] / (w.res * w.res)
        torch.cuda.empty_cache()
        rec.update(compare_paths(X, torch, s, w, rec["value"], stream, flush, args, full_plain=False))
    torch.cuda.empty_cache()
    return rec


def bench_scene(args):
    import torch
    import __graft_entry__ as G
    import xray_projection_render_gb300 as X
    from xray_projection_render_gb300 import workloads as W

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    G.build()
    from xray_projection_render_gb300.sharding import job_time, shard
    w = make_workload(args.workload, W, args.views, args.res)
    march = resolve_march(args, w)
    is_voxel = w.volume is not None
    my_angles = shard(w.angles, rank, world)  # view k on rank k mod N, no exchange
    wm = dataclasses.replace(w, angles=my_angles)
    n_my = len(my_angles)
    res = w.res
    img = res * res
    dev = torch.device("cuda", local)
    stream = torch.cuda.current_stream(dev)
    vols = [torch.from_numpy(w.volume).to(dev)] if is_voxel else []
    scene = X.Scene(w.obj, w.deformation, vols)
    out = torch.empty((n_my, res, res), device=dev, dtype=torch.float32)
    flush = torch.empty(64 * 1024 * 1024, device=dev, dtype=torch.float32)  # 256 MiB > L2
    kw = dict(resolution=res, ds=w.ds, R=w.R, fov=w.fov, volume_path=args.volume_path,
              integration=args.integration)

    prop = None
    if march == "proposal":
        prop = X.Proposal(scene, my_angles, resolution=res, ds=w.ds, R=w.R, fov=w.fov, segment=64)
    step = scene_step(X, scene, w, my_angles, march, out, stream, prop, args.volume_path,
                      args.integration, args.plain_fp64)
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    # exact sample count of one step (counter pass, untimed, on a view subset)
    nstat = max(1, min(8, n_my))
    _, samples, fp64 = X.render(scene, my_angles[:nstat], stats=True, **kw)
    samples_step = samples * n_my / nstat
    evals_step = None
    if march != "plain" and not is_voxel:
        # evaluations the march actually makes (density + certificate per
        # evaluation, or one density per dense sample)
        _, pst = X.render_proposal(scene, prop, my_angles[:nstat], resolution=res, ds=w.ds, R=w.R,
                                   fov=w.fov, segment=64, refine=march == "proposal",
                                   trace=_trace_mode(march), stats=True, integration=args.integration)
        evals_step = (pst["evaluations"] + pst["dense_samples"]) * n_my / nstat
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        t_local = _event_time(torch, step, args.steps, stream, flush)
    t_step, rays_total = job_time(t_local, n_my * img, dev)
    value = rays_total / t_step / 1e6

    # error of the timed step's images against FP64, on the CPU baseline
    # leg's rays (the oracle renders them once; rank 0's views)
    cb = None
    if rank == 0:
        if args.no_cpu_baseline:
            rng = np.random.default_rng(1234)
            rays = draw_rays(rng, n_my, res, 20000)
            ref = oracle_rays(wm, my_angles, rays, integration=args.integration)
        else:
            cb, rays, ref = cpu_baseline(wm, args.cpu_seconds, integration=args.integration)
        err = error_vs_fp64(out, rays, ref, res)

    # end to end through the host-facing C ABI, pinned host buffers, inputs
    # uploaded and images read back inside the timed region
    e2e_times = []
    out_host = None if args.no_e2e else torch.empty((n_my, res, res), dtype=torch.float32).pin_memory()
    if is_voxel and args.integration == "simple":
        # the reference's own entry point (uniform-step integrator only)
        cams21 = X.xray_camera_params(my_angles, w.R, w.fov)
        h2d = int(w.volume.nbytes + cams21.nbytes)
        path = "RenderVolumeProjectionsCUDA, pinned host buffers"
        if not args.no_e2e:
            vol_host = torch.from_numpy(w.volume).pin_memory()

        def e2e_call():
            X.render_volume_projections(vol_host.numpy(), cams21, res, w.ds, out=out_host)
    elif is_voxel:
        h2d = int(w.volume.nbytes) + n_my * 192
        path = "xrp_scene_create (host volume) + xrp_render, pinned host buffers"
        if not args.no_e2e:
            vol_host = torch.from_numpy(w.volume).pin_memory()

        def e2e_call():
            with X.Scene(w.obj, w.deformation, [vol_host.numpy()]) as s2:
                X.render(s2, my_angles, out=out_host, **kw)
    else:
        obj_json = json.dumps(w.obj)
        def_json = json.dumps(w.deformation) if w.deformation else None
        h2d = len(obj_json) + (len(def_json) if def_json else 0) + n_my * 192
        path = ("xrp_scene_create + " + ("xrp_render" if march == "plain" else "xrp_render_proposal")
                + ", pinned host output")

        def e2e_call():
            with X.Scene(obj_json, def_json) as s2:
                if march == "plain":
                    X.render(s2, my_angles, out=out_host, **kw)
                else:  # the network trained on the resident scene applies to this copy
                    X.render_proposal(s2, prop, my_angles, resolution=res, ds=w.ds, R=w.R,
                                      fov=w.fov, segment=64, refine=march == "proposal",
                                      trace=_trace_mode(march), out=out_host,
                                      integration=args.integration)
    if not args.no_e2e:
        e2e_call()  # warm
        for _ in range(max(1, min(args.steps, 3))):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            e2e_call()
            e2e_times.append(time.perf_counter() - t0)
    t_e2e, _ = job_time(float(np.mean(e2e_times)) if e2e_times else float("nan"), 0, dev)
    e2e_value = rays_total / t_e2e / 1e6

    peaks = measured_peaks()
    fp32_peak = fp32_peak_tflops(torch)
    fps = FLOPS[args.workload]
    if evals_step is None:
        achieved = samples_step * fps / t_step / 1e12
        work = "lattice samples evaluated x FLOPs per sample"
    else:
        # a certificate evaluation adds the bound (about 12 FLOPs beyond the
        # density, sharing its deformation and geometry)
        achieved = evals_step * (fps + 12) / t_step / 1e12
        work = ("evaluations the march makes (counter pass) x (FLOPs per sample + 12 for the "
                "certificate); the plain integrator would evaluate samples_per_step")
    fp32_roof = {"bound": "fp32", "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                 "frac": achieved / fp32_peak if fp32_peak else None,
                 "peak_source": "measured in this run: CUDA-core SGEMM, TF32 off",
                 "flops_per_sample": fps, "work": work, "evaluations_per_step": evals_step}
    roof = dict(fp32_roof)
    if is_voxel and args.volume_path == "gather":
        # the voxel kernel's binding unit is the texture path: two tld4
        # gathers (16 B each) per evaluated sample, against the gather rate
        # measured in this run by xrp_probe_gather_rate
        import ctypes
        from xray_projection_render_gb300 import _lib as XL
        gr = ctypes.c_double(0.0)
        XL.check(XL.load().xrp_probe_gather_rate(ctypes.byref(gr)), "xrp_probe_gather_rate")
        g_ach = 2.0 * samples_step / t_step
        roof = {"bound": "tex", "achieved": g_ach * 16 / 1e9, "peak": gr.value * 16 / 1e9, "unit": "GB/s",
                "frac": g_ach / gr.value if gr.value else None,
                "peak_source": "measured in this run: tld4 gathers on an L1-resident layered texture",
                "note": "gathered bytes (2 x 16 B per sample) vs the measured gather throughput",
                "fp32": fp32_roof}
    traffic = TRAFFIC_PER_VIEW.get(args.workload) if march == "plain" else None
    cfg = workload_config(w, march, world, args.workload, args.integration)
    if is_voxel:
        cfg["volume_path"] = args.volume_path
    elif march == "plain":
        cfg["plain_fp64"] = args.plain_fp64
    line = {
        "metric": (VOXEL_METRIC if args.workload == "voxel" else
                   HEADLINE_METRIC if args.workload == "lattice" else f"Mrays/s on 1 GB300 ({w.name})"),
        "value": value, "unit": "Mrays/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_step * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded)", "config": cfg, "path": MARCH_PATHS[march],
        "e2e": {"value": e2e_value, "unit": "Mrays/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": int(n_my * img * 4), "path": path},
        "gpu_launches": args.steps * launches_per_step(march, n_my * img, is_voxel, args.integration,
                                                       args.plain_fp64, non_affine(w.deformation)),
        "roofline": dict(roof, **{
            "traffic": traffic * n_my if traffic else None,
            "traffic_note": ("constant: DRAM bytes per view from an ncu capture of the same kernel "
                             "on 8 views, times the views") if traffic else "not captured for this path",
            "samples_per_step": samples_step,
            "fp64_fallback_fraction": fp64 / max(samples, 1),
            "hbm_peak_gbs_measured": peaks.get("hbm_gbs")}),
        "clocks": clk.summary(),
    }
    if rank == 0:
        line["error_vs_fp64"] = err
        if cb is not None:
            line["cpu_baseline"] = cb
    if (rank == 0 and world == 1 and not args.no_compare and not is_voxel and march != "plain"
            and args.integration == "simple"):
        del out
        torch.cuda.empty_cache()
        line.update(compare_paths(X, torch, scene, w, value, stream, flush, args))
        if args.workload == "lattice" and not (args.views or args.res):
            scene.close()
            line["gyroid"] = secondary_gyroid(X, torch, W, stream, flush, args)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if prop is not None:
        prop.close()
    scene.close()
    if world > 1:
        torch.distributed.destroy_process_group()


def bench_batched(args):
    """The batch of 64 seeded scenes (1-200 primitives, resolution 256/512/1024,
    8-128 views, ds 0.005) in one persistent launch per step, replayed from
    the CUDA graph xrp_batch_create captured (autotuned tile shape and grid)."""
    import torch
    import __graft_entry__ as G
    import xray_projection_render_gb300 as X
    from xray_projection_render_gb300 import workloads as W
    from xray_projection_render_gb300.sharding import job_time, shard
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    G.build()
    ws = shard(W.batched_scenes(args.scenes), rank, world)  # scene k on rank k mod N
    if args.res or args.views:  # reduced copies (profiling)
        ws = [W.reduced(w, args.res or w.res, args.views or None) for w in ws]
    ds = 0.005
    scenes = [X.Scene(w.obj, w.deformation) for w in ws]
    items = [(s, w.angles, w.res) for s, w in zip(scenes, ws)]
    dev = torch.device("cuda", local)
    stream = torch.cuda.current_stream(dev)
    flush = torch.empty(64 * 1024 * 1024, device=dev, dtype=torch.float32)
    march = args.march if args.march != "auto" else "trace"
    trace = _trace_mode(march)
    b = X.Batch(items, ds=ds, autotune=True, trace=trace, integration=args.integration)
    info = b.info()
    for _ in range(args.warmup):
        b.render(stream)
    torch.cuda.synchronize()
    # samples per step: each scene's counter pass on one view, scaled
    samples = 0.0
    for s, w in zip(scenes, ws):
        _, n, _ = X.render(s, w.angles[:1], resolution=w.res, ds=ds, stats=True,
                           integration=args.integration)
        samples += n * len(w.angles)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    times = []
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            flush.fill_(1.0)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            b.render(stream)
            e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1) * 1e-3)
    t_step = float(np.mean(times))
    rays = info["rays"]
    # the same work as one xrp_render_device call per scene (for comparison)
    seq_out = torch.empty(max(len(w.angles) * w.res * w.res for w in ws), device=dev)
    for rep in range(2):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for s, w in zip(scenes, ws):
            X.render(s, w.angles, resolution=w.res, ds=ds, out=seq_out, stream=stream)
        torch.cuda.synchronize()
        t_seq = time.perf_counter() - t0
    t_step, rays = job_time(t_step, rays, dev)
    rays = int(rays)
    value = rays / t_step / 1e6
    # end to end: a new batch through the public API (scene flattening and
    # upload, batch creation without tuning, graph replay, every item's
    # images copied to pinned host memory)
    e2e_times, d2h = [], 0
    if not args.no_e2e:
        outs = [torch.empty((len(w.angles), w.res, w.res), dtype=torch.float32).pin_memory() for w in ws]
        d2h = sum(o.numel() * 4 for o in outs)
        objs = [(json.dumps(w.obj), json.dumps(w.deformation) if w.deformation else None) for w in ws]
        h2d = sum(len(o) + (len(d) if d else 0) for o, d in objs) + sum(len(w.angles) * 192 for w in ws)
        from xray_projection_render_gb300 import _lib as XL
        for rep in range(1 + max(1, min(args.steps, 2))):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            sc2 = [X.Scene(o, d) for o, d in objs]
            with X.Batch([(s2, w.angles, w.res) for s2, w in zip(sc2, ws)], ds=ds, autotune=False,
                         trace=trace, integration=args.integration) as b2:
                b2.render()
                for k, o in enumerate(outs):
                    XL.check(XL.load().xrp_batch_copy_item(b2._h, k, ctypes_ptr(o)), "xrp_batch_copy_item")
            for s2 in sc2:
                s2.close()
            if rep:
                e2e_times.append(time.perf_counter() - t0)
    t_e2e = float(np.mean(e2e_times)) if e2e_times else float("nan")
    fp32_peak = fp32_peak_tflops(torch)
    line = {
        "metric": BATCH_METRIC,
        "value": value, "unit": "Mrays/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_step * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded, seed 4)",
        "config": batched_config(args.scenes, world, args.integration),
        "batch": {"scenes": len(ws), "rays": rays, "tile": f'{info["tile_w"]}x{info["tile_h"]}',
                  "blocks_per_sm": info["blocks_per_sm"], "autotune_ms": info["tune_ms"],
                  "graph": "one CUDA graph replay per step",
                  "march": {"trace": "certificate tracing (ray bounds: every scene is affine)",
                            "ball": "certificate tracing (ball certificates)"}.get(march, "plain"),
                  "per_scene_calls_mrays": info["rays"] / t_seq / 1e6},
        "e2e": {"value": rays / t_e2e / 1e6 if e2e_times else None, "unit": "Mrays/s",
                "h2d_bytes_per_step": h2d if e2e_times else 0, "d2h_bytes_per_step": d2h,
                "path": "xrp_scene_create x64 + xrp_batch_create (no tuning) + xrp_batch_render + "
                        "xrp_batch_copy_item into pinned host memory"},
        "gpu_launches": args.steps,
        "roofline": {"bound": "fp32", "achieved": None, "peak": fp32_peak, "unit": "TFLOP/s",
                     "frac": None, "traffic": None,
                     "note": "per-sample work varies with each scene's candidate lists; "
                             "samples per step reported instead",
                     "samples_per_step": samples, "samples_per_s": samples / t_step},
        "clocks": clk.summary(),
    }
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline_multi(ws[:8], args.cpu_seconds, args.integration)
    if rank == 0:
        # error of the replayed batch against FP64: seeded rays of the first
        # eight items, from the items' images (copied back after the timing)
        worst_rel, worst_abs, nrays = 0.0, 0.0, 0
        rng = np.random.default_rng(4321)
        for k, w in enumerate(ws[:8]):
            rays = draw_rays(rng, len(w.angles), w.res, 2500)
            host = b.item(k)
            got = host[rays[:, 0], rays[:, 1], rays[:, 2]].astype(np.float64)
            ref = oracle_rays(dataclasses.replace(w, ds=ds), w.angles, rays, integration=args.integration)
            d = np.abs(got - ref)
            worst_rel = max(worst_rel, float(np.max(d / ref)))
            worst_abs = max(worst_abs, float(np.max(d)))
            nrays += len(rays)
        line["error_vs_fp64"] = {"max_rel": worst_rel, "max_abs": worst_abs, "rays": nrays,
                                 "items": "first 8 of the batch"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    b.close()
    for s in scenes:
        s.close()
    if world > 1:
        torch.distributed.destroy_process_group()


def bench_small_kernel(args):
    """Device-side image finishing (64 images of 1024^2, 4 B read and 2 + 2 B
    written per pixel: HBM-bound) or the volume export of the deformed
    lattice at 256^3 (SM-bound), timed with CUDA events, inputs resident."""
    import torch
    import __graft_entry__ as G
    import xray_projection_render_gb300 as X
    from xray_projection_render_gb300 import workloads as W
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    G.build()
    dev = torch.device("cuda", local)
    stream = torch.cuda.current_stream(dev)
    flush = torch.empty(64 * 1024 * 1024, device=dev, dtype=torch.float32)
    peaks = measured_peaks()
    if args.workload == "finish":
        n, res = 64, 1024
        img = torch.rand((n, res, res), device=dev)
        step = lambda: X.finish_images(img, stream=stream)  # noqa: E731
        units, unit = n * res * res, "Mpixels/s"
        bytes_per_unit = 4 + 2 + 2
        metric = "Mpixels/s of device-side image finishing (64 images of 1024^2)"
        cfg = {"workload": "finish_64x1024^2", "images": n, "res": res}
    else:
        w = W.deformed_lattice()
        res = 256
        scene = X.Scene(w.obj, w.deformation)
        step = lambda: X.voxelize_scene(scene, res)  # noqa: E731  (host copies included)
        units, unit = res ** 3, "Mvoxels/s"
        bytes_per_unit = None
        metric = "Mvoxels/s of the volume export (deformed lattice, 256^3, host copy included)"
        cfg = {"workload": "voxelize_lattice_256^3", "res": res}
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    times = []
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            flush.fill_(1.0)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            step()
            e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1) * 1e-3)
    t = float(np.mean(times))
    line = {"metric": metric, "value": units / t / 1e6, "unit": unit, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)", "config": cfg,
            "gpu_launches": args.steps, "clocks": clk.summary()}
    if bytes_per_unit:
        ach = units * bytes_per_unit / t / 1e9
        pk = peaks.get("hbm_gbs")
        line["roofline"] = {"bound": "hbm", "achieved": ach, "peak": pk, "unit": "GB/s",
                            "frac": ach / pk if pk else None, "traffic": None,
                            "peak_source": "MEASURED_PEAKS.json hbm_gbs"}
    print(json.dumps(line), flush=True)


def ctypes_ptr(t):
    import ctypes
    return ctypes.c_void_p(t.data_ptr())


BATCH_METRIC = "Mrays/s on 1 GB300 (64 uneven scenes, one persistent launch per step)"


def batched_config(scenes, world, integration="simple"):
    return {"workload": f"batched_scenes_{scenes}", "scenes": scenes, "ds": 0.005,
            "integrator": integration, "R": 4.0, "fov": 40.0,
            "scene_definition": "collections of 1-200 seeded primitives, resolution 256/512/1024, "
                                "8-128 views (seed 4)",
            "l2": "flushed before every timed step (256 MiB write); output > L2",
            "parallelism": f"scenes k mod {world}"}


def cpu_baseline_multi(ws, seconds, integration="simple"):
    """The oracle on seeded random rays spread over several scenes."""
    parts = [cpu_baseline(w, seconds / len(ws), integration=integration)[0] for w in ws]
    rays_s = len(ws) / sum(1.0 / p["value"] for p in parts)  # equal rays per scene
    out = dict(parts[0])
    out["value"] = rays_s
    out["sample"] = f"{len(ws)} scenes of the batch, seeded random rays each ({seconds:.0f} s total)"
    return out


def _trace_mode(march):
    """render_proposal / Batch `trace` argument of a --march choice."""
    return {"trace": True, "ball": "ball"}.get(march, False)


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.impl == "reference_gpu":
        return run_reference_gpu(args)
    if args.workload == "batched":
        return bench_batched(args)
    if args.workload in ("finish", "voxelize"):
        return bench_small_kernel(args)
    return bench_scene(args)


if __name__ == "__main__":
    main()
