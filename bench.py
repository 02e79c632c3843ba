"""Benchmark: Mrays/s of the GB300 projection engine on the voxel-grid workload.

Workload (one step = one pass of the hot path over one batch): the 256^3 FP32
grid of 64 seeded Gaussians rendered from 180 views (azimuth 0, 2, ..., 358
degrees, polar 90) at 1024x1024 with the uniform-step integrator, ds = half a
voxel (2/256/2), R = 4, fov = 40 -- 188.7 M rays per step.

value     : device throughput, volume resident in HBM, output to a device
            buffer, L2 flushed (256 MiB write) before every timed step, each
            step timed with CUDA events on the launching stream.
e2e       : the same metric through the reference ABI call
            RenderVolumeProjectionsCUDA with pinned host buffers (volume
            upload and image download inside the timed region).
roofline  : the voxel kernel is bound by its texture gathers (two tld4 of
            16 B per sample, the exact sample count from a counter pass):
            achieved gathered bytes/s against the gather throughput measured
            in this run (xrp_probe_gather_rate, L1-resident texture).  The
            FP32 view (58 FLOPs per sample against a CUDA-core SGEMM with
            TF32 off, measured in this run) is kept under "fp32"; the
            analytic workloads report the FP32 view.
cpu_baseline / --impl reference: the FP64 CPU restatement of the reference
            path (oracle/), on all host cores, on a seeded ray subset.

Multi-GPU: the path has no exchange step; N processes render disjoint view
subsets (view k on rank k mod N) with no collective ("scaling": "weak").
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

FLOPS_PER_SAMPLE = 58  # 8 common (position + accumulate) + 50 trilinear
METRIC = "Mrays/s on 1 GB300 (uniform-step integrator, voxel grid 256^3, 180 views x 1024^2)"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="engine", choices=["engine", "reference"])
    p.add_argument("--workload", default="voxel",
                   choices=["voxel", "cube", "lattice", "gyroid", "batched", "finish", "voxelize"],
                   help="voxel (default, the headline), one of the analytic scenes, the batch "
                        "of 64 uneven scenes (one persistent launch replayed from a CUDA graph), "
                        "device-side image finishing of 64 images of 1024^2, or the volume "
                        "export of the deformed lattice at 256^3")
    p.add_argument("--scenes", type=int, default=64, help="batched: number of scenes")
    p.add_argument("--march", default="plain",
                   choices=["plain", "trace", "ball", "certificate", "proposal"],
                   help="analytic scenes: plain integrator, per-ray certificate tracing (ray bounds "
                        "for affine deformation chains), tracing with ball certificates only, "
                        "segment march with certificates and no network, or the trained proposal")
    p.add_argument("--views", type=int, default=0, help="view count (0: the workload's)")
    p.add_argument("--res", type=int, default=0, help="resolution (0: the workload's)")
    p.add_argument("--cpu-seconds", type=float, default=12.0)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-e2e", action="store_true", help="skip the host-buffer ABI timing")
    p.add_argument("--volume-path", default="gather", choices=["gather", "loads"],
                   help="voxel reads: texture gathers (default) or per-tap loads")
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


def cpu_baseline(workload, seconds, threads=None):
    """FP64 oracle on a seeded subset of the workload's rays, all host cores."""
    from oracle import oracle as O
    threads = threads or os.cpu_count() or 1
    rng = np.random.default_rng(1234)
    if workload.volume is not None:
        from xray_projection_render_gb300 import engine  # camera rows only (host code)
        cams21 = engine.xray_camera_params(workload.angles, workload.R, workload.fov)
        scene = O.VolumeABIScene(workload.volume)

        def render(rays):
            scene.render_rays(cams21, workload.res, np.float32(workload.ds), rays, nthreads=threads)
    else:
        scene = O.Scene(workload.obj, workload.deformation)

        def render(rays):
            O.render(scene, workload.angles, workload.res, workload.ds, R=workload.R,
                     fov=workload.fov, rays=rays, nthreads=threads)

    def run(n):
        rays = np.stack([rng.integers(0, len(workload.angles), n), rng.integers(0, workload.res, n),
                         rng.integers(0, workload.res, n)], 1).astype(np.int32)
        t = time.perf_counter()
        render(rays)
        return time.perf_counter() - t

    n = 2000
    dt = run(n)
    n2 = int(max(2000, min(40_000_000, n * seconds / max(dt, 1e-3))))
    dt2 = run(n2)
    return {"value": n2 / dt2 / 1e6, "unit": "Mrays/s", "cores": threads, "kind": "port",
            "sample": f"{n2} seeded random rays of {workload.name} ({dt2:.1f} s)"}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from xray_projection_render_gb300 import workloads as W
    if args.workload in ("finish", "voxelize"):
        print(json.dumps({"impl": "reference", "unavailable":
                          "the reference runs this step in Go on the host (PNG / raw writing); "
                          "no CPU arm is timed for it here"}), flush=True)
        return
    if args.workload == "batched":
        ws = W.batched_scenes(64)[:8]
        w = W.Workload("batched_scenes_64", None, None, [], 0, 0.005)
        measure = lambda sec: cpu_baseline_multi(ws, sec)  # noqa: E731
    else:
        w = make_workload(args.workload, W, args.views, args.res)
        measure = lambda sec: cpu_baseline(w, sec)  # noqa: E731
    vals = []
    for i in range(args.warmup + args.steps):
        cb = measure(max(2.0, args.cpu_seconds / max(1, args.steps)))
        if i >= args.warmup:
            vals.append(cb["value"])
    v = float(np.median(vals))
    cb["value"] = v
    line = {"impl": "reference",
            "metric": METRIC if args.workload == "voxel" else f"Mrays/s on 1 GB300 ({w.name})",
            "value": v, "unit": "Mrays/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded)",
            "config": {"workload": w.name, "views": len(w.angles), "res": w.res, "ds": w.ds},
            "cpu_baseline": cb,
            "e2e": {"value": v, "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# Algorithmic FP32 work per evaluated sample (FMA = 2), from the per-item
# table of the benchmark definitions: common 8 + object terms.
FLOPS = {
    "voxel": 58,     # 50 trilinear
    "cube": 54,      # sphere 9 + box 9 + cylinder 23 + collection 3 + clip 2
    "lattice": 437,  # linear deformation 18 + fold/bounds 27 + 16 cylinders x 23 + 16
    "gyroid": 53,    # gyroid 13 (+6 SFU) + sigmoid 5 (+2 SFU) + fold/bounds 27
}


# DRAM bytes (read + write) of the render kernel per view, from the ncu
# captures summarised in profiles/ (small cases scaled by view count: the
# grid streams through L2 once per view, so traffic grows with the views).
TRAFFIC = {
    "voxel": {"bytes_per_view": (404.93e6 + 47.01e6) / 8,
              "source": "profiles/k_voxel_gather_voxel256_8x1024.md (8-view capture, x views)"},
    "lattice": {"bytes_per_view": (0.611e6 + 0.472e6) / 2 * 4,
                "source": "profiles/k_render_lattice_2x512.md (2 views at 512^2, x views x 4)"},
}


def make_workload(name, W, views, res):
    if name == "voxel":
        return W.voxel_blobs(res or 1024, views or 180)
    if name == "cube":
        w = W.cube_minus_sphere_cylinder(res or 512)
    elif name == "lattice":
        w = W.deformed_lattice(res or 1024, 360)
    elif name == "gyroid":
        w = W.gyroid_sigmoid(res or 2048, 720)
    else:
        raise ValueError(name)
    if views:
        w = W.reduced(w, w.res, views)
    return w


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
    trace = _trace_mode(args)
    b = X.Batch(items, ds=ds, autotune=True, trace=trace)
    info = b.info()
    for _ in range(args.warmup):
        b.render(stream)
    torch.cuda.synchronize()
    # samples per step: each scene's counter pass on one view, scaled
    samples = 0.0
    for s, w in zip(scenes, ws):
        _, n, _ = X.render(s, w.angles[:1], resolution=w.res, ds=ds, stats=True)
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
                         trace=trace) as b2:
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
        "metric": "Mrays/s on 1 GB300 (64 uneven scenes, one persistent launch per step)",
        "value": value, "unit": "Mrays/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_step * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded, seed 4)",
        "config": {"workload": "batched_scenes_64", "scenes": len(ws), "rays": rays, "ds": ds,
                   "integrator": "simple", "R": 4.0, "fov": 40.0,
                   "l2": "flushed before every timed step (256 MiB write); output > L2",
                   "tile": f'{info["tile_w"]}x{info["tile_h"]}', "blocks_per_sm": info["blocks_per_sm"],
                   "autotune_ms": info["tune_ms"], "graph": "one CUDA graph replay per step",
                   "march": {"trace": "certificate tracing (ray bounds: every scene is affine)",
                             "ball": "certificate tracing (ball certificates)"}.get(args.march, "plain"),
                   "per_scene_calls_mrays": info["rays"] / t_seq / 1e6,
                   "parallelism": f"scenes k mod {world}"},
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
        line["cpu_baseline"] = cpu_baseline_multi(ws[:8], args.cpu_seconds)
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


def cpu_baseline_multi(ws, seconds):
    """The oracle on seeded random rays spread over several scenes."""
    parts = [cpu_baseline(w, seconds / len(ws)) for w in ws]
    rays_s = len(ws) / sum(1.0 / p["value"] for p in parts)  # equal rays per scene
    out = dict(parts[0])
    out["value"] = rays_s
    out["sample"] = f"{len(ws)} scenes of the batch, seeded random rays each ({seconds:.0f} s total)"
    return out


def _trace_mode(args):
    """render_proposal / Batch `trace` argument of a --march choice."""
    return {"trace": True, "ball": "ball"}.get(args.march, False)


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "batched":
        return bench_batched(args)
    if args.workload in ("finish", "voxelize"):
        return bench_small_kernel(args)
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
    is_voxel = w.volume is not None
    my_angles = shard(w.angles, rank, world)  # view k on rank k mod N, no exchange
    n_my = len(my_angles)
    res = w.res
    img = res * res
    dev = torch.device("cuda", local)
    stream = torch.cuda.current_stream(dev)
    vols = [torch.from_numpy(w.volume).to(dev)] if is_voxel else []
    scene = X.Scene(w.obj, w.deformation, vols)
    out = torch.empty((n_my, res, res), device=dev, dtype=torch.float32)
    flush = torch.empty(64 * 1024 * 1024, device=dev, dtype=torch.float32)  # 256 MiB > L2
    kw = dict(resolution=res, ds=w.ds, R=w.R, fov=w.fov, volume_path=args.volume_path)

    prop = None
    if args.march == "proposal":
        prop = X.Proposal(scene, my_angles, resolution=res, ds=w.ds, R=w.R, fov=w.fov, segment=64)

    def step():
        if args.march == "plain":
            X.render(scene, my_angles, out=out, stream=stream, **kw)
        else:
            X.render_proposal(scene, prop, my_angles, resolution=res, ds=w.ds, R=w.R, fov=w.fov,
                              segment=64, refine=args.march == "proposal",
                              trace=_trace_mode(args), out=out, stream=stream)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    # exact sample count of one step (counter pass, untimed, on a view subset)
    nstat = max(1, min(8, n_my))
    _, samples, fp64 = X.render(scene, my_angles[:nstat], stats=True, **kw)
    samples_step = samples * n_my / nstat
    evals_step = None
    if args.march != "plain" and not is_voxel:
        # evaluations the march actually makes (density + certificate radius
        # per evaluation, or one density per dense sample)
        _, pst = X.render_proposal(scene, prop, my_angles[:nstat], resolution=res, ds=w.ds, R=w.R,
                                   fov=w.fov, segment=64, refine=args.march == "proposal",
                                   trace=_trace_mode(args), stats=True)
        evals_step = (pst["evaluations"] + pst["dense_samples"]) * n_my / nstat
    if world > 1:
        torch.distributed.barrier()
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
    t_step, rays_total = job_time(float(np.mean(times)), n_my * img, dev)
    value = rays_total / t_step / 1e6

    # end to end through the host-facing C ABI, pinned host buffers, inputs
    # uploaded and images read back inside the timed region
    e2e_times = []
    out_host = None if args.no_e2e else torch.empty((n_my, res, res), dtype=torch.float32).pin_memory()
    if is_voxel:
        cams21 = X.xray_camera_params(my_angles, w.R, w.fov)
        h2d = int(w.volume.nbytes + cams21.nbytes)
        path = "RenderVolumeProjectionsCUDA, pinned host buffers"
        if not args.no_e2e:
            vol_host = torch.from_numpy(w.volume).pin_memory()

        def e2e_call():
            X.render_volume_projections(vol_host.numpy(), cams21, res, w.ds, out=out_host)
    else:
        obj_json = json.dumps(w.obj)
        def_json = json.dumps(w.deformation) if w.deformation else None
        h2d = len(obj_json) + (len(def_json) if def_json else 0) + n_my * 192
        path = "xrp_scene_create + xrp_render, pinned host output"

        def e2e_call():
            with X.Scene(obj_json, def_json) as s2:
                if args.march == "plain":
                    X.render(s2, my_angles, out=out_host, **kw)
                else:  # the network trained on the resident scene applies to this copy
                    X.render_proposal(s2, prop, my_angles, resolution=res, ds=w.ds, R=w.R,
                                      fov=w.fov, segment=64, refine=args.march == "proposal",
                                      trace=_trace_mode(args), out=out_host)
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
        # a certificate evaluation adds the radius (about 12 FLOPs beyond
        # the density, sharing its deformation and geometry)
        achieved = evals_step * (fps + 12) / t_step / 1e12
        work = ("evaluations the march makes (counter pass) x (FLOPs per sample + 12 for the "
                "certificate radius); the plain integrator would evaluate samples_per_step")
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
    line = {
        "metric": METRIC if args.workload == "voxel" else f"Mrays/s on 1 GB300 ({w.name})",
        "value": value, "unit": "Mrays/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_step * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded)",
        "config": {"workload": w.name, "views": len(w.angles), "res": res, "ds": w.ds,
                   "integrator": "simple", "R": w.R, "fov": w.fov,
                   "march": None if is_voxel else args.march,
                   "l2": "flushed before every timed step (256 MiB write)",
                   "volume_path": args.volume_path if is_voxel else None,
                   "parallelism": f"views k mod {world}"},
        "e2e": {"value": e2e_value, "unit": "Mrays/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": int(n_my * img * 4), "path": path},
        # plain: one render launch per step (all views); march modes: per
        # launch group of at most 8 M rays, the march, its FP64 pass and
        # the exp pass
        "gpu_launches": args.steps * (1 if (args.march == "plain" or is_voxel)
                                      else 3 * -(-n_my * img // (1 << 23))),
        "roofline": dict(roof, **{
                     "traffic": TRAFFIC.get(args.workload, {}).get("bytes_per_view", 0) * n_my or None,
                     "traffic_source": TRAFFIC.get(args.workload, {}).get("source"),
                     "samples_per_step": samples_step,
                     "fp64_fallback_fraction": fp64 / max(samples, 1),
                     "hbm_peak_gbs_measured": peaks.get("hbm_gbs")}),
        "clocks": clk.summary(),
    }
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(w, args.cpu_seconds)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if prop is not None:
        prop.close()
    scene.close()
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
