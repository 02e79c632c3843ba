"""The proposal march on the GPU: the tensor-core training step against the
FP64 network of oracle/mlp.py; the march against the FP64 oracle (every
sample is evaluated or covered by a certificate, so the bar is the plain
integrator's 1e-5 relative, with or without the network); and what the
trained network changes in work and speed against the march without it."""
import time

import numpy as np
import pytest

from oracle import mlp as M
from oracle import oracle as O
from xray_projection_render_gb300 import workloads as W

pytestmark = pytest.mark.gpu

REL_TOL = 1e-5  # relative transmittance error vs the FP64 oracle, as the plain integrator


@pytest.fixture(scope="module")
def X():
    import __graft_entry__ as g
    g.build()
    import xray_projection_render_gb300 as X
    return X


def _oracle(w):
    return O.render(O.Scene(w.obj, w.deformation), w.angles, w.res, w.ds, R=w.R, fov=w.fov)


def test_mlp_grad_matches_fp64_oracle(X):
    rng = np.random.default_rng(5)
    a = rng.uniform(-1, 1, (1000, 3))
    b = a + rng.normal(0, 0.1, (1000, 3))
    bits = M.bf16_bits(M.segment_features(a, b))
    Xv = M.from_bf16_bits(bits)
    y = (rng.uniform(size=1000) < 0.3).astype(np.float32)
    p = M.init_params(3).astype(np.float32)
    grad, loss, logits = X.mlp_grad(p, bits, y, pos_weight=8.0)
    l_ref, z_ref, g_ref = M.forward_backward(p.astype(np.float64), Xv, y, 8.0, emulate=True)
    assert abs(loss - l_ref) <= 1e-4 * abs(l_ref)
    assert np.max(np.abs(logits - z_ref)) <= 1e-3 * (1 + np.max(np.abs(z_ref)))
    rel = np.linalg.norm(grad - g_ref) / np.linalg.norm(g_ref)
    assert rel <= 5e-3, rel
    for name, (o, n) in M.OFF.items():
        gr = g_ref[o:o + n]
        d = np.linalg.norm(grad[o:o + n] - gr) / max(np.linalg.norm(gr), 1e-30)
        assert d <= 2e-2, (name, d)


def test_mlp_grad_small_batches_and_padding(X):
    # rows not a multiple of the 128-row tile: padded rows contribute nothing
    rng = np.random.default_rng(6)
    for rows in (1, 37, 129):
        bits = M.bf16_bits(rng.normal(size=(rows, 64)))
        y = (rng.uniform(size=rows) < 0.5).astype(np.float32)
        p = M.init_params(rows).astype(np.float32)
        grad, loss, _ = X.mlp_grad(p, bits, y, pos_weight=2.0)
        l_ref, _, g_ref = M.forward_backward(p.astype(np.float64), M.from_bf16_bits(bits), y, 2.0)
        assert abs(loss - l_ref) <= 1e-4 * abs(l_ref)
        assert np.linalg.norm(grad - g_ref) <= 5e-3 * np.linalg.norm(g_ref)


CASES = {
    "gyroid_sigmoid": lambda: W.reduced(W.gyroid_sigmoid(), 48, 2),
    "deformed_lattice": lambda: W.reduced(W.deformed_lattice(), 40, 2),
    "cube_minus_sphere_cylinder": lambda: W.cube_minus_sphere_cylinder(48),
    "batched_scene0": lambda: W.reduced(W.batched_scenes(1)[0], 48, 2),
}


def _affine_collection():
    # every primitive under a chain of affine steps (ray certificates)
    coll = {"type": "object_collection", "objects": [
        {"type": "sphere", "center": [0.1, -0.2, 0.05], "radius": 0.4, "rho": 0.7},
        {"type": "box", "center": [0.0, 0.2, 0.0], "sides": [0.5, 0.3, 0.9], "rho": 0.5},
        {"type": "cylinder", "p0": [-0.5, -0.5, -0.2], "p1": [0.5, 0.4, 0.3], "radius": 0.1},
        {"type": "parallelepiped", "origin": [0.0, 0.0, 0.0], "v0": [0.4, 0.1, 0.0],
         "v1": [0.0, 0.5, 0.1], "v2": [0.1, 0.0, 0.3], "rho": 0.9},
        {"type": "gyroid", "center": [0.0, 0.0, 0.0], "scale": 0.1, "thickness": 0.2, "rho": 1.0}]}
    deform = {"type": "composed", "deformations": [
        {"type": "affine", "matrix": [[1.1, 0.0, 0.1], [0.0, 0.9, 0.0], [0.05, 0.0, 1.0]]},
        {"type": "rigid", "displacements": [0.05, -0.1, 0.02]},
        {"type": "linear", "strains": [0.02, -0.01, 0.05, 0.01, 0.0, 0.03]}]}
    return W.Workload("affine_collection", coll, deform, [(10.0, 80.0), (200.0, 120.0)], 48, 0.004)


GAUSS = {"type": "gaussian", "amplitudes": [0.1, -0.05, 0.02], "sigmas": [0.3, 0.3, 0.5],
         "centers": [0.0, 0.1, 0.0]}


def _gaussian_collection():
    # every primitive under a gaussian chain (curve certificates)
    w = _affine_collection()
    return W.Workload("gaussian_collection", w.obj, GAUSS, w.angles, w.res, w.ds)


def _gaussian_lattice():
    base = W.reduced(W.deformed_lattice(), 40, 2)
    return W.Workload("gaussian_lattice", base.obj, GAUSS, base.angles, base.res, base.ds)


TRACE_CASES = dict(CASES, affine_collection=_affine_collection, gaussian_collection=_gaussian_collection,
                   gaussian_lattice=_gaussian_lattice)


@pytest.mark.parametrize("mode", [True, "ball"])
@pytest.mark.parametrize("integration", ["simple", "hierarchical"])
@pytest.mark.parametrize("name", sorted(TRACE_CASES))
def test_certificate_tracing_matches_oracle(X, name, integration, mode):
    """Tracing with ray bounds (affine chains), curve bounds (the gyroid's
    sigmoid chain, gaussian chains) and with ball certificates only."""
    w = TRACE_CASES[name]()
    ref = O.render(O.Scene(w.obj, w.deformation), w.angles, w.res, w.ds, R=w.R, fov=w.fov,
                   integration=integration)
    with X.Scene(w.obj, w.deformation) as s:
        img, st = X.render_proposal(s, None, w.angles, resolution=w.res, ds=w.ds, R=w.R, fov=w.fov,
                                    trace=mode, stats=True, integration=integration)
    assert np.max(np.abs(img - ref) / ref) <= REL_TOL
    assert st["evaluations"] > 0 and st["fp64_list_overflow"] == 0


def test_ray_certificates_evaluate_less_than_balls(X):
    # the lattice (linear strain): the ray bound jumps straight to the next
    # strut or cell face instead of approaching it geometrically
    w = W.reduced(W.deformed_lattice(), 64, 2)
    with X.Scene(w.obj, w.deformation) as s:
        kw = dict(resolution=w.res, ds=w.ds, R=w.R, fov=w.fov, stats=True)
        a, st_ray = X.render_proposal(s, None, w.angles, trace=True, **kw)
        b, st_ball = X.render_proposal(s, None, w.angles, trace="ball", **kw)
    assert np.max(np.abs(a - b) / b) <= 2 * REL_TOL
    assert 2 * st_ray["evaluations"] < st_ball["evaluations"]
    print(f"\nevaluations: ray {st_ray['evaluations']}, ball {st_ball['evaluations']}")


def test_curve_certificates_evaluate_less_than_balls(X):
    # the gyroid under the sigmoid: the curve bound reaches the band edge in
    # a step or two where balls approach it geometrically
    w = W.reduced(W.gyroid_sigmoid(), 96, 2)
    with X.Scene(w.obj, w.deformation) as s:
        kw = dict(resolution=w.res, ds=w.ds, R=w.R, fov=w.fov, stats=True)
        a, st_curve = X.render_proposal(s, None, w.angles, trace=True, **kw)
        b, st_ball = X.render_proposal(s, None, w.angles, trace="ball", **kw)
    assert np.max(np.abs(a - b) / b) <= 2 * REL_TOL
    assert 2 * st_curve["evaluations"] < st_ball["evaluations"]
    print(f"\nevaluations: curve {st_curve['evaluations']}, ball {st_ball['evaluations']}")


@pytest.mark.parametrize("name", sorted(CASES))
@pytest.mark.parametrize("segment,refine", [(32, False), (128, False), (64, True), (256, True)])
def test_certificate_march_matches_oracle(X, name, segment, refine):
    w = CASES[name]()
    ref = _oracle(w)
    with X.Scene(w.obj, w.deformation) as s:
        img, st = X.render_proposal(s, None, w.angles, resolution=w.res, ds=w.ds, R=w.R, fov=w.fov,
                                    segment=segment, refine=refine, stats=True)
        plain = X.render(s, w.angles, resolution=w.res, ds=w.ds, R=w.R, fov=w.fov)
    assert np.max(np.abs(img - ref) / ref) <= REL_TOL
    assert np.max(np.abs(plain - ref) / ref) <= REL_TOL
    assert st["routed_dense"] == 0 and st["mlp_rounds"] == 0
    if not refine:
        assert st["subdivided"] == 0 and st["refined"] == 0
        assert st["certified"] + st["dense"] == st["segments"]
    if name == "gyroid_sigmoid" or (name == "cube_minus_sphere_cylinder" and segment == 32):
        assert st["certified"] > 0
    if refine and name == "gyroid_sigmoid":
        assert st["refined"] > 0


def test_certificate_march_device_path_and_options(X):
    import torch
    w = W.cube_minus_sphere_cylinder(40)
    ref = O.render(O.Scene(w.obj, w.deformation), w.angles, w.res, w.ds, R=w.R, fov=w.fov,
                   density_multiplier=1.7, flat_field=0.3)
    with X.Scene(w.obj) as s:
        out = torch.empty(len(w.angles) * w.res * w.res, device="cuda", dtype=torch.float32)
        X.render_proposal(s, None, w.angles, resolution=w.res, ds=w.ds, R=w.R, fov=w.fov,
                          density_multiplier=1.7, flat_field=0.3, out=out)
        torch.cuda.synchronize()
        img = out.cpu().numpy().reshape(ref.shape)
    assert np.max(np.abs(img - ref) / ref) <= REL_TOL


def test_proposal_rejects_unsupported(X):
    w = W.cube_minus_sphere_cylinder(16)
    with X.Scene(w.obj) as s:
        from xray_projection_render_gb300._lib import EngineError
        with pytest.raises(EngineError):
            X.render_proposal(s, None, w.angles, resolution=16, ds=w.ds, segment=48)
        vol = W.gaussian_blob_volume(8, 2, seed=1)
        with X.Scene({"type": "voxel_grid", "volume": 0}, volumes=[vol]) as sv:
            with pytest.raises(EngineError):
                X.render_proposal(sv, None, w.angles, resolution=16, ds=w.ds)


@pytest.fixture(scope="module")
def gyroid_trained(X):
    w = W.reduced(W.gyroid_sigmoid(), 96, 4)
    s = X.Scene(w.obj, w.deformation)
    P = X.Proposal(s, w.angles, resolution=w.res, ds=w.ds, R=w.R, fov=w.fov, segment=128,
                   train_rays=16384, val_rays=8192, steps=1000, seed=1)
    yield w, s, P
    P.close()
    s.close()


def _work(st):
    # samples evaluated, a certificate evaluation counted as two
    return st["dense_samples"] + 2 * st["evaluations"]


def test_trained_proposal_is_exact_and_routes(X, gyroid_trained):
    w, s, P = gyroid_trained
    info = P.info()
    assert info["train_rows"] > 0 and np.isfinite(info["final_loss"])
    ref = _oracle(w)
    kw = dict(resolution=w.res, ds=w.ds, R=w.R, fov=w.fov, stats=True)
    img, st = X.render_proposal(s, P, w.angles, **kw)
    ref_only, st_r = X.render_proposal(s, None, w.angles, segment=info["segment"], **kw)
    dense_only, st_d = X.render_proposal(s, None, w.angles, segment=info["segment"], refine=False,
                                         **kw)
    for im in (img, ref_only, dense_only):
        assert np.max(np.abs(im - ref) / ref) <= REL_TOL
    assert st["mlp_rounds"] > 0 and st["routed_dense"] + st["subdivided"] > 0
    # the network's routing against the two fixed policies: far less work
    # than integrating every uncertified segment densely, and within 5 % of
    # refining every one (which it does not beat: the certificates already
    # settle what it could skip; measured 1.3 % above)
    assert _work(st) < 0.5 * _work(st_d)
    assert _work(st) <= 1.05 * _work(st_r)
    print(f"\nwork: proposal {_work(st)}, refinement only {_work(st_r)}, dense only {_work(st_d)}"
          f"\nproposal {st}\ninfo {info}")


def test_proposal_speed_against_plain_and_without_network(X, gyroid_trained):
    """Times the plain integrator, the march without the network and the
    proposal on the same rays (device output).  Prints the three rates; the
    assertions are on the results, which must agree whatever the speed."""
    import torch
    w, s, P = gyroid_trained
    res, views = 256, w.angles[:4]
    n = len(views) * res * res
    outs = [torch.empty(n, device="cuda", dtype=torch.float32) for _ in range(3)]

    def timed(fn, reps=3):
        fn()
        torch.cuda.synchronize()
        t = time.perf_counter()
        for _ in range(reps):
            fn()
        torch.cuda.synchronize()
        return (time.perf_counter() - t) / reps

    kw = dict(resolution=res, ds=w.ds, R=w.R, fov=w.fov)
    t_plain = timed(lambda: X.render(s, views, out=outs[0], **kw))
    t_prop = timed(lambda: X.render_proposal(s, P, views, out=outs[1], **kw))
    t_cert = timed(lambda: X.render_proposal(s, None, views, segment=P.info()["segment"],
                                             refine=False, out=outs[2], **kw))
    print(f"\nplain {n / t_plain / 1e6:.1f} Mrays/s, march without network {n / t_cert / 1e6:.1f}, "
          f"proposal {n / t_prop / 1e6:.1f}")
    a, b, c = (o.cpu().numpy() for o in outs)
    assert np.max(np.abs(b - a) / a) <= 2 * REL_TOL
    assert np.max(np.abs(c - a) / a) <= 2 * REL_TOL


def test_certificate_tracing_options(X):
    # multiplier and flat field, device output, both integrators
    import torch
    w = W.reduced(W.gyroid_sigmoid(), 40, 2)
    for integration in ("simple", "hierarchical"):
        ref = O.render(O.Scene(w.obj, w.deformation), w.angles, w.res, w.ds, R=w.R, fov=w.fov,
                       density_multiplier=1.7, flat_field=0.3, integration=integration)
        with X.Scene(w.obj, w.deformation) as s:
            out = torch.empty(len(w.angles) * w.res * w.res, device="cuda", dtype=torch.float32)
            X.render_proposal(s, None, w.angles, resolution=w.res, ds=w.ds, R=w.R, fov=w.fov,
                              density_multiplier=1.7, flat_field=0.3, trace=True,
                              integration=integration, out=out)
            torch.cuda.synchronize()
            img = out.cpu().numpy().reshape(ref.shape)
        assert np.max(np.abs(img - ref) / ref) <= REL_TOL


@pytest.mark.parametrize("obj", [
    {"type": "object_collection", "objects": []},
    {"type": "sphere", "center": [9.0, 9.0, 9.0], "radius": 0.5, "rho": 1.0},
    {"type": "sphere", "center": [0.0, 0.0, 0.0], "radius": 0.5, "rho": 0.0},
], ids=["empty", "outside", "zero_rho"])
def test_tracing_and_march_on_empty_support(X, obj):
    # nothing to integrate: every pixel is exp(-flat_field), as the oracle says
    angles = [(0.0, 90.0), (40.0, 60.0)]
    ref = O.render(O.Scene(obj), angles, 24, 0.01, flat_field=0.25)
    assert np.allclose(ref, np.exp(-0.25))
    with X.Scene(obj) as s:
        for kw in (dict(trace=True), dict(refine=False, segment=32), dict(refine=True)):
            img = X.render_proposal(s, None, angles, resolution=24, ds=0.01, flat_field=0.25, **kw)
            assert np.max(np.abs(img - ref) / ref) <= REL_TOL, kw


def test_tracing_coarse_step(X):
    # ds comparable to the object: few samples, long certificate jumps clamp at k1
    w = W.cube_minus_sphere_cylinder(32)
    for ds in (0.05, 0.2):
        ref = O.render(O.Scene(w.obj), w.angles, 32, ds)
        with X.Scene(w.obj) as s:
            img = X.render_proposal(s, None, w.angles, resolution=32, ds=ds, trace=True)
        assert np.max(np.abs(img - ref) / ref) <= REL_TOL


@pytest.mark.parametrize("name", ["deformed_lattice", "cube_minus_sphere_cylinder", "batched_scene0",
                                  "affine_collection", "gaussian_collection", "gaussian_lattice"])
def test_ray_tracing_matches_plain_at_scale(X, name):
    """Ray certificates with the device's approximate reciprocals and square
    roots, on ~0.6 M rays per scene: traced renders equal the plain
    integrator's (itself checked against the oracle) within the summation
    tolerance."""
    w = TRACE_CASES[name]()
    angles = (w.angles * 4)[:4]
    angles = [(a + 37.0 * k, p) for k, (a, p) in enumerate(angles)]
    res = 384
    with X.Scene(w.obj, w.deformation) as s:
        kw = dict(resolution=res, ds=w.ds, R=w.R, fov=w.fov)
        plain = X.render(s, angles, **kw)
        traced, st = X.render_proposal(s, None, angles, trace=True, stats=True, **kw)
    assert st["fp64_list_overflow"] == 0
    assert np.max(np.abs(traced - plain) / plain) <= 2 * REL_TOL


def test_tracing_large_scene_reads_nodes_from_global_memory(X):
    """A scene whose node table exceeds the 32 KB staged in shared memory
    (300 primitives): the tracing kernel reads the global table."""
    rng = np.random.default_rng(21)
    objs = []
    for _ in range(300):
        c = rng.uniform(-0.8, 0.8, 3).tolist()
        objs.append({"type": "sphere", "center": c, "radius": float(rng.uniform(0.02, 0.08)),
                     "rho": 1.0 if rng.uniform() < 0.7 else -1.0})
    w = W.Workload("many_spheres", {"type": "object_collection", "objects": objs}, None,
                   [(10.0, 80.0), (200.0, 120.0)], 48, 0.005)
    ref = _oracle(w)
    with X.Scene(w.obj, w.deformation) as s:
        for mode in (True, "ball"):
            img = X.render_proposal(s, None, w.angles, resolution=w.res, ds=w.ds, R=w.R, fov=w.fov,
                                    trace=mode)
            assert np.max(np.abs(img - ref) / ref) <= REL_TOL
