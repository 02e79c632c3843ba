"""Parity at the benchmarked sizes.

The deformed lattice (360 views x 1024^2, ds 0.002, up to 3,480 samples per
ray) and the gyroid under the sigmoid deformation (720 views x 2048^2,
ds 0.001) are rendered on the GPU at full resolution and full step by every
march path -- plain integrator, certificate tracing with ray and ball
certificates, the segment march with and without the trained network, the
traced batch and both integrators -- and compared with the FP64 oracle on
seeded rays drawn over the rendered views.  The sample positions' FP32
error grows with the distance along the ray, so these sizes are where the
guard bands are tightest.

The tracing and plain paths render every view of the workload; the slower
marches render an evenly strided subset of its views at the same
resolution and step (the per-ray arithmetic does not depend on which other
views share the call).  Bar: 1e-5 relative on transmittance for every path.
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

REL_TOL = 1e-5
RAYS = 30000


@pytest.fixture(scope="module")
def X():
    import torch
    torch.cuda.set_device(0)
    import __graft_entry__ as g
    g.build()
    import xray_projection_render_gb300 as X
    return X


def W():
    from xray_projection_render_gb300 import workloads
    return workloads


@pytest.fixture(scope="module")
def lattice(X):
    w = W().deformed_lattice()
    s = X.Scene(w.obj, w.deformation)
    yield w, s
    s.close()


@pytest.fixture(scope="module")
def gyroid(X):
    w = W().gyroid_sigmoid()
    s = X.Scene(w.obj, w.deformation)
    yield w, s
    s.close()


@pytest.fixture(scope="module")
def gyroid_fine(X):
    w = W().gyroid_fine_sigmoid()
    s = X.Scene(w.obj, w.deformation)
    yield w, s
    s.close()


def _rays(nviews, res, n, seed):
    rng = np.random.default_rng(seed)
    return np.stack([rng.integers(0, nviews, n), rng.integers(0, res, n),
                     rng.integers(0, res, n)], 1).astype(np.int32)


def _pick(out, rays, res):
    """The transmittances at (view, i, j) of a device image stack [view][i][j]."""
    import torch
    idx = (torch.from_numpy(rays[:, 0].astype(np.int64)) * res * res
           + torch.from_numpy(rays[:, 1].astype(np.int64)) * res
           + torch.from_numpy(rays[:, 2].astype(np.int64))).to(out.device)
    return out.reshape(-1)[idx].cpu().numpy().astype(np.float64)


def _check(got, ref, what):
    assert np.all(np.isfinite(got)), what
    rel = np.abs(got - ref) / ref
    k = int(rel.argmax())
    assert rel.max() <= REL_TOL, f"{what}: max rel error {rel.max():.3g} at ray {k}"
    return float(rel.max())


def _render(X, s, w, angles, integration="simple", march="plain", prop=None):
    """Device render of `angles` at the workload's resolution and step;
    returns the device image stack and the march's counters (or None)."""
    import torch
    out = torch.empty((len(angles), w.res, w.res), device="cuda", dtype=torch.float32)
    kw = dict(resolution=w.res, ds=w.ds, R=w.R, fov=w.fov, integration=integration)
    st = None
    if march == "plain":
        X.render(s, angles, out=out, **kw)
    elif march in ("trace", "ball"):
        _, st = X.render_proposal(s, None, angles, trace=True if march == "trace" else "ball",
                                  out=out, stats=True, **kw)
    elif march == "segments":
        _, st = X.render_proposal(s, None, angles, segment=64, refine=False, out=out, stats=True,
                                  **kw)
    elif march == "proposal":
        _, st = X.render_proposal(s, prop, angles, out=out, stats=True, **kw)
    else:
        raise ValueError(march)
    torch.cuda.synchronize()
    if st is not None:
        assert st["fp64_list_overflow"] == 0, f"{march}: the FP64 list overflowed"
    return out, st


def _oracle(w, angles, rays, integration="simple", ds=None):
    # the oracle holds one scene at a time: build it right before rendering
    return O.render(O.Scene(w.obj, w.deformation), angles, w.res, ds or w.ds, R=w.R, fov=w.fov,
                    integration=integration, rays=rays)


def _subset(w, views):
    return list(w.angles[:: max(1, len(w.angles) // views)][:views])


@pytest.mark.parametrize("march", ["plain", "trace", "ball"])
def test_lattice_every_view(X, lattice, march):
    w, s = lattice
    rays = _rays(len(w.angles), w.res, RAYS, seed=31)
    out, st = _render(X, s, w, w.angles, march=march)
    err = _check(_pick(out, rays, w.res), _oracle(w, w.angles, rays), f"lattice {march}")
    print(f"\nlattice {march}: max rel {err:.2e} over {RAYS} rays; counters {st}")


def test_lattice_segment_march_and_proposal(X, lattice):
    w, s = lattice
    angles = _subset(w, 12)
    rays = _rays(len(angles), w.res, RAYS, seed=32)
    ref = _oracle(w, angles, rays)
    out, _ = _render(X, s, w, angles, march="segments")
    _check(_pick(out, rays, w.res), ref, "lattice segment march")
    with X.Proposal(s, angles[:4], resolution=w.res, ds=w.ds, R=w.R, fov=w.fov, segment=64) as P:
        out, st = _render(X, s, w, angles, march="proposal", prop=P)
    err = _check(_pick(out, rays, w.res), ref, "lattice proposal")
    assert st["mlp_rounds"] > 0
    print(f"\nlattice proposal: max rel {err:.2e}; counters {st}")


@pytest.mark.parametrize("march", ["plain", "trace"])
def test_lattice_hierarchical(X, lattice, march):
    w, s = lattice
    angles = _subset(w, 16)
    rays = _rays(len(angles), w.res, RAYS // 2, seed=33)
    out, _ = _render(X, s, w, angles, integration="hierarchical", march=march)
    _check(_pick(out, rays, w.res), _oracle(w, angles, rays, "hierarchical"),
           f"lattice hierarchical {march}")


@pytest.mark.parametrize("march", ["trace", "ball"])
def test_gyroid_every_view_traced(X, gyroid, march):
    """Curve certificates (the sigmoid chain is not affine) and balls."""
    import torch
    w, s = gyroid
    rays = _rays(len(w.angles), w.res, RAYS, seed=51)
    out, st = _render(X, s, w, w.angles, march=march)
    err = _check(_pick(out, rays, w.res), _oracle(w, w.angles, rays), f"gyroid {march}")
    print(f"\ngyroid {march} (720 x 2048^2): max rel {err:.2e}; counters {st}")
    del out
    torch.cuda.empty_cache()


@pytest.mark.parametrize("march", ["plain", "segments"])
def test_gyroid_view_subset(X, gyroid, march):
    w, s = gyroid
    angles = _subset(w, 12)
    rays = _rays(len(angles), w.res, RAYS, seed=52)
    out, _ = _render(X, s, w, angles, march=march)
    _check(_pick(out, rays, w.res), _oracle(w, angles, rays), f"gyroid {march}")


def test_gyroid_proposal(X, gyroid):
    w, s = gyroid
    angles = _subset(w, 8)
    rays = _rays(len(angles), w.res, RAYS, seed=53)
    with X.Proposal(s, angles[:2], resolution=w.res, ds=w.ds, R=w.R, fov=w.fov, segment=64) as P:
        out, st = _render(X, s, w, angles, march="proposal", prop=P)
    err = _check(_pick(out, rays, w.res), _oracle(w, angles, rays), "gyroid proposal")
    print(f"\ngyroid proposal: max rel {err:.2e}; counters {st}")


@pytest.mark.parametrize("march", ["plain", "trace"])
def test_gyroid_hierarchical(X, gyroid, march):
    w, s = gyroid
    angles = _subset(w, 8)
    rays = _rays(len(angles), w.res, RAYS // 2, seed=54)
    out, _ = _render(X, s, w, angles, integration="hierarchical", march=march)
    _check(_pick(out, rays, w.res), _oracle(w, angles, rays, "hierarchical"),
           f"gyroid hierarchical {march}")


@pytest.mark.parametrize("trace", [True, "ball"])
def test_traced_batch_at_full_size(X, lattice, gyroid, trace):
    """One persistent launch over the lattice (24 views at 1024^2) and the
    gyroid (6 views at 2048^2) at their full resolutions.  A batch shares one
    step, so both items use the lattice's ds 0.002 (the oracle renders them
    with the same step)."""
    wl, sl = lattice
    wg, sg = gyroid
    al, ag = _subset(wl, 24), _subset(wg, 6)
    ds = wl.ds
    with X.Batch([(sl, al, wl.res), (sg, ag, wg.res)], ds=ds, trace=trace) as b:
        b.render()
        for k, (w, angles, seed) in enumerate(((wl, al, 61), (wg, ag, 62))):
            img = b.item(k)
            rays = _rays(len(angles), w.res, RAYS // 2, seed=seed)
            got = img[rays[:, 0], rays[:, 1], rays[:, 2]].astype(np.float64)
            ref = _oracle(w, angles, rays, ds=ds)
            _check(got, ref, f"batch item {k} trace={trace}")


@pytest.mark.parametrize("march", ["plain", "trace"])
@pytest.mark.parametrize("integration", ["simple", "hierarchical"])
def test_launch_groups_overlap(X, lattice, march, integration, monkeypatch):
    """A call of several launch groups (8 M rays each, 2 M hierarchical; 12
    views of 1024^2 make two, or six) runs each group's FP64 pass on the
    side stream beside the next group's march.  The images equal those of
    the one-stream schedule (XRP_FB_OVERLAP=0) within 1e-5, on the
    device and the host path, also when every list overflows (a 64-entry
    list: tracing renders the call again, the plain mode marches the rays
    that lost a sample again), and match the oracle."""
    import torch
    w, s = lattice
    angles = _subset(w, 12)
    kw = dict(resolution=w.res, ds=w.ds, R=w.R, fov=w.fov, integration=integration)

    def render(host):
        if march == "plain":
            if host:
                return X.render(s, angles, plain_fp64="list", **kw)
            out = torch.empty((len(angles), w.res, w.res), device="cuda", dtype=torch.float32)
            X.render(s, angles, out=out, plain_fp64="list", **kw)
        else:
            if host:
                return X.render_proposal(s, None, angles, trace=True, **kw)
            out = torch.empty((len(angles), w.res, w.res), device="cuda", dtype=torch.float32)
            X.render_proposal(s, None, angles, trace=True, out=out, **kw)
        torch.cuda.synchronize()
        return out.cpu().numpy()

    dev = render(False)
    host = render(True)
    monkeypatch.setenv("XRP_FB_OVERLAP", "0")
    serial = render(False)
    monkeypatch.setenv("XRP_FB_OVERLAP", "1")
    monkeypatch.setenv("XRP_FALLBACK_LIST", "64")
    full = render(False)
    monkeypatch.delenv("XRP_FALLBACK_LIST")
    # the FP64 values are added to the optical depths in another order (and a
    # re-marched ray sums them inside the march): FP32 rounding, a few 1e-6
    for a, what in ((host, "host"), (serial, "one stream"), (full, "full lists")):
        np.testing.assert_allclose(a, dev, rtol=REL_TOL, atol=1e-7, err_msg=what)
    rays = _rays(len(angles), w.res, 8000, seed=35)
    ref = _oracle(w, angles, rays, integration)
    got = dev[rays[:, 0], rays[:, 1], rays[:, 2]].astype(np.float64)
    _check(got, ref, f"lattice {march} {integration}, overlapped groups")


@pytest.mark.parametrize("integration", ["simple", "hierarchical"])
@pytest.mark.parametrize("march", ["plain", "trace", "ball"])
def test_gyroid_fine_every_march(X, gyroid_fine, march, integration):
    """The example scene's gyroid (scale 0.1: a lattice of sheets) under the
    sigmoid deformation, at the benchmarked 2048^2 and ds 0.001, on four of
    its views: every march and both integrators against the oracle."""
    w, s = gyroid_fine
    angles = _subset(w, 4)
    rays = _rays(len(angles), w.res, 20000, seed=41)
    out, st = _render(X, s, w, angles, integration=integration, march=march)
    err = _check(_pick(out, rays, w.res), _oracle(w, angles, rays, integration),
                 f"fine gyroid {march} {integration}")
    print(f"\nfine gyroid {march} {integration}: max rel {err:.2e}; counters {st}")


def test_certificate_kind_probe(X, gyroid, gyroid_fine):
    """Calls of at least 2^22 rays over a non-affine chain pick curve or ball
    certificates from their evaluation counts on a small probe: curves for
    the scale-8 gyroid (one smooth band), balls for the scale-0.1 one (a
    lattice of sheets, where a curve evaluation's extra cost does not pay)."""
    import torch
    for (w, s), want_ball in ((gyroid, False), (gyroid_fine, True)):
        angles = w.angles[:1]  # one 2048^2 view: 2^22 rays
        out = torch.empty((1, w.res, w.res), device="cuda", dtype=torch.float32)
        kw = dict(resolution=w.res, ds=w.ds, R=w.R, fov=w.fov, out=out, stats=True)
        _, auto = X.render_proposal(s, None, angles, trace=True, **kw)
        _, ball = X.render_proposal(s, None, angles, trace="ball", **kw)
        assert (auto["evaluations"] == ball["evaluations"]) == want_ball, (w.name, auto, ball)
