"""Batched rendering (xrp_batch_*): many scenes of uneven resolution and
view count in one persistent launch replayed from a CUDA graph.  Each
item's images must equal what xrp_render produces for it alone, and match
the FP64 oracle within 1e-5 relative."""
import numpy as np
import pytest

from oracle import oracle as O
from xray_projection_render_gb300 import workloads as W

pytestmark = pytest.mark.gpu

REL_TOL = 1e-5


@pytest.fixture(scope="module")
def X():
    import __graft_entry__ as g
    g.build()
    import xray_projection_render_gb300 as X
    return X


def _items():
    ws = [W.reduced(w, r, v) for w, r, v in zip(W.batched_scenes(4), (48, 24, 64, 17), (3, 5, 1, 2))]
    ws.append(W.cube_minus_sphere_cylinder(40))
    ws.append(W.reduced(W.deformed_lattice(), 32, 2))
    ws.append(W.reduced(W.gyroid_sigmoid(), 20, 1))
    return ws


@pytest.mark.parametrize("integration", ["simple", "hierarchical"])
@pytest.mark.parametrize("autotune", [True, False])
def test_batch_equals_single_renders(X, integration, autotune):
    ws = _items()
    ds = 0.005
    scenes = [X.Scene(w.obj, w.deformation) for w in ws]
    try:
        with X.Batch([(s, w.angles, w.res) for s, w in zip(scenes, ws)], ds=ds,
                     integration=integration, autotune=autotune) as b:
            b.render()
            b.render()  # replay of the same graph
            info = b.info()
            assert info["tile_w"] * info["tile_h"] == 32
            assert info["rays"] == sum(len(w.angles) * w.res ** 2 for w in ws)
            if autotune:
                assert info["tune_candidates"] >= 4
            for k, (s, w) in enumerate(zip(scenes, ws)):
                # the batch kernel re-evaluates undecided samples in FP64
                # inside the march, like plain_fp64="inplace": bit for bit
                single = X.render(s, w.angles, resolution=w.res, ds=ds, integration=integration,
                                  plain_fp64="inplace")
                assert np.array_equal(b.item(k), single), w.name
                # the FP64 list adds those samples after the march
                listed = X.render(s, w.angles, resolution=w.res, ds=ds, integration=integration,
                                  plain_fp64="list")
                np.testing.assert_allclose(b.item(k), listed, rtol=2e-6, atol=1e-7, err_msg=w.name)
    finally:
        for s in scenes:
            s.close()


def test_batch_matches_oracle(X):
    ws = _items()
    ds = 0.005
    scenes = [X.Scene(w.obj, w.deformation) for w in ws]
    try:
        with X.Batch([(s, w.angles, w.res) for s, w in zip(scenes, ws)], ds=ds) as b:
            b.render()
            for k in (0, 4, 5):
                w = ws[k]
                ref = O.render(O.Scene(w.obj, w.deformation), w.angles, w.res, ds, R=w.R, fov=w.fov)
                assert np.max(np.abs(b.item(k) - ref) / ref) <= REL_TOL
    finally:
        for s in scenes:
            s.close()


def test_batch_rejects_bad_items(X):
    from xray_projection_render_gb300._lib import EngineError
    w = W.cube_minus_sphere_cylinder(16)
    with X.Scene(w.obj) as s:
        with pytest.raises(EngineError):
            X.Batch([(s, w.angles, 0)], ds=0.01)
        with pytest.raises(EngineError):
            X.Batch([(s, w.angles, 16)], ds=-1.0)


def test_batch_with_certificate_tracing(X):
    ws = _items()
    ds = 0.005
    scenes = [X.Scene(w.obj, w.deformation) for w in ws]
    try:
        with X.Batch([(s, w.angles, w.res) for s, w in zip(scenes, ws)], ds=ds, trace=True) as b:
            b.render()
            for k, (s, w) in enumerate(zip(scenes, ws)):
                single = X.render(s, w.angles, resolution=w.res, ds=ds)
                # same samples, summed in another order (runs of equal density)
                assert np.max(np.abs(b.item(k) - single) / single) <= 2 * REL_TOL, w.name
            w = ws[4]
            ref = O.render(O.Scene(w.obj, w.deformation), w.angles, w.res, ds, R=w.R, fov=w.fov)
            assert np.max(np.abs(b.item(4) - ref) / ref) <= REL_TOL
        # without the gyroid (sigmoid chain) every scene is affine: ray bounds
        with X.Batch([(s, w.angles, w.res) for s, w in zip(scenes[:6], ws[:6])], ds=ds, trace=True) as br:
            br.render()
            for k, (s, w) in enumerate(zip(scenes[:6], ws[:6])):
                single = X.render(s, w.angles, resolution=w.res, ds=ds)
                assert np.max(np.abs(br.item(k) - single) / single) <= 2 * REL_TOL, w.name
        with X.Batch([(s, w.angles, w.res) for s, w in zip(scenes, ws)], ds=ds, trace="ball") as bb:
            bb.render()
            for k, (s, w) in enumerate(zip(scenes, ws)):
                single = X.render(s, w.angles, resolution=w.res, ds=ds)
                assert np.max(np.abs(bb.item(k) - single) / single) <= 2 * REL_TOL, w.name
        with X.Batch([(s, w.angles, w.res) for s, w in zip(scenes, ws)], ds=ds, trace=True,
                     integration="hierarchical") as bh:
            bh.render()
            for k, (s, w) in enumerate(zip(scenes, ws)):
                single = X.render(s, w.angles, resolution=w.res, ds=ds, integration="hierarchical")
                assert np.max(np.abs(bh.item(k) - single) / single) <= 2 * REL_TOL, w.name
    finally:
        for s in scenes:
            s.close()


def test_batch_with_empty_and_outside_scenes(X):
    objs = [{"type": "object_collection", "objects": []},
            {"type": "sphere", "center": [9.0, 9.0, 9.0], "radius": 0.5, "rho": 1.0},
            W.cube_minus_sphere_cylinder(8).obj]
    angles = [(0.0, 90.0), (40.0, 60.0)]
    scenes = [X.Scene(o) for o in objs]
    try:
        for trace in (False, True):
            with X.Batch([(s, angles, r) for s, r in zip(scenes, (16, 20, 24))], ds=0.01,
                         flat_field=0.25, trace=trace) as b:
                b.render()
                for k, (o, r) in enumerate(zip(objs, (16, 20, 24))):
                    ref = O.render(O.Scene(o), angles, r, 0.01, flat_field=0.25)
                    assert np.max(np.abs(b.item(k) - ref) / ref) <= REL_TOL
    finally:
        for s in scenes:
            s.close()
