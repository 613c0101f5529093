"""Launch tuning (vxr_tuning) changes speed, never results; the autotuner's cache.

Every tuning renders the same bits as the defaults (G-buffer, reservoirs, frame,
accumulator), for a single view and for a batch: among them the shadow tracer without its
visibility early-out and with its shared-memory brick cache (the calibration frame and
the frames that read the cached bricks' opacity masks)."""
import json

import pytest

from conftest import assert_records_equal

pytestmark = pytest.mark.gpu

ODD = dict(tile_x=32, tile_y=4, persistent=1, shadow_refill=16, shadow_burst=16, list_blocks_per_sm=4, occupancy=1,
           shadow_schedule=1, shadow_early_out=0, brick_cache=0)
ODD2 = dict(tile_x=8, tile_y=16, persistent=1, shadow_refill=1, shadow_burst=1, list_blocks_per_sm=1, occupancy=0,
            shadow_schedule=1, shadow_early_out=1, brick_cache=128)
# the shadow tracer's shared-memory brick cache (calibration frame, then the table)
CACHED = dict(tile_x=16, tile_y=8, persistent=0, shadow_refill=8, shadow_burst=4, list_blocks_per_sm=16, occupancy=0,
              shadow_schedule=0, shadow_early_out=0, brick_cache=1024)


def _cam(f):
    return (110.0 + 4.0 * f, 150.0 - 1.5 * f, 10.0 + 2.0 * f), (128.0, 120.0, 128.0)


def _snap(v):
    return [v.read_gbuffer(0), v.read_reservoirs(0), v.read_reservoirs(1), v.read_frame(), v.read_accum()]


@pytest.mark.parametrize("model", ["area", "point"])
def test_tuning_does_not_change_results(lib, cuda_device, scene0, model):
    w, _ = scene0
    lm = lib.LIGHTS_POINT if model == "point" else lib.LIGHTS_AREA
    desc = lib.view_desc(150, 70, lm, accumulate=1)
    views = [lib.View(w, desc) for _ in range(4)]
    try:
        views[1].set_tuning(lib.tuning(**ODD))
        views[2].set_tuning(lib.tuning(**ODD2))
        views[3].set_tuning(lib.tuning(**CACHED))
        assert views[1].get_tuning().as_dict() == ODD
        for f in range(4):
            for v in views:
                v.lookat(*_cam(f))
                v.render()
            snaps = []
            for v in views:
                v.wait()
                snaps.append(_snap(v))
            for other in snaps[1:]:
                for name, a, b in zip(("gbuffer", "candidates", "spatial", "frame", "accum"), other, snaps[0]):
                    assert_records_equal(name, a, b, f"[{model} frame {f}]")
    finally:
        for v in views:
            v.close()


def test_tuning_rejects_bad_values(lib, cuda_device, scene0):
    v = lib.View(scene0[0], lib.view_desc(32, 32))
    try:
        for bad in (dict(tile_x=5, tile_y=5), dict(tile_x=64, tile_y=32), dict(tile_x=32, tile_y=16), dict(persistent=2), dict(shadow_refill=0),
                    dict(shadow_refill=33), dict(shadow_burst=0), dict(shadow_burst=65), dict(list_blocks_per_sm=0), dict(occupancy=2),
                    dict(shadow_schedule=2), dict(shadow_early_out=2), dict(brick_cache=100), dict(brick_cache=64),
                    dict(brick_cache=4096)):
            with pytest.raises(lib.VxrError):
                v.set_tuning(lib.tuning(**bad))
    finally:
        v.close()


def test_autotune_caches_a_result(lib, cuda_device, scene0, tmp_path):
    from smallproject_gb300 import autotune as at
    w, _ = scene0
    desc = lib.view_desc(128, 72, lib.LIGHTS_AREA)
    path = str(tmp_path / "tune.json")
    t, rep = at.autotune(w, desc, _cam, frames=2, rounds=1, cache_path=path)
    assert rep["ms"] > 0 and rep["ms"] <= rep["default_ms"] * 1.2 and rep["evaluated"] >= 10
    cache = json.load(open(path))
    key = at.config_key(w, desc)
    assert key in cache
    t2, rep2 = at.autotune(w, desc, _cam, cache_path=path)   # served from the cache
    assert t2.as_dict() == t.as_dict() and rep2 == cache[key]
    v = lib.View(w, desc)
    try:
        assert at.apply_cached(v, w, cache_path=path)
        assert v.get_tuning().as_dict() == t.as_dict()
    finally:
        v.close()


def test_batch_tuning_keeps_results(lib, cuda_device, scene0):
    """Two batches over identical views, one with an unusual tuning, render the same bits;
    then the batch autotuner runs on one of them."""
    from smallproject_gb300 import autotune as at
    w, _ = scene0
    descs = [lib.view_desc(96, 64, lib.LIGHTS_AREA, accumulate=1), lib.view_desc(64, 40, lib.LIGHTS_POINT, accumulate=1)]
    va = [lib.View(w, d) for d in descs]
    vb = [lib.View(w, d) for d in descs]
    ba = lib.Batch(va, graph=True)
    bb = lib.Batch(vb, graph=False)
    cams = [lambda f, i=i: ((100.0 + 7 * i + f, 150.0, 5.0 * i + f), (128.0, 120.0, 128.0)) for i in range(2)]
    try:
        bb.set_tuning(lib.tuning(**ODD))
        for f in range(3):
            for i in range(2):
                p, t = cams[i](f)
                va[i].lookat(p, t)
                vb[i].lookat(p, t)
            ba.render()
            bb.render()
            ba.wait()
            bb.wait()
            for i in range(2):
                for name, x, y in zip(("gbuffer", "candidates", "spatial", "frame", "accum"), _snap(vb[i]), _snap(va[i])):
                    assert_records_equal(name, x, y, f"[batch view {i} frame {f}]")
        t, rep = at.autotune_batch(ba, cams, frames=1, rounds=1)
        assert rep["ms"] > 0 and rep["evaluated"] >= 10
    finally:
        ba.close()
        bb.close()
        for v in va + vb:
            v.close()
