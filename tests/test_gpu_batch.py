"""Batched rendering (vxr_batch): several views with their own worlds, resolutions and
light models rendered as one frame must give, per view, exactly what rendering that view
alone gives (the alone path is itself bit-exact against the oracle, test_gpu_parity.py).

Compared bit for bit after every frame: G-buffer, candidate and spatial reservoirs, the
shaded frame and the accumulator. Cameras move between frames so temporal reuse runs."""
import pytest

from conftest import assert_records_equal

pytestmark = pytest.mark.gpu


def _world(lib, seed, emitters, extent=256, mode=0):
    w = lib.World()
    d = lib.scene_preset(0, seed=seed, emitters=emitters, extent=extent, emitter_mode=mode)
    w.generate(d)
    return w, d


# (scene seed, emitters, width, height, light model, accumulate, spatial, temporal)
SPECS = [
    (11, 64, 160, 90, "point", 1, 1, 1),
    (12, 300, 96, 64, "area", 1, 1, 1),
    (13, 17, 77, 41, "area", 0, 1, 1),       # ragged tiles
    (14, 1000, 128, 72, "point", 1, 0, 1),   # spatial off
    (15, 5, 64, 48, "area", 1, 1, 0),        # temporal off
]


def _cam(i, f):
    return (100.0 + 9.0 * i + 5.0 * f, 150.0 - 2.0 * f, 20.0 * i + 3.0 * f), (128.0, 110.0 + i, 128.0)


def _make_views(lib, worlds, specs):
    views = []
    for (seed, ne, W, H, lm, acc, sp, tp), (w, _) in zip(specs, worlds):
        model = lib.LIGHTS_POINT if lm == "point" else lib.LIGHTS_AREA
        views.append(lib.View(w, lib.view_desc(W, H, model, accumulate=acc, spatial=sp, temporal=tp,
                                               rng_seed=0x9E3779B9 ^ seed)))
    return views


def _snapshot(v):
    return dict(g=v.read_gbuffer(0), c=v.read_reservoirs(0), h=v.read_reservoirs(1), f=v.read_frame(),
                a=v.read_accum())


def _compare(a, b, ctx):
    assert_records_equal("gbuffer", a["g"], b["g"], ctx)
    assert_records_equal("candidates", a["c"], b["c"], ctx)
    assert_records_equal("spatial", a["h"], b["h"], ctx)
    assert_records_equal("frame", a["f"], b["f"], ctx)
    assert_records_equal("accum", a["a"], b["a"], ctx)


@pytest.mark.parametrize("graph,chains", [(False, 1), (True, 1), (False, 2), (True, 3), (True, 5)],
                         ids=["launches", "graph", "launches-2-chains", "graph-3-chains", "graph-5-chains"])
def test_batch_matches_single_views(lib, cuda_device, graph, chains):
    """chains > 1: the views split into groups whose stages run on parallel branches."""
    worlds = [_world(lib, s[0], s[1]) for s in SPECS]
    alone = _make_views(lib, worlds, SPECS)
    batched = _make_views(lib, worlds, SPECS)
    batch = lib.Batch(batched, graph=graph, chains=chains)
    try:
        for f in range(4):
            for i, (va, vb) in enumerate(zip(alone, batched)):
                p, t = _cam(i, f)
                va.lookat(p, t)
                vb.lookat(p, t)
                va.render()
            batch.render()
            ms = batch.wait()
            assert ms > 0.0
            for i, (va, vb) in enumerate(zip(alone, batched)):
                va.wait()
                vb.wait()
                _compare(_snapshot(vb), _snapshot(va),
                         f"[view {i} {SPECS[i][4]} frame {f} graph={graph} chains={chains}]")
    finally:
        batch.close()
        for v in alone + batched:
            v.close()


def test_batch_tile_shape_and_mixed_sizes(lib, cuda_device):
    """A 32x4 batch tile against the default 16x8 of the single views, and a 512^3 world
    next to a 256^3 one, each view in a chain of its own."""
    specs = [(21, 200, 120, 80, "area", 1, 1, 1), (22, 40, 200, 30, "point", 1, 1, 1)]
    worlds = [_world(lib, 21, 200, extent=512, mode=1), _world(lib, 22, 40)]
    alone = _make_views(lib, worlds, specs)
    batched = _make_views(lib, worlds, specs)
    batch = lib.Batch(batched, tile=(32, 4), graph=True, chains=2)
    try:
        for f in range(3):
            for i, (va, vb) in enumerate(zip(alone, batched)):
                p, t = _cam(i, f)
                va.lookat(p, t)
                vb.lookat(p, t)
                va.render()
            batch.render()
            batch.wait()
            for i, (va, vb) in enumerate(zip(alone, batched)):
                va.wait()
                _compare(_snapshot(vb), _snapshot(va), f"[view {i} frame {f}]")
    finally:
        batch.close()
        for v in alone + batched:
            v.close()


def test_batch_rejects_bad_arguments(lib, cuda_device):
    w, _ = _world(lib, 31, 8)
    v = lib.View(w, lib.view_desc(32, 32))
    try:
        with pytest.raises(lib.VxrError):
            lib.Batch([v, v])
        with pytest.raises(lib.VxrError):
            lib.Batch([v], tile=(5, 5))
        with pytest.raises(lib.VxrError):
            lib.Batch([v] * 17)
        with pytest.raises(lib.VxrError):
            lib.Batch([v], chains=2)   # more chains than views
    finally:
        v.close()
