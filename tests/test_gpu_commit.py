"""Incremental world commits (vxr_world_commit: World::Commit + the commit kernel): after
edits, only the changed bricks (and the grid when it changed) go to the device, and the
incrementally updated copy renders exactly what a freshly uploaded copy of the same world
renders (G-buffer, reservoirs, frame, bit for bit), which also checks the rebuilt uber
grid and skip tables."""
import numpy as np
import pytest

from conftest import assert_records_equal

pytestmark = pytest.mark.gpu

EMIT = (40 << 16) | (0xF << 12) | 0x0F8   # emitter payload: strength 40, opaque, orange


def _world(lib):
    w = lib.World()
    w.generate(lib.scene_preset(0, seed=21, emitters=48))
    return w


def _edits(w, step):
    """Deterministic edits of four kinds (the same sequence for both worlds)."""
    rng = np.random.default_rng(100 + step)
    for _ in range(40):                           # voxels inside existing terrain bricks
        x, z = (int(v) for v in rng.integers(8, 248, 2))
        y = int(rng.integers(40, 90))
        w.set(x, y, z, 0 if rng.random() < 0.5 else 0xF5A3)
    for i in range(3):                            # a floating block: splits empty cells
        x0, y0, z0 = 60 + 37 * i + step * 9, 150 + 4 * step, 90 + 23 * i
        for x in range(x0, x0 + 5):
            for y in range(y0, y0 + 3):
                for z in range(z0, z0 + 4):
                    w.set(x, y, z, 0xF9C6)
    w.set(120 + step, 158 + step, 128, EMIT)      # a new emitter (light list change)
    for x in range(64, 72):                       # clear a whole 8^3 cell: frees its brick
        for y in range(56, 64):
            for z in range(64, 72):
                w.set(x, y, z, 0)


def _render(lib, w, pos, tgt):
    v = lib.View(w, lib.view_desc(96, 64, lib.LIGHTS_AREA, temporal=0, spatial=1, rng_seed=77))
    try:
        v.lookat(pos, tgt)
        v.render()
        v.wait()
        return dict(g=v.read_gbuffer(0), c=v.read_reservoirs(0), h=v.read_reservoirs(1), f=v.read_frame())
    finally:
        v.close()


def test_commit_sends_only_changes_and_renders_like_a_fresh_upload(lib, cuda_device):
    a = _world(lib)
    pos, tgt = (100.0, 170.0, 20.0), (128.0, 100.0, 128.0)
    _render(lib, a, pos, tgt)                      # first frame: everything sent
    n, grid, full = a.pending()
    assert (n, grid, full) == (0, False, False)
    for step in range(3):
        _edits(a, step)
        n, grid, full = a.pending()
        assert not full and grid and 0 < n < 200, (step, n, grid, full)
        sent, everything = a.commit()
        assert (sent, everything) == (n, False), (step, sent, n)
        assert a.pending() == (0, False, False)
        b = _world(lib)                            # the same world, built and sent whole
        for s in range(step + 1):
            _edits(b, s)
        ra, rb = _render(lib, a, pos, tgt), _render(lib, b, pos, tgt)
        ctx = f"[after edit round {step}]"
        assert_records_equal("gbuffer", ra["g"], rb["g"], ctx)
        assert_records_equal("candidates", ra["c"], rb["c"], ctx)
        assert_records_equal("spatial", ra["h"], rb["h"], ctx)
        assert_records_equal("frame", ra["f"], rb["f"], ctx)
        b.close()


def test_render_commits_pending_edits(lib, cuda_device):
    """A frame rendered after edits commits them first (incrementally)."""
    w = _world(lib)
    pos, tgt = (100.0, 170.0, 20.0), (128.0, 100.0, 128.0)
    _render(lib, w, pos, tgt)
    w.set(130, 60, 130, 0xF777)
    n, grid, full = w.pending()
    assert n >= 1 and not full
    _render(lib, w, pos, tgt)
    assert w.pending() == (0, False, False)
    w.upload()                                     # an explicit full upload still works
    assert w.pending() == (0, False, False)


def _moves(lib, w):
    _, _, lights = w.arrays()
    idx = [k for k in range(len(lights)) if lights["size"][k] == 1][:6]
    for n, i in enumerate(idx):
        w.move_light(i, 70 + 23 * n, 140 + 3 * n, 60 + 29 * n)
    return idx


def test_moved_lights_render_like_a_fresh_upload(lib, cuda_device):
    """Lights moved with vxr_world_move_light and committed incrementally (a few bricks,
    the light table) render exactly like the same world sent whole."""
    pos, tgt = (100.0, 170.0, 20.0), (128.0, 100.0, 128.0)
    a = _world(lib)
    _render(lib, a, pos, tgt)
    moved = _moves(lib, a)
    assert len(moved) == 6
    n, _, full = a.pending()
    assert 0 < n <= 24 and not full
    ra = _render(lib, a, pos, tgt)
    b = _world(lib)
    _moves(lib, b)
    rb = _render(lib, b, pos, tgt)
    for key, name in (("g", "gbuffer"), ("c", "candidates"), ("h", "spatial"), ("f", "frame")):
        assert_records_equal(name, ra[key], rb[key], "[moved lights]")
    a.close()
    b.close()


@pytest.mark.parametrize("spatial", [0, 1])
def test_moving_a_light_resets_temporal_reuse_only_without_spatial(lib, cuda_device, spatial):
    w = _world(lib)
    v = lib.View(w, lib.view_desc(64, 48, lib.LIGHTS_AREA, spatial=spatial, temporal=1))
    try:
        v.lookat((100.0, 170.0, 20.0), (128.0, 100.0, 128.0))
        for _ in range(3):
            v.render()
        v.wait()
        _moves(lib, w)
        k = v.begin_frame()
        assert (k.restirtemporalframe == 0) == (spatial == 0), k.restirtemporalframe
    finally:
        v.close()
        w.close()
