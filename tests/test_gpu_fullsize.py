"""The headline workload at its full size (config 3: 1920 x 1080, the 1024^3 fBm world
with 65,536 emitters, area lights, the bench's camera path): three whole consecutive
frames against the C oracle (all host cores), every stage bit for bit - primary rays,
candidates with visibility and temporal reuse, spatial reuse, shading with its
visibility rays, the history reservoirs and the accumulator; a band of rows of a first
frame; and a size-independent property: a very different launch tuning on a second view
changes no bit of any stage over several frames (the persistent work queues at full
load)."""
import numpy as np
import pytest

from conftest import assert_records_equal
from oracle import binding as ob

pytestmark = pytest.mark.gpu

W, H = 1920, 1080
BAND = (536, 548)            # rows compared with the oracle
PATH = 300                   # frames of the bench's camera path
ODD = dict(tile_x=32, tile_y=4, persistent=1, shadow_refill=16, shadow_burst=16, list_blocks_per_sm=4, occupancy=1,
           shadow_schedule=1)


@pytest.fixture(scope="module")
def scene3(lib):
    w = lib.World()
    d = lib.scene_preset(3)
    w.generate(d)
    return w, d


def test_full_frame_band_matches_oracle(lib, cuda_device, scene3):
    w, d = scene3
    g, b, l = w.arrays()
    assert len(l) == 65536
    port = ob.Renderer("port", ob.WorldArrays(g, b, l), W, H, False)
    view = lib.View(w, lib.view_desc(W, H, lib.LIGHTS_AREA, accumulate=1))
    y0, y1 = BAND
    rows = slice(y0 * W, y1 * W)
    try:
        view.lookat(*lib.camera_path(d, 1, 150, PATH))
        k = view.begin_frame()
        assert k.restirtemporalframe == 0
        port.frame_start()
        view.stage(lib.STAGE_ALBEDO)
        port.stage(k, 1, y0, y1)
        gv = view.read_gbuffer(0)
        assert_records_equal("gbuffer", gv[rows], port.gbuffer(0)[rows], f"[rows {y0}-{y1}]")
        assert (gv["voxel"][rows] != 0).mean() > 0.2          # the band sees terrain
        view.stage(lib.STAGE_CANDIDATES)
        port.stage(k, 2, y0, y1)
        assert_records_equal("candidates", view.read_reservoirs(0)[rows], port.reservoirs(0)[rows], f"[rows {y0}-{y1}]")
        assert_records_equal("seed", view.read_gbuffer(0)["seed"][rows], port.gbuffer(0)["seed"][rows], "")
        view.end_frame()
        view.wait()
    finally:
        port.close()
        view.close()


def test_whole_frames_match_oracle(lib, cuda_device, scene3):
    w, d = scene3
    g, b, l = w.arrays()
    port = ob.Renderer("port", ob.WorldArrays(g, b, l), W, H, False)
    view = lib.View(w, lib.view_desc(W, H, lib.LIGHTS_AREA, accumulate=1))
    try:
        for f in range(3):
            view.lookat(*lib.camera_path(d, 1, 150 + f, PATH))
            k = view.begin_frame()
            assert (k.restirtemporalframe > 0) == (f > 0)   # temporal reuse from the second frame on
            port.frame_start()
            ctx = f"[1920x1080 config 3, frame {f}]"
            for s in range(1, 6):
                view.stage(s)
                port.stage(k, s)
                if s == 1:
                    assert_records_equal("gbuffer", view.read_gbuffer(0), port.gbuffer(0), ctx)
                elif s == 2:
                    assert_records_equal("candidates", view.read_reservoirs(0), port.reservoirs(0), ctx)
                    assert_records_equal("seed", view.read_gbuffer(0)["seed"], port.gbuffer(0)["seed"], ctx)
                elif s == 3:
                    assert_records_equal("spatial", view.read_reservoirs(1), port.reservoirs(1), ctx)
                    assert_records_equal("seed", view.read_gbuffer(0)["seed"], port.gbuffer(0)["seed"], ctx)
                elif s == 4:
                    assert_records_equal("frame", view.read_frame(), port.image(0), ctx)
                    assert_records_equal("history", view.read_reservoirs(1), port.reservoirs(2), ctx)
                else:
                    assert_records_equal("accum", view.read_accum(), port.image(1), ctx)
            view.end_frame()
            view.wait()
        fr = view.read_frame()
        assert (fr[:, :3] > 0).mean() > 0.2
    finally:
        port.close()
        view.close()


def test_full_frames_do_not_depend_on_launch_tuning(lib, cuda_device, scene3):
    w, d = scene3
    desc = lib.view_desc(W, H, lib.LIGHTS_AREA, accumulate=1)
    views = [lib.View(w, desc), lib.View(w, desc)]
    try:
        views[1].set_tuning(lib.tuning(**ODD))
        for f in range(4):
            for v in views:
                v.lookat(*lib.camera_path(d, 1, 150 + f, PATH))
                v.render()
            snaps = []
            for v in views:
                v.wait()
                snaps.append([v.read_gbuffer(0), v.read_reservoirs(0), v.read_reservoirs(1), v.read_frame(),
                              v.read_accum()])
            for name, a, b in zip(("gbuffer", "candidates", "spatial", "frame", "accum"), snaps[1], snaps[0]):
                assert_records_equal(name, a, b, f"[1920x1080 frame {f}]")
            assert np.isfinite(snaps[0][3]).all() and (snaps[0][3][:, :3] > 0).mean() > 0.2
    finally:
        for v in views:
            v.close()
