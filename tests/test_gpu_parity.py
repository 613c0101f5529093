"""Bit-exact parity of the CUDA render path (libvxr.so, sm_103a) with the CPU oracle.

Every stage output of every frame is compared bit for bit: G-buffer (voxel, dist
bits, side, seed), candidate and spatial reservoirs (all fields), the shaded frame
and the accumulator. The oracle itself is pinned against the reference's kernel
source (test_oracle_ref.py)."""
import numpy as np
import pytest

from conftest import assert_records_equal
from oracle import binding as ob

pytestmark = pytest.mark.gpu

CONSTS = dict(numberOfCandidates=32, numberOfMaxTemporalImportance=20, spatialRadius=30, spatialTaps=5)


def _run_parity(lib, scene, arrays, W, H, point, frames, cams, accumulate=1, spatial=1, temporal=1):
    world, _ = scene
    view = lib.View(world, lib.view_desc(W, H, lib.LIGHTS_POINT if point else lib.LIGHTS_AREA,
                                         accumulate=accumulate, spatial=spatial, temporal=temporal))
    port = ob.Renderer("port", arrays, W, H, point)
    try:
        for f in range(frames):
            pos, tgt = cams(f)
            view.lookat(pos, tgt)
            k = view.begin_frame()
            port.frame_start()
            ctx = f"[{'point' if point else 'area'} {W}x{H} frame {f}]"
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
    finally:
        port.close()
        view.close()


def _orbit(f):
    return (128.0 + 6.0 * f, 160.0 - 2.0 * f, 3.0 * f), (128.0, 128.0, 128.0)


@pytest.mark.parametrize("point", [True, False], ids=["point", "area"])
def test_stage_parity_config0(lib, cuda_device, scene0, world0_arrays, point):
    _run_parity(lib, scene0, world0_arrays, 320, 180, point, 4, _orbit)


def test_stage_parity_odd_resolution(lib, cuda_device, scene0, world0_arrays):
    # ragged tiles: width/height not multiples of the 16x8 block
    _run_parity(lib, scene0, world0_arrays, 77, 41, False, 3, _orbit)


def test_stage_parity_toggles_off(lib, cuda_device, scene0, world0_arrays):
    _run_parity(lib, scene0, world0_arrays, 96, 64, False, 3, _orbit, accumulate=0, spatial=0, temporal=0)


def test_stage_parity_inside_world(lib, cuda_device, scene0, world0_arrays):
    # camera inside the map, looking down: primary rays start inside the grid
    _run_parity(lib, scene0, world0_arrays, 128, 96, True, 3,
                lambda f: ((100.0 + f, 90.0, 100.0), (140.0, 40.0, 150.0)))


@pytest.fixture(scope="module")
def scene_big(lib):
    """A 1024^3 world (config 1's terrain scaled x4, 4,096 emitters in the air) and its arrays."""
    w = lib.World()
    d = lib.scene_preset(1)
    w.generate(d)
    g, b, l = w.arrays()
    return (w, d), ob.WorldArrays(g, b, l)


@pytest.mark.parametrize("point", [False, True], ids=["area", "point"])
def test_stage_parity_1024_world(lib, cuda_device, scene_big, point):
    """The full 1024^3 map (all 32^3 uber cells, 128^3 grid, ~100k bricks), thousands of
    emitters, a camera on the config's spline: every stage bit for bit."""
    scene, arrays = scene_big
    d = scene[1]
    _run_parity(lib, scene, arrays, 96, 54, point, 3, lambda f: lib.camera_path(d, 1, 10 + f, 120))
