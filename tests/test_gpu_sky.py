"""Sky-dome sampling (vxr_view_set_sky; ris.cl:197-211, 254-290; tools.cl:6-28, 54-70,
130-144) on the GPU against the reference's own shading kernel compiled for the CPU with
skyDomeSampling = 1 (golden frames tests/golden/config0_sky_48x32.npz for area lights and
config0_sky_point_48x32.npz for point lights, made by tests/golden/make_golden.py from the
synthetic sky of tests/golden/sky_inputs.py):
background pixels, sky seen through translucent voxels and the sky-light ray, bit for
bit, with the accumulator; then the batched path with a sky view beside a sky-less one,
against the same views rendered alone."""
import os
import sys

import numpy as np
import pytest

from conftest import ROOT, assert_records_equal

sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
import sky_inputs  # noqa: E402

pytestmark = pytest.mark.gpu

FIXTURES = {"area": os.path.join(ROOT, "tests", "golden", "config0_sky_48x32.npz"),
            "point": os.path.join(ROOT, "tests", "golden", "config0_sky_point_48x32.npz")}


def _scene(lib):
    w = lib.World()
    w.generate(lib.scene_preset(0))
    sky_inputs.add_panel(w)
    return w


def _set_sky(view):
    view.set_sky(sky_inputs.sky_texture(), sky_inputs.SKY_LIGHT, sky_inputs.LIGHT_SCALE, sky_inputs.blue_noise())


@pytest.mark.parametrize("model", ["area", "point"])
def test_sky_dome_reproduces_reference(lib, cuda_device, model):
    fx = dict(np.load(FIXTURES[model]))
    w = _scene(lib)
    assert tuple(int(v) for v in fx["checksum"]) == w.checksum(), "scene drifted from the fixture"
    W, H, F = int(fx["W"]), int(fx["H"]), int(fx["frames"])
    view = lib.View(w, lib.view_desc(W, H, lib.LIGHTS_POINT if model == "point" else lib.LIGHTS_AREA, accumulate=1))
    _set_sky(view)
    seen = {"background": 0, "translucent": 0}
    try:
        for f in range(F):
            cam = fx[f"camera{f}"]
            view.lookat(cam[:3], cam[3:])
            k = view.begin_frame()
            assert bytes(k) == fx[f"consts{f}"].tobytes(), "camera constants differ from the reference driver's"
            for s in (lib.STAGE_ALBEDO, lib.STAGE_CANDIDATES, lib.STAGE_SPATIAL, lib.STAGE_SHADE, lib.STAGE_ACCUMULATE):
                view.stage(s)
            g = view.read_gbuffer(0)
            assert_records_equal("gbuffer", g, fx[f"gbuffer{f}"], f"frame {f}")
            assert_records_equal("frame", view.read_frame(), fx[f"frame{f}"], f"frame {f}")
            assert_records_equal("accum", view.read_accum(), fx[f"accum{f}"], f"frame {f}")
            view.end_frame()
            view.wait()
            v = g["voxel"] & 0xFFFFFF
            seen["background"] += int((v == 0).sum())
            seen["translucent"] += int((((v >> 12) & 15) != 15).sum() - (v == 0).sum())
    finally:
        view.close()
        w.close()
    assert min(seen.values()) > 0.2 * W * H * F, seen


def test_sky_off_again_matches_no_sky(lib, cuda_device):
    """Turning the sky off (set_sky(None)) gives the frames of a view that never had one."""
    w = _scene(lib)
    a = lib.View(w, lib.view_desc(40, 24, lib.LIGHTS_POINT, accumulate=1))
    b = lib.View(w, lib.view_desc(40, 24, lib.LIGHTS_POINT, accumulate=1))
    _set_sky(b)
    try:
        for f in range(3):
            if f == 1:
                b.set_sky(None)
            for v in (a, b):
                v.lookat((130.0 + f, 150.0, 30.0), (128.0, 130.0, 230.0))
                v.render()
                v.wait()
            same = np.array_equal(a.read_frame().view(np.uint32), b.read_frame().view(np.uint32))
            assert same == (f >= 1), f"frame {f}"
    finally:
        a.close()
        b.close()
        w.close()


@pytest.mark.parametrize("graph", [False, True], ids=["launches", "graph"])
def test_batch_with_sky_matches_single_views(lib, cuda_device, graph):
    """vxr_batch with one sky view and one without: the shading launch takes the sky
    variant, the recorded graphs follow a sky switched off and on again, and every view
    renders what it renders alone."""
    w = _scene(lib)
    specs = [(48, 32, lib.LIGHTS_AREA, True), (40, 24, lib.LIGHTS_POINT, False)]
    alone = [lib.View(w, lib.view_desc(W, H, m, accumulate=1)) for W, H, m, _ in specs]
    batched = [lib.View(w, lib.view_desc(W, H, m, accumulate=1)) for W, H, m, _ in specs]
    for (_, _, _, sky), va, vb in zip(specs, alone, batched):
        if sky:
            _set_sky(va)
            _set_sky(vb)
    batch = lib.Batch(batched, graph=graph)
    try:
        for f in range(5):
            if f == 2:            # sky off for one frame, then on again
                alone[0].set_sky(None)
                batched[0].set_sky(None)
            if f == 3:
                _set_sky(alone[0])
                _set_sky(batched[0])
            for i, (va, vb) in enumerate(zip(alone, batched)):
                p, t = (126.0 + 3.0 * i + 2.0 * f, 150.0, 30.0 + f), (128.0, 135.0, 230.0)
                va.lookat(p, t)
                vb.lookat(p, t)
                va.render()
            batch.render()
            batch.wait()
            for i, (va, vb) in enumerate(zip(alone, batched)):
                va.wait()
                vb.wait()
                ctx = f"[view {i} frame {f} graph={graph}]"
                assert_records_equal("frame", vb.read_frame(), va.read_frame(), ctx)
                assert_records_equal("accum", vb.read_accum(), va.read_accum(), ctx)
    finally:
        batch.close()
        for v in alone + batched:
            v.close()
        w.close()


def test_load_sky_from_hdr_file(lib, cuda_device, tmp_path):
    """scene_io.load_sky (LoadSky from a Radiance file) renders the same bits as setting
    the texture it builds, with its sky lights, by hand."""
    from smallproject_gb300 import scene_io as io
    rng = np.random.default_rng(9)
    rgb = (rng.random((32, 64, 3)) * 2.0).astype(np.float32)
    path = str(tmp_path / "sky.hdr")
    io.write_hdr(path, rgb)
    bn = sky_inputs.blue_noise()
    w = _scene(lib)
    a = lib.View(w, lib.view_desc(48, 32, lib.LIGHTS_AREA))
    b = lib.View(w, lib.view_desc(48, 32, lib.LIGHTS_AREA))
    try:
        tex = io.load_sky(a, path, bn, scale=1.25, light_scale=0.75)
        assert np.array_equal(tex, io.sky_texture(io.read_hdr(path), scale=1.25))
        b.set_sky(tex, lib.sky_lights(tex), 0.75, bn)
        for v in (a, b):
            v.lookat((126.0, 150.0, 30.0), (128.0, 140.0, 230.0))
            v.render()
            v.wait()
        assert_records_equal("frame", a.read_frame(), b.read_frame(), "load_sky")
        assert (a.read_frame()[:, :3] > 0).mean() > 0.3
    finally:
        a.close()
        b.close()
        w.close()
