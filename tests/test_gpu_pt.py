"""The reference's ground-truth mode (renderPathTracer / render_di_gfxexp,
kernels.cl:177-260) on the GPU (VXR_STAGE_PATH_TRACE) against the reference's own kernel
compiled for the CPU (golden frames in tests/golden/config0_pt_48x32.npz, made by
tests/golden/make_golden.py): the frame of every stratum and the accumulator, bit for
bit."""
import os

import numpy as np
import pytest

from conftest import ROOT, assert_records_equal

pytestmark = pytest.mark.gpu

FIXTURE = os.path.join(ROOT, "tests", "golden", "config0_pt_48x32.npz")


def test_path_tracer_reproduces_reference(lib, cuda_device):
    fx = dict(np.load(FIXTURE))
    emitters, mode, seed = (int(v) for v in fx["scene"])
    w = lib.World()
    w.generate(lib.scene_preset(0, emitters=emitters, emitter_mode=mode, seed=seed))
    assert tuple(int(v) for v in fx["checksum"]) == w.checksum(), "scene generator drifted from the fixture"
    W, H, F = int(fx["W"]), int(fx["H"]), int(fx["frames"])
    view = lib.View(w, lib.view_desc(W, H, lib.LIGHTS_AREA, accumulate=1))
    nonzero = 0
    try:
        for f in range(F):
            cam = fx[f"camera{f}"]
            view.lookat(cam[:3], cam[3:])
            k = view.begin_frame()
            assert bytes(k) == fx[f"consts{f}"].tobytes(), "camera constants differ from the reference driver's"
            view.stage(lib.STAGE_PATH_TRACE)
            img = view.read_frame()
            assert_records_equal("frame", img, fx[f"frame{f}"], f"frame {f}")
            view.stage(lib.STAGE_ACCUMULATE)
            assert_records_equal("accum", view.read_accum(), fx[f"accum{f}"], f"frame {f}")
            view.end_frame()
            view.wait()
            nonzero += int((img[:, :3].sum(1) > 0).sum())
    finally:
        view.close()
        w.close()
    assert nonzero > 0.1 * W * H * F   # the fixture exercises the emitter hits
