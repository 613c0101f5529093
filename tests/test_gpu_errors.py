"""Device-side failure detection without a GPU fault: a kernel that meets an impossible
input raises a bit in the view's error word, clamps the value and goes on; the host
reads the word at vxr_view_wait, reports VXR_E_DEVICE once and clears it. The input
comes from the host: a reservoir naming a light beyond the light list, written through
the stage-level access between the spatial and shading stages. The tensor-core inference
of the learned proposal bounds every mbarrier wait: with the test hook its waits run out
with no MMA in flight, and the frame reports flag 16, stays finite, and later frames are
clean."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _cam(f):
    return (128.0 + 4.0 * f, 160.0, 10.0 + f), (128.0, 120.0, 128.0)


def test_shading_light_index_error_is_reported_once(lib, cuda_device, scene0):
    w, _ = scene0
    nl = len(w.arrays()[2])
    v = lib.View(w, lib.view_desc(64, 48, lib.LIGHTS_AREA))
    try:
        v.lookat(*_cam(0))
        v.render()
        v.wait()
        v.lookat(*_cam(1))
        v.begin_frame()
        for s in (lib.STAGE_ALBEDO, lib.STAGE_CANDIDATES, lib.STAGE_SPATIAL):
            v.stage(s)
        h = v.read_reservoirs(1)
        live = (h["streamLength"] > 0) & (h["sumOfWeights"] > 0) & (h["pHat"] > 0)
        assert live.sum() > 10
        h["lightIndex"][live] = nl + 7
        v.write_reservoirs(1, h)
        v.stage(lib.STAGE_SHADE)
        v.stage(lib.STAGE_ACCUMULATE)
        v.end_frame()
        with pytest.raises(lib.VxrError) as e:
            v.wait()
        assert e.value.code == -5                                   # VXR_E_DEVICE
        assert "device error flags 0x8 (8: shading light index)" in str(e.value)
        assert np.isfinite(v.read_frame()).all()          # clamped, not faulted
        # the bad index also sits in the history the next temporal pass reads: empty it,
        # then later frames are clean (the word was cleared when it was reported)
        v.write_reservoirs(1, np.zeros_like(h))
        for f in (2, 3):
            v.lookat(*_cam(f))
            v.render()
            v.wait()
    finally:
        v.close()


def test_tensor_core_wait_timeout_is_reported_once(lib, cuda_device):
    w = lib.World()
    w.generate(lib.scene_preset(0, emitters=2048, emitter_mode=1))
    w.cluster_lights(256, seed=3, iters=6)
    v = lib.View(w, lib.view_desc(96, 64, lib.LIGHTS_AREA, num_candidates=8))
    try:
        v.proposal_enable(seed=7, batch=4096, inference=2)
        v.proposal_use(True)
        v.lookat(*_cam(0))
        v.render()
        v.wait()
        v.proposal_test_timeout(True)
        v.lookat(*_cam(1))
        v.render()
        with pytest.raises(lib.VxrError) as e:
            v.wait()
        assert e.value.code == -5                                   # VXR_E_DEVICE
        assert "device error flags 0x10 (16: tensor-core wait gave up)" in str(e.value)
        assert np.isfinite(v.read_frame()).all()
        v.proposal_test_timeout(False)
        for f in (2, 3):
            v.lookat(*_cam(f))
            v.render()
            v.wait()
        assert np.isfinite(v.read_frame()).all() and v.read_frame()[:, :3].max() > 0
    finally:
        v.close()
