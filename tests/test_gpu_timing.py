"""Per-kernel timing (vxr_view_kernel_timing / vxr_view_kernel_stats) and the work
counts of a frame (vxr_view_work_counts)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_kernel_timing_counts_every_launch(lib, cuda_device, scene0):
    w, _ = scene0
    v = lib.View(w, lib.view_desc(160, 90, lib.LIGHTS_AREA, accumulate=1))
    try:
        v.lookat((110.0, 150.0, 10.0), (128.0, 120.0, 128.0))
        v.render()
        v.wait()
        v.kernel_timing(True)
        v.kernel_stats(reset=True)
        for f in range(3):
            v.lookat((110.0 + f, 150.0, 10.0 + f), (128.0, 120.0, 128.0))
            v.render()
        v.wait()
        st = v.kernel_stats(reset=True)
        for k in ("albedo", "compact_hits", "ris_candidates", "shadow_candidates", "temporal", "spatial",
                  "shade_request", "shadow_shading", "shade_finish"):
            assert st[k][1] == 3 and st[k][0] > 0.0, (k, st[k])
        assert st["accumulate"][1] == 0 and st["proposal_infer"][1] == 0   # fused / not enabled
        # stage times cover the kernels of the stage
        sums, counts = v.stage_stats(reset=True)
        cand = st["compact_hits"][0] + st["ris_candidates"][0] + st["shadow_candidates"][0] + st["temporal"][0]
        assert cand <= sums[1] * 1.05 + 0.05
        hits, rc, rs = v.work_counts()
        assert 0 < hits <= 160 * 90 and 0 < rc <= hits and 0 < rs <= hits
        # timing off: nothing recorded
        v.kernel_timing(False)
        v.render()
        v.wait()
        assert all(c == 0 for _, c in v.kernel_stats().values())
    finally:
        v.close()


def test_pipelined_images_equal_synchronous_ones(lib, cuda_device, scene0):
    """vxr_view_render_to_host_async returns, image for image, what vxr_view_render_to_host
    returns for the same camera sequence (two views with the same seed), with frame f + 1
    enqueued before image f is waited for; a ticket older than the four in flight is
    rejected."""
    w, _ = scene0
    W, H = 128, 72
    va = lib.View(w, lib.view_desc(W, H, lib.LIGHTS_AREA, accumulate=1, rng_seed=9))
    vb = lib.View(w, lib.view_desc(W, H, lib.LIGHTS_AREA, accumulate=1, rng_seed=9))
    bufs = [lib.PinnedBuffer(W * H * 4) for _ in range(2)]
    sync = lib.PinnedBuffer(W * H * 4)
    try:
        cams = [((110.0 + 3 * f, 150.0, 10.0 + 2 * f), (128.0, 120.0, 128.0)) for f in range(6)]
        want = []
        for pos, tgt in cams:
            va.render_to_host(pos, tgt, sync.array)
            want.append(sync.array.copy())
        tickets = [vb.render_to_host_async(*cams[0], bufs[0].array)]
        for f in range(1, len(cams)):
            tickets.append(vb.render_to_host_async(*cams[f], bufs[f % 2].array))
            vb.image_wait(tickets[f - 1])
            assert (bufs[(f - 1) % 2].array.view("u4") == want[f - 1].view("u4")).all(), f - 1
        vb.image_wait(tickets[-1])
        assert (bufs[(len(cams) - 1) % 2].array.view("u4") == want[-1].view("u4")).all()
        with pytest.raises(lib.VxrError):
            vb.image_wait(tickets[0])    # six images ago: no longer tracked
        with pytest.raises(lib.VxrError):
            vb.image_wait(tickets[-1] + 1)   # not issued
    finally:
        for b in bufs + [sync]:
            b.close()
        va.close()
        vb.close()


def test_overlapped_frames_equal_stage_by_stage_ones(lib, cuda_device, scene0):
    """vxr_view_render starts a frame's primary rays beside the previous frame's shading
    when the frames follow each other with no other call on the view; the images, G-buffer
    planes and reservoirs equal those of the same frames rendered stage by stage (every
    stage in order on the view's stream), bit for bit."""
    w, _ = scene0
    W, H = 320, 180
    va = lib.View(w, lib.view_desc(W, H, lib.LIGHTS_AREA, accumulate=1, rng_seed=5))
    vb = lib.View(w, lib.view_desc(W, H, lib.LIGHTS_AREA, accumulate=1, rng_seed=5))
    try:
        for f in range(8):
            pos, tgt = (100.0 + 4 * f, 150.0, 10.0 + 3 * f), (128.0, 120.0, 128.0)
            va.lookat(pos, tgt)
            va.render()
            vb.lookat(pos, tgt)
            vb.begin_frame()
            for s in (lib.STAGE_ALBEDO, lib.STAGE_CANDIDATES, lib.STAGE_SPATIAL, lib.STAGE_SHADE,
                      lib.STAGE_ACCUMULATE):
                vb.stage(s)
            vb.end_frame()
        va.wait()
        vb.wait()
        assert np.array_equal(va.read_frame().view(np.uint32), vb.read_frame().view(np.uint32))
        assert np.array_equal(va.read_accum().view(np.uint32), vb.read_accum().view(np.uint32))
        bits = lambda a: np.ascontiguousarray(a).view(np.uint8)
        for which in (0, 1):
            assert np.array_equal(bits(va.read_gbuffer(which)), bits(vb.read_gbuffer(which)))
        for role in (0, 1):
            assert np.array_equal(bits(va.read_reservoirs(role)), bits(vb.read_reservoirs(role)))
    finally:
        va.close()
        vb.close()
