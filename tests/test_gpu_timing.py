"""Per-kernel timing (vxr_view_kernel_timing / vxr_view_kernel_stats) and the work
counts of a frame (vxr_view_work_counts)."""
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
