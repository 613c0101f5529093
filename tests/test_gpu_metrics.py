"""Converged reference (FP64 running sum of shaded frames) and the MSE / MAE metric
(mse.cpp:33-65) on the GPU, against numpy restatements."""
import numpy as np
import pytest

from oracle import metrics

pytestmark = pytest.mark.gpu


def test_sum64_and_error_match_numpy(lib, cuda_device, scene0):
    world, _ = scene0
    W, H = 128, 72
    pos, tgt = (128.0, 160.0, 0.0), (128.0, 128.0, 128.0)
    ref = lib.View(world, lib.view_desc(W, H, lib.LIGHTS_AREA, spatial=0, temporal=0, accumulate=0))
    ref.lookat(pos, tgt)
    ref.sum64_reset()
    acc = np.zeros((W * H, 3), np.float64)
    K = 6
    for _ in range(K):
        ref.render()
        ref.sum64_add()
        acc += ref.read_frame()[:, :3].astype(np.float64)
    n, mean = ref.sum64_mean()
    assert n == K
    want = acc * (1.0 / K)
    assert np.array_equal(mean, want)
    # a ReSTIR view of the same camera, several frames of reuse, error of frame and accumulator
    img = lib.View(world, lib.view_desc(W, H, lib.LIGHTS_AREA, accumulate=1))
    img.lookat(pos, tgt)
    for _ in range(4):
        img.render()
    img.wait()
    gt = mean.astype(np.float32)
    for which, data in ((0, img.read_frame()), (1, img.read_accum())):
        mse, mae = img.error_vs(ref, which)
        wmse, wmae = metrics.mse_mae(gt, data)
        assert mse == pytest.approx(wmse, rel=1e-12, abs=1e-300) and mae == pytest.approx(wmae, rel=1e-12)
        assert mse > 0.0
    img.close()
    ref.close()


def test_reuse_lowers_error_against_converged(lib, cuda_device, scene0):
    """Sanity of the estimator chain: ReSTIR with reuse has lower MSE against the
    converged render than a single frame of plain RIS (same candidate count)."""
    world, _ = scene0
    W, H = 160, 96
    pos, tgt = (128.0, 150.0, 20.0), (128.0, 100.0, 128.0)
    ref = lib.View(world, lib.view_desc(W, H, lib.LIGHTS_AREA, spatial=0, temporal=0, accumulate=0))
    ref.lookat(pos, tgt)
    ref.sum64_reset()
    for _ in range(256):
        ref.render()
        ref.sum64_add()
    plain = lib.View(world, lib.view_desc(W, H, lib.LIGHTS_AREA, spatial=0, temporal=0, accumulate=0, rng_seed=99))
    plain.lookat(pos, tgt)
    plain.render()
    restir = lib.View(world, lib.view_desc(W, H, lib.LIGHTS_AREA, accumulate=0, rng_seed=99))
    restir.lookat(pos, tgt)
    for _ in range(8):
        restir.render()
    e_plain = plain.error_vs(ref, 0)[0]
    e_restir = restir.error_vs(ref, 0)[0]
    assert e_restir < e_plain, (e_restir, e_plain)
    for v in (ref, plain, restir):
        v.close()
