"""Learned candidate proposal on the GPU: gradients of both trainers (FP32 CUDA cores,
BF16 tensor cores) against the FP64 restatement (oracle/proposal_ref.py), BF16 inference
probabilities against FP64, checkpoint round trip, unbiasedness of the learned source
pdf, the gain of a trained network over the uniform source at equal candidate count, and
online training inside the rendered frame."""
import numpy as np
import pytest

from oracle import proposal_ref as pr

pytestmark = pytest.mark.gpu


def _samples(rng, n, lo=0.0, hi=256.0):
    pos = rng.uniform(lo, hi, (n, 3)).astype(np.float32)
    code = rng.integers(0, 6, n).astype(np.uint32)
    s = np.zeros((n, 4), np.float32)
    s[:, :3] = pos
    s[:, 3] = code.view(np.float32)
    return s


@pytest.fixture(scope="module")
def clustered_view(lib, cuda_device):
    w = lib.World()
    w.generate(lib.scene_preset(0))
    w.cluster_lights(16, seed=3, iters=6)
    v = lib.View(w, lib.view_desc(96, 64, lib.LIGHTS_AREA))
    v.proposal_enable(seed=7, batch=4096)
    yield w, v
    v.close()


def _grad_case(lib, w, v, rng, B, bf16_operands=False):
    n, K, H = v.proposal_shape()
    params = v.proposal_params().astype(np.float64)
    # make the encoding and biases non-trivial so every tensor's gradient is exercised
    L = pr.layout(H, K)
    o, sz = L["enc"]
    params[o:o + sz] = rng.normal(0, 0.5, sz)
    for b in ("b1", "b2", "b3", "b4"):
        o, sz = L[b]
        params[o:o + sz] = rng.normal(0, 0.1, sz)
    v.proposal_set_params(params.astype(np.float32))
    p32 = v.proposal_params().astype(np.float64)
    s = _samples(rng, B)
    t = rng.integers(0, K, B).astype(np.uint32)
    wt = rng.uniform(0.0, 2.0, B).astype(np.float32)
    wt[::9] = 0.0
    loss, g = v.proposal_grad(s, t, wt)
    rloss, rg, L = pr.loss_and_grad(p32, s, t, wt.astype(np.float64), H, K, bf16_operands=bf16_operands)
    return loss, g, rloss, rg, L, (s, t, wt)


def _rel(g, rg, L, name):
    o, sz = L[name]
    a, b = g[o:o + sz].astype(np.float64), rg[o:o + sz]
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-12)


# FP32 trainer: relative error per tensor < 1e-3 against FP64. Tensor-core trainer: its
# operands are BF16, so it is checked against the FP64 gradient of the same BF16-rounded
# network (oracle bf16_operands: inputs, weights, activations and the back-propagated
# gradients rounded where the kernel rounds them) at < 1e-2 per tensor, and against the
# exact FP64 gradient at < 0.15 (what BF16 operands cost; ReLU masks flip near zero).
NAMES = ("enc", "W1", "b1", "W2", "b2", "W3", "b3", "W4", "b4")


def test_fp32_gradients_match_fp64(lib, clustered_view):
    w, _ = clustered_view
    v = lib.View(w, lib.view_desc(96, 64, lib.LIGHTS_AREA))
    try:
        v.proposal_enable(seed=7, batch=4096, training=1)
        loss, g, rloss, rg, L, _ = _grad_case(lib, w, v, np.random.default_rng(1), 250)
        assert loss == pytest.approx(rloss, rel=1e-4)
        for name in NAMES:
            assert _rel(g, rg, L, name) < 1e-3, (name, _rel(g, rg, L, name))
    finally:
        v.close()


@pytest.mark.parametrize("clusters", [16, 256])
def test_tensor_core_gradients_match_fp64(lib, clustered_view, world256, clusters):
    w = clustered_view[0] if clusters == 16 else world256
    v = lib.View(w, lib.view_desc(64, 48, lib.LIGHTS_AREA))
    try:
        v.proposal_enable(seed=7, batch=4096, training=2)
        assert v.proposal_shape()[1] == clusters
        # 250 / 1000 samples: ragged last tiles of 16, one and several CTAs
        B = 250 if clusters == 16 else 1000
        loss, g, rloss, rg, L, (s, t, wt) = _grad_case(lib, w, v, np.random.default_rng(1), B, bf16_operands=True)
        assert loss == pytest.approx(rloss, rel=2e-3)
        for name in NAMES:
            assert _rel(g, rg, L, name) < 1e-2, (name, _rel(g, rg, L, name))
        _, K, H = v.proposal_shape()
        p32 = v.proposal_params().astype(np.float64)
        _, rg64, _ = pr.loss_and_grad(p32, s, t, wt.astype(np.float64), H, K)
        for name in NAMES:
            assert _rel(g, rg64, L, name) < 0.15, (name, _rel(g, rg64, L, name))
    finally:
        v.close()


def test_inference_probabilities_match_fp64(lib, clustered_view):
    w, v = clustered_view
    n, K, H = v.proposal_shape()
    rng = np.random.default_rng(2)
    s = _samples(rng, 300)
    probs = v.proposal_probs(s)
    ref = pr.softmax(pr.forward(v.proposal_params().astype(np.float64), s, H, K)[-1])
    assert np.allclose(probs.sum(1), 1.0, atol=1e-3)
    # BF16 weights/activations and FP16 logits: absolute error on probabilities
    assert np.abs(probs - ref).max() < 2e-2


def test_checkpoint_round_trip(lib, clustered_view, tmp_path):
    w, v = clustered_view
    p0 = v.proposal_params()
    v.proposal_save(tmp_path / "prop.bin")
    v.proposal_set_params(np.zeros_like(p0))
    v.proposal_load(tmp_path / "prop.bin")
    assert np.array_equal(v.proposal_params(), p0)


def _converged_mean(lib, world, learned, frames, pos, tgt, seed, W=96, H=64, train_view=None, inference=0, share=1):
    v = lib.View(world, lib.view_desc(W, H, lib.LIGHTS_AREA, spatial=0, temporal=0, accumulate=0, rng_seed=seed))
    v.lookat(pos, tgt)
    if learned:
        v.proposal_enable(seed=5, batch=4096, inference=inference, pixels_per_eval=share)
        if train_view is not None:
            v.proposal_set_params(train_view.proposal_params())
        v.proposal_use(True)
    v.sum64_reset()
    for _ in range(frames):
        v.render()
        v.sum64_add()
    n, mean = v.sum64_mean()
    v.close()
    return mean


def test_learned_source_is_unbiased(lib, cuda_device):
    """Spatial/temporal off: RIS is unbiased for any source pdf > 0, so the learned
    (untrained, random) proposal and the uniform one converge to the same image."""
    w = lib.World()
    w.generate(lib.scene_preset(0))
    w.cluster_lights(16, seed=3, iters=6)
    pos, tgt = (128.0, 150.0, 20.0), (128.0, 100.0, 128.0)
    a = _converged_mean(lib, w, False, 384, pos, tgt, 11)
    b = _converged_mean(lib, w, True, 384, pos, tgt, 12)
    ma, mb = a.mean(), b.mean()
    assert ma > 0 and abs(ma - mb) / ma < 0.03, (ma, mb)


def test_trained_proposal_beats_uniform(lib, cuda_device):
    """Many emitters (config 3 lights), a short online training on the plain method's
    reservoirs: at equal candidate count the learned source lowers the single-frame MSE
    against the converged render."""
    w = lib.World()
    w.generate(lib.scene_preset(3))
    w.cluster_lights(256, seed=1, iters=6)
    d = lib.scene_preset(3)
    pos, tgt = lib.camera_path(d, 1, 0, 300)
    W, H = 192, 108
    ref = lib.View(w, lib.view_desc(W, H, lib.LIGHTS_AREA, spatial=0, temporal=0, accumulate=0, rng_seed=77))
    ref.lookat(pos, tgt)
    ref.sum64_reset()
    for _ in range(1024):
        ref.render()
        ref.sum64_add()
    trainer = lib.View(w, lib.view_desc(W, H, lib.LIGHTS_AREA, rng_seed=5))
    trainer.lookat(pos, tgt)
    trainer.proposal_enable(seed=2, batch=8192)
    losses = []
    for it in range(60):
        trainer.render()
        losses.append(trainer.proposal_train(2))
    assert np.mean(losses[-10:]) < np.mean(losses[:5])
    errs = {}
    for learned in (False, True):
        v = lib.View(w, lib.view_desc(W, H, lib.LIGHTS_AREA, spatial=0, temporal=0, accumulate=0, rng_seed=31))
        v.lookat(pos, tgt)
        if learned:
            v.proposal_enable(seed=2, batch=8192)
            v.proposal_set_params(trainer.proposal_params())
            v.proposal_use(True)
        e = []
        for _ in range(16):
            v.render()
            e.append(v.error_vs(ref, 0)[0])
        errs[learned] = float(np.mean(e))
        v.close()
    assert errs[True] < errs[False], errs
    trainer.close()
    ref.close()


@pytest.fixture(scope="module")
def world256(lib, cuda_device):
    w = lib.World()
    w.generate(lib.scene_preset(0, emitters=2048, emitter_mode=1))
    w.cluster_lights(256, seed=3, iters=6)
    return w


def test_tcgen05_inference_matches_mma_and_fp64(lib, world256):
    """The tcgen05 / TMEM inference kernel (256 clusters) against the mma.sync kernel with
    the same parameters and against the FP64 forward pass; 600 samples = 3 tiles of 128
    per CTA half, the last one partial."""
    a = lib.View(world256, lib.view_desc(64, 48, lib.LIGHTS_AREA))
    b = lib.View(world256, lib.view_desc(64, 48, lib.LIGHTS_AREA))
    try:
        a.proposal_enable(seed=7, batch=4096, inference=1)
        b.proposal_enable(seed=7, batch=4096, inference=2)
        b.proposal_set_params(a.proposal_params())
        n, K, H = b.proposal_shape()
        assert K == 256
        rng = np.random.default_rng(3)
        s = _samples(rng, 600, 0.0, 1000.0)
        pa = a.proposal_probs(s)
        pb = b.proposal_probs(s)
        ref = pr.softmax(pr.forward(b.proposal_params().astype(np.float64), s, H, K)[-1])
        assert np.allclose(pb.sum(1), 1.0, atol=1e-3)
        assert np.abs(pb - ref).max() < 2e-2
        assert np.abs(pb - pa).max() < 1e-2
    finally:
        a.close()
        b.close()


@pytest.mark.parametrize("share", [1, 2, 4, 8])
def test_tcgen05_learned_source_is_unbiased(lib, world256, share):
    """The tcgen05 inference kernel (256 clusters) samples candidates with the probability
    it reports: with spatial and temporal reuse off its learned source and the uniform
    one converge to the same image (a source pdf that differed from the sampling
    frequencies would bias the RIS estimate). share = 2 / 4 / 8: runs of up to two / four /
    eight consecutive hit pixels sample from one network evaluation (the run's first)."""
    pos, tgt = (110.0, 150.0, 10.0), (128.0, 110.0, 128.0)
    a = _converged_mean(lib, world256, False, 384, pos, tgt, 21)
    b = _converged_mean(lib, world256, True, 384, pos, tgt, 22, inference=2, share=share)
    ma, mb = a.mean(), b.mean()
    assert ma > 0 and abs(ma - mb) / ma < 0.03, (ma, mb)


def test_tcgen05_learned_render_runs_clean(lib, world256):
    """Frames rendered with the tcgen05 inference: no device error flag, finite image."""
    v = lib.View(world256, lib.view_desc(200, 120, lib.LIGHTS_AREA, num_candidates=12))
    try:
        v.proposal_enable(seed=5, batch=8192, inference=2)
        v.lookat((110.0, 150.0, 10.0), (128.0, 110.0, 128.0))
        for _ in range(3):
            v.render()
            v.proposal_train(1)
        v.proposal_use(True)
        for f in range(3):
            v.lookat((110.0 + f, 150.0, 10.0), (128.0, 110.0, 128.0))
            v.render()
        v.wait()
        img = v.read_frame()
        assert np.isfinite(img).all() and img[..., :3].max() > 0
    finally:
        v.close()


@pytest.mark.parametrize("lag", [0, 1])
def test_online_training_inside_the_frame(lib, cuda_device, lag):
    """A learned view that trains itself: each vxr_view_render ends with one training
    step on that frame's own final reservoirs (timed as proposal_train). Starting from
    random parameters, after 80 such frames its single-frame MSE against the converged
    render is below the uniform source's at the same candidate count. lag = 1: a frame's
    inference uses the weights of the step two frames back (published copies)."""
    w = lib.World()
    w.generate(lib.scene_preset(3))
    w.cluster_lights(256, seed=1, iters=6)
    d = lib.scene_preset(3)
    pos, tgt = lib.camera_path(d, 1, 0, 300)
    W, H = 192, 108
    ref = lib.View(w, lib.view_desc(W, H, lib.LIGHTS_AREA, spatial=0, temporal=0, accumulate=0, rng_seed=77))
    ref.lookat(pos, tgt)
    ref.sum64_reset()
    for _ in range(1024):
        ref.render()
        ref.sum64_add()
    errs = {}
    for learned in (False, True):
        v = lib.View(w, lib.view_desc(W, H, lib.LIGHTS_AREA, num_candidates=8, rng_seed=31))
        v.lookat(pos, tgt)
        if learned:
            v.proposal_enable(seed=2, batch=8192, training_lag=lag)
            v.proposal_use(True)
            v.proposal_online(1)
            p0 = v.proposal_params()
            v.kernel_timing(True)
            for _ in range(80):
                v.render()
            v.wait()
            v.kernel_timing(False)
            ks = v.kernel_stats(reset=True)
            assert ks["proposal_train"][1] == 80 and ks["proposal_train"][0] > 0
            assert not np.array_equal(v.proposal_params(), p0)
        e = []
        for _ in range(24):
            v.render()
            e.append(v.error_vs(ref, 0)[0])
        errs[learned] = float(np.median(e))
        v.close()
    ref.close()
    assert errs[True] < errs[False], errs


@pytest.mark.parametrize("lag", [0, 1])
def test_online_training_weights_reach_the_right_frame(lib, world256, lag):
    """With one online training step per frame, the inference of frame f uses the
    parameters after step f - 1 (training_lag = 0) or after step f - 2 (training_lag = 1,
    the published copies; the initial parameters before that). Checked bit for bit: the
    candidates a training view draws in frames 1 and 2 equal, pixel for pixel, those of
    views that never train and hold the expected parameters (same camera and seeds; one
    network evaluation per pixel, so no draw depends on the hit list's order)."""
    W, H = 96, 64
    pos, tgt = (110.0, 150.0, 10.0), (128.0, 110.0, 128.0)

    def make(params=None, online=0):
        v = lib.View(world256, lib.view_desc(W, H, lib.LIGHTS_AREA, num_candidates=4, rng_seed=41))
        v.lookat(pos, tgt)
        v.proposal_enable(seed=3, batch=4096, training_lag=lag)
        if params is not None:
            v.proposal_set_params(params)
        v.proposal_use(True)
        v.proposal_online(online)
        return v

    tv = make(online=1)
    p0 = tv.proposal_params()
    got, after = [], [p0]
    for f in range(3):
        tv.render()
        tv.wait()
        got.append(tv.proposal_candidates(4))
        after.append(tv.proposal_params())      # after step f
    tv.close()
    assert not np.array_equal(after[1], p0) and not np.array_equal(after[2], after[1])
    for f in (1, 2):
        want_params = after[f - lag] if f - lag >= 1 else p0   # step f - 1 - lag, or the initial
        rv = make(params=want_params)
        for g in range(f + 1):
            rv.render()
            rv.wait()
        hits, cand = rv.proposal_candidates(4)
        rv.close()
        # the hit list's order depends on the compaction's atomics: compare per pixel
        ga, gc = got[f]
        oa, ob = np.argsort(ga), np.argsort(hits)
        assert np.array_equal(ga[oa], hits[ob]), f
        assert np.array_equal(gc[:, oa], cand[:, ob]), (f, lag)


def test_overlapped_learned_frames_equal_stage_by_stage_ones(lib, world256):
    """A learned view's front half (primary rays, hit list, inference, candidates and
    their visibility) runs beside the previous frame's shading when frames follow each
    other through vxr_view_render; with the same network (no training in the frames; one
    evaluation per pixel, so no draw depends on the hit list's order) the images,
    G-buffer planes and reservoirs equal those of frames rendered stage by stage."""
    W, H = 240, 136
    trainer = lib.View(world256, lib.view_desc(W, H, lib.LIGHTS_AREA, num_candidates=4))
    trainer.proposal_enable(seed=5, batch=8192, inference=2)
    trainer.lookat((110.0, 150.0, 10.0), (128.0, 110.0, 128.0))
    for _ in range(3):
        trainer.render()
        trainer.proposal_train(1)
    params = trainer.proposal_params()
    trainer.close()
    views = []
    try:
        for _ in range(2):
            v = lib.View(world256, lib.view_desc(W, H, lib.LIGHTS_AREA, num_candidates=4, accumulate=1, rng_seed=17))
            v.proposal_enable(seed=5, batch=8192, inference=2)
            v.proposal_set_params(params)
            v.proposal_use(True)
            views.append(v)
        va, vb = views
        for f in range(6):
            pos, tgt = (104.0 + 3 * f, 150.0, 10.0 + 2 * f), (128.0, 110.0, 128.0)
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
        bits = lambda a: np.ascontiguousarray(a).view(np.uint8)
        assert np.array_equal(bits(va.read_frame()), bits(vb.read_frame()))
        assert np.array_equal(bits(va.read_accum()), bits(vb.read_accum()))
        for which in (0, 1):
            assert np.array_equal(bits(va.read_gbuffer(which)), bits(vb.read_gbuffer(which)))
        for role in (0, 1):
            assert np.array_equal(bits(va.read_reservoirs(role)), bits(vb.read_reservoirs(role)))
    finally:
        for v in views:
            v.close()
