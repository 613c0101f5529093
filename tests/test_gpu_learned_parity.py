"""The learned candidate path bit for bit against the C oracle, given the proposal's draws.

The proposal's network and sampler are checked with tolerances and unbiasedness tests
(test_gpu_proposal.py); everything after the draw is the reference's arithmetic: the
candidate kernel weighs each drawn emitter with p_hat / p_src, keeps one by weighted
reservoir sampling, traces its visibility, reuses temporally, then the spatial and
shading stages run. The oracle (oracle/vxr_oracle.c) runs the same stages with the same
candidates (read back through vxr_view_proposal_read_candidates), and every stage output
of every frame must match bit for bit - for the mma.sync and the tcgen05 inference, with
one network evaluation per hit pixel and per two."""
import numpy as np
import pytest

from conftest import assert_records_equal
from oracle import binding as ob

pytestmark = pytest.mark.gpu


def _orbit(f):
    return (120.0 + 5.0 * f, 150.0 - 2.0 * f, 8.0 + 3.0 * f), (128.0, 118.0, 128.0)


@pytest.mark.parametrize("clusters,inference,share", [(16, 1, 1), (256, 2, 1), (256, 2, 2), (256, 2, 4), (256, 2, 8)])
def test_learned_frames_match_oracle_given_candidates(lib, cuda_device, clusters, inference, share):
    w = lib.World()
    if clusters == 256:
        w.generate(lib.scene_preset(0, emitters=2048, emitter_mode=1))
    else:
        w.generate(lib.scene_preset(0))
    w.cluster_lights(clusters, seed=3, iters=6)
    g, b, l = w.arrays()
    W, H = 128, 80
    view = lib.View(w, lib.view_desc(W, H, lib.LIGHTS_AREA, accumulate=1, num_candidates=8))
    port = ob.Renderer("port", ob.WorldArrays(g, b, l), W, H, False)
    try:
        view.proposal_enable(seed=11, batch=4096, inference=inference, pixels_per_eval=share)
        view.proposal_use(True)
        for f in range(3):
            view.lookat(*_orbit(f))
            k = view.begin_frame()
            port.frame_start()
            ctx = f"[learned, {clusters} clusters, inference {inference}, share {share}, frame {f}]"
            view.stage(lib.STAGE_ALBEDO)
            port.stage(k, 1)
            assert_records_equal("gbuffer", view.read_gbuffer(0), port.gbuffer(0), ctx)
            view.stage(lib.STAGE_CANDIDATES)
            K = min(k.numberOfCandidates, k.numberOfLights)
            hits, cand = view.proposal_candidates(K)
            assert len(hits) > 100 and (cand[:, :, 0] < len(l)).all()
            pdf = cand[:, :, 1].view(np.float32)
            assert (pdf > 0).all() and (pdf <= 1).all()
            idx = np.zeros((K, W * H), np.uint32)
            p = np.ones((K, W * H), np.float32)
            idx[:, hits] = cand[:, :, 0]
            p[:, hits] = pdf
            port.set_candidates(idx, p)
            port.stage(k, 2)
            assert_records_equal("candidates", view.read_reservoirs(0), port.reservoirs(0), ctx)
            assert_records_equal("seed", view.read_gbuffer(0)["seed"], port.gbuffer(0)["seed"], ctx)
            for s in (3, 4, 5):
                view.stage(s)
                port.stage(k, s)
            assert_records_equal("spatial", view.read_reservoirs(1), port.reservoirs(2), ctx)
            assert_records_equal("frame", view.read_frame(), port.image(0), ctx)
            assert_records_equal("accum", view.read_accum(), port.image(1), ctx)
            view.end_frame()
            view.wait()
        # the learned frames differ from the uniform source's: the proposal was used
        assert (idx[:, hits] != 0).any()
    finally:
        port.close()
        view.close()


def _shading_points(k, gb, W):
    """Shading points (float64) and side codes (axis * 2 + facing) of the given pixels."""
    pix = np.arange(len(gb))
    x, y = pix % W, pix // W
    E, p0, p1, p2 = (np.array(v[:], np.float64) for v in (k.E, k.p0, k.p1, k.p2))
    u = (x * k.oneOverRes[0])[:, None]
    v = (y * k.oneOverRes[1])[:, None]
    D = p0 + (p1 - p0) * u + (p2 - p0) * v - E
    D /= np.linalg.norm(D, axis=1, keepdims=True)
    side = gb["side"].astype(np.int64)
    comp = D[np.arange(len(gb)), np.minimum(side, 2)]
    code = side * 2 + (comp > 0)
    return E + D * gb["dist"][:, None].astype(np.float64), code


def _runs(sp, code, hits, group, dist):
    """Runs of the hit list as the pairing kernel forms them (aligned groups of `group`
    entries, a run extended while an entry is on the first one's voxel side within `dist`
    of it in every coordinate), and whether any test sat within 1 % of `dist`."""
    runs, unsure = [], False
    n = len(hits)
    for g0 in range(0, n, group):
        m = min(group, n - g0)
        start = 0
        for q in range(1, m):
            a, b = hits[g0 + start], hits[g0 + q]
            gap = np.abs(sp[a] - sp[b]).max()
            unsure |= code[a] == code[b] and abs(gap - dist) <= 0.01 * dist
            if not (code[a] == code[b] and gap <= dist):
                runs.append((g0 + start, q - start))
                start = q
        runs.append((g0 + start, m - start))
    return runs, unsure


@pytest.mark.parametrize("group,dist", [(2, 2.0), (2, 1e30), (4, 2.0), (8, 2.0), (8, 1e30)])
def test_shared_evaluations_pair_only_compatible_pixels(lib, cuda_device, group, dist):
    """pixels_per_eval = 2, 4 or 8: the hit list in aligned groups of that many entries; a run
    of entries on the voxel side of its first entry, within share_distance voxels of it in
    every coordinate, shares one network evaluation. Pixels of one run draw from one
    distribution, so an emitter two of them drew carries the same source pdf in both;
    pixels of different runs evaluate separately."""
    w = lib.World()
    w.generate(lib.scene_preset(0, emitters=2048, emitter_mode=1))
    w.cluster_lights(256, seed=3, iters=6)
    W, H = 160, 96
    view = lib.View(w, lib.view_desc(W, H, lib.LIGHTS_AREA, num_candidates=32))
    try:
        view.proposal_enable(seed=11, batch=4096, inference=2, pixels_per_eval=group, share_distance=dist)
        # large random parameters: the distribution changes visibly between shading points
        p = view.proposal_params()
        view.proposal_set_params(np.random.default_rng(5).normal(0.0, 0.3, p.shape).astype(p.dtype))
        view.proposal_use(True)
        view.lookat(*_orbit(1))
        k = view.begin_frame()
        view.stage(lib.STAGE_ALBEDO)
        view.stage(lib.STAGE_CANDIDATES)
        K = min(k.numberOfCandidates, k.numberOfLights)
        hits, cand = view.proposal_candidates(K)
        rows = view.proposal_rows()
        sp, code = _shading_points(k, view.read_gbuffer(0), W)
        view.end_frame()
        view.wait()
        # the frame's evaluation count is its number of runs (a group with a test within 1 %
        # of share_distance may split either way)
        n_runs, n_unsure = 0, 0
        for g0 in range(0, len(hits), group):
            sub, unsure = _runs(sp, code, hits[g0:g0 + group], group, dist)
            n_runs += len(sub)
            n_unsure += int(unsure)
        assert abs(rows - n_runs) <= n_unsure * (group - 1), (rows, n_runs, n_unsure)
        assert rows < len(hits)

        def same_pdfs(i, j):
            """(the two entries drew a common emitter, every common one has equal pdfs)"""
            m = cand[:, i, 0][:, None] == cand[:, j, 0][None, :]
            if not m.any():
                return False, False
            ia, ib = np.nonzero(m)
            return True, bool((cand[ia, i, 1] == cand[ib, j, 1]).all())

        inside, across = [], []
        n = len(hits)
        for g0 in range(0, n, group):
            sub, unsure = _runs(sp, code, hits[g0:g0 + group], group, dist)
            if unsure:
                continue
            run_of = {}
            for r, (s0, ln) in enumerate(sub):
                for q in range(ln):
                    run_of[g0 + s0 + q] = r
            ids = sorted(run_of)
            for x in range(len(ids)):
                for y in range(x + 1, len(ids)):
                    common, equal = same_pdfs(ids[x], ids[y])
                    if common:
                        (inside if run_of[ids[x]] == run_of[ids[y]] else across).append(equal)
        assert len(inside) > 200
        assert all(inside)
        if dist < 1e29:
            assert len(across) > 20
            assert np.mean(across) < 0.05
    finally:
        view.close()
