"""Pin the C oracle (oracle/vxr_oracle.c) to the reference's own render-path kernels
(cl/*.cl compiled for the CPU by oracle/ref_build.py): every stage output bit-exact,
both light models, several frames with temporal and spatial reuse, plus fuzzed single
rays through all three DDA variants. Skipped where the reference oracle cannot be
built (no reference checkout and no generated source)."""
import numpy as np
import pytest

from conftest import assert_records_equal
from oracle import binding as ob

KNOBS = dict(numberOfCandidates=32, numberOfMaxTemporalImportance=20, spatialRadius=30, spatialTaps=5)


@pytest.fixture(scope="module")
def ref_lib():
    lib = ob.load_ref()
    if lib is None:
        pytest.skip("reference oracle unavailable on this machine")
    return lib


def _frames(arrays, W, H, point, nframes, cams, **flags):
    port = ob.Renderer("port", arrays, W, H, point)
    ref = ob.Renderer("ref", arrays, W, H, point)
    cam = ob.CameraPath(W, H)
    opts = dict(spatial=1, temporal=1, accumulate=1)
    opts.update(flags)
    try:
        for f in range(nframes):
            pos, tgt = cams(f)
            cam.lookat(pos, tgt)
            k = cam.begin(numberOfLights=len(arrays.lights), **KNOBS, **opts)
            port.frame_start()
            ref.frame_start()
            ctx = f"[{'point' if point else 'area'} frame {f}]"
            for s in range(1, 6):
                port.stage(k, s)
                ref.stage(k, s)
                if s == 1:
                    assert_records_equal("gbuffer", port.gbuffer(0), ref.gbuffer(0), ctx)
                elif s == 2:
                    got, want = port.reservoirs(0), ref.reservoirs(0)
                    assert_records_equal("candidates", got, want, ctx)
                    assert_records_equal("seed", port.gbuffer(0)["seed"], ref.gbuffer(0)["seed"], ctx)
                elif s == 3:
                    assert_records_equal("spatial", port.reservoirs(1), ref.reservoirs(1), ctx)
                elif s == 4:
                    assert_records_equal("frame", port.image(0), ref.image(0), ctx)
                    assert_records_equal("history", port.reservoirs(2), ref.reservoirs(2), ctx)
                else:
                    assert_records_equal("accum", port.image(1), ref.image(1), ctx)
            # the GPU layout stores no W: W must equal sumOfWeights / max(1e-5, pHat * M) exactly
            r = ref.reservoirs(2)
            den = np.maximum(np.float32(1e-5), (r["pHat"] * r["streamLength"].astype(np.float32)).astype(np.float32))
            derived = (r["sumOfWeights"] / den).astype(np.float32)
            assert np.array_equal(derived.view(np.uint32), r["adjustedWeight"].view(np.uint32)), ctx
            cam.end()
    finally:
        port.close()
        ref.close()


def _orbit(f):
    return (128.0 + 7.0 * f, 158.0 - 1.5 * f, 2.0 * f), (128.0, 128.0, 128.0)


@pytest.mark.parametrize("point", [True, False], ids=["point", "area"])
def test_port_matches_reference_config0(ref_lib, world0_arrays, point):
    _frames(world0_arrays, 200, 120, point, 4, _orbit)


def test_port_matches_reference_inside_world(ref_lib, world0_arrays):
    _frames(world0_arrays, 120, 80, False, 3, lambda f: ((100.0 + 2 * f, 90.0, 100.0), (140.0, 40.0, 150.0)))


def test_port_matches_reference_no_reuse(ref_lib, world0_arrays):
    _frames(world0_arrays, 96, 64, False, 2, _orbit, spatial=0, temporal=0, accumulate=0)


def test_port_matches_reference_translucent(ref_lib, lib):
    """A scene with translucent voxels and a solid emitter brick (size-8 light)."""
    w = lib.World()
    w.box(0, 0, 0, 64, 8, 64, 0xF888)                                          # opaque floor
    w.box(10, 8, 10, 30, 20, 12, 0x7F44)                                        # translucent wall, alpha 7
    w.box(40, 8, 40, 44, 30, 44, 0x3488)                                        # faint pillar, alpha 3
    w.box(16, 24, 16, 24, 32, 24, (5 << 16) | 0xFFFF)                          # 8^3 emitter brick -> size 8
    for i in range(6):
        w.set(5 + 9 * i, 12 + i, 50, (3 << 16) | 0xF0F7)                        # single-voxel emitters
    w.optimize()
    w.scan_lights()
    g, b, l = w.arrays()
    assert 8 in set(l["size"].tolist()) and 1 in set(l["size"].tolist())
    arrays = ob.WorldArrays(g, b, l)
    _frames(arrays, 96, 72, False, 3, lambda f: ((-20.0 + f, 40.0, -15.0), (32.0, 8.0, 32.0)))
    _frames(arrays, 64, 48, True, 2, lambda f: ((-20.0 + f, 40.0, -15.0), (32.0, 8.0, 32.0)))


def test_port_matches_reference_zero_and_one_light(ref_lib, lib):
    w = lib.World()
    w.box(0, 0, 0, 64, 8, 64, 0xF888)
    w.scan_lights()
    g, b, l = w.arrays()
    _frames(ob.WorldArrays(g, b, l), 48, 32, False, 2, lambda f: ((32.0, 30.0, -10.0), (32.0, 0.0, 32.0)))
    w.set(30, 12, 30, (9 << 16) | 0xFFFF)
    w.scan_lights()
    g, b, l = w.arrays()
    assert len(l) == 1
    _frames(ob.WorldArrays(g, b, l), 48, 32, False, 3, lambda f: ((32.0 + f, 30.0, -10.0), (32.0, 0.0, 32.0)))


@pytest.mark.parametrize("mode", [0, 1, 2])
def test_single_ray_traversal_matches_reference(ref_lib, world0_arrays, mode):
    rng = np.random.default_rng(7 + mode)
    port = ob.Renderer("port", world0_arrays, 4, 4, False)
    ref = ob.Renderer("ref", world0_arrays, 4, 4, False)
    n = 4000
    origins = np.concatenate([rng.uniform(-300, 1300, (n // 2, 3)),            # mostly outside the map
                              rng.uniform(0, 256, (n // 2, 3))]).astype(np.float32)
    dirs = rng.normal(size=(n, 3)).astype(np.float32)
    dirs[::7, 0] = 0.0                                                           # axis-aligned components
    dirs[::11, 1] = 1e-9
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    for i in range(n):
        steps = int(rng.choice([128, 999999, 12]))
        through = int(rng.choice([0, 0x7F44, 0xF888]))
        a = port.trace(mode, origins[i], dirs[i], steps, through, 0xFFFF)
        b = ref.trace(mode, origins[i], dirs[i], steps, through, 0xFFFF)
        assert a[0] == b[0] and a[2] == b[2] and np.float32(a[1]).view(np.uint32) == np.float32(b[1]).view(np.uint32), \
            (i, origins[i], dirs[i], a, b)
