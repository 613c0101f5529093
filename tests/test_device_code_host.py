"""The product's device-side traversal and trig (smallproject_gb300/csrc/device.cuh),
compiled for the host CPU by tests/native/build_devhost.py, against the oracle:
- trace<MODE> (primary rays, shadow rays, trace-through) bit-exact with the oracle's
  DDA for fuzzed rays;
- the resumable walker used by the persistent shadow tracer bit-exact with trace<1>;
- sincos_vx identical to the oracle's sin/cos on reachable tap angles.
A CPU check of the GPU code's arithmetic; the GPU tests check the compiled kernels."""
import ctypes as C
import os
import sys

import numpy as np
import pytest

from conftest import ROOT
from oracle import binding as ob

sys.path.insert(0, os.path.join(ROOT, "tests", "native"))
import build_devhost  # noqa: E402


@pytest.fixture(scope="module")
def dh():
    path = build_devhost.build()
    if path is None:
        pytest.skip("CUDA headers unavailable")
    lib = C.CDLL(path)
    P = C.c_void_p
    F = C.POINTER(C.c_float)
    lib.dh_trace.restype = C.c_uint32
    lib.dh_trace.argtypes = [C.c_int, P, P, P, F, F, C.c_int, C.c_uint32, C.c_uint32, F, C.POINTER(C.c_uint32)]
    lib.dh_walk.restype = C.c_uint32
    lib.dh_walk.argtypes = [P, P, P, F, F, C.c_int, F, C.POINTER(C.c_uint32), C.POINTER(C.c_int), C.POINTER(C.c_int)]
    lib.dh_sincos.argtypes = [C.c_float, F, F]
    lib.dh_walk_burst.restype = C.c_uint32
    lib.dh_walk_burst.argtypes = [P, P, P, F, F, C.c_int, C.c_int, F, C.POINTER(C.c_uint32), C.POINTER(C.c_int)]
    lib.dh_area_sample.argtypes = [C.c_int, F, F, C.c_uint32, F]
    lib.dh_trace_skip.restype = C.c_uint32
    lib.dh_trace_skip.argtypes = [C.c_int, P, P, P, P, P, P, F, F, C.c_int, C.c_uint32, C.c_uint32, F,
                                  C.POINTER(C.c_uint32)]
    lib.dh_walk_skip.argtypes = [P, P, P, P, F, F, C.c_int, F, C.POINTER(C.c_uint32), C.POINTER(C.c_int)]
    lib.dh_shadow.restype = C.c_int
    lib.dh_shadow.argtypes = [P, P, P, P, F, F, C.c_uint32, C.c_uint32, C.c_int, C.POINTER(C.c_int)]
    return lib


def _rays(n, seed, lo=-300.0, hi=1300.0, inside=(0.0, 256.0)):
    rng = np.random.default_rng(seed)
    o = np.concatenate([rng.uniform(lo, hi, (n // 2, 3)), rng.uniform(*inside, (n - n // 2, 3))]).astype(np.float32)
    d = rng.normal(size=(n, 3)).astype(np.float32)
    d[::7, 0] = 0.0
    d[::13, 2] = 1e-9
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return o, d.astype(np.float32), rng


def _f3(v):
    return (C.c_float * 3)(*[float(x) for x in v])


@pytest.mark.parametrize("mode", [0, 1, 2])
def test_device_trace_matches_oracle(dh, world0_arrays, mode):
    wa = world0_arrays
    port = ob.Renderer("port", wa, 4, 4, False)
    o, d, rng = _rays(3000, 100 + mode)
    for i in range(len(o)):
        steps = int(rng.choice([128, 999999, 9]))
        through = int(rng.choice([0, 0x7F44, 0xF888]))
        dist, side = C.c_float(0), C.c_uint32(0)
        v = dh.dh_trace(mode, wa.grid.ctypes.data, wa.uber.ctypes.data, wa.bricks.ctypes.data, _f3(o[i]), _f3(d[i]),
                        steps, through, 0xFFFF, C.byref(dist), C.byref(side))
        want = port.trace(mode, o[i], d[i], steps, through, 0xFFFF)
        assert (v, side.value) == (want[0], want[2]) and \
            np.float32(dist.value).view(np.uint32) == np.float32(want[1]).view(np.uint32), (i, o[i], d[i])


def test_walker_matches_recursive_trace(dh, world0_arrays):
    wa = world0_arrays
    o, d, rng = _rays(6000, 7)
    # shadow-ray-like rays: from just above the terrain surface towards random points
    total_visits = 0
    for i in range(len(o)):
        steps = int(rng.choice([128, 128, 999999, 5, 1]))
        dist, side = C.c_float(0), C.c_uint32(0)
        v = dh.dh_trace(1, wa.grid.ctypes.data, wa.uber.ctypes.data, wa.bricks.ctypes.data, _f3(o[i]), _f3(d[i]),
                        steps, 0, 0, C.byref(dist), C.byref(side))
        dist2, side2, st, nv = C.c_float(0), C.c_uint32(0), C.c_int(0), C.c_int(0)
        v2 = dh.dh_walk(wa.grid.ctypes.data, wa.uber.ctypes.data, wa.bricks.ctypes.data, _f3(o[i]), _f3(d[i]), steps,
                        C.byref(dist2), C.byref(side2), C.byref(st), C.byref(nv))
        total_visits += nv.value
        if st.value == 1:
            assert v == v2 and side.value == side2.value and \
                np.float32(dist.value).view(np.uint32) == np.float32(dist2.value).view(np.uint32), (i, o[i], d[i])
        else:
            assert v == 0, (i, o[i], d[i], v)
    assert total_visits > 10000


def test_walker_bursts_match_single_visits(dh, world0_arrays):
    """walk_run(n) (the shadow tracer's bursts) ends exactly like n single visits."""
    wa = world0_arrays
    o, d, rng = _rays(4000, 19)
    for i in range(len(o)):
        steps = int(rng.choice([128, 999999, 7, 1]))
        burst = int(rng.choice([1, 2, 3, 4, 8, 16, 64]))
        dist, side = C.c_float(0), C.c_uint32(0)
        v = dh.dh_trace(1, wa.grid.ctypes.data, wa.uber.ctypes.data, wa.bricks.ctypes.data, _f3(o[i]), _f3(d[i]),
                        steps, 0, 0, C.byref(dist), C.byref(side))
        d2, s2, st = C.c_float(0), C.c_uint32(0), C.c_int(0)
        v2 = dh.dh_walk_burst(wa.grid.ctypes.data, wa.uber.ctypes.data, wa.bricks.ctypes.data, _f3(o[i]), _f3(d[i]),
                              steps, burst, C.byref(d2), C.byref(s2), C.byref(st))
        if st.value == 1:
            assert v == v2 and side.value == s2.value and \
                np.float32(dist.value).view(np.uint32) == np.float32(d2.value).view(np.uint32), (i, burst)
        else:
            assert v == 0, (i, burst)


def brick_boxes(bricks, nonzero=False):
    """Per brick the box of its opaque voxels (type nibble 15), or of its non-zero voxels,
    packed as the GPU builds them at upload (build_brick_boxes_kernel): low x, y, z in
    bits 0-8, high (inclusive) in bits 9-17, 3 bits each; 0xFFFFFFFF when there is none."""
    b4 = bricks.reshape(-1, 8, 8, 8)                                   # [n, z, y, x]
    op = (b4 != 0) if nonzero else (((b4 >> 12) & 15) == 15)
    out = np.full(len(op), 0xFFFFFFFF, np.uint32)
    for i in np.nonzero(op.any(axis=(1, 2, 3)))[0]:
        z, y, x = np.nonzero(op[i])
        lo, hi = (x.min(), y.min(), z.min()), (x.max(), y.max(), z.max())
        out[i] = sum(int(v) << (3 * a) for a, v in enumerate(lo)) | sum(int(v) << (9 + 3 * a) for a, v in enumerate(hi))
    return out


def uber_boxes0(grid, bricks):
    """Per uber cell (x + z*32 + y*1024) the box of its non-zero voxels (brick-less non-zero
    grid cells whole, bricks by their non-zero box), 5 bits per corner coordinate: low
    x, y, z in bits 0-14, high (inclusive) in bits 15-29; 0xFFFFFFFF when empty (the GPU
    builds the same at upload, build_uber_boxes_kernel)."""
    g = grid.reshape(128, 128, 128).astype(np.int64)                  # [gy, gz, gx]
    bb = brick_boxes(bricks, nonzero=True).astype(np.int64)
    lo = np.full((128, 128, 128, 3), 99, np.int64)
    hi = np.full((128, 128, 128, 3), -1, np.int64)
    gy, gz, gx = np.meshgrid(np.arange(128), np.arange(128), np.arange(128), indexing="ij")
    base = np.stack([(gx & 3) * 8, (gy & 3) * 8, (gz & 3) * 8], -1)    # x, y, z in the uber cell
    solid = ((g & 1) == 0) & (g != 0)
    lo[solid] = base[solid]
    hi[solid] = base[solid] + 7
    isb = (g & 1) == 1
    box = bb[g[isb] >> 1]
    ok = box != 0xFFFFFFFF
    sel = tuple(a[ok] for a in np.nonzero(isb))
    box = box[ok]
    lo[sel] = base[sel] + np.stack([box & 7, (box >> 3) & 7, (box >> 6) & 7], -1)
    hi[sel] = base[sel] + np.stack([(box >> 9) & 7, (box >> 12) & 7, (box >> 15) & 7], -1)
    lo = lo.reshape(32, 4, 32, 4, 32, 4, 3).min(axis=(1, 3, 5))       # [uy, uz, ux, 3]
    hi = hi.reshape(32, 4, 32, 4, 32, 4, 3).max(axis=(1, 3, 5))
    packed = sum(lo[..., a] << (5 * a) for a in range(3)) + sum(hi[..., a] << (15 + 5 * a) for a in range(3))
    return np.ascontiguousarray(np.where(hi[..., 0] >= 0, packed, 0xFFFFFFFF).astype(np.uint32).reshape(-1))


def _surface_rays(wa, n, seed):
    """Rays from just above the terrain of world0 towards random points: the shape of
    shadow rays (they leave a surface and cross bricks near it)."""
    rng = np.random.default_rng(seed)
    g = wa.grid.reshape(128, 128, 128)                                   # [y, z, x]
    occ = g != 0
    o = np.zeros((n, 3), np.float32)
    for i in range(n):
        x, z = int(rng.integers(0, 256)), int(rng.integers(0, 256))
        col = np.nonzero(occ[:, z // 8, x // 8])[0]
        top = (int(col.max()) * 8 + 8) if len(col) else 0
        o[i] = (x + rng.random(), top + rng.uniform(-6.0, 3.0), z + rng.random())
    tgt = rng.uniform([0, 0, 0], [256, 160, 256], (n, 3)).astype(np.float32)
    d = tgt - o
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return o, d.astype(np.float32), rng


def test_walker_brick_skipping_is_exact(dh, world0_arrays):
    """Skipping bricks whose opaque-voxel box the ray's line misses (by more than the
    slack) changes no walk result (status, distance bits, side), and skips bricks on
    surface-leaving rays."""
    wa = world0_arrays
    boxes = brick_boxes(wa.bricks)
    assert (boxes != 0xFFFFFFFF).any()
    o1, d1, rng = _rays(3000, 41)
    o2, d2, _ = _surface_rays(wa, 3000, 43)
    o, d = np.concatenate([o1, o2]), np.concatenate([d1, d2])
    saved = hits = 0
    for i in range(len(o)):
        steps = int(rng.choice([128, 128, 999999, 5, 1]))
        da, sa, sta, nva = C.c_float(0), C.c_uint32(0), C.c_int(0), C.c_int(0)
        dh.dh_walk(wa.grid.ctypes.data, wa.uber.ctypes.data, wa.bricks.ctypes.data, _f3(o[i]), _f3(d[i]), steps,
                   C.byref(da), C.byref(sa), C.byref(sta), C.byref(nva))
        db, sb, nvb = C.c_float(0), C.c_uint32(0), C.c_int(0)
        stb = dh.dh_walk_skip(wa.grid.ctypes.data, wa.uber.ctypes.data, wa.bricks.ctypes.data, boxes.ctypes.data,
                              _f3(o[i]), _f3(d[i]), steps, C.byref(db), C.byref(sb), C.byref(nvb))
        assert sta.value == stb and sa.value == sb.value and \
            np.float32(da.value).view(np.uint32) == np.float32(db.value).view(np.uint32), (i, o[i], d[i], steps)
        saved += nva.value - nvb.value
        hits += stb == 1
    assert hits > 500 and saved > 10000


@pytest.mark.parametrize("mode", [0, 1, 2])
def test_trace_brick_skipping_matches_oracle(dh, world0_arrays, mode):
    """trace<0> skipping bricks whose non-zero-voxel box the ray misses, and with a budget
    that cannot run out whole uber cells likewise (primary rays), with every box table
    given to every mode, still matches the oracle's DDA bit for bit."""
    wa = world0_arrays
    box, box0 = brick_boxes(wa.bricks), brick_boxes(wa.bricks, nonzero=True)
    ub0 = uber_boxes0(wa.grid, wa.bricks)
    assert (box0 != 0xFFFFFFFF).any() and (ub0 != 0xFFFFFFFF).any()
    port = ob.Renderer("port", wa, 4, 4, False)
    o1, d1, rng = _rays(2000, 200 + mode)
    o2, d2, _ = _surface_rays(wa, 2000, 300 + mode)
    o, d = np.concatenate([o1, o2]), np.concatenate([d1, d2])
    for i in range(len(o)):
        steps = int(rng.choice([128, 999999, 9]))
        through = int(rng.choice([0, 0x7F44, 0xF888]))
        dist, side = C.c_float(0), C.c_uint32(0)
        v = dh.dh_trace_skip(mode, wa.grid.ctypes.data, wa.uber.ctypes.data, wa.bricks.ctypes.data, box.ctypes.data,
                             box0.ctypes.data, ub0.ctypes.data, _f3(o[i]), _f3(d[i]), steps, through, 0xFFFF,
                             C.byref(dist), C.byref(side))
        want = port.trace(mode, o[i], d[i], steps, through, 0xFFFF)
        assert (v, side.value) == (want[0], want[2]) and \
            np.float32(dist.value).view(np.uint32) == np.float32(want[1]).view(np.uint32), (i, o[i], d[i])


def test_device_sincos_matches_oracle(dh):
    rng = np.random.default_rng(5)
    s = rng.integers(0, 2 ** 32, 50000, dtype=np.uint64).astype(np.uint32)
    a = (s.astype(np.float32) * np.float32(2.3283064365387e-10)).astype(np.float32) * np.float32(6.28318530717958647692528)
    for x in a.astype(np.float32):
        sn, cs = C.c_float(), C.c_float()
        dh.dh_sincos(float(x), C.byref(sn), C.byref(cs))
        osn, ocs = ob.sincos(float(x))
        assert np.float32(sn.value) == np.float32(osn) and np.float32(cs.value) == np.float32(ocs), x


def test_area_sample_per_axis_matches_per_face(dh):
    """The per-axis area-light sample (one facing face per axis) against the per-face
    form, bit for bit: point, weight, face and the advanced RNG state. Shading points
    far away, near the cube, inside its slabs, on its face planes, and inside it."""
    rng = np.random.default_rng(11)
    n = 60000
    out_a = np.zeros(6, np.float32)
    out_b = np.zeros(6, np.float32)
    pa = out_a.ctypes.data_as(C.POINTER(C.c_float))
    pb = out_b.ctypes.data_as(C.POINTER(C.c_float))
    for i in range(n):
        size = float(rng.choice([1.0, 8.0]))
        c = np.floor(rng.uniform(0, 1000, 3)).astype(np.float32) + np.float32(0.5 * size)
        mode = i % 5
        if mode == 0:
            sp = rng.uniform(0, 1024, 3)
        elif mode == 1:
            sp = c + rng.normal(0, 3 * size, 3)
        elif mode == 2:      # inside one or two slabs
            sp = c + rng.uniform(-0.5 * size, 0.5 * size, 3) * (rng.random(3) < 0.5) + rng.normal(0, 5, 3) * (rng.random(3) < 0.5)
        elif mode == 3:      # exactly on a face plane
            sp = c + rng.normal(0, 4, 3)
            ax = rng.integers(3)
            sp[ax] = c[ax] + rng.choice([-0.5, 0.5]) * size
        else:                # inside the cube
            sp = c + rng.uniform(-0.5 * size, 0.5 * size, 3)
        sp = sp.astype(np.float32)
        lg = (C.c_float * 4)(float(c[0]), float(c[1]), float(c[2]), size)
        spo = _f3(sp)
        seed = int(rng.integers(1, 2 ** 32))
        dh.dh_area_sample(0, lg, spo, seed, pa)
        dh.dh_area_sample(1, lg, spo, seed, pb)
        assert out_a.view(np.uint32).tolist() == out_b.view(np.uint32).tolist(), (i, c, size, sp, seed, out_a, out_b)


def _candidate_shadow_rays(wa, lights, W, H, cam_path, point):
    """The candidate stage's shadow rays of two oracle frames: origin = shading point +
    0.1 N, direction towards the selected sample on the emitter, and the emitter."""
    r = ob.Renderer("port", wa, W, H, point)
    cam = ob.CameraPath(W, H)
    out = []
    for f in range(2):
        cam.lookat(*cam_path(f))
        k = cam.begin(numberOfLights=len(lights), numberOfCandidates=32, numberOfMaxTemporalImportance=20,
                      spatialRadius=30, spatialTaps=5, spatial=1, temporal=1, accumulate=0)
        r.frame_start()
        r.stage(k, 1)
        r.stage(k, 2)
        g, res = r.gbuffer(0), r.reservoirs(0)
        cam.end()
        E, p0, p1, p2 = (np.array(v, np.float32) for v in (k.E, k.p0, k.p1, k.p2))
        idx = np.nonzero((g["voxel"] != 0) & (res["streamLength"] > 0) & (res["pHat"] > 0))[0]
        u = (idx % W).astype(np.float32) * np.float32(k.oneOverRes[0])
        v = (idx // W).astype(np.float32) * np.float32(k.oneOverRes[1])
        D = p0 + (p1 - p0) * u[:, None] + (p2 - p0) * v[:, None] - E
        D /= np.linalg.norm(D, axis=1, keepdims=True)
        sp = E + D * g["dist"][idx][:, None]
        side = g["side"][idx]
        n = np.arange(len(idx))
        sp[n, side] += np.where(D[n, side] > 0, np.float32(-0.1), np.float32(0.1))
        L = res["positionOnVoxel"][idx] - sp
        L /= np.linalg.norm(L, axis=1, keepdims=True)
        out.append((sp.astype(np.float32), L.astype(np.float32), res["lightIndex"][idx]))
    r.close()
    return [np.concatenate(x) for x in zip(*out)]


def _early_out_case(dh, wa, lights, O, D, LI):
    box = brick_boxes(wa.bricks)
    n = C.c_int()
    diff = visits = visits_early = visible = 0
    for i in range(len(O)):
        lt = lights[LI[i]]
        o, d = _f3(O[i]), _f3(D[i])
        a = dh.dh_shadow(wa.grid.ctypes.data, wa.uber.ctypes.data, wa.bricks.ctypes.data, box.ctypes.data, o, d,
                         int(lt["position"]), int(lt["size"]), 0, C.byref(n))
        visits += n.value
        b = dh.dh_shadow(wa.grid.ctypes.data, wa.uber.ctypes.data, wa.bricks.ctypes.data, box.ctypes.data, o, d,
                         int(lt["position"]), int(lt["size"]), 1, C.byref(n))
        visits_early += n.value
        diff += a != b
        visible += a
    return diff, visits, visits_early, visible


def test_shadow_early_out_is_exact(dh, world0_arrays):
    """The visibility early-out (walk_target: stop as occluded once the step budget left is
    below the grid-cell distance to the emitter) never changes a visibility result: the
    candidate shadow rays of oracle frames (point and area lights) and surface-leaving
    rays towards random emitters of world0."""
    wa = world0_arrays
    lights = wa.lights

    def orbit(f):
        return (128.0 + 40.0 * f, 170.0, -60.0 + 30.0 * f), (128.0, 100.0, 128.0)

    total = [0, 0, 0]
    for point in (True, False):
        O, D, LI = _candidate_shadow_rays(wa, lights, 160, 96, orbit, point)
        diff, v0, v1, _ = _early_out_case(dh, wa, lights, O, D, LI)
        assert diff == 0
        total = [total[0] + len(O), total[1] + v0, total[2] + v1]
    rng = np.random.default_rng(3)
    o, _, _ = _surface_rays(wa, 3000, 9)
    LI = rng.integers(0, len(lights), len(o))
    ex = lights["position"][LI] % 1024
    ez = (lights["position"][LI] // 1024) % 1024
    ey = lights["position"][LI] // (1024 * 1024)
    tgt = np.stack([ex, ey, ez], 1).astype(np.float32) + np.float32(0.5)
    d = tgt - o
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    diff, v0, v1, vis = _early_out_case(dh, wa, lights, o, d, LI)
    assert diff == 0 and vis > 0
    assert total[2] <= total[1] and v1 <= v0


@pytest.mark.slow
def test_shadow_early_out_is_exact_config3(dh):
    """The same on the benchmark scene (config 3: 1024^3 terrain, 65,536 emitters in
    blobs): every candidate shadow ray of two 240 x 135 frames along the camera path."""
    hs = ob.HostScene(3)
    wa = ob.WorldArrays(hs.grid, hs.bricks, hs.lights)
    O, D, LI = _candidate_shadow_rays(wa, hs.lights, 240, 135, lambda f: hs.camera_path(1, 150 + f, 300), False)
    assert len(O) > 20000
    diff, v0, v1, _ = _early_out_case(dh, wa, hs.lights, O, D, LI)
    assert diff == 0 and v1 < v0
