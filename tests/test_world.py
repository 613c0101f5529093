"""Host voxel store (World::Set/Get/OptimizeBricks/FindLightsInWord semantics) and the
procedural scenes, against the oracle's restatement of the same functions."""
import numpy as np
import pytest

from oracle import binding as ob


def _store():
    lib = ob.load_port()
    return lib, lib.orc_store_create()


def test_set_get_matches_restated_world(lib):
    olib, st = _store()
    w = lib.World()
    rng = np.random.default_rng(3)
    ops = []
    for _ in range(6000):
        x, y, z = (int(v) for v in rng.integers(0, 40, 3))
        r = rng.random()
        v = 0 if r < 0.3 else (int(rng.integers(1, 255)) << 16 | 0xF123 if r < 0.35 else int(rng.integers(1, 0xFFFF)))
        ops.append((x, y, z, v))
    ops += [(x, 3, z, 0xF00F) for x in range(8, 16) for z in range(8, 16)]           # fills a whole brick layer
    ops += [(1100, 3, 4, 5), (3, 2000, 4, 5)]                                          # outside the map: ignored
    for x, y, z, v in ops:
        w.set(x, y, z, v)
        olib.orc_store_set(st, x, y, z, v)
    for x in range(0, 41):
        for y in (0, 3, 7, 8, 21, 39):
            for z in range(0, 41, 3):
                assert w.get(x, y, z) == olib.orc_store_get(st, x, y, z), (x, y, z)
    # incremental light list (AddLight / RemoveLight order)
    _, _, lights = w.arrays()
    cap = 100000
    out = np.zeros(cap, ob.LIGHT_DTYPE)
    n = olib.orc_store_lights(st, out.ctypes.data, cap)
    assert n == len(lights)
    assert np.array_equal(out[:n], lights)
    olib.orc_store_destroy(st)


def test_optimize_and_scan_lights(lib):
    olib, st = _store()
    w = lib.World()
    w.box(0, 0, 0, 32, 8, 32, 0xF777)                     # 4x4 uniform bricks -> solid cells
    w.box(8, 8, 8, 16, 16, 16, (7 << 16) | 0xFFFF)        # one uniform emitter brick -> size-8 light
    w.set(3, 9, 3, (2 << 16) | 0xF00F)                    # single emitter voxel
    w.set(5, 2, 5, 0)                                     # hole keeps its brick
    for (x1, y1, z1, x2, y2, z2, v) in [(0, 0, 0, 32, 8, 32, 0xF777), (8, 8, 8, 16, 16, 16, (7 << 16) | 0xFFFF)]:
        for y in range(y1, y2):
            for z in range(z1, z2):
                for x in range(x1, x2):
                    olib.orc_store_set(st, x, y, z, v)
    olib.orc_store_set(st, 3, 9, 3, (2 << 16) | 0xF00F)
    olib.orc_store_set(st, 5, 2, 5, 0)
    r1 = w.optimize()
    r2 = olib.orc_store_optimize(st)
    assert r1 == r2 and r1 > 0
    n = w.scan_lights()
    g, b, l = w.arrays()
    cap = 10000
    out = np.zeros(cap, ob.LIGHT_DTYPE)
    m = olib.orc_scan_lights(g.ctypes.data, np.ascontiguousarray(b.reshape(-1)).ctypes.data, out.ctypes.data, cap)
    assert n == m == len(l)
    assert np.array_equal(out[:m], l)
    assert sorted(set(l["size"].tolist())) == [1, 8]
    for x, y, z in [(0, 0, 0), (5, 2, 5), (12, 12, 12), (3, 9, 3), (31, 7, 31), (40, 1, 1)]:
        assert w.get(x, y, z) == olib.orc_world_get(g.ctypes.data, np.ascontiguousarray(b.reshape(-1)).ctypes.data,
                                                    x, y, z)
    olib.orc_store_destroy(st)


def test_scene_is_deterministic_and_pinned(lib):
    """The config-0 scene regenerates to the same canonical content (checksums pinned)."""
    a, b = lib.World(), lib.World()
    a.generate(lib.scene_preset(0))
    b.generate(lib.scene_preset(0))
    assert a.checksum() == b.checksum()
    g, br, l = a.arrays()
    assert len(l) == 64 and set(l["size"].tolist()) == {1}
    # every emitter voxel sits 1..8 voxels above the terrain column
    d = lib.scene_preset(0)
    for li in l:
        p = int(li["position"])
        x, z, y = p % 1024, (p // 1024) % 1024, p // (1024 * 1024)
        h = lib.scene_height(d, x, z)
        assert h <= y <= h + 7 and a.get(x, y, z) == int(li["voxel"])
        assert (int(li["voxel"]) >> 16) & 255 >= 1 and (int(li["voxel"]) >> 12) & 15 == 15


def test_scene_presets(lib):
    for cfg, n, mode in [(1, 4096, 1), (3, 65536, 2)]:
        d = lib.scene_preset(cfg)
        assert d.emitters == n and d.emitter_mode == mode and d.extent == 1024
    d = lib.scene_preset(4)
    assert d.octaves == 6 and abs(d.cave_threshold - 0.6) < 1e-6 and d.emitters == 1048576


def test_world_checksum_ignores_brick_numbering(lib):
    a, b = lib.World(), lib.World()
    a.box(0, 0, 0, 20, 5, 20, 0xF321)
    for y in reversed(range(5)):
        for z in reversed(range(20)):
            for x in reversed(range(20)):
                b.set(x, y, z, 0xF321)
    assert a.checksum() == b.checksum()


def test_camera_constants_match_oracle(lib):
    """Per-frame constants (LookAt, corners, frustum planes, R0, counters) bit-exact."""
    W, H = 1280, 720
    cam = lib.Camera(0x12345678)
    ocam = ob.CameraPath(W, H, 0x12345678)
    d = lib.scene_preset(1)
    for f in range(12):
        pos, tgt = lib.camera_path(d, 5, f, 120)
        cam.lookat(pos, tgt)
        ocam.lookat(pos, tgt)
        k = cam.begin_frame(W, H)
        ko = ocam.begin()
        a = bytes(k)
        b = bytes(ob.copy_consts(ko, type(k)))
        assert a == b, f"frame {f}"
        cam.end_frame()
        ocam.end()


def test_pending_commit_before_any_device_copy(lib):
    """Without a device copy the next commit is a full one: every brick and the grid."""
    w = lib.World()
    w.generate(lib.scene_preset(0))
    n, grid, full = w.pending()
    assert full and grid and n == len(w.arrays()[1])
    w.set(5, 5, 5, 0xF123)
    assert w.pending()[2]
    w.close()


def test_move_light_restores_and_remembers_voxels(lib):
    """vxr_world_move_light (World::MoveLights for one light): the emitter voxel moves,
    the voxel it covered comes back, the list keeps its order, brick lights stay put."""
    w = lib.World()
    w.generate(lib.scene_preset(0, seed=5, emitters=12))
    _, _, lights = w.arrays()
    i = next(k for k in range(len(lights)) if lights["size"][k] == 1)
    p0 = int(lights["position"][i])
    v = int(lights["voxel"][i])
    x0, z0, y0 = p0 % 1024, (p0 // 1024) % 1024, p0 // (1024 * 1024)
    assert w.get(x0, y0, z0) == v
    # onto a solid voxel: the solid voxel is remembered and restored later
    w.set(30, 200, 30, 0xF321)
    w.move_light(i, 30, 200, 30)
    assert w.get(30, 200, 30) == v and w.get(x0, y0, z0) == 0
    _, _, after = w.arrays()
    assert len(after) == len(lights) and int(after["position"][i]) == 30 + 30 * 1024 + 200 * 1024 * 1024
    assert np.array_equal(np.delete(after, i), np.delete(lights, i))
    w.move_light(i, x0, y0, z0)
    assert w.get(x0, y0, z0) == v and w.get(30, 200, 30) == 0xF321
    with pytest.raises(lib.VxrError):
        w.move_light(len(lights), 1, 1, 1)
    w.close()


def test_add_brick_solid_cell_and_brick_lights(lib):
    """vxr_world_add_brick (World::AddBrick, world.h:308-352): the cell turns solid and its
    brick is recycled; emitter voxels that were in it leave the light list, an emitter
    value joins it as one size-8 light at the cell's corner, replacing that cell's old
    brick light; a non-emitter leaves none; out-of-grid cells are ignored."""
    w = lib.World()
    em = 3 << 16 | 0xF0F0
    w.set(17, 9, 25, em)
    w.set(18, 9, 25, 0x0123)
    w.set(3, 3, 3, em)
    before = w.brick_count()
    assert len(w.arrays()[2]) == 2
    w.add_brick(2, 1, 3, 5 << 16 | 0xFFFF)               # the cell of (17, 9, 25)
    assert w.brick_count() == before - 1
    assert all(w.get(16 + i, 8 + i, 24 + i) == 5 << 16 | 0xFFFF for i in range(8))
    pos = 2 * 8 + 3 * 8 * 1024 + 1 * 8 * 1024 * 1024
    lights = w.arrays()[2]
    assert sorted(zip(lights["position"].tolist(), lights["size"].tolist())) == [(3 + 3 * 1024 + 3 * 1024 * 1024, 1), (pos, 8)]
    w.add_brick(2, 1, 3, 0xF777)                          # a solid emitter cell replaced: its light goes
    assert w.arrays()[2]["position"].tolist() == [3 + 3 * 1024 + 3 * 1024 * 1024]
    assert w.get(20, 12, 30) == 0xF777
    w.add_brick(128, 0, 0, em)                            # outside the grid
    assert len(w.arrays()[2]) == 1
    w.close()
