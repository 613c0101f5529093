"""Scene and frame files (smallproject_gb300/scene_io.py): .vx worlds as the reference's
MyGameScene::SaveWorld / LoadWorld write and read them (sprite format, one frame,
stamped with | 0xF000), .dat frames as saveScreenBuffer writes them."""
import os

import numpy as np
import pytest

from smallproject_gb300 import scene_io as io

REF_SCENES = "/root/reference/scene_export"


def _lightset(lights):
    return sorted(zip(lights["position"].tolist(), lights["voxel"].tolist(), lights["size"].tolist()))


def test_vx_world_round_trip(lib, tmp_path):
    a = lib.World()
    a.generate(lib.scene_preset(0, seed=3, emitters=40))
    a.set(0, 0, 0, 0xF123)
    path = str(tmp_path / "world.vx")
    io.save_world_vx(a, path, (256, 160, 256))
    b = lib.World()
    b.set(500, 500, 500, 0xF777)                   # cleared by the load
    assert io.load_world_vx(b, path) == (256, 160, 256)
    va, vb = io.region(a, (0, 0, 0), (256, 160, 256)), io.region(b, (0, 0, 0), (256, 160, 256))
    assert np.array_equal(vb, np.where(va != 0, va | 0xF000, 0))
    assert b.get(500, 500, 500) == 0
    # emitters stamped in draw-list order become the same set of lights
    assert _lightset(b.arrays()[2]) == _lightset(a.arrays()[2])
    a.close()
    b.close()


def test_vx_payload2_and_stamp_order(lib, tmp_path):
    """2-byte payloads keep the low 16 bits; entries are stamped in file order, the last
    one at a position wins; the draw list's position packing is x | y << 10 | z << 20."""
    pos = np.array([0, 0, 5 | 6 << 10 | 7 << 20, 5 | 6 << 10 | 7 << 20, 1023 | 1023 << 10 | 1023 << 20], np.uint32)
    vox = np.array([0, 0, 0x0ABC, 0x1234, 0x0F00], np.uint32)
    path = str(tmp_path / "s.vx")
    io.write_vx(path, [((1024, 1024, 1024), pos, vox | 0xFF0000)], payload=2)
    pls, frames = io.read_vx(path)
    assert pls == 2 and np.array_equal(frames[0][2], vox)
    w = lib.World()
    io.load_world_vx(w, path)
    assert w.get(0, 0, 0) == 0xF000
    assert w.get(5, 6, 7) == 0xF234
    assert w.get(1023, 1023, 1023) == 0xFF00
    w.close()


@pytest.mark.skipif(not os.path.isdir(REF_SCENES), reason="the reference's scene files are not present")
@pytest.mark.parametrize("scene", ["nolights", "randomscatteroffset10"])
def test_reference_world_files_load(lib, scene):
    """The reference's own exported worlds (2-byte payload) load with LoadWorld's
    semantics: every draw-list entry stamped in order with | 0xF000, including the
    size / 4 zero entries its CreateSprite writes first (so the origin becomes 0xF000)."""
    path = os.path.join(REF_SCENES, scene, "grid.vx")
    pls, frames = io.read_vx(path)
    assert pls == 2 and len(frames) == 1
    size, pos, vox = frames[0]
    lead = size[0] * size[1] * size[2] // 4
    assert not pos[:lead].any() and not vox[:lead].any() and (pos[lead:] != 0).any()
    w = lib.World()
    io.load_world_vx(w, path)
    vol = io.region(w, (0, 0, 0), tuple(min(s, 1024) for s in size))
    x, y, z = pos[lead:] & 1023, (pos[lead:] >> 10) & 1023, pos[lead:] >> 20
    last = {}
    for px, py, pz, v in zip(x.tolist(), y.tolist(), z.tolist(), vox[lead:].tolist()):
        last[(px, py, pz)] = v | 0xF000
    keys = np.array(list(last.keys()))
    assert np.array_equal(vol[keys[:, 0], keys[:, 1], keys[:, 2]], np.array(list(last.values()), np.uint32))
    expect = len(last) + (0 if (0, 0, 0) in last else 1)
    assert int((vol != 0).sum()) == expect
    w.close()


def test_dat_frame_round_trip(tmp_path):
    rng = np.random.default_rng(2)
    img = rng.random((12 * 7, 4), dtype=np.float32)
    path = str(tmp_path / "f.dat")
    io.write_frame_dat(path, img, 12, 7)
    assert os.path.getsize(path) == 8 + 16 * 12 * 7
    w, h, back = io.read_frame_dat(path)
    assert (w, h) == (12, 7) and np.array_equal(back, img)
    with open(path, "r+b") as f:
        f.truncate(100)
    with pytest.raises(ValueError):
        io.read_frame_dat(path)
