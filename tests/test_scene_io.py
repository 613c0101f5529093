"""Scene and frame files (smallproject_gb300/scene_io.py): .vx worlds as the reference's
MyGameScene::SaveWorld / LoadWorld write and read them (sprite format, one frame,
stamped with | 0xF000), .dat frames as saveScreenBuffer writes them."""
import os
import re
import struct

import numpy as np
import pytest

from smallproject_gb300 import scene_io as io

from oracle.ref_build import DEFAULT_REF

REF_SCENES = os.path.join(DEFAULT_REF, "scene_export")


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


# --- MagicaVoxel .vox (SpriteManager::LoadSprite without the large-model flag) ---------

REF_TEMPLATE = os.path.join(DEFAULT_REF, "template", "world.cpp")
REF_CORNELL = os.path.join(REF_SCENES, "cornellbox")


def _chunk(name, content=b"", children=b""):
    return name + struct.pack("<ii", len(content), len(children)) + content + children


def _vox_file(path, chunks, version=150):
    body = b"".join(chunks)
    with open(path, "wb") as f:
        f.write(b"VOX " + struct.pack("<i", version) + _chunk(b"MAIN", b"", body))
    return str(path)


def _size(x, y, z):
    return _chunk(b"SIZE", struct.pack("<iii", x, y, z))


def _xyzi(vox):
    return _chunk(b"XYZI", struct.pack("<I", len(vox)) + bytes(np.array(vox, np.uint8).ravel()))


def test_vox_default_palette_structure():
    pal = io.vox_default_palette()
    assert pal[0] == 0 and (pal[1:] >> 24 == 0xFF).all()
    assert pal[1] == 0xFFFFFFFF and pal[2] == 0xFFCCFFFF          # blue steps first
    assert pal[7] == 0xFFFFCCFF and pal[37] == 0xFFFFFFCC          # then green, then red
    assert len(np.unique(pal[1:])) == 255 and 0xFF000000 not in pal  # black left out


@pytest.mark.skipif(not os.path.isfile(REF_TEMPLATE), reason="the reference's sources are not present")
def test_vox_default_palette_matches_reference():
    """The generated palette equals the reference's default_palette table, read as text
    from template/world.cpp."""
    src = open(REF_TEMPLATE).read()
    m = re.search(r"default_palette\[256\]\s*=\s*\{(.*?)\};", src, re.S)
    table = np.array([int(v, 16) for v in re.findall(r"0x[0-9a-fA-F]+", m.group(1))], np.uint32)
    assert np.array_equal(table, io.vox_default_palette())


def test_vox_colour_rounding():
    c = np.array([0x000000, 0x000008, 0x000009, 0x0000F8, 0x0000FF, 0x00FF00, 0xFF0000, 0x778899], np.uint32)
    assert io.vox_colour(c).tolist() == [1, 1, 0x100, 0xF00, 0xF00, 0x0F0, 0x00F, 0xA87]


def test_vox_frames_axes_palette_and_order(tmp_path):
    """PACK frame count, one frame per SIZE + XYZI, MagicaVoxel's y and z swapped, colour
    index i coloured by palette entry i - 1 of the RGBA chunk, last write to a cell wins,
    draw list z outer then y then x, skipped chunks stepped over by their content size."""
    rng = np.random.default_rng(5)
    pal = rng.integers(0, 2**32, 256, dtype=np.uint64).astype(np.uint32)
    path = _vox_file(tmp_path / "m.vox", [
        _chunk(b"PACK", struct.pack("<i", 2)),
        _size(3, 4, 2), _xyzi([(1, 3, 1, 5), (0, 0, 0, 2), (2, 0, 1, 9), (2, 0, 1, 7)]),
        _chunk(b"MATL", bytes(range(20))), _chunk(b"nTRN", bytes(28)),
        _size(1, 1, 1), _xyzi([(0, 0, 0, 1)]),
        _chunk(b"RGBA", pal.tobytes()),
    ])
    f0, f1 = io.read_vox(path)
    assert f0[0] == (3, 2, 4) and f1[0] == (1, 1, 1)
    # engine (x, y, z) = MagicaVoxel (x, z, y)
    assert f0[1].tolist() == [0, 2 | 1 << 10, 1 | 1 << 10 | 3 << 20]
    assert f0[2].tolist() == io.vox_colour(pal[[1, 6, 4]]).tolist()
    assert f1[1].tolist() == [0] and f1[2].tolist() == io.vox_colour(pal[[0]]).tolist()


def test_vox_default_palette_and_unknown_chunk(tmp_path):
    """Without an RGBA chunk the default palette colours the voxels, indexed by i - 1 as
    well. A chunk the reader does not know moves it past the 12-byte header only: here its
    zero content then reads as the end marker, so the RGBA chunk after it is never seen."""
    path = _vox_file(tmp_path / "d.vox", [
        _size(2, 2, 2), _xyzi([(0, 0, 0, 3), (1, 1, 1, 216)]),
        _chunk(b"NOTE", bytes(16)), _chunk(b"RGBA", bytes(1024)),
    ])
    (size, pos, vox), = io.read_vox(path)
    assert size == (2, 2, 2) and pos.tolist() == [0, 1 | 1 << 10 | 1 << 20]
    assert vox.tolist() == io.vox_colour(io.vox_default_palette()[[2, 215]]).tolist()


@pytest.mark.parametrize("case", ["magic", "version", "main", "no_size", "pack_more", "pack_less", "outside", "truncated"])
def test_vox_errors(tmp_path, case):
    one = [_size(2, 2, 2), _xyzi([(0, 0, 0, 1)])]
    files = {
        "magic": lambda p: open(p, "wb").write(b"VOXX" + bytes(30)) and str(p),
        "version": lambda p: _vox_file(p, one, version=200),
        "main": lambda p: open(p, "wb").write(b"VOX " + struct.pack("<i", 150) + b"MAIX" + bytes(20)) and str(p),
        "no_size": lambda p: _vox_file(p, [_xyzi([(0, 0, 0, 1)])]),
        "pack_more": lambda p: _vox_file(p, one + one),
        "pack_less": lambda p: _vox_file(p, [_chunk(b"PACK", struct.pack("<i", 2))] + one),
        "outside": lambda p: _vox_file(p, [_size(2, 2, 2), _xyzi([(0, 2, 0, 1)])]),
        "truncated": lambda p: _vox_file(p, [_size(2, 2, 2), _chunk(b"XYZI", struct.pack("<I", 5) + bytes(8))]),
    }
    path = files[case](tmp_path / "bad.vox")
    with pytest.raises(ValueError):
        io.read_vox(str(path))


def test_stamp_sprite_dispatch(lib, tmp_path):
    """LoadSprite picks the .vx reader when the path contains ".vx", else .vox; the frame
    is stamped at the origin given with | 0xF000."""
    vox = _vox_file(tmp_path / "s.vox", [_size(2, 3, 4), _xyzi([(1, 2, 3, 1)])])
    vx = str(tmp_path / "s.vx")
    io.write_vx(vx, [((2, 4, 3), np.array([1 | 3 << 10 | 2 << 20], np.uint32), np.array([0x123], np.uint32))])
    w = lib.World()
    assert io.stamp_sprite(w, vox, (10, 20, 30)) == (2, 4, 3)
    assert io.stamp_sprite(w, vx, (100, 0, 0)) == (2, 4, 3)
    assert w.get(11, 23, 32) == 0xF001                      # index 1 reads entry 0 (empty): black -> 1
    assert w.get(101, 3, 2) == 0xF123
    w.close()


def test_world_frame_wraps_like_get(lib):
    """World::CreateSprite over a box that crosses the map edge and one wider than the
    map: coordinates wrap modulo 1024 and positions pack with wrap-around, checked
    against a dense listing of the same box."""
    w = lib.World()
    for p, v in [((1021, 2, 3), 0x111), ((2, 0, 1), 0x222), ((1023, 3, 0), 0x333), ((5, 1, 2), 0x444)]:
        w.set(*p, v)
    w.add_brick(0, 0, 1, 0x555)                             # a solid cell: 512 voxels
    for origin, size in [((1020, 0, 0), (8, 4, 4)), ((0, 0, 0), (1030, 4, 4)), ((1016, 0, 8), (1040, 8, 9))]:
        _, pos, val = io.world_frame(w, origin, size)
        vol = io.region(w, origin, size)
        x, y, z = (a.astype(np.uint64) for a in np.nonzero(vol))
        assert np.array_equal(pos, ((x + (y << 10) + (z << 20)) & 0xFFFFFFFF).astype(np.uint32))
        assert np.array_equal(val, vol[np.nonzero(vol)])
    w.close()


@pytest.mark.skipif(not os.path.isdir(REF_CORNELL), reason="the reference's scene files are not present")
def test_reference_cornell_box_export(lib):
    """The reference's Cornell box world rebuilt from its own cornell-box.vox (read_vox,
    stamped at the origin), with CreateCornellBoxWorld's colour replacement (12-bit
    colours 0x050, 0xDA7, 0x700 -> 0x0F0, 0xFFF, 0xF00, set without the 0xF000 bits) and
    its 16 x 16 ceiling bricks (AddBrick at by = 31, value 0xFFFF)
    (cornellboxscene.cpp:12-107), exported as MyGameScene::SaveWorld did for the file in
    the same folder (box 1027 x 260 x 1027, wider than the map): the draw list equals
    grid.vx's after its leading zero entries, entry for entry."""
    w = lib.World()
    assert io.stamp_sprite(w, os.path.join(REF_CORNELL, "cornell-box.vox")) == (255, 255, 255)
    x, y, z, v = io.world_voxels(w)
    colour = v & 0xFFF
    repl = {0x050: 0x0F0, 0xDA7: 0xFFF, 0x700: 0xF00}
    hit = np.isin(colour, list(repl))
    new = np.zeros(len(colour), np.uint32)
    for k, c in repl.items():
        new[colour == k] = c
    w.stamp((x[hit] | y[hit] << 10 | z[hit] << 20).astype(np.uint32), new[hit])
    for bx in range(64 // 8, 192 // 8):
        for bz in range(64 // 8, 192 // 8):
            w.add_brick(bx, 248 // 8, bz, 0xFFFF)
    size, pos, val = io.world_frame(w, (0, 0, 0), (1027, 260, 1027))
    pls, frames = io.read_vx(os.path.join(REF_CORNELL, "grid.vx"))
    fsize, fpos, fvox = frames[0]
    lead = fsize[0] * fsize[1] * fsize[2] // 4
    assert pls == 2 and fsize == size
    assert np.array_equal(fpos[lead:], pos) and np.array_equal(fvox[lead:], val & 0xFFFF)
    w.close()


def _tool_metrics(gt, img, w, h):
    """The comparison tool's loops (mse.cpp:19-63), one pixel at a time, float32 terms
    and a Python float (double) accumulator."""
    f = np.float32
    mse = mae = en = 0.0
    for i in range(len(gt)):
        dg = [f(gt[i, c]) - f(img[i, c]) for c in range(3)]
        sq = [f(v * v) for v in dg]
        mse += float(f(f(sq[0] + sq[1]) + sq[2]))
        ab = [f(abs(v)) for v in dg]
        mae += float(f(f(ab[0] + ab[1]) + ab[2]))
        en += float(f(f(f(img[i, 0]) + f(img[i, 1])) + f(img[i, 2])) / f(3.0))
    n = len(gt)
    return f(mse / (n * 3)), f(mae / (n * 3)), f(en / w / h)


def test_frame_metrics_match_the_comparison_tool(tmp_path):
    rng = np.random.default_rng(4)
    w, h = 23, 17
    gt = (rng.random((w * h, 4)) * 3).astype(np.float32)
    img = (gt + rng.normal(0, 0.2, gt.shape)).astype(np.float32)
    io.write_frame_dat(str(tmp_path / "gt.dat"), gt, w, h)
    io.write_frame_dat(str(tmp_path / "img.dat"), img, w, h)
    _, _, g = io.read_frame_dat(str(tmp_path / "gt.dat"))
    _, _, d = io.read_frame_dat(str(tmp_path / "img.dat"))
    mse, mae, en = _tool_metrics(g, d, w, h)
    assert io.frame_mse(g, d) == mse and io.frame_mae(g, d) == mae and io.frame_energy(d, w, h) == en
    assert io.frame_mse(g, g) == 0.0 and io.frame_mae(g, g) == 0.0
