"""MagicaVoxel scenes through the reference's large-model path (LoadSprite(path, true),
template/world.cpp:1039-1137): smallproject_gb300/vox_scene.py against the reference's
own vendored opengametools reader (lib/ogt_vox.h, compiled by oracle/ref_build.py when
the reference checkout is present) on seeded scene graphs, and its sprite frame against
a loop-by-loop restatement of the reference's placement over ogt's own scene."""
import os
import struct

import numpy as np
import pytest

from oracle import binding as ob
from oracle.ref_build import DEFAULT_REF
from smallproject_gb300 import scene_io as io
from smallproject_gb300 import vox_scene as vs

needs_ogt = pytest.mark.skipif(ob.load_ogt() is None, reason="the reference's ogt_vox is not present")
CORNELL = os.path.join(DEFAULT_REF, "scene_export", "cornellbox", "cornell-box.vox")


# ---- a .vox writer (chunk layout of the MagicaVoxel format) --------------------------

def _dict(d):
    out = struct.pack("<I", len(d))
    for k, v in d.items():
        k, v = k.encode(), str(v).encode()
        out += struct.pack("<I", len(k)) + k + struct.pack("<I", len(v)) + v
    return out


def _chunk(name, content):
    return name + struct.pack("<ii", len(content), 0) + content


def _model(grid):
    """SIZE + XYZI of a uint8[sz, sy, sx] index grid."""
    sz, sy, sx = grid.shape
    z, y, x = np.nonzero(grid)
    xyzi = np.stack([x, y, z, grid[z, y, x]], axis=1).astype(np.uint8)
    return _chunk(b"SIZE", struct.pack("<III", sx, sy, sz)) + \
        _chunk(b"XYZI", struct.pack("<I", len(xyzi)) + xyzi.tobytes())


def _trn(nid, child, layer=0, frame=None, attrs=None):
    return _chunk(b"nTRN", struct.pack("<I", nid) + _dict(attrs or {}) +
                  struct.pack("<IIII", child, 0xFFFFFFFF, layer, 1) + _dict(frame or {}))


def _grp(nid, children):
    return _chunk(b"nGRP", struct.pack("<I", nid) + _dict({}) + struct.pack("<I", len(children)) +
                  struct.pack(f"<{len(children)}I", *children))


def _shp(nid, model):
    return _chunk(b"nSHP", struct.pack("<I", nid) + _dict({}) + struct.pack("<II", 1, model) + _dict({}))


def _write(path, chunks):
    body = b"".join(chunks)
    with open(path, "wb") as f:
        f.write(b"VOX " + struct.pack("<i", 150) + b"MAIN" + struct.pack("<ii", 0, len(body)) + body)
    return str(path)


VALID_R = [r0 | (r1 << 2) for r0 in range(3) for r1 in range(3) if r0 != r1]


def _random_scene(path, seed, imap=None, palette=True):
    """Models (one duplicate, one empty), a root transform, a group of transforms with
    rotations and translations, a nested group, a hidden node, layers, materials and an
    unknown chunk."""
    rng = np.random.default_rng(seed)
    grids = []
    for _ in range(3):
        s = rng.integers(1, 7, 3)
        g = np.where(rng.random((s[2], s[1], s[0])) < 0.4, rng.integers(1, 256, (s[2], s[1], s[0])), 0).astype(np.uint8)
        g.flat[0] = rng.integers(1, 256)
        grids.append(g)
    grids.append(grids[0].copy())                        # duplicate of model 0
    chunks = [_model(g) for g in grids]
    chunks.append(_chunk(b"SIZE", struct.pack("<III", 2, 2, 2)) + _chunk(b"XYZI", struct.pack("<I", 0)))  # empty
    if palette:
        chunks.append(_chunk(b"RGBA", rng.integers(0, 256, 1024, dtype=np.uint8).tobytes()))
    if imap is not None:
        chunks.append(_chunk(b"IMAP", imap.tobytes()))
    nodes, nid = [], 2
    kids = []
    for k in range(int(rng.integers(2, 6))):
        tid, sid = nid, nid + 1
        nid += 2
        frame = {"_t": " ".join(str(int(v)) for v in rng.integers(-40, 40, 3))}
        if rng.random() < 0.8:
            frame["_r"] = int(rng.choice(VALID_R)) | (int(rng.integers(0, 8)) << 4)
        attrs = {"_hidden": 1} if rng.random() < 0.2 else {}
        nodes.append(_trn(tid, sid, int(rng.integers(0, 2)), frame, attrs))
        nodes.append(_shp(sid, int(rng.integers(0, 5))))   # model 4 is the empty one
        kids.append(tid)
    # a nested group under a rotated transform
    gt, gg = nid, nid + 1
    nid += 2
    inner = []
    for k in range(2):
        tid, sid = nid, nid + 1
        nid += 2
        nodes.append(_trn(tid, sid, 0, {"_t": f"{k * 7} -3 {2 * k}", "_r": int(rng.choice(VALID_R))}))
        nodes.append(_shp(sid, k + 1))
        inner.append(tid)
    nodes.append(_trn(gt, gg, 0, {"_t": "5 6 -7", "_r": int(rng.choice(VALID_R)) | 0x30}))
    nodes.append(_grp(gg, inner))
    kids.append(gt)
    chunks += [_trn(0, 1, 0, {}), _grp(1, kids)] + nodes
    chunks.append(_chunk(b"LAYR", struct.pack("<i", 0) + _dict({"_name": "a"}) + struct.pack("<i", -1)))
    chunks.append(_chunk(b"LAYR", struct.pack("<i", 1) + _dict({"_hidden": 1}) + struct.pack("<i", -1)))
    chunks.append(_chunk(b"MATL", struct.pack("<i", 5) + _dict({"_type": "_metal", "_rough": "0.5"})))
    chunks.append(_chunk(b"rOBJ", bytes(range(40))))
    return _write(path, chunks)


def _same_scene(got, want):
    gm, gi, gp = got
    wm, wi, wp = want
    assert len(gm) == len(wm) and all(np.array_equal(a, b) for a, b in zip(gm, wm))
    assert [m for m, _ in gi] == [m for m, _ in wi]
    for (_, a), (_, b) in zip(gi, wi):
        assert np.array_equal(a.astype(np.float32), b)
    assert np.array_equal(gp, wp)


def _reference_frame(models, instances, pal):
    """World.cpp:1041-1129 loop by loop over ogt's scene (mat4::FromColumnMajor of the
    instance transform: M[r][c] = t[c][r]; translation M[r][3])."""
    lo, hi = [0xFFFFFF] * 3, [-0xFFFFFF] * 3
    for mid, t in instances:
        sz, sy, sx = models[mid].shape
        M = [[float(t[c][r]) for c in range(4)] for r in range(4)]
        pos = [int(M[r][3]) for r in range(3)]
        size = [int(M[r][0] * sx + M[r][1] * sy + M[r][2] * sz + M[r][3] * 0.0) for r in range(3)]
        lo = [min(lo[i], pos[i], pos[i] + size[i]) for i in range(3)]
        hi = [max(hi[i], pos[i], pos[i] + size[i]) for i in range(3)]
    S = [hi[i] + 1 - lo[i] for i in range(3)]
    S[1], S[2] = S[2], S[1]
    buf = {}
    for mid, t in instances:
        m = models[mid]
        sz, sy, sx = m.shape
        M = [[float(t[c][r]) for c in range(4)] for r in range(4)]
        pos = [int(M[r][3]) - lo[r] for r in range(3)]
        MX, MY, MZ = ([int(M[r][c]) for c in range(3)] for r in range(3))
        for z in range(sz):
            for y in range(sy):
                for x in range(sx):
                    v = int(m[z, y, x])
                    if not v:
                        continue
                    px = MX[0] * x + MX[1] * y + MX[2] * z + pos[0]
                    py = MY[0] * x + MY[1] * y + MY[2] * z + pos[1]
                    pz = MZ[0] * x + MZ[1] * y + MZ[2] * z + pos[2]
                    buf[px + pz * S[0] + py * S[0] * S[1]] = v
    pos_out, vox_out = [], []
    for i in sorted(buf):
        x, y, z = i % S[0], (i // S[0]) % S[1], i // (S[0] * S[1])
        r, g, b = (int(c) for c in pal[buf[i]][:3])
        blue, green, red = min(15, (r + 7) >> 4), min(15, (g + 7) >> 4), min(15, (b + 7) >> 4)
        p = (red << 8) + (green << 4) + blue
        pos_out.append((x + (y << 10) + (z << 20)) & 0xFFFFFFFF)
        vox_out.append(p if p else 1)
    return tuple(S), np.array(pos_out, np.uint32), np.array(vox_out, np.uint32)


@needs_ogt
@pytest.mark.parametrize("seed", range(12))
def test_scene_graph_matches_ogt_vox(tmp_path, seed):
    """Models, flattened instance transforms, instance order and palette as the
    reference's ogt_vox_read_scene gives them, on seeded scene graphs (rotations,
    translations, nested groups, hidden nodes, a duplicate and an empty model, layers,
    materials, a skipped chunk; the default palette on odd seeds)."""
    path = _random_scene(tmp_path / "s.vox", seed, palette=seed % 2 == 0)
    want = ob.ogt_scene(path)
    _same_scene(vs.read_vox_scene(path), want)
    size, pos, vox = vs.large_model_frame(path)
    wsize, wpos, wvox = _reference_frame(*want)
    assert size == wsize and np.array_equal(pos, wpos) and np.array_equal(vox, wvox)


@needs_ogt
@pytest.mark.parametrize("kind", ["keeps_empty", "fills_empty"])
def test_index_map_matches_ogt_vox(tmp_path, kind):
    """IMAP: the palette in display order and the voxel indices remapped (a map whose
    inverse sends 0 to 0 keeps empty cells empty; any other fills them, as ogt does)."""
    rng = np.random.default_rng(3)
    imap = rng.permutation(256).astype(np.uint8)
    if kind == "keeps_empty":
        imap = np.concatenate([rng.permutation(np.arange(1, 256)), [0]]).astype(np.uint8)
    path = _random_scene(tmp_path / "m.vox", 40, imap=imap)
    want = ob.ogt_scene(path)
    _same_scene(vs.read_vox_scene(path), want)
    size, pos, vox = vs.large_model_frame(path)
    wsize, wpos, wvox = _reference_frame(*want)
    assert size == wsize and np.array_equal(pos, wpos) and np.array_equal(vox, wvox)


@pytest.mark.skipif(not os.path.isfile(CORNELL), reason="the reference's scene files are not present")
def test_cornell_box_both_branches():
    """cornell-box.vox (one model, no scene graph): the large-model frame lists the same
    voxels as the default branch (read_vox), one larger per axis, with red and blue of
    every colour exchanged; against ogt too when it is built."""
    size, pos, vox = vs.large_model_frame(CORNELL)
    (dsize, dpos, dvox), = io.read_vox(CORNELL)
    assert size == tuple(s + 1 for s in dsize) and np.array_equal(pos, dpos)
    swapped = ((dvox & 0xF) << 8) | (dvox & 0xF0) | ((dvox >> 8) & 0xF)
    assert np.array_equal(vox, np.where(swapped == 0, 1, swapped))
    if ob.load_ogt() is not None:
        _same_scene(vs.read_vox_scene(CORNELL), ob.ogt_scene(CORNELL))


@pytest.mark.parametrize("case", ["rotation", "frames", "no_size", "shape_models", "no_instances", "magic"])
def test_scene_errors(tmp_path, case):
    g = np.ones((2, 2, 2), np.uint8)
    chunks = {
        "rotation": [_model(g), _trn(0, 1, 0, {"_r": 0}), _shp(1, 0)],          # rows 0 and 1 both x
        "frames": [_model(g), _chunk(b"nTRN", struct.pack("<I", 0) + _dict({}) +
                                     struct.pack("<IIII", 1, 0xFFFFFFFF, 0, 2) + _dict({}) + _dict({}))],
        "no_size": [_chunk(b"XYZI", struct.pack("<I", 1) + bytes(4))],
        "shape_models": [_model(g), _chunk(b"nSHP", struct.pack("<I", 0) + _dict({}) + struct.pack("<III", 2, 0, 0))],
        "no_instances": [_model(g), _model(g * 2)],                            # two models, no graph
    }
    if case == "magic":
        path = str(tmp_path / "x.vox")
        open(path, "wb").write(b"VOX " + struct.pack("<i", 200) + bytes(12))
    else:
        path = _write(tmp_path / "x.vox", chunks[case])
    with pytest.raises(ValueError):
        vs.large_model_frame(path)


def test_sprite_dispatch_large_model(lib, tmp_path):
    """load_sprite / stamp_sprite with large_model=True take the opengametools path."""
    g = np.zeros((1, 1, 3), np.uint8)
    g[0, 0] = (1, 0, 9)
    path = _write(tmp_path / "d.vox", [_model(g), _trn(0, 1, 0, {"_t": "4 5 6"}), _shp(1, 0)])
    (size, pos, vox), = io.load_sprite(path, large_model=True)
    assert (size, pos.tolist()) == ((4, 2, 2), [0, 2])
    w = lib.World()
    io.stamp_sprite(w, path, (10, 10, 10), large_model=True)
    assert w.get(10, 10, 10) == 0xF000 | int(vox[0]) and w.get(12, 10, 10) == 0xF000 | int(vox[1])
    w.close()


def test_cyclic_scene_graph_is_rejected(tmp_path):
    """A transform node whose child leads back to it: ValueError (ogt_vox recurses
    without end)."""
    g = np.ones((1, 1, 1), np.uint8)
    path = _write(tmp_path / "c.vox", [_model(g), _trn(0, 1), _grp(1, [2, 0]), _shp(2, 0)])
    with pytest.raises(ValueError):
        vs.read_vox_scene(path)
