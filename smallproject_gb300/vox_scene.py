"""MagicaVoxel scenes as the reference's SpriteManager::LoadSprite reads them with its
large-model flag (template/world.cpp:1039-1137): the file is parsed by the third-party
opengametools reader vendored with the reference (lib/ogt_vox.h,
ogt_vox_read_scene), then every instance is placed with its flattened transform into
one sprite frame.

The reader's published algorithm, restated here (read_vox_scene):

* header "VOX " and version 150, then 12-byte chunk headers (id, content bytes, children
  bytes) while at least 12 bytes remain. MAIN has no content. SIZE sets the size of the
  next models; XYZI adds a model (voxels x + y * sx + z * sx * sy, MagicaVoxel axes, the
  last write to a cell wins) or, with no voxels, an empty model. RGBA replaces the
  palette. nTRN, nGRP, nSHP, LAYR, MATL and IMAP are parsed field by field (dictionaries:
  a pair count, then length-prefixed key and value strings; keys compare
  case-insensitively). Every other chunk is skipped by its content size.
* nTRN frame attributes: `_r` packs a signed permutation (bits 0-1: column of row 0's
  non-zero entry, 2-3: row 1's, row 2 takes the remaining column; bits 4-6 negate rows
  0-2); `_t` holds three integers read like C's "%i". The rows are stored as the
  transform's columns; the translation is the last row.
* With scene nodes, instances come from a walk from node 0: a transform node multiplies
  its transform by its parent's (child * parent), a group node passes its transform to
  each child, a shape node makes one instance of its model unless the model is empty.
  Without nodes and with exactly one model, that model gets one identity instance.
* IMAP reorders the palette into display order and remaps the voxel indices; then the
  palette is rotated so that index i holds file entry i - 1 (index 0: entry 255 with
  alpha 0). Identical models are merged into the first, empty models dropped and the
  instances renumbered, and the instances are sorted by model index (stable here; the C
  library's qsort leaves the order of equal keys to the platform).

Hidden nodes and layers are read but, as in the reference, every instance is placed.
Inputs that make the C code assert or read out of bounds raise ValueError here.
"""
import re
import struct

import numpy as np

from .scene_io import vox_default_palette

_VECTORS = np.array([[1, 0, 0], [0, 1, 0], [0, 0, 1], [0, 0, 0]], np.float64)
_ROW2 = {3: 2, 5: 1, 6: 0}        # (1 << row0) | (1 << row1) -> row 2's column
_MAX_DICT_PAIRS, _MAX_DICT_BYTES = 256, 4096


class _Reader:
    def __init__(self, data, path):
        self.d, self.off, self.path = data, 0, path

    def remaining(self):
        return len(self.d) - self.off

    def bytes(self, n):
        if self.off + n > len(self.d):
            raise ValueError(f"{self.path}: chunk content truncated at byte {self.off}")
        b = self.d[self.off:self.off + n]
        self.off += n
        return b

    def u32(self):
        return struct.unpack("<I", self.bytes(4))[0]

    def i32(self):
        return struct.unpack("<i", self.bytes(4))[0]

    def dict(self):
        n = self.u32()
        if n > _MAX_DICT_PAIRS:
            raise ValueError(f"{self.path}: dictionary of {n} pairs")
        out, used = [], 0
        for _ in range(n):
            k = self.bytes(self.u32())
            v = self.bytes(self.u32())
            used += len(k) + len(v) + 2
            if used > _MAX_DICT_BYTES:
                raise ValueError(f"{self.path}: dictionary larger than {_MAX_DICT_BYTES} bytes")
            out.append((k.decode("latin-1"), v.decode("latin-1")))
        return out


def _get(d, key, default=None):
    for k, v in d:
        if k.lower() == key.lower():
            return v
    return default


def _c_atoi(s):
    m = re.match(r"\s*([+-]?\d+)", s)
    return int(m.group(1)) if m else 0


def _c_scan_ints(s, count):
    """Integers read like sscanf(s, "%i %i %i"): decimal, 0x hex or leading-0 octal,
    stopping at the first field that does not parse (the rest stay 0)."""
    out = [0] * count
    pos = 0
    for i in range(count):
        m = re.compile(r"\s*([+-]?)(0[xX][0-9a-fA-F]+|0[0-7]*|[1-9][0-9]*)").match(s, pos)
        if not m:
            break
        sign, body = m.group(1), m.group(2)
        v = int(body, 16) if body[:2].lower() == "0x" else (int(body, 8) if body.startswith("0") else int(body))
        out[i] = (-v if sign == "-" else v)
        pos = m.end()
    return out


def _frame_transform(rot, trans, path):
    """_r / _t strings -> 4 x 4 transform (rows: the rotation's columns, then the
    translation)."""
    t = np.eye(4, dtype=np.float64)
    if rot is not None:
        bits = _c_atoi(rot) & 0xFFFFFFFF
        r0, r1 = bits & 3, (bits >> 2) & 3
        key = (1 << r0) | (1 << r1)
        if key not in _ROW2:
            raise ValueError(f"{path}: invalid rotation {rot!r}")
        rows = [_VECTORS[r0].copy(), _VECTORS[r1].copy(), _VECTORS[_ROW2[key]].copy()]
        for i in range(3):
            if bits & (1 << (4 + i)):
                rows[i] = -rows[i]
        for c in range(3):             # t[c][r] = row r's component c
            for r in range(3):
                t[c][r] = rows[r][c]
    if trans is not None:
        t[3][:3] = _c_scan_ints(trans, 3)
    return t


def _walk(nodes, models, path):
    """generate_instances_for_node from node 0 without group output (flattened
    transforms), depth first in child order, with an explicit stack."""
    instances, stack = [], [(0, np.eye(4), 0)]
    while stack:
        node_id, transform, depth = stack.pop()
        if depth > 4096:
            raise ValueError(f"{path}: scene graph too deep or cyclic")
        node = nodes.get(node_id)
        if node is None:              # referenced but never defined: no instance
            continue
        if node[0] == "trn":
            _, t, child = node
            stack.append((child, t @ transform, depth + 1))
        elif node[0] == "grp":
            for c in reversed(node[1]):
                stack.append((c, transform, depth + 1))
        elif node[1] < len(models) and models[node[1]] is not None:
            instances.append([node[1], transform])
    return instances


def read_vox_scene(path):
    """ogt_vox_read_scene (lib/ogt_vox.h:847-1449) without group output: (models,
    instances, palette). models: list of uint8[sz, sy, sx] colour-index arrays in
    MagicaVoxel axes; instances: list of (model index, 4 x 4 float64 transform, rows:
    the rotation's columns then the translation), sorted by model index; palette:
    uint8[256, 4] RGBA with index i = file entry i - 1."""
    with open(path, "rb") as f:
        data = f.read()
    r = _Reader(data, path)
    if len(data) < 8 or data[:4] != b"VOX " or struct.unpack_from("<I", data, 4)[0] != 150:
        raise ValueError(f"{path}: not a version-150 .vox file")
    r.off = 8
    # the default palette in file order: the table's entries 1-255, then opaque black
    pal = vox_default_palette().view(np.uint8).reshape(256, 4)[np.r_[1:256, 0]].copy()
    pal[255, 3] = 255
    models, nodes, imap = [], {}, None
    size = (0, 0, 0)
    while r.remaining() >= 12:
        cid, csize = r.bytes(4), r.u32()
        r.u32()
        if cid == b"MAIN":
            continue
        if cid == b"SIZE":
            size = (r.u32(), r.u32(), r.u32())
        elif cid == b"XYZI":
            n = r.u32()
            sx, sy, sz = size
            if n == 0:
                models.append(None)
                continue
            if not (sx and sy and sz):
                raise ValueError(f"{path}: XYZI chunk without a SIZE")
            k = min(r.remaining() // 4, n)
            v = np.frombuffer(data, np.uint8, 4 * k, r.off).reshape(k, 4).astype(np.int64)
            r.off = min(len(data), r.off + 4 * n)
            if k and ((v[:, 0] >= sx).any() or (v[:, 1] >= sy).any() or (v[:, 2] >= sz).any()):
                raise ValueError(f"{path}: voxel outside the model size {size}")
            grid = np.zeros(sx * sy * sz, np.uint8)
            cell = v[:, 0] + v[:, 1] * sx + v[:, 2] * sx * sy
            _, last = np.unique(cell[::-1], return_index=True)     # the last write to a cell wins
            keep = k - 1 - last
            grid[cell[keep]] = v[keep, 3]
            models.append(grid.reshape(sz, sy, sx))
        elif cid == b"RGBA":
            pal = np.frombuffer(r.bytes(1024), np.uint8).reshape(256, 4).copy()
        elif cid == b"nTRN":
            nid = r.u32()
            r.dict()
            child, reserved, _layer, frames = r.u32(), r.u32(), r.u32(), r.u32()
            if reserved != 0xFFFFFFFF or frames != 1:
                raise ValueError(f"{path}: transform node {nid} with {frames} frames")
            fd = r.dict()
            nodes[nid] = ("trn", _frame_transform(_get(fd, "_r"), _get(fd, "_t"), path), child)
        elif cid == b"nGRP":
            nid = r.u32()
            r.dict()
            nodes[nid] = ("grp", [r.u32() for _ in range(r.u32())])
        elif cid == b"nSHP":
            nid = r.u32()
            r.dict()
            if r.u32() != 1:
                raise ValueError(f"{path}: shape node {nid} without exactly one model")
            mid = r.u32()
            r.dict()
            nodes[nid] = ("shp", mid)
        elif cid == b"IMAP":
            imap = np.frombuffer(r.bytes(256), np.uint8).copy()
        elif cid == b"LAYR":
            r.i32()
            r.dict()
            r.i32()
        elif cid == b"MATL":
            r.i32()
            r.dict()
        else:
            r.off = min(len(data), r.off + csize)
    instances = []
    if nodes:
        instances = _walk(nodes, models, path)
    elif len(models) == 1:
        if models[0] is None:
            raise ValueError(f"{path}: the only model is empty")
        instances.append([0, np.eye(4)])
    if imap is not None:
        inverse = np.zeros(256, np.uint8)
        inverse[imap] = np.arange(256, dtype=np.uint8)
        pal = pal[(imap.astype(np.int64) + 255) & 255]
        models = [None if m is None else (1 + inverse[m].astype(np.int64)).astype(np.uint8) for m in models]
    pal = pal[np.r_[255, 0:255]].copy()        # index i = entry i - 1; index 0 transparent
    pal[0, 3] = 0
    for i in range(len(models)):               # merge identical models into the first
        for j in range(i + 1, len(models)):
            if models[i] is not None and models[j] is not None and models[i].shape == models[j].shape \
                    and np.array_equal(models[i], models[j]):
                models[j] = None
                for inst in instances:
                    if inst[0] == j:
                        inst[0] = i
    remap, out = {}, []
    for i, m in enumerate(models):             # drop empty models
        if m is not None:
            remap[i] = len(out)
            out.append(m)
    for inst in instances:
        inst[0] = remap[inst[0]]
    instances.sort(key=lambda t: t[0])
    return out, [(m, t) for m, t in instances], pal


def large_model_frame(path):
    """The one sprite frame LoadSprite(path, largeModel = true) builds
    (world.cpp:1041-1129): (size (x, y, z), pos uint32[n], voxels uint32[n]).

    Every instance is placed (hidden ones too) at its integer translation minus the
    corner of all instances' boxes, its voxels rotated by the transform, MagicaVoxel's
    y and z swapped into the frame; a later instance overwrites an earlier one. Voxel
    colour = the palette colour of its index with red and blue exchanged: blue from
    (r + 7) >> 4, green from (g + 7) >> 4, red from (b + 7) >> 4, each clamped to 15, and 1
    for black. The draw list runs z outer, then y, then x."""
    models, instances, pal = read_vox_scene(path)
    if not instances:
        raise ValueError(f"{path}: no instances")
    lo, hi, placed = np.full(3, 0xFFFFFF, np.int64), np.full(3, -0xFFFFFF, np.int64), []
    for mid, t in instances:
        sz, sy, sx = models[mid].shape
        pos = np.trunc(t[3, :3]).astype(np.int64)
        ext = np.trunc(np.array([sx, sy, sz], np.float64) @ t[:3, :3]).astype(np.int64)
        lo = np.minimum(lo, np.minimum(pos, pos + ext))
        hi = np.maximum(hi, np.maximum(pos, pos + ext))
    S = (hi + 1) - lo                            # MagicaVoxel axes; the frame swaps y and z
    fx, fy, fz = int(S[0]), int(S[2]), int(S[1])
    for mid, t in instances:
        m = models[mid]
        z, y, x = np.nonzero(m)                  # model order: z outer, y, x inner
        local = np.stack([x, y, z], axis=1).astype(np.float64)
        p = np.trunc(local @ t[:3, :3]).astype(np.int64) + (np.trunc(t[3, :3]).astype(np.int64) - lo)
        placed.append((p[:, 0] + p[:, 2] * fx + p[:, 1] * fx * fy, m[z, y, x]))
    idx = np.concatenate([a for a, _ in placed])
    val = np.concatenate([b for _, b in placed])
    if idx.size and (idx.min() < 0 or idx.max() >= fx * fy * fz):
        raise ValueError(f"{path}: an instance lies outside the frame")
    cells, last = np.unique(idx[::-1], return_index=True)      # later instances win
    v = val[len(idx) - 1 - last].astype(np.int64)
    c = pal[v].astype(np.int64)
    blue = np.minimum(15, (c[:, 0] + 7) >> 4)
    green = np.minimum(15, (c[:, 1] + 7) >> 4)
    red = np.minimum(15, (c[:, 2] + 7) >> 4)
    colour = (red << 8) | (green << 4) | blue
    colour = np.where(colour == 0, 1, colour).astype(np.uint32)
    X, Y, Z = cells % fx, (cells // fx) % fy, cells // (fx * fy)
    pos = ((X + (Y << 10) + (Z << 20)) & 0xFFFFFFFF).astype(np.uint32)
    return (fx, fy, fz), pos, colour
