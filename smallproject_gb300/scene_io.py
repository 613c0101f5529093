"""Scene and frame files of the reference, the data formats on either side of the render
path:

* ``.vx`` worlds and sprites: gzip stream of int32 payload size (2 or 4 bytes per voxel),
  int32 frame count, then per frame int32 size x, y, z, uint32 draw-list length n, n
  uint32 positions ``x | y << 10 | z << 20`` and n voxels (SpriteManager::LoadSprite /
  SaveSprite, template/world.cpp:1005-1035, 1307-1327). A world file is one frame
  (MyGameScene::SaveWorld / LoadWorld, mygamescene.cpp:110-134); loading clears the world
  and stamps the draw list at the origin with ``| 0xF000`` (World::StampSpriteTo,
  world.cpp:1545-1563), entries in file order.
* ``.vox`` sprites (MagicaVoxel): read as SpriteManager::LoadSprite reads them without
  its large-model flag (world.cpp:1140-1296), into the same frame format (read_vox).
  The large-model branch (the third-party opengametools ogt_vox reader, with scene-graph
  transforms) has no caller in the reference that enables it and is not provided.
* ``.dat`` frames: uint32 width, uint32 height, then width * height float4 pixels, row
  by row (saveScreenBuffer, mygame.cpp:518-549; the reference appends a time stamp to
  the file name, these functions use the name given).

Files written by the reference's World::CreateSprite (world.cpp:1347-1386) begin with
size_x * size_y * size_z / 4 zero entries (its draw list is created with that many
elements, then appended to), so loading one stamps 0xF000 at the origin before the real
voxels; ``load_world_vx`` reproduces this, ``save_world_vx`` writes no such entries.
"""
import gzip
import struct

import numpy as np

STAMP_MASK = 0xF000


def read_vx(path):
    """(payload bytes, frames) of a .vx file; frames: [(size (x, y, z), pos uint32[n],
    voxels uint32[n]), ...]."""
    with gzip.open(path, "rb") as f:
        data = f.read()
    pls, nframes = struct.unpack_from("<ii", data, 0)
    if pls not in (2, 4):
        raise ValueError(f"{path}: payload size {pls}: only 2 and 4 bytes per voxel are known")
    off = 8
    frames = []
    for _ in range(nframes):
        sx, sy, sz, n = struct.unpack_from("<iiiI", data, off)
        off += 16
        pos = np.frombuffer(data, np.uint32, n, off).copy()
        off += 4 * n
        vox = np.frombuffer(data, np.uint16 if pls == 2 else np.uint32, n, off).astype(np.uint32)
        off += pls * n
        frames.append(((sx, sy, sz), pos, vox))
    if off != len(data):
        raise ValueError(f"{path}: {len(data) - off} bytes after the last frame")
    return pls, frames


def write_vx(path, frames, payload=4):
    """Write frames [(size, pos, voxels), ...] as a .vx file (payload 2 keeps the low 16
    bits of each voxel)."""
    if payload not in (2, 4):
        raise ValueError("payload must be 2 or 4 bytes")
    with gzip.open(path, "wb", compresslevel=6) as f:     # zlib's default, as gzopen(.., "wb")
        f.write(struct.pack("<ii", payload, len(frames)))
        for size, pos, vox in frames:
            pos = np.ascontiguousarray(pos, np.uint32)
            vox = np.ascontiguousarray(vox, np.uint32)
            f.write(struct.pack("<iiiI", *(int(s) for s in size), len(pos)))
            f.write(pos.tobytes())
            f.write((vox & 0xFFFF).astype(np.uint16).tobytes() if payload == 2 else vox.tobytes())


def region(world, origin, size):
    """Dense voxels of the box [origin, origin + size) of a world, indexed [x, y, z];
    coordinates wrap modulo 1024 like World::Get (world.h:293-306)."""
    grid, bricks, _ = world.arrays()
    g = grid.reshape(128, 128, 128)                       # [gy, gz, gx]
    ox, oy, oz = (int(v) for v in origin)
    sx, sy, sz = (int(v) for v in size)
    # broadcast index vectors: x along axis 0, y along 1, z along 2
    xi, yi, zi = (np.arange(o, o + n) & 1023 for o, n in ((ox, sx), (oy, sy), (oz, sz)))
    cell = g[(yi >> 3)[None, :, None], (zi >> 3)[None, None, :], (xi >> 3)[:, None, None]]
    out = cell >> 1
    isb = (cell & 1) == 1
    if isb.any():
        local = ((xi & 7)[:, None, None] + (yi & 7)[None, :, None] * 8 + (zi & 7)[None, None, :] * 64).astype(np.int32)
        local = np.broadcast_to(local, cell.shape)
        out[isb] = bricks[cell[isb] >> 1, local[isb]]
    return out.astype(np.uint32)


def world_voxels(world):
    """Every non-zero voxel of a world: (x, y, z, value) arrays, from its solid cells and
    bricks (no dense pass over the 1024^3 map)."""
    grid, bricks, _ = world.arrays()
    i = np.flatnonzero(grid).astype(np.int64)                # cell = bx + bz * 128 + by * 128^2
    c = grid[i]
    bx, bz, by = i & 127, (i >> 7) & 127, i >> 14
    lx, ly, lz = (np.arange(512) & 7), (np.arange(512) >> 3) & 7, np.arange(512) >> 6
    solid = (c & 1) == 0
    vs = np.repeat(c[solid] >> 1, 512)
    xs = (bx[solid, None] * 8 + lx).ravel()
    ys = (by[solid, None] * 8 + ly).ravel()
    zs = (bz[solid, None] * 8 + lz).ravel()
    bv = bricks[c[~solid] >> 1]                              # [n, 512]
    k, j = np.nonzero(bv)
    xb = bx[~solid][k] * 8 + lx[j]
    yb = by[~solid][k] * 8 + ly[j]
    zb = bz[~solid][k] * 8 + lz[j]
    return (np.concatenate([xs, xb]), np.concatenate([ys, yb]), np.concatenate([zs, zb]),
            np.concatenate([vs, bv[k, j]]).astype(np.uint32))


def _box_coords(w, o, n):
    """Box coordinates s in [0, n) with (s + o) mod 1024 == w, for world coordinates w:
    (index into w, s) pairs; more than one s per w when the box is wider than the map."""
    first = (w - o) & 1023
    reps = np.maximum(0, (n - first + 1023) // 1024)
    idx = np.repeat(np.arange(len(w)), reps)
    k = np.arange(len(idx)) - np.repeat(np.cumsum(reps) - reps, reps)
    return idx, first[idx] + 1024 * k


def world_frame(world, origin, size):
    """One frame of a world's box as World::CreateSprite lists it (world.cpp:1347-1386):
    the non-zero voxels, box x outer, then y, then z; World::Get wraps coordinates modulo
    1024, and the position x + (y << 10) + (z << 20) is packed with unsigned wrap-around,
    as the reference does for boxes wider than the map (without CreateSprite's leading
    zero entries)."""
    x, y, z, v = world_voxels(world)
    (ox, oy, oz), (sx, sy, sz) = (tuple(int(a) for a in t) for t in (origin, size))
    i, bx = _box_coords(x.astype(np.int64), ox, sx)
    j, by = _box_coords(y[i].astype(np.int64), oy, sy)
    i, bx = i[j], bx[j]
    j, bz = _box_coords(z[i].astype(np.int64), oz, sz)
    i, bx, by = i[j], bx[j], by[j]
    order = np.lexsort((bz, by, bx))
    bx, by, bz, val = bx[order], by[order], bz[order], v[i[order]]
    pos = ((bx + (by << 10) + (bz << 20)) & 0xFFFFFFFF).astype(np.uint32)
    return (sx, sy, sz), pos, val


def save_world_vx(world, path, size, origin=(0, 0, 0), payload=4):
    """MyGameScene::SaveWorld: the box [origin, origin + size) as a one-frame .vx."""
    write_vx(path, [world_frame(world, origin, size)], payload)


def load_world_vx(world, path, frame=0):
    """MyGameScene::LoadWorld: clear the world, stamp frame `frame` of the file at the
    origin with | 0xF000, entries in file order. Returns the file's frame size."""
    _, frames = read_vx(path)
    size, pos, vox = frames[frame]
    # runs of identical entries set the same voxel to the same value again, which changes
    # nothing: stamp each run once (the leading zero entries of reference-made files)
    keep = np.ones(len(pos), bool)
    keep[1:] = (pos[1:] != pos[:-1]) | (vox[1:] != vox[:-1])
    world.clear()
    world.stamp(pos[keep], vox[keep], (0, 0, 0), STAMP_MASK)
    return size


def vox_default_palette():
    """MagicaVoxel's default palette as uint32 RGBA (r in the low byte), indexed by colour
    index: entry 0 empty; 1-215 the 6 x 6 x 6 cube of levels ff, cc, 99, 66, 33, 00 with
    blue varying fastest, then green, then red, black left out; 216-255 ten-step ramps
    (ee dd bb aa 88 77 55 44 22 11) of red, green, blue and grey."""
    lv = [0xFF, 0xCC, 0x99, 0x66, 0x33, 0x00]
    ramp = [0xEE, 0xDD, 0xBB, 0xAA, 0x88, 0x77, 0x55, 0x44, 0x22, 0x11]
    pal = [0]
    for r in lv:
        for g in lv:
            for b in lv:
                if r or g or b:
                    pal.append(0xFF000000 | b << 16 | g << 8 | r)
    pal += [0xFF000000 | c for c in ramp]                      # red
    pal += [0xFF000000 | c << 8 for c in ramp]                 # green
    pal += [0xFF000000 | c << 16 for c in ramp]                # blue
    pal += [0xFF000000 | c << 16 | c << 8 | c for c in ramp]   # grey
    assert len(pal) == 256
    return np.array(pal, np.uint32)


def vox_colour(c):
    """The reference's 12-bit voxel colour of RGBA palette entries (2- and 4-byte
    payloads, world.cpp:1267-1272): each channel (v + 7) >> 4 clamped to 15, red in bits
    8-11, green 4-7, blue 0-3; a colour that rounds to black becomes 1."""
    c = np.asarray(c, np.uint32)
    blue = np.minimum(15, (((c >> 16) & 255) + 7) >> 4)
    green = np.minimum(15, (((c >> 8) & 255) + 7) >> 4)
    red = np.minimum(15, ((c & 255) + 7) >> 4)
    p = (red << 8) | (green << 4) | blue
    return np.where(p == 0, 1, p).astype(np.uint32)


# chunks whose content the reference's reader skips (materials, scene graph, layers)
_VOX_SKIPPED = (b"MATT", b"MATL", b"nTRN", b"nGRP", b"nSHP", b"LAYR")


def read_vox(path):
    """Frames of a MagicaVoxel .vox file as SpriteManager::LoadSprite reads one without
    its large-model flag (template/world.cpp:1140-1296): [(size (x, y, z), pos uint32[n],
    voxels uint32[n]), ...], one frame per XYZI chunk, in the sprite format of read_vx.

    * Header "VOX ", version 150, then a MAIN chunk whose two size fields are ignored.
    * Chunks of 12-byte headers (name, content bytes, children bytes) until the end of the
      file or a header whose name starts with a zero byte. PACK sets the frame count
      (default 1); SIZE starts a frame and swaps y and z (MagicaVoxel's z is up); XYZI
      fills it with colour indices at x + z * sx + y * sx * sy (sizes after the swap);
      RGBA replaces the palette; MATT, MATL, nTRN, nGRP, nSHP and LAYR are skipped by
      their content size. Any other chunk moves the reader past its 12-byte header
      only, as the reference does.
    * Voxel colour = vox_colour(palette[index - 1]), for the default palette as for an
      RGBA chunk. The draw list runs z outer, then y, then x.

    Where the reference has undefined behaviour this raises ValueError instead: more or
    fewer XYZI chunks than PACK announced, XYZI without SIZE, voxels outside the size,
    truncated chunk content."""
    with open(path, "rb") as f:
        data = f.read()
    if len(data) < 20 or data[:4] != b"VOX ":
        raise ValueError(f"{path}: bad header")
    version = struct.unpack_from("<i", data, 4)[0]
    if version != 150:
        raise ValueError(f"{path}: bad version ({version})")
    if data[8:12] != b"MAIN":
        raise ValueError(f"{path}: no MAIN chunk")
    off = 20
    palette = vox_default_palette()
    frame_count = 1
    size = None
    models = []

    def take(n):
        nonlocal off
        if off + n > len(data):
            raise ValueError(f"{path}: chunk content truncated at byte {off}")
        b = data[off:off + n]
        off += n
        return b

    while off + 12 <= len(data):
        name = data[off:off + 4]
        content = struct.unpack_from("<i", data, off + 4)[0]
        off += 12
        if name[0] == 0:
            break
        if name == b"PACK":
            frame_count = struct.unpack("<i", take(4))[0]
        elif name == b"SIZE":
            sx, sy, sz = struct.unpack("<iii", take(12))
            size = (sx, sz, sy)
        elif name == b"XYZI":
            if size is None:
                raise ValueError(f"{path}: XYZI chunk without SIZE")
            n = struct.unpack("<I", take(4))[0]
            xyzi = np.frombuffer(take(4 * n), np.uint8).reshape(n, 4).astype(np.int64)
            sx, sy, sz = size
            if n and ((xyzi[:, 0] >= sx).any() or (xyzi[:, 2] >= sy).any() or (xyzi[:, 1] >= sz).any()):
                raise ValueError(f"{path}: voxel outside the model size {size}")
            if len(models) == frame_count:
                raise ValueError(f"{path}: bad frame count")
            buf = np.zeros(sx * sy * sz, np.uint8)
            cell = xyzi[:, 0] + xyzi[:, 2] * sx + xyzi[:, 1] * sx * sy
            _, last = np.unique(cell[::-1], return_index=True)      # the last write to a cell wins
            keep = n - 1 - last
            buf[cell[keep]] = xyzi[keep, 3]
            models.append((size, buf))
            size = None
        elif name == b"RGBA":
            palette = np.frombuffer(take(1024), np.uint32).copy()
        elif name in _VOX_SKIPPED:
            take(content)
    if len(models) != frame_count:
        raise ValueError(f"{path}: {len(models)} models for a frame count of {frame_count}")
    frames = []
    for (sx, sy, sz), buf in models:
        i = np.flatnonzero(buf)                                  # z outer, y, x inner
        x, y, z = i % sx, (i // sx) % sy, i // (sx * sy)
        pos = (x | (y << 10) | (z << 20)).astype(np.uint32)
        frames.append(((sx, sy, sz), pos, vox_colour(palette[buf[i].astype(np.int64) - 1])))
    return frames


def load_sprite(path):
    """SpriteManager::LoadSprite: the frames of a .vx (read_vx) or .vox (read_vox) file."""
    return read_vx(path)[1] if ".vx" in str(path) else read_vox(path)    # strstr(path, ".vx")


def stamp_sprite(world, path, origin=(0, 0, 0), frame=0):
    """LoadSprite + StampSpriteTo: stamp frame `frame` of a sprite file into the world at
    `origin` with | 0xF000, entries in draw-list order. Returns the frame's size."""
    size, pos, vox = load_sprite(path)[frame]
    world.stamp(pos, vox, origin, STAMP_MASK)
    return size


def write_frame_dat(path, rgba, width, height):
    """saveScreenBuffer: uint32 width, height, then float4 pixels row by row."""
    a = np.ascontiguousarray(rgba, np.float32).reshape(height * width, 4)
    with open(path, "wb") as f:
        f.write(struct.pack("<II", width, height))
        f.write(a.tobytes())


def read_frame_dat(path):
    """(width, height, float32[height * width, 4]) of a .dat frame file."""
    with open(path, "rb") as f:
        data = f.read()
    w, h = struct.unpack_from("<II", data, 0)
    if len(data) != 8 + 16 * w * h:
        raise ValueError(f"{path}: {len(data)} bytes for a {w} x {h} frame")
    return w, h, np.frombuffer(data, np.float32, 4 * w * h, 8).reshape(w * h, 4).copy()
