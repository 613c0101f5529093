"""Scene and frame files of the reference, the data formats on either side of the render
path:

* ``.vx`` worlds and sprites: gzip stream of int32 payload size (2 or 4 bytes per voxel),
  int32 frame count, then per frame int32 size x, y, z, uint32 draw-list length n, n
  uint32 positions ``x | y << 10 | z << 20`` and n voxels (SpriteManager::LoadSprite /
  SaveSprite, template/world.cpp:1005-1035, 1307-1327). A world file is one frame
  (MyGameScene::SaveWorld / LoadWorld, mygamescene.cpp:110-134); loading clears the world
  and stamps the draw list at the origin with ``| 0xF000`` (World::StampSpriteTo,
  world.cpp:1545-1563), entries in file order.
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
    """Dense voxels of the box [origin, origin + size) of a world, indexed [x, y, z]."""
    grid, bricks, _ = world.arrays()
    g = grid.reshape(128, 128, 128)                       # [gy, gz, gx]
    ox, oy, oz = (int(v) for v in origin)
    sx, sy, sz = (int(v) for v in size)
    # broadcast index vectors: x along axis 0, y along 1, z along 2
    xs, ys, zs = np.arange(ox, ox + sx), np.arange(oy, oy + sy), np.arange(oz, oz + sz)
    xi, yi, zi = np.minimum(xs, 1023), np.minimum(ys, 1023), np.minimum(zs, 1023)
    cell = g[(yi >> 3)[None, :, None], (zi >> 3)[None, None, :], (xi >> 3)[:, None, None]]
    out = cell >> 1
    isb = (cell & 1) == 1
    if isb.any():
        local = ((xi & 7)[:, None, None] + (yi & 7)[None, :, None] * 8 + (zi & 7)[None, None, :] * 64).astype(np.int32)
        local = np.broadcast_to(local, cell.shape)
        out[isb] = bricks[cell[isb] >> 1, local[isb]]
    inside = (xs < 1024)[:, None, None] & (ys < 1024)[None, :, None] & (zs < 1024)[None, None, :]
    return np.where(inside, out, 0).astype(np.uint32)


def world_frame(world, origin, size):
    """One frame of a world's box as World::CreateSprite lists it: the non-zero voxels
    in x, then y, then z order (without CreateSprite's leading zero entries)."""
    vol = region(world, origin, size)
    x, y, z = np.nonzero(vol)                             # row-major: x outer, z inner
    pos = (x.astype(np.uint32) | (y.astype(np.uint32) << 10) | (z.astype(np.uint32) << 20))
    return tuple(int(s) for s in size), pos, vol[x, y, z]


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
