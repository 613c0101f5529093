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
  With the large-model flag the reference parses the file with the third-party
  opengametools reader instead and places every instance of the scene graph
  (vox_scene.py, load_sprite(path, large_model=True)).
* ``.dat`` frames: uint32 width, uint32 height, then width * height float4 pixels, row
  by row (saveScreenBuffer, mygame.cpp:518-549; the reference appends a time stamp to
  the file name, these functions use the name given).
* frame comparison as the reference's MSE tool does it (mse.cpp:19-63): frame_mse,
  frame_mae, frame_energy, with its float / double arithmetic.
* ``.hdr`` sky domes (Radiance RGBE, the format World::LoadSky reads through
  stb_image's stbi_loadf, world.cpp:803-876): read_hdr / write_hdr, and sky_texture for
  LoadSky's conversion to the texture of vxr_view_set_sky.

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


def load_sprite(path, large_model=False):
    """SpriteManager::LoadSprite: the frames of a .vx file (read_vx), else of a .vox file:
    with large_model the one frame of its scene (vox_scene.large_model_frame, the
    opengametools path), without it read_vox."""
    if ".vx" in str(path):                                   # strstr(path, ".vx")
        return read_vx(path)[1]
    if large_model:
        from .vox_scene import large_model_frame
        return [large_model_frame(path)]
    return read_vox(path)


def stamp_sprite(world, path, origin=(0, 0, 0), frame=0, large_model=False):
    """LoadSprite + StampSpriteTo: stamp frame `frame` of a sprite file into the world at
    `origin` with | 0xF000, entries in draw-list order. Returns the frame's size."""
    size, pos, vox = load_sprite(path, large_model)[frame]
    world.stamp(pos, vox, origin, STAMP_MASK)
    return size


def _rgbe_to_float(rgbe):
    """RGBE bytes [..., 4] -> float32 [..., 3]: c * 2^(e - 136), 0 where e == 0."""
    e = rgbe[..., 3].astype(np.int32)
    f = np.where(e != 0, np.ldexp(np.float32(1.0), e - 136), 0.0).astype(np.float32)
    return rgbe[..., :3].astype(np.float32) * f[..., None]


def read_hdr(path):
    """float32[h, w, 3] linear RGB of a Radiance .hdr file, as stb_image's stbi_loadf
    decodes one: a "#?RADIANCE" or "#?RGBE" signature, header lines up to an empty one
    among which FORMAT=32-bit_rle_rgbe must appear, the resolution line "-Y h +X w"
    (the only orientation read), then h scanlines. Images narrower than 8 or 32768 and
    wider are flat RGBE; otherwise each scanline starts 2, 2, width (16 bits) and holds
    the four byte planes in runs (count > 128: count - 128 copies of one byte, else
    count literal bytes). A scanline without that start switches to flat RGBE from the
    first pixel of the image on, as stb_image does. Channel = byte * 2^(e - 136)."""
    with open(path, "rb") as f:
        data = f.read()
    off = 0

    def line():
        nonlocal off
        end = data.find(b"\n", off)
        if end < 0:
            end = len(data)
        s = data[off:end]
        off = end + 1
        return s.decode("latin-1")

    if line() not in ("#?RADIANCE", "#?RGBE"):
        raise ValueError(f"{path}: not a Radiance HDR file")
    valid = False
    while True:
        if off >= len(data):
            raise ValueError(f"{path}: header without end")
        t = line()
        if t == "":
            break
        valid |= t == "FORMAT=32-bit_rle_rgbe"
    if not valid:
        raise ValueError(f"{path}: unsupported format")
    parts = line().split()
    if len(parts) != 4 or parts[0] != "-Y" or parts[2] != "+X":
        raise ValueError(f"{path}: unsupported orientation")
    h, w = int(parts[1]), int(parts[3])
    if h < 1 or w < 1:
        raise ValueError(f"{path}: bad size")
    buf = np.frombuffer(data, np.uint8, len(data) - off, off)
    pos = 0

    def flat(first_pixel, p0):
        need = 4 * (w * h - first_pixel)
        if p0 + need > len(buf):
            raise ValueError(f"{path}: truncated pixel data")
        return buf[p0:p0 + need].reshape(-1, 4)

    out = np.zeros((h * w, 4), np.uint8)
    if w < 8 or w >= 32768:
        out[:] = flat(0, 0)
        return _rgbe_to_float(out).reshape(h, w, 3)
    for j in range(h):
        if pos + 4 > len(buf):
            raise ValueError(f"{path}: truncated scanline {j}")
        c1, c2, ln = int(buf[pos]), int(buf[pos + 1]), int(buf[pos + 2])
        if c1 != 2 or c2 != 2 or (ln & 0x80):
            out[0] = buf[pos:pos + 4]
            out[1:] = flat(1, pos + 4)
            break
        if (ln << 8 | int(buf[pos + 3])) != w:
            raise ValueError(f"{path}: invalid decoded scanline length")
        pos += 4
        row = np.empty((4, w), np.uint8)
        for k in range(4):
            i = 0
            while i < w:
                if pos >= len(buf):
                    raise ValueError(f"{path}: truncated run data")
                count = int(buf[pos])
                pos += 1
                if count > 128:
                    count -= 128
                    if count > w - i or pos >= len(buf):
                        raise ValueError(f"{path}: bad RLE data")
                    row[k, i:i + count] = buf[pos]
                    pos += 1
                else:
                    if count > w - i or pos + count > len(buf):
                        raise ValueError(f"{path}: bad RLE data")
                    row[k, i:i + count] = buf[pos:pos + count]
                    pos += count
                i += count
        out[j * w:(j + 1) * w] = row.T
    return _rgbe_to_float(out).reshape(h, w, 3)


def float_to_rgbe(rgb):
    """float [..., 3] -> RGBE bytes [..., 4] (shared exponent of the largest channel,
    mantissas truncated: v = m * 2^e with m in [0.5, 1), byte = c * m * 256 / v)."""
    rgb = np.asarray(rgb, np.float32)
    v = rgb.max(axis=-1)
    m, e = np.frexp(v)
    ok = v >= np.float32(1e-32)
    scale = np.where(ok, m * np.float32(256.0) / np.where(ok, v, 1), 0).astype(np.float32)
    out = np.zeros(rgb.shape[:-1] + (4,), np.uint8)
    out[..., :3] = np.where(ok[..., None], (rgb * scale[..., None]).astype(np.int64), 0).clip(0, 255)
    out[..., 3] = np.where(ok, e + 128, 0)
    return out


def write_hdr(path, rgb, rle=True):
    """Write float [h, w, 3] as a Radiance .hdr file (header, "-Y h +X w", run-length
    scanlines when rle and 8 <= w < 32768, flat RGBE otherwise)."""
    rgb = np.asarray(rgb, np.float32)
    h, w, _ = rgb.shape
    px = float_to_rgbe(rgb).reshape(h, w, 4)
    parts = [f"#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n-Y {h} +X {w}\n".encode()]
    if not rle or w < 8 or w >= 32768:
        parts.append(px.tobytes())
    else:
        for j in range(h):
            parts.append(bytes([2, 2, w >> 8, w & 255]))
            for k in range(4):
                plane = px[j, :, k].tobytes()
                i = 0
                while i < w:
                    r = 1
                    while i + r < w and r < 127 and plane[i + r] == plane[i]:
                        r += 1
                    if r >= 3:
                        parts.append(bytes([128 + r, plane[i]]))
                        i += r
                        continue
                    s = i                      # literal block up to the next run of 3
                    while i < w and i - s < 128:
                        if i + 2 < w and plane[i] == plane[i + 1] == plane[i + 2]:
                            break
                        i += 1
                    parts.append(bytes([i - s]) + plane[s:i])
    with open(path, "wb") as f:
        f.write(b"".join(parts))


def _sky_directions(h, w):
    """Per texel of a w x h sky image, LoadSky's direction (cos p cos t, sin p, cos p sin t)
    with t = (x - w/2) / w * 2 pi, p = -(y - h/2) / h * pi, in binary32 (cos and sin
    correctly rounded)."""
    f = np.float32
    x = np.arange(w, dtype=f)[None, :]
    y = np.arange(h, dtype=f)[:, None]
    fw, fh, pi = f(w), f(h), f(3.14159265358979323846264)
    t = ((x - f(0.5) * fw) / fw * f(2)) * pi
    p = (-(y - f(0.5) * fh) / fh) * pi
    ct, st = np.cos(t.astype(np.float64)).astype(f), np.sin(t.astype(np.float64)).astype(f)
    cp, sp = np.cos(p.astype(np.float64)).astype(f), np.sin(p.astype(np.float64)).astype(f)
    return cp * ct, np.broadcast_to(sp, (h, w)), cp * st


def sky_texture(rgb, scale=1.5, artificial_sun=True, debug_lights=False):
    """World::LoadSky's texture (world.cpp:803-870) from decoded HDR pixels
    float[h, w, 3]: optionally the debug-light marks (red 10 where -D.x > 0.97, else green
    10 where -D.z > 0.97), then the artificial sun (rgb 24, 24, 18 where D . L > 0.999,
    L = normalize(2, 1.5, 3); on by default, as Game::artificialSun), then
    scale * (r, g, b, 1) per texel: the float32[h, w, 4] texture of vxr_view_set_sky.
    LoadSky's checkerboard option is not provided: on its first row the reference
    divides by a zero D.y."""
    px = np.array(rgb, np.float32)
    h, w, _ = px.shape
    f = np.float32
    if debug_lights or artificial_sun:
        dx, dy, dz = _sky_directions(h, w)
        if debug_lights:
            red = -dx > f(0.97)
            green = ~red & (-dz > f(0.97))
            px[red] = (10, 0, 0)
            px[green] = (0, 10, 0)
        if artificial_sun:
            L = np.array([2.0, 1.5, 3.0], f)
            L = L * (f(1.0) / np.sqrt(np.float32((L[0] * L[0] + L[1] * L[1]) + L[2] * L[2])))
            sun = ((dx * L[0] + dy * L[1]) + dz * L[2]) > f(0.999)
            px[sun] = (24, 24, 18)
    return (np.concatenate([px, np.ones((h, w, 1), f)], axis=2) * f(scale)).astype(f)


def load_sky(view, path, blue_noise, scale=1.5, light_scale=2.0, artificial_sun=True, seed=0x12345678):
    """World::LoadSky + the sky fields of World::Render's parameters (world.cpp:803-870,
    2185-2189) for one view: decode the .hdr file, build LoadSky's texture (scale 1.5 and
    the artificial sun by default, as Game::skyDomeScale / Game::artificialSun), integrate
    its sky lights (UpdateSkylights, vxr_sky_lights with `seed`) and turn the view's sky
    dome on with skyLightScale = light_scale (Game::skyDomeLightScale, 2.0) and the
    blue-noise tables `blue_noise` (uint32[327680]). Returns the texture."""
    from .vxr import sky_lights
    tex = sky_texture(read_hdr(path), scale=scale, artificial_sun=artificial_sun)
    view.set_sky(tex, sky_lights(tex, seed), light_scale, blue_noise)
    return tex


def _pixel_sum(per_pixel):
    """Sequential double accumulation in pixel order (the reference's `total +=` loop;
    numpy's sum would add pairwise)."""
    return float(np.cumsum(per_pixel.astype(np.float64))[-1]) if per_pixel.size else 0.0


def frame_mse(gt, img):
    """CalculateMSE of the reference's frame-comparison tool (mse.cpp:33-48) for two
    float[N, 4] frames: per pixel the squared differences of r, g, b in float, summed in
    float, accumulated in double, divided by 3N, returned as a float."""
    g = np.asarray(gt, np.float32).reshape(-1, 4)[:, :3]
    d = np.asarray(img, np.float32).reshape(-1, 4)[:, :3]
    y = (g - d) * (g - d)
    return np.float32(_pixel_sum((y[:, 0] + y[:, 1]) + y[:, 2]) / (len(y) * 3))


def frame_mae(gt, img):
    """CalculateRMAE of the same tool (mse.cpp:50-63): the mean absolute difference of r,
    g, b, computed like frame_mse (no normalisation despite the name)."""
    g = np.asarray(gt, np.float32).reshape(-1, 4)[:, :3]
    d = np.asarray(img, np.float32).reshape(-1, 4)[:, :3]
    y = np.abs(g - d)
    return np.float32(_pixel_sum((y[:, 0] + y[:, 1]) + y[:, 2]) / (len(y) * 3))


def frame_energy(img, width, height):
    """energyInRaster (mse.cpp:19-31): the mean over pixels of (r + g + b) / 3 in float,
    accumulated in double, divided by the width, then by the height."""
    v = np.asarray(img, np.float32).reshape(-1, 4)
    return np.float32(_pixel_sum(((v[:, 0] + v[:, 1]) + v[:, 2]) / np.float32(3.0)) / width / height)


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
