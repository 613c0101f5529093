"""Host side of the sky dome: Radiance .hdr files (scene_io.read_hdr / write_hdr) against
the reference's own stb_image (lib/stb_image.h, compiled by oracle/ref_build.py where
the reference checkout is present), LoadSky's texture (scene_io.sky_texture) and
UpdateSkylights (vxr_sky_lights)."""
import struct

import numpy as np
import pytest

from oracle import binding as ob
from smallproject_gb300 import scene_io as io

needs_stb = pytest.mark.skipif(ob.load_stb() is None, reason="the reference's stb_image is not present")


def _sky_image(h, w, seed):
    rng = np.random.default_rng(seed)
    img = (rng.random((h, w, 3)) * np.array([1.0, 20.0, 0.003])).astype(np.float32)
    img[1, 3:200] = (0.25, 4.0, 1e-3)          # long runs (longer than 127 where w allows)
    img[2] = 0.0                               # black: exponent 0
    return img


def _rle_scanline_file(path, w, planes):
    with open(path, "wb") as f:
        f.write(f"#?RGBE\nGAMMA=1\nFORMAT=32-bit_rle_rgbe\n\n-Y 1 +X {w}\n".encode())
        f.write(bytes([2, 2, w >> 8, w & 255]) + b"".join(planes))


@needs_stb
@pytest.mark.parametrize("h,w,rle", [(7, 300, True), (5, 64, False), (3, 5, True), (4, 8, True)])
def test_read_hdr_matches_stb_image(tmp_path, h, w, rle):
    """Files from our writer and from stbi_write_hdr decode identically through read_hdr
    and the reference's stbi_loadf (flat, run-length, narrow images)."""
    img = _sky_image(h, w, h * w)
    for name, write in (("ours.hdr", lambda p: io.write_hdr(p, img, rle=rle)), ("stb.hdr", lambda p: ob.stb_write_hdr(p, img))):
        p = str(tmp_path / name)
        write(p)
        want = ob.stb_loadf(p)
        got = io.read_hdr(p)
        assert want is not None and want.shape == (h, w, 3)
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), name
    q = io._rgbe_to_float(io.float_to_rgbe(img))
    assert np.array_equal(io.read_hdr(str(tmp_path / "ours.hdr")), q)


@needs_stb
def test_read_hdr_hand_made_runs_and_fallback(tmp_path):
    """Byte-level files: runs, literals and a scanline without the 2, 2 marker (decoded
    flat from the first pixel on, as stb_image does), against stbi_loadf and by value."""
    p = str(tmp_path / "runs.hdr")
    _rle_scanline_file(p, 8, [bytes([136, 5]), bytes([8]) + bytes(range(8)),
                              bytes([130, 1, 6, 1, 2, 3, 4, 5, 6]), bytes([136, 129])])
    got = io.read_hdr(p)
    assert np.array_equal(got, ob.stb_loadf(p))
    f = np.float32(2.0 ** (129 - 136))
    assert got[0, :, 0].tolist() == [5 * f] * 8 and got[0, :, 1].tolist() == [i * f for i in range(8)]
    assert got[0, :, 2].tolist() == [f, f, 1 * f, 2 * f, 3 * f, 4 * f, 5 * f, 6 * f]
    flat = str(tmp_path / "flat.hdr")
    px = np.arange(8 * 2 * 4, dtype=np.uint8).reshape(16, 4) | np.uint8(0x80)
    with open(flat, "wb") as fh:
        fh.write(b"#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n-Y 2 +X 8\n" + px.tobytes())
    assert np.array_equal(io.read_hdr(flat), ob.stb_loadf(flat))


@pytest.mark.parametrize("case", ["signature", "format", "orientation", "length", "truncated", "bad_run"])
def test_read_hdr_errors(tmp_path, case):
    p = str(tmp_path / "bad.hdr")
    head = b"#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n-Y 1 +X 8\n"
    body = {
        "signature": b"#?RADIANCX\nFORMAT=32-bit_rle_rgbe\n\n-Y 1 +X 8\n" + bytes(32),
        "format": b"#?RADIANCE\nFORMAT=32-bit_rle_xyze\n\n-Y 1 +X 8\n" + bytes(32),
        "orientation": b"#?RADIANCE\nFORMAT=32-bit_rle_rgbe\n\n+Y 1 +X 8\n" + bytes(32),
        "length": head + bytes([2, 2, 0, 9]) + bytes(40),
        "truncated": head + bytes([2, 2, 0, 8, 136, 1]),
        "bad_run": head + bytes([2, 2, 0, 8, 137, 1]) + bytes(40),
    }[case]
    with open(p, "wb") as f:
        f.write(body)
    with pytest.raises(ValueError):
        io.read_hdr(p)


def test_sky_texture_scale_sun_and_debug_lights():
    rgb = np.full((64, 128, 3), 0.5, np.float32)
    t = io.sky_texture(rgb, scale=2.0)
    assert t.dtype == np.float32 and t.shape == (64, 128, 4)
    assert (t[..., 3] == 2.0).all()
    sun = t[..., 0] == 48.0
    assert 1 <= sun.sum() <= 8 and (t[sun][:, 2] == 36.0).all()
    assert ((t[~sun][:, :3]) == 1.0).all()
    dx, dy, dz = io._sky_directions(64, 128)
    L = np.array([2.0, 1.5, 3.0]) / np.linalg.norm([2.0, 1.5, 3.0])
    assert (dx * L[0] + dy * L[1] + dz * L[2])[sun].min() > 0.998
    d = io.sky_texture(rgb, scale=1.0, artificial_sun=False, debug_lights=True)
    assert (d[..., 0] == 10).sum() > 0 and (d[..., 1] == 10).sum() > 0
    assert ((d[..., 0] == 10) & (d[..., 1] == 10)).sum() == 0
    plain = io.sky_texture(rgb, scale=1.0, artificial_sun=False)
    assert (plain[..., :3] == 0.5).all()


def test_sky_lights_constant_and_hemisphere(lib):
    """UpdateSkylights: a constant sky integrates to itself for every normal; a sky bright
    only above its horizon (z-up: theta < pi/2, the upper half of the rows) gives the
    +z normal (skyLight[3], shading's +y) nearly all of it, -z nearly none, the side
    normals half."""
    h, w = 32, 64
    const = np.concatenate([np.full((h, w, 3), 0.75, np.float32), np.ones((h, w, 1), np.float32)], axis=2)
    l = lib.sky_lights(const)
    assert l.shape == (6, 4) and np.allclose(l[:, :3], 0.75, rtol=1e-5) and (l[:, 3] == 0).all()
    half = const.copy()
    half[h // 2:, :, :3] = 0.0
    half[: h // 2, :, :3] = 1.0
    l = lib.sky_lights(half)[:, 0]
    assert l[3] > 0.9 and l[2] < 0.1
    assert all(0.4 < l[i] < 0.6 for i in (0, 1, 4, 5))
    assert np.array_equal(lib.sky_lights(half, seed=5), lib.sky_lights(half, seed=5))
    assert not np.array_equal(lib.sky_lights(half, seed=5), lib.sky_lights(half, seed=6))


def test_sky_inputs_are_deterministic():
    """The fixture's synthetic inputs are exact (hash-built), so both hosts build the
    same bits: spot values."""
    import os
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
    import sky_inputs
    t, bn = sky_inputs.sky_texture(), sky_inputs.blue_noise()
    assert t.shape == (32, 64, 4) and bn.shape == (327680,) and bn.max() <= 255
    assert struct.pack("<4f", *t[0, 0]) == struct.pack("<4f", *t[0, 0].astype(np.float64).astype(np.float32))
    assert (t[..., 3] == 1.5).all() and (t[..., :3] < 3.0).all()
