"""Seeded sky-dome inputs of the sky parity fixture (tests/golden/config0_sky_48x32.npz),
shared by tests/golden/make_golden.py and tests/test_gpu_sky.py.

The reference's sky is an HDR file that is not available (assets/sky_15.hdr), so the
texture, the blue-noise tables and the sky lights here are synthetic: integer hashes
turned into floats with exact arithmetic, so that x86 and Arm hosts build the same bits.
The scene is the config-0 scene plus a translucent panel (alpha 8) in front of the
fixture's cameras, so that sky seen through translucent voxels is exercised as well as
the background and the sky-light rays.
"""
import numpy as np

SKY_W, SKY_H = 64, 32
SKY_SCALE = 1.5             # World::LoadSky brightness scale (skyDomeScale)
LIGHT_SCALE = 0.5           # skyLightScale (mygame.cpp:46)
# skyLight: one colour per axis normal (exact binary32 values)
SKY_LIGHT = np.array([[0.75, 0.5, 0.25, 0.0], [1.0, 0.875, 0.5, 0.0], [0.125, 0.25, 0.375, 0.0],
                      [2.0, 1.75, 1.5, 0.0], [0.5, 0.625, 0.75, 0.0], [0.25, 0.125, 1.0, 0.0]], np.float32)
PANEL = (100, 110, 70, 156, 150, 71)   # x1, y1, z1, x2, y2, z2 (half-open box)
PANEL_VOXEL = 0x85AC                    # alpha 8, rgb 5, 10, 12


def _hash(i):
    """Wang's 32-bit integer hash, elementwise."""
    i = np.asarray(i, np.uint32)
    i = (i ^ np.uint32(61)) ^ (i >> np.uint32(16))
    i = i * np.uint32(9)
    i = i ^ (i >> np.uint32(4))
    i = i * np.uint32(0x27D4EB2D)
    return i ^ (i >> np.uint32(15))


def sky_texture():
    """float32[SKY_H, SKY_W, 4]: SKY_SCALE * (r, g, b, 1) with r, g, b in [0, 2)."""
    v = (_hash(np.arange(SKY_W * SKY_H * 3, dtype=np.uint32) + np.uint32(1000)) & np.uint32(0xFFFF))
    rgb = v.astype(np.float32).reshape(SKY_H, SKY_W, 3) * np.float32(2.0 / 65536.0)
    return np.concatenate([rgb, np.ones((SKY_H, SKY_W, 1), np.float32)], axis=2) * np.float32(SKY_SCALE)


def blue_noise():
    """uint32[327680] in the reference's layout, 8-bit entries: sequence, scrambling,
    ranking."""
    out = np.zeros(327680, np.uint32)
    out[:65536] = _hash(np.arange(65536, dtype=np.uint32) + np.uint32(7)) & np.uint32(255)
    out[65536:196608] = _hash(np.arange(131072, dtype=np.uint32) + np.uint32(70001)) & np.uint32(255)
    out[196608:] = _hash(np.arange(131072, dtype=np.uint32) + np.uint32(900001)) & np.uint32(255)
    return out


def add_panel(world):
    """The translucent panel, set voxel by voxel (vxr_world_box)."""
    world.box(*PANEL, PANEL_VOXEL)
