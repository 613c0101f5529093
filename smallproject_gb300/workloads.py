"""Benchmark workloads built on the C ABI (no reference counterpart: the reference's
demo scenes are hand-built games).

config 2: eight independent scenes and views rendered as one batch per frame. From one
seed: world sizes drawn from {256^3, 512^3, 1024^3}, emitter counts log-uniform in
[16, 65536], resolutions from {640x360, 1280x720, 1920x1080}, point or area lights at
random; each view follows its own seeded Catmull-Rom camera path.

config 4 (stress, plain method): four 3840x2160 views of one 1024^3 world (fBm of 6
octaves with caves, 1,048,576 emitters in a glowing layer plus 10% scattered), area
lights, each view on its own camera path.
"""
import numpy as np

from . import vxr as _v

RESOLUTIONS = ((640, 360), (1280, 720), (1920, 1080))
EXTENTS = (256, 512, 1024)


def config2_specs(seed=3, views=8, scale=1.0):
    """Scene / view specifications of config 2 (scale < 1 shrinks resolutions for tests)."""
    rng = np.random.default_rng(seed)
    specs = []
    for i in range(views):
        ext = int(rng.choice(EXTENTS))
        ne = int(round(float(np.exp(rng.uniform(np.log(16.0), np.log(65536.0))))))
        w, h = RESOLUTIONS[int(rng.integers(len(RESOLUTIONS)))]
        point = bool(rng.integers(2))
        specs.append({"extent": ext, "emitters": ne, "width": max(16, int(w * scale)), "height": max(16, int(h * scale)),
                      "light_model": "point" if point else "area", "scene_seed": seed * 1000 + i,
                      "path_seed": seed * 100 + i})
    return specs


def build_config2(seed=3, views=8, scale=1.0):
    """(worlds, views, scene descs, specs) of config 2; views are created on the current device."""
    worlds, vlist, descs = [], [], []
    specs = config2_specs(seed, views, scale)
    for sp in specs:
        d = _v.scene_preset(1, extent=sp["extent"], seed=sp["scene_seed"], emitters=sp["emitters"],
                            emitter_mode=1)
        w = _v.World()
        w.generate(d)
        model = _v.LIGHTS_POINT if sp["light_model"] == "point" else _v.LIGHTS_AREA
        v = _v.View(w, _v.view_desc(sp["width"], sp["height"], model, rng_seed=sp["scene_seed"]))
        worlds.append(w)
        vlist.append(v)
        descs.append(d)
    return worlds, vlist, descs, specs


def config2_cameras(descs, specs, frames=60):
    """Camera function per view: f -> (pos, target) on the view's own path."""
    return [lambda f, d=d, s=s: _v.camera_path(d, s["path_seed"], f % frames, frames) for d, s in zip(descs, specs)]


def build_config4(views=4, scale=1.0):
    """(world, views, scene desc, path seeds) of config 4 (the plain method)."""
    d = _v.scene_preset(4)
    w = _v.World()
    w.generate(d)
    W, H = max(16, int(3840 * scale)), max(16, int(2160 * scale))
    vlist = [_v.View(w, _v.view_desc(W, H, _v.LIGHTS_AREA, rng_seed=5000 + i)) for i in range(views)]
    return w, vlist, d, [500 + i for i in range(views)]
