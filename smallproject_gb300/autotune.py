"""Launch autotuner for the render path (no reference counterpart: the reference's
work-group size is fixed, template/template.cpp:1700-1754).

Tunes the launch parameters of vxr_tuning - pixel-stage tile shape, persistent tile
queue on/off, shadow-tracer refill threshold and burst length, blocks per SM of the
hit-list kernels, register cap of the shadow tracer and candidate kernels - per configuration, by timing whole frames on the GPU, and caches the
winner in a JSON file keyed by device, resolution, light model, candidate count and the
world's size class. Every setting renders the same bits (the kernels' per-pixel
arithmetic does not depend on them), so tuning changes speed only.

Brick cache: the DDA reads bricks through the L1 data cache; the kernels use no shared
memory for it (at most 4 bytes per block), so the L1/shared split already gives the
whole array to L1 and there is no software brick cache to size.

Search: coordinate descent from the library defaults, `rounds` passes over the
parameters in a fixed order, each candidate timed over `frames` frames (after one
warm-up frame) on a scratch view of the same world and description, so the caller's
view keeps its own history.
"""
import json
import math
import os

from . import vxr as _v

SPACE = [
    ("tile", [(16, 8), (32, 4), (8, 16), (32, 8), (16, 16), (64, 2)]),
    ("persistent", [0, 1]),
    ("shadow_refill", [4, 8, 16, 24]),
    ("shadow_burst", [2, 4, 8, 16]),
    ("list_blocks_per_sm", [4, 8, 16, 32]),
    ("occupancy", [0, 1]),
    ("shadow_schedule", [0, 1]),
    ("shadow_early_out", [0, 1]),
    ("brick_cache", [0, 256, 1024]),
]


def default_cache_path():
    return os.environ.get("VXR_TUNE_CACHE", os.path.join(os.path.expanduser("~"), ".cache", "vxr_tuning.json"))


def _world_class(world):
    """(log2 emitters, log2 bricks) of the world, read without copying its arrays."""
    lib = _v.load()
    g = _v.C.POINTER(_v.C.c_uint32)()
    b = _v.C.POINTER(_v.C.c_uint32)()
    nb = _v.C.c_uint32()
    lp = _v.C.POINTER(_v.Light)()
    nl = _v.C.c_uint32()
    _v.check(lib.vxr_world_arrays(world.h, _v.C.byref(g), _v.C.byref(b), _v.C.byref(nb), _v.C.byref(lp),
                                  _v.C.byref(nl)))
    return int(math.log2(max(1, nl.value))), int(math.log2(max(1, nb.value)))


def config_key(world, desc):
    """Cache key: device, resolution, light model, candidates, log2 lights, log2 bricks."""
    name, sms, cc = _v.device_info()
    lg, bg = _world_class(world)
    model = "point" if desc.light_model == _v.LIGHTS_POINT else "area"
    return f"{name}|sm{cc[0]}{cc[1]}x{sms}|{desc.width}x{desc.height}|{model}|c{desc.num_candidates}|l{lg}|b{bg}"


def _to_tuning(d):
    t = _v.tuning()
    t.tile_x, t.tile_y = d["tile"]
    for k in ("persistent", "shadow_refill", "shadow_burst", "list_blocks_per_sm", "occupancy", "shadow_schedule",
              "shadow_early_out", "brick_cache"):
        setattr(t, k, d.get(k, getattr(t, k)))
    return t


def _from_tuning(t):
    return {"tile": (t.tile_x, t.tile_y), "persistent": t.persistent, "shadow_refill": t.shadow_refill,
            "shadow_burst": t.shadow_burst, "list_blocks_per_sm": t.list_blocks_per_sm, "occupancy": t.occupancy,
            "shadow_schedule": t.shadow_schedule, "shadow_early_out": t.shadow_early_out, "brick_cache": t.brick_cache}


def time_view(view, t, cams, frames, start=0):
    """GPU ms per frame of `view` rendered with tuning `t` along camera function cams(f)."""
    view.set_tuning(t)
    pos, tgt = cams(start)
    view.lookat(pos, tgt)
    view.render()
    view.wait()
    view.timer_begin()
    for f in range(frames):
        pos, tgt = cams(start + 1 + f)
        view.lookat(pos, tgt)
        view.render()
    ms = view.timer_end()
    view.wait()
    return ms / frames


def load_cache(path=None):
    path = path or default_cache_path()
    try:
        with open(path) as fh:
            return json.load(fh)
    except (OSError, ValueError):
        return {}


def save_cache(cache, path=None):
    path = path or default_cache_path()
    os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
    tmp = path + ".tmp"
    with open(tmp, "w") as fh:
        json.dump(cache, fh, indent=1, sort_keys=True)
    os.replace(tmp, path)


def autotune(world, desc, cams, frames=6, rounds=2, cache_path=None, force=False):
    """Best tuning for (world, desc) along camera path cams(f) -> (pos, target).

    Returns (vxr.Tuning, report dict). Reads and updates the JSON cache unless force."""
    key = config_key(world, desc)
    cache = load_cache(cache_path)
    if not force and key in cache:
        return _to_tuning(cache[key]["tuning"]), cache[key]
    scratch = _v.View(world, desc)
    try:
        best = _from_tuning(_v.tuning())
        timings = {}

        def measure(cand):
            k = json.dumps(cand, sort_keys=True)
            if k not in timings:
                timings[k] = time_view(scratch, _to_tuning(cand), cams, frames, start=len(timings) * (frames + 1))
            return timings[k]

        best_ms = measure(best)
        for _ in range(rounds):
            changed = False
            for name, values in SPACE:
                for val in values:
                    cand = dict(best)
                    cand[name] = val
                    ms = measure(cand)
                    if ms < best_ms * 0.995:
                        best, best_ms, changed = cand, ms, True
            if not changed:
                break
        default_ms = measure(_from_tuning(_v.tuning()))
    finally:
        scratch.close()
    report = {"tuning": best, "ms": best_ms, "default_ms": default_ms, "evaluated": len(timings), "frames": frames}
    cache[key] = report
    save_cache(cache, cache_path)
    return _to_tuning(best), report


def apply_cached(view, world, cache_path=None):
    """Set the cached tuning of this configuration on `view`; False when none is cached."""
    cache = load_cache(cache_path)
    key = config_key(world, view.desc)
    if key not in cache:
        return False
    view.set_tuning(_to_tuning(cache[key]["tuning"]))
    return True


def autotune_batch(batch, cams_list, frames=4, rounds=1):
    """Tune a vxr_batch in place (its views render the timed frames). cams_list[i](f) is
    view i's camera. Returns (vxr.Tuning, report dict); the batch keeps the winner."""
    step = [0]

    def measure(cand):
        batch.set_tuning(_to_tuning(cand))
        total = 0.0
        for f in range(frames + 1):
            for v, cams in zip(batch.views, cams_list):
                pos, tgt = cams(step[0])
                v.lookat(pos, tgt)
            step[0] += 1
            batch.render()
            ms = batch.wait()
            if f:
                total += ms
        return total / frames

    best = _from_tuning(_v.tuning())
    best["tile"] = tuple(best["tile"])
    best_ms = measure(best)
    evaluated = 1
    for _ in range(rounds):
        changed = False
        for name, values in SPACE:
            for val in values:
                if best[name] == val:
                    continue
                cand = dict(best)
                cand[name] = val
                ms = measure(cand)
                evaluated += 1
                if ms < best_ms * 0.995:
                    best, best_ms, changed = cand, ms, True
        if not changed:
            break
    batch.set_tuning(_to_tuning(best))
    return _to_tuning(best), {"tuning": best, "ms": best_ms, "evaluated": evaluated, "frames": frames}
