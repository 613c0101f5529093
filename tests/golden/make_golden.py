"""Generate tests/golden/*.npz from the reference oracle (the reference's own
render-path kernel source compiled for the CPU, oracle/_ref).

Each fixture: the config-0 scene (regenerated by the library; its canonical checksum
is stored and asserted), a small frame size, a few frames with a moving camera, and
for every frame the frame constants plus every stage output of the reference:
G-buffer after renderAlbedo, reservoirs after perPixelInitialSampling and after
perPixelSpatialResampling (as left by renderRIS), the shaded frame and the
accumulator. The path-tracer fixture holds, per frame, the frame of the reference's
ground-truth mode (renderPathTracer, GFXEXP) and the accumulator after it. The sky
fixture renders the config-0 scene with a translucent panel and the sky dome on
(synthetic sky inputs of tests/golden/sky_inputs.py) and holds, per frame, the shaded
frame and the accumulator.

Usage: python tests/golden/make_golden.py [fixture names]   (all by default; needs the
reference checkout or a previously generated oracle/_ref/vxref_gen.inc)
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

CASES = [
    # name, W, H, point, frames
    ("config0_area_48x32", 48, 32, False, 3),
    ("config0_point_48x32", 48, 32, True, 3),
]
# the path tracer's scene: config 0 with 4,096 emitters (seed 6, blob mode), so that
# hemisphere samples hit emitters in a useful share of pixels
PT_CASES = [("config0_pt_48x32", 48, 32, 8, dict(emitters=4096, emitter_mode=1, seed=6))]
SKY_CASES = [("config0_sky_48x32", 48, 32, 3, False), ("config0_sky_point_48x32", 48, 32, 3, True)]
KNOBS = dict(numberOfCandidates=32, numberOfMaxTemporalImportance=20, spatialRadius=30, spatialTaps=5,
             spatial=1, temporal=1, accumulate=1)


def camera(f):
    return (126.0 + 5.0 * f, 150.0 - 1.0 * f, 30.0 + 2.0 * f), (128.0, 100.0, 128.0)


def sky_camera(f):
    """Toward the horizon: background, the translucent panel and terrain in one view."""
    return (126.0 + 5.0 * f, 150.0 - 1.0 * f, 30.0 + 2.0 * f), (128.0, 140.0 - 10.0 * f, 230.0)


def main():
    import smallproject_gb300 as vx
    from oracle import binding as ob
    sys.path.insert(0, HERE)
    import sky_inputs
    if ob.load_ref() is None:
        sys.exit("reference oracle unavailable")
    w = vx.World()
    w.generate(vx.scene_preset(0))
    ck = w.checksum()
    g, b, l = w.arrays()
    arrays = ob.WorldArrays(g, b, l)
    only = set(sys.argv[1:])
    for name, W, H, point, F in CASES:
        if only and name not in only:
            continue
        ref = ob.Renderer("ref", arrays, W, H, point)
        cam = ob.CameraPath(W, H)
        out = {"checksum": np.array(ck, np.uint64), "W": W, "H": H, "point": int(point), "frames": F}
        for f in range(F):
            pos, tgt = camera(f)
            cam.lookat(pos, tgt)
            k = cam.begin(numberOfLights=len(l), **KNOBS)
            out[f"consts{f}"] = np.frombuffer(bytes(k), np.uint8)
            out[f"camera{f}"] = np.array(pos + tgt, np.float32)
            ref.frame_start()
            for s in range(1, 6):
                ref.stage(k, s)
                if s == 1:
                    out[f"gbuffer{f}"] = ref.gbuffer(0)
                elif s == 2:
                    out[f"candidates{f}"] = ref.reservoirs(0)
                    out[f"seed_cand{f}"] = ref.gbuffer(0)["seed"]
                elif s == 3:
                    out[f"seed_spatial{f}"] = ref.gbuffer(0)["seed"]
                elif s == 4:
                    out[f"spatial{f}"] = ref.reservoirs(1)
                    out[f"frame{f}"] = ref.image(0)
                else:
                    out[f"accum{f}"] = ref.image(1)
            cam.end()
        ref.close()
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
        print("wrote", name)
    for name, W, H, F, scene in PT_CASES:
        if only and name not in only:
            continue
        wp = vx.World()
        wp.generate(vx.scene_preset(0, **scene))
        gp, bp, lp = wp.arrays()
        ref = ob.Renderer("ref", ob.WorldArrays(gp, bp, lp), W, H, False)
        cam = ob.CameraPath(W, H)
        out = {"checksum": np.array(wp.checksum(), np.uint64), "W": W, "H": H, "frames": F,
               "scene": np.array([scene["emitters"], scene["emitter_mode"], scene["seed"]], np.uint32)}
        for f in range(F):
            pos, tgt = camera(f)
            cam.lookat(pos, tgt)
            k = cam.begin(numberOfLights=len(lp), **KNOBS)
            out[f"consts{f}"] = np.frombuffer(bytes(k), np.uint8)
            out[f"camera{f}"] = np.array(pos + tgt, np.float32)
            ref.frame_start()
            ref.stage(k, 6)
            out[f"frame{f}"] = ref.image(0)
            ref.stage(k, 5)
            out[f"accum{f}"] = ref.image(1)
            cam.end()
        ref.close()
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
        print("wrote", name)
    for name, W, H, F, point in SKY_CASES:
        if only and name not in only:
            continue
        ws = vx.World()
        ws.generate(vx.scene_preset(0))
        sky_inputs.add_panel(ws)
        gs, bs, ls = ws.arrays()
        ref = ob.Renderer("ref", ob.WorldArrays(gs, bs, ls), W, H, point)
        ref.set_sky(sky_inputs.sky_texture(), sky_inputs.SKY_LIGHT, sky_inputs.LIGHT_SCALE, sky_inputs.blue_noise())
        cam = ob.CameraPath(W, H)
        out = {"checksum": np.array(ws.checksum(), np.uint64), "W": W, "H": H, "frames": F, "point": int(point)}
        for f in range(F):
            pos, tgt = sky_camera(f)
            cam.lookat(pos, tgt)
            k = cam.begin(numberOfLights=len(ls), **KNOBS)
            out[f"consts{f}"] = np.frombuffer(bytes(k), np.uint8)
            out[f"camera{f}"] = np.array(pos + tgt, np.float32)
            ref.frame_start()
            for s in range(1, 6):
                ref.stage(k, s)
            out[f"gbuffer{f}"] = ref.gbuffer(0)
            out[f"frame{f}"] = ref.image(0)
            out[f"accum{f}"] = ref.image(1)
            cam.end()
        ref.close()
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
        print("wrote", name)


if __name__ == "__main__":
    main()
