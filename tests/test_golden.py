"""Committed golden vectors from the reference's own kernel source (tests/golden,
made by tests/golden/make_golden.py): the C oracle on the CPU and the CUDA path on
the GPU must reproduce every stage output bit for bit."""
import glob
import os

import numpy as np
import pytest

from conftest import ROOT, assert_records_equal
from oracle import binding as ob

# the render-path fixtures (the path tracer and the sky dome have their own GPU tests,
# test_gpu_pt.py and test_gpu_sky.py: the C oracle restates neither)
FIXTURES = sorted(f for f in glob.glob(os.path.join(ROOT, "tests", "golden", "*.npz"))
                  if "_pt_" not in f and "_sky_" not in f)


def _load(path):
    return dict(np.load(path))


def _consts(raw, cls):
    k = cls()
    import ctypes as C
    C.memmove(C.byref(k), raw.tobytes(), C.sizeof(k))
    return k


def _check_scene(lib, scene0, fx):
    assert tuple(int(v) for v in fx["checksum"]) == scene0[0].checksum(), "scene generator drifted from the fixture"


@pytest.mark.parametrize("path", FIXTURES, ids=[os.path.basename(p) for p in FIXTURES])
def test_oracle_reproduces_golden(lib, scene0, world0_arrays, path):
    fx = _load(path)
    _check_scene(lib, scene0, fx)
    W, H, point, F = int(fx["W"]), int(fx["H"]), bool(fx["point"]), int(fx["frames"])
    port = ob.Renderer("port", world0_arrays, W, H, point)
    for f in range(F):
        k = _consts(fx[f"consts{f}"], ob.FrameConsts)
        port.frame_start()
        for s in range(1, 6):
            port.stage(k, s)
            if s == 1:
                assert_records_equal("gbuffer", port.gbuffer(0)[["voxel", "dist", "side"]],
                                     fx[f"gbuffer{f}"][["voxel", "dist", "side"]], f"frame {f}")
            elif s == 2:
                assert_records_equal("candidates", port.reservoirs(0), fx[f"candidates{f}"], f"frame {f}")
                assert_records_equal("seed", port.gbuffer(0)["seed"], fx[f"seed_cand{f}"], f"frame {f}")
            elif s == 3:
                assert_records_equal("seed", port.gbuffer(0)["seed"], fx[f"seed_spatial{f}"], f"frame {f}")
            elif s == 4:
                assert_records_equal("spatial", port.reservoirs(1), fx[f"spatial{f}"], f"frame {f}")
                assert_records_equal("frame", port.image(0), fx[f"frame{f}"], f"frame {f}")
            else:
                assert_records_equal("accum", port.image(1), fx[f"accum{f}"], f"frame {f}")
    port.close()


@pytest.mark.gpu
@pytest.mark.parametrize("path", FIXTURES, ids=[os.path.basename(p) for p in FIXTURES])
def test_cuda_reproduces_golden(lib, cuda_device, scene0, path):
    fx = _load(path)
    _check_scene(lib, scene0, fx)
    W, H, point, F = int(fx["W"]), int(fx["H"]), bool(fx["point"]), int(fx["frames"])
    view = lib.View(scene0[0], lib.view_desc(W, H, lib.LIGHTS_POINT if point else lib.LIGHTS_AREA, accumulate=1))
    for f in range(F):
        cam = fx[f"camera{f}"]
        view.lookat(cam[:3], cam[3:])
        k = view.begin_frame()
        assert bytes(k) == fx[f"consts{f}"].tobytes(), "camera constants differ from the reference driver's"
        for s in range(1, 6):
            view.stage(s)
            if s == 1:
                assert_records_equal("gbuffer", view.read_gbuffer(0)[["voxel", "dist", "side"]],
                                     fx[f"gbuffer{f}"][["voxel", "dist", "side"]], f"frame {f}")
            elif s == 2:
                assert_records_equal("candidates", view.read_reservoirs(0), fx[f"candidates{f}"], f"frame {f}")
                assert_records_equal("seed", view.read_gbuffer(0)["seed"], fx[f"seed_cand{f}"], f"frame {f}")
            elif s == 3:
                assert_records_equal("seed", view.read_gbuffer(0)["seed"], fx[f"seed_spatial{f}"], f"frame {f}")
            elif s == 4:
                assert_records_equal("spatial", view.read_reservoirs(1), fx[f"spatial{f}"], f"frame {f}")
                assert_records_equal("frame", view.read_frame(), fx[f"frame{f}"], f"frame {f}")
            else:
                assert_records_equal("accum", view.read_accum(), fx[f"accum{f}"], f"frame {f}")
        view.end_frame()
        view.wait()
    view.close()
