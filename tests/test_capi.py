"""The C-ABI library: loads, exports every symbol include/vxr.h declares, and rejects
bad arguments with status codes (no GPU needed)."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from conftest import ROOT


def _declared():
    src = open(os.path.join(ROOT, "include", "vxr.h")).read()
    src = re.sub(r"/\*.*?\*/", " ", src, flags=re.S)
    return sorted(set(re.findall(r"\b(vxr_[a-z0-9_]+)\s*\(", src)) - {"vxr_world", "vxr_view"})


def test_library_exports_every_declared_symbol(lib):
    so = C.CDLL(lib.LIB_PATH)
    missing = [s for s in _declared() if not hasattr(so, s)]
    assert not missing, missing
    # and the Python binding covers them all
    assert set(_declared()) <= set(lib.exported_symbols()), set(_declared()) - set(lib.exported_symbols())


def test_struct_layouts_match_header(lib):
    from smallproject_gb300 import vxr as V
    assert C.sizeof(V.FrameConsts) == 44 * 4
    assert C.sizeof(V.ReservoirRec) == 48 and C.sizeof(V.GBufferRec) == 16 and C.sizeof(V.Light) == 12
    assert C.sizeof(V.SceneDesc) == 20 * 4 and C.sizeof(V.ViewDesc) == 13 * 4
    assert C.sizeof(V.ProposalDesc) == 13 * 4


def test_proposal_defaults_and_new_entry_points_check_arguments(lib):
    from smallproject_gb300 import vxr as V
    L = lib.load()
    d = V.ProposalDesc()
    assert L.vxr_proposal_default_desc(C.byref(d)) == 0
    assert (d.hidden, d.table_log2, d.res0, d.res1, d.batch, d.seed, d.inference, d.training, d.pixels_per_eval,
            d.training_lag) == (64, 16, 32, 128, 65536, 1, 0, 0, 1, 0)
    assert abs(d.epsilon - 0.1) < 1e-7 and abs(d.learning_rate - 1e-3) < 1e-9 and d.share_distance == 2.0
    t = C.c_uint64()
    n = C.c_uint32()
    img = (C.c_float * 4)()
    p3 = (C.c_float * 3)()
    assert L.vxr_view_render_to_host_async(None, p3, p3, img, C.byref(t)) == lib.vxr.VXR_E_INVALID
    assert L.vxr_view_image_wait(None, 0) == lib.vxr.VXR_E_INVALID
    assert L.vxr_view_proposal_rows(None, C.byref(n)) == lib.vxr.VXR_E_INVALID
    h = C.c_void_p()
    arr = (C.c_void_p * 1)(None)
    assert L.vxr_batch_create(arr, 1, 0, 0, 1 | (2 << 8), C.byref(h)) == lib.vxr.VXR_E_INVALID   # 2 chains, 1 view


def test_invalid_arguments_return_status(lib):
    L = lib.load()
    assert L.vxr_world_create(None) == lib.vxr.VXR_E_INVALID
    assert b"null" in L.vxr_last_error()
    w = lib.World()
    out = C.c_uint32()
    assert L.vxr_world_get(None, 0, 0, 0, C.byref(out)) == lib.vxr.VXR_E_INVALID
    d = lib.scene_preset(0)
    d.extent = 4
    with pytest.raises(lib.VxrError):
        w.generate(d)
    with pytest.raises(lib.VxrError):
        lib.scene_preset(9)
    bad = np.zeros(1, lib.LIGHT_DTYPE)
    bad["position"] = 1024 ** 3
    with pytest.raises(lib.VxrError):
        w.set_lights(bad)
    vd = lib.view_desc(0, 10)
    h = C.c_void_p()
    assert L.vxr_view_create(w.h, C.byref(vd), C.byref(h)) == lib.vxr.VXR_E_INVALID
    assert L.vxr_view_stage(None, 1) == lib.vxr.VXR_E_INVALID
    # batches and tuning: argument checks that need no device
    assert L.vxr_batch_create(None, 1, 0, 0, 0, C.byref(h)) == lib.vxr.VXR_E_INVALID
    arr = (C.c_void_p * 1)(None)
    assert L.vxr_batch_create(arr, 0, 0, 0, 0, C.byref(h)) == lib.vxr.VXR_E_INVALID
    assert L.vxr_batch_create(arr, 17, 0, 0, 0, C.byref(h)) == lib.vxr.VXR_E_INVALID
    assert L.vxr_batch_create(arr, 1, 0, 0, 2, C.byref(h)) == lib.vxr.VXR_E_INVALID
    assert L.vxr_batch_create(arr, 1, 5, 5, 0, C.byref(h)) == lib.vxr.VXR_E_INVALID
    assert L.vxr_batch_create(arr, 1, 0, 0, 0, C.byref(h)) == lib.vxr.VXR_E_INVALID   # null view
    assert L.vxr_batch_render(None) == lib.vxr.VXR_E_INVALID
    assert L.vxr_batch_wait(None, None) == lib.vxr.VXR_E_INVALID
    assert L.vxr_batch_destroy(None) == lib.vxr.VXR_OK
    t = lib.tuning()
    assert (t.tile_x, t.tile_y, t.persistent, t.shadow_refill, t.shadow_burst, t.list_blocks_per_sm, t.occupancy,
            t.shadow_schedule, t.shadow_early_out, t.brick_cache) == \
        (16, 8, 0, 8, 4, 16, 0, 0, 0, 0)
    assert L.vxr_view_set_tuning(None, C.byref(t)) == lib.vxr.VXR_E_INVALID
    assert L.vxr_batch_set_tuning(None, C.byref(t)) == lib.vxr.VXR_E_INVALID
    assert L.vxr_default_tuning(None) == lib.vxr.VXR_E_INVALID


def test_autotune_cache_roundtrip(tmp_path):
    from smallproject_gb300 import autotune as at
    from smallproject_gb300 import vxr as V
    d = {"tile": [32, 4], "persistent": 1, "shadow_refill": 16, "shadow_burst": 2, "list_blocks_per_sm": 8, "occupancy": 1,
         "shadow_schedule": 1, "shadow_early_out": 0, "brick_cache": 256}
    t = at._to_tuning(d)
    assert isinstance(t, V.Tuning) and at._from_tuning(t) == {**d, "tile": (32, 4)}
    path = str(tmp_path / "c.json")
    assert at.load_cache(path) == {}
    at.save_cache({"k": {"tuning": d, "ms": 1.0}}, path)
    assert at.load_cache(path)["k"]["tuning"] == d
    # every candidate of the search space is a valid tuning
    for name, values in at.SPACE:
        for val in values:
            dd = dict(d)
            dd[name] = list(val) if isinstance(val, tuple) else val
            tt = at._to_tuning(dd)
            assert (tt.tile_x * tt.tile_y) % 32 == 0 and tt.tile_x * tt.tile_y <= 1024


def test_out_of_map_set_is_ignored(lib):
    w = lib.World()
    w.set(1024, 0, 0, 0xF111)
    w.set(0, 5000, 0, 0xF111)
    assert w.get(0, 0, 0) == 0
    g, b, l = w.arrays()
    assert not g.any() and len(l) == 0


def test_worldapi_shim_compiles_links_and_runs(lib, tmp_path):
    """The C++ shim that replaces worldapi.h's World-backed bodies (tests/native/
    worldapi_shim.cpp) builds against include/vxr.h alone, links libvxr.so and drives the
    world through Plot / Box / Read / ClearWorld."""
    import subprocess
    exe = str(tmp_path / "shim")
    libdir = os.path.dirname(lib.LIB_PATH)
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-I" + os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "native", "worldapi_shim.cpp"), "-L" + libdir, "-lvxr",
                        "-Wl,-rpath," + libdir, "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.split() == ["f888", "f123", "0", "0"]
