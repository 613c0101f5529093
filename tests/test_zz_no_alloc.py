"""vxr_render_frame_noalloc: one frame rendered without any allocation by the library,
for callers that cannot call cudaMalloc (they own every device buffer themselves).

The test owns the device buffers (allocated here through torch, as such a caller would
through its own allocator), renders two different frames in a row through the C ABI,
and requires each to match, bit for bit, the same frame rendered by the regular view
path (vxr_view_*, temporal reuse and accumulation off). A third call, bracketed by
cudaMemGetInfo, must leave the device's free memory unchanged."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dev(torch, arr):
    t = torch.from_numpy(np.ascontiguousarray(arr).view(np.int32).reshape(-1).copy())
    return t.to("cuda")


def test_noalloc_matches_view_path_twice(lib, cuda_device, scene0):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("torch without CUDA")
    world, _ = scene0
    W, H = 160, 96
    g, b, l = world.arrays()
    d_grid = _dev(torch, g)
    d_bricks = _dev(torch, b)
    d_lights = _dev(torch, l.view(np.uint32))
    d_out = torch.zeros(W * H * 4, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()

    view = lib.View(world, lib.view_desc(W, H, lib.LIGHTS_AREA, temporal=0, accumulate=0))
    L = lib.load()
    cams = [((128.0, 160.0, 0.0), (128.0, 128.0, 128.0)), ((60.0, 120.0, 40.0), (150.0, 60.0, 170.0))]
    for pos, tgt in cams:
        view.lookat(pos, tgt)
        k = view.begin_frame()
        for s in (lib.STAGE_ALBEDO, lib.STAGE_CANDIDATES, lib.STAGE_SPATIAL, lib.STAGE_SHADE):
            view.stage(s)
        view.end_frame()
        view.wait()
        want = view.read_frame()
        rc = L.vxr_render_frame_noalloc(C.c_void_p(d_grid.data_ptr()), C.c_void_p(d_bricks.data_ptr()), len(b),
                                        C.c_void_p(d_lights.data_ptr()), len(l), lib.LIGHTS_AREA, C.byref(k),
                                        C.c_void_p(d_out.data_ptr()), None)
        assert rc == 0, L.vxr_last_error().decode()
        got = d_out.cpu().numpy().reshape(-1, 4)
        assert (want[:, 3] > 0).any() and (want[:, :3] > 0).any()
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), \
            f"{int((got != want).any(axis=1).sum())} pixels differ"
    # the promise itself: after a first call, a further call changes the device's free
    # memory by nothing (no cudaMalloc, no lazily grown buffer, no library allocator)
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    rc = L.vxr_render_frame_noalloc(C.c_void_p(d_grid.data_ptr()), C.c_void_p(d_bricks.data_ptr()), len(b),
                                    C.c_void_p(d_lights.data_ptr()), len(l), lib.LIGHTS_AREA, C.byref(k),
                                    C.c_void_p(d_out.data_ptr()), None)
    assert rc == 0, L.vxr_last_error().decode()
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
    view.close()


def test_noalloc_rejects_oversize(lib, cuda_device, scene0):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("torch without CUDA")
    world, _ = scene0
    g, b, l = world.arrays()
    d_grid = _dev(torch, g)
    d_bricks = _dev(torch, b)
    d_lights = _dev(torch, l.view(np.uint32))
    d_out = torch.zeros(4, dtype=torch.float32, device="cuda")
    cam = lib.Camera()
    cam.lookat((128.0, 160.0, 0.0), (128.0, 128.0, 128.0))
    k = cam.begin_frame(512, 512)                                   # 262,144 px > 65,536
    k.numberOfLights, k.numberOfCandidates, k.spatialRadius, k.spatialTaps = len(l), 32, 30, 5
    L = lib.load()
    rc = L.vxr_render_frame_noalloc(C.c_void_p(d_grid.data_ptr()), C.c_void_p(d_bricks.data_ptr()), len(b),
                                    C.c_void_p(d_lights.data_ptr()), len(l), lib.LIGHTS_AREA, C.byref(k),
                                    C.c_void_p(d_out.data_ptr()), None)
    assert rc == lib.vxr.VXR_E_INVALID and b"exceeds the fixed scratch" in L.vxr_last_error()
    k2 = cam.begin_frame(64, 64)
    k2.numberOfLights, k2.numberOfCandidates, k2.spatialRadius, k2.spatialTaps = len(l), 32, 30, 5
    rc = L.vxr_render_frame_noalloc(C.c_void_p(d_grid.data_ptr()), C.c_void_p(d_bricks.data_ptr()), 1,
                                    C.c_void_p(d_lights.data_ptr()), len(l), lib.LIGHTS_AREA, C.byref(k2),
                                    C.c_void_p(d_out.data_ptr()), None)
    assert rc == lib.vxr.VXR_E_INVALID and b"brick" in L.vxr_last_error()
