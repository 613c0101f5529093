import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a); runs the CUDA path")
    config.addinivalue_line("markers", "slow: longer CPU case")


@pytest.fixture(scope="session")
def lib():
    from smallproject_gb300 import build as B
    B.build()
    import smallproject_gb300 as vx
    return vx


@pytest.fixture(scope="session")
def cuda_device(lib):
    """Skips unless a CUDA device is visible (GPU tests are marked gpu anyway)."""
    import ctypes
    try:
        rt = ctypes.CDLL("libcuda.so.1")
        n = ctypes.c_int(0)
        if rt.cuInit(0) != 0 or rt.cuDeviceGetCount(ctypes.byref(n)) != 0 or n.value == 0:
            pytest.skip("no CUDA device")
    except OSError:
        pytest.skip("no CUDA driver")
    return True


@pytest.fixture(scope="session")
def scene0(lib):
    """Config-0 world (256^3 fBm terrain, 64 emitters) and its arrays."""
    w = lib.World()
    d = lib.scene_preset(0)
    w.generate(d)
    return w, d


@pytest.fixture(scope="session")
def world0_arrays(scene0):
    from oracle import binding as ob
    g, b, l = scene0[0].arrays()
    return ob.WorldArrays(g, b, l)


def bits(a):
    a = np.asarray(a)
    return a.view(np.uint32) if a.dtype.kind == "f" else a


def assert_records_equal(name, got, want, ctx=""):
    """Bit-exact comparison of structured (or plain) arrays with a useful message."""
    if got.dtype.names:
        for f in want.dtype.names:
            g, w = bits(got[f]), bits(want[f])
            d = g != w
            if d.ndim > 1:
                d = d.any(axis=1)
            if d.any():
                idx = np.nonzero(d)[0]
                raise AssertionError(f"{ctx} {name}.{f}: {d.sum()} of {len(d)} differ; first {idx[:5].tolist()}: "
                                     f"got {got[f][idx[0]]!r} want {want[f][idx[0]]!r}")
    else:
        d = bits(got) != bits(want)
        if d.ndim > 1:
            d = d.any(axis=-1)
        if d.any():
            idx = np.nonzero(d.reshape(-1))[0]
            raise AssertionError(f"{ctx} {name}: {d.sum()} differ; first {idx[:5].tolist()}")
