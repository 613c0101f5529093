"""The worldapi.h shim (tests/native/worldapi_shim.cpp, the code of the integration guide)
driving a render: a world built through Plot / Box, the camera through LookAt, frames
through RenderFrame / CommitFrame, the image read back - a C++ caller of libvxr.so with
no Python in the loop."""
import os
import subprocess

import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu


def test_worldapi_shim_renders(lib, cuda_device, tmp_path):
    exe = str(tmp_path / "shim")
    libdir = os.path.dirname(lib.LIB_PATH)
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-I" + os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "native", "worldapi_shim.cpp"), "-L" + libdir, "-lvxr",
                        "-Wl,-rpath," + libdir, "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([exe, "render"], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stdout + out.stderr
    lit, bad, mx = out.stdout.split()
    assert int(lit) > 100 and int(bad) == 0 and float(mx) > 0.0
