"""bench.py with N > 1 ranks, on the CPU over gloo (torch.distributed.run, two ranks,
rendezvous on 127.0.0.1): the multi-rank helpers, and the reference arm, whose rank 0
alone times the reference's CPU path and prints the one JSON line while the other ranks
exit 0 without work."""
import json
import os
import socket
import subprocess
import sys

import pytest

from conftest import ROOT
from oracle.ref_build import DEFAULT_REF


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _torchrun(args, timeout):
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), *args]
    env = dict(os.environ, OMP_NUM_THREADS="2", CUDA_VISIBLE_DEVICES="")
    r = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=timeout)
    lines = [json.loads(line) for line in r.stdout.splitlines() if line.startswith("{")]
    return r, lines


def test_multi_rank_helpers_gloo():
    r, lines = _torchrun([os.path.join(ROOT, "tests", "dist_worker.py")], 180)
    assert r.returncode == 0, r.stderr[-3000:]
    assert sorted(d["rank"] for d in lines) == [0, 1]
    for d in lines:
        assert d["world"] == 2 and d["max"] == 3.0            # the slowest rank's time everywhere
        assert d["quality"] == {"learned_at_equal_mse": {"candidates": 4}} and d["params"] == [0.25, -1.5]


@pytest.mark.skipif(not os.path.isdir(DEFAULT_REF) and not os.path.isfile(
    os.path.join(ROOT, "oracle", "_ref", "vxref_gen.inc")), reason="the reference oracle cannot be built here")
def test_reference_arm_two_ranks():
    r, lines = _torchrun(["bench.py", "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "0",
                          "--config", "0", "--width", "64", "--height", "48"], 600)
    assert r.returncode == 0, r.stderr[-3000:]
    assert len(lines) == 1, lines                               # rank 0 alone prints
    d = lines[0]
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["unit"] == "ms/frame" and d["value"] > 0
    assert d["cpu_baseline"]["value"] == d["value"] and d["e2e"]["h2d_bytes_per_step"] == 0
    assert "whole 64x48 frames" in d["cpu_baseline"]["sample"] and d["opencl_cpu_runtime"]["status"]
