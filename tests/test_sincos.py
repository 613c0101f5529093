"""The fixed sin/cos of the spatial taps (oracle restatement; the CUDA kernel uses the
same formula and is compared bit-exactly on the GPU): accuracy against the correctly
rounded values over angles u * 2pi reachable from the xorshift stream."""
import math

import numpy as np

from oracle import binding as ob


def test_sincos_accuracy_on_reachable_angles():
    rng = np.random.default_rng(11)
    s = rng.integers(0, 2 ** 32, 20000, dtype=np.uint64).astype(np.uint32)
    s = np.concatenate([s, np.array([0, 1, 2 ** 31, 2 ** 32 - 1, 2 ** 30, 3 * 2 ** 30], np.uint32)])
    u = (s.astype(np.float32) * np.float32(2.3283064365387e-10)).astype(np.float32)
    a = (u * np.float32(6.28318530717958647692528)).astype(np.float32)
    worst = 0
    for x in a:
        sn, cs = ob.sincos(float(x))
        for got, ref in ((sn, math.sin(float(x))), (cs, math.cos(float(x)))):
            r32 = np.float32(ref)
            ulp = np.spacing(np.float32(max(abs(r32), 1e-30)))
            err = abs(np.float32(got) - r32) / ulp if abs(ref) > 1e-6 else abs(got - ref) / 1e-7
            worst = max(worst, float(err))
    assert worst <= 2.0, worst
