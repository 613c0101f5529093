"""Benchmark workload definitions (no GPU needed): config 2's eight mixed views."""
from smallproject_gb300 import workloads as wl


def test_config2_specs_follow_the_definition():
    a = wl.config2_specs(seed=3)
    assert a == wl.config2_specs(seed=3) and a != wl.config2_specs(seed=4)
    assert len(a) == 8
    for s in a:
        assert s["extent"] in (256, 512, 1024)
        assert 16 <= s["emitters"] <= 65536
        assert (s["width"], s["height"]) in wl.RESOLUTIONS
        assert s["light_model"] in ("point", "area")
    small = wl.config2_specs(seed=3, scale=0.1)
    assert all(x["width"] == max(16, int(y["width"] * 0.1)) for x, y in zip(small, a))
