"""The bench's quality-protocol decisions (bench.decide, bench.boot_ci, bench.boot_ratio)
on synthetic per-seed MSE samples, on the CPU: which learned configuration counts as
"equal MSE" to plain at 32 candidates, and which one is the equal-time point."""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import bench  # noqa: E402


def _groups(rng, median, seeds=40, frames=16, tail=(0.0, 0)):
    """Per-seed arrays of per-frame MSEs: lognormal around `median`; tail = (factor, n)
    puts a firefly frame (factor x the median) into each of the first n seeds."""
    g = [median * np.exp(0.15 * rng.standard_normal(frames)) for _ in range(seeds)]
    for i in range(tail[1]):
        g[i][3] = median * tail[0]
    return g


def _point(method, k, ms, groups):
    allf = np.concatenate(groups)
    return {"method": method, "candidates": k, "ms": ms, "mse": float(allf.mean()),
            "mse_ci95": bench.boot_ci(groups, np.mean), "mse_median": float(np.median(allf)),
            "mse_median_ci95": bench.boot_ci(groups, np.median)}


def _table(spec, seed=0):
    """spec: key -> (ms, median MSE, (firefly factor, seeds with a firefly))"""
    rng = np.random.default_rng(seed)
    groups, table = {}, {}
    for key, (ms, med, tail) in spec.items():
        fam, k = key.rsplit("_", 1)
        groups[key] = _groups(rng, med, tail=tail)
        table[key] = _point("plain" if fam == "plain" else fam, int(k), ms, groups[key])
    return table, groups


def test_boot_intervals_cover_the_statistic():
    rng = np.random.default_rng(3)
    g = _groups(rng, 0.05)
    lo, hi = bench.boot_ci(g, np.mean)
    m = float(np.concatenate(g).mean())
    assert lo <= m <= hi and hi - lo < 0.2 * m
    # the same distribution against itself: the ratio interval holds 1
    lo, hi = bench.boot_ratio(g, _groups(rng, 0.05), np.median)
    assert lo < 1.0 < hi


def test_equal_mse_needs_both_intervals_and_picks_the_fastest():
    table, groups = _table({
        "plain_32": (5.1, 0.048, (100.0, 8)),  # a heavy-tailed plain mean (≈ 2.2 x its median)
        "learned_2": (4.3, 0.043, (0.0, 0)),   # both ratios below 1
        "learned_4": (4.5, 0.040, (0.0, 0)),
        "learned2_2": (4.2, 0.060, (0.0, 0)),  # mean ratio < 1 (plain's tail), median ratio > 1
        "learned4_2": (4.1, 0.040, (800.0, 1)),  # a firefly of its own: mean interval above 1
    })
    eq, eq_mean, eq_med, mono, fams, et = bench.decide(table, groups)
    assert eq["method"] == "learned" and eq["candidates"] == 2
    assert table["learned2_2"]["mse_ratio_ci95"][1] <= 1.0 < table["learned2_2"]["median_mse_ratio_ci95"][1]
    assert eq_mean["method"] == "learned2"         # the mean alone would have taken it
    assert table["learned4_2"]["mse_ratio_ci95"][1] > 1.0
    assert eq_med["method"] == "learned4"          # the median alone would have taken the firefly point
    assert mono


def test_equal_time_takes_the_largest_time_not_above_plain_per_family():
    table, groups = _table({
        "plain_32": (5.0, 0.048, (0.0, 0)),
        "learned_4": (4.5, 0.040, (0.0, 0)),
        "learned_8": (4.9, 0.036, (0.0, 0)),
        "learned_12": (5.2, 0.035, (0.0, 0)),       # slower than plain: not an equal-time point
        "learned2_8": (4.8, 0.037, (0.0, 0)),
        "learned2_12": (5.0, 0.034, (0.0, 0)),      # equal to plain's time: allowed
    })
    eq, eq_mean, eq_med, mono, fams, et = bench.decide(table, groups)
    assert fams["learned"]["candidates"] == 8 and fams["learned2"]["candidates"] == 12
    assert et is fams["learned2"]                   # the one closest to plain's time
    assert eq["candidates"] == 4 and eq["method"] == "learned"


def test_no_learned_point_qualifies():
    table, groups = _table({"plain_32": (5.0, 0.030, (0.0, 0)), "learned_2": (4.0, 0.060, (0.0, 0)),
                            "learned_4": (4.2, 0.050, (0.0, 0))})
    eq, eq_mean, eq_med, mono, fams, et = bench.decide(table, groups)
    assert eq is None and eq_mean is None and eq_med is None
    assert et["candidates"] == 4
