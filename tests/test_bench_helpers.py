"""bench.py's host-side helpers, without a GPU: the harmonic mean, the launch
count, the clock-sample summary, the byte models' step split and the parity
check against the reference's fixture (with a stand-in for the C ABI)."""
import hashlib

import numpy as np

import bench


def test_hmean_gteps():
    # two searches of 2e9 and 4e9 directed edges (1e9, 2e9 undirected), 1 s each
    assert abs(bench.hmean_gteps([2e9, 4e9], [1.0, 1.0]) - 2 / (1 / 1.0 + 1 / 2.0)) < 1e-12
    assert bench.hmean_gteps([0, 0], [1.0, 1.0]) == 0.0


def test_count_launches():
    n = 1 << 20
    steps = [dict(kind="td", edges=10), dict(kind="td", edges=(n >> 3) + 1),
             dict(kind="e", edges=0), dict(kind="bu", edges=7), dict(kind="c", edges=0),
             dict(kind="td", edges=n >> 3)]
    # init + final decide, 2 per step, one more for the bitmap top-down step
    assert bench.count_launches([steps], n) == 2 + 2 * len(steps) + 1
    assert bench.count_launches([steps, steps[:1]], n) == (2 + 13) + (2 + 2)
    assert bench.count_launches([], n) == 0


def test_clock_summary_skips_samples_before_the_timed_region():
    c = bench.ClockSampler(0)
    c.lines = ["900, 2070, 300.0, 0x0, Not Active, Not Active, Not Active, Not Active",
               "2070, 2070, 900.5, 0x0, Not Active, Not Active, Not Active, Active",
               "2055, 2070, 910.0, 0x0, Not Active, Not Active, Not Active, Not Active",
               "[N/A], 2070, 0, 0x0, Not Active, Not Active, Not Active, Not Active",
               "short line"]
    c.skip = 1
    s = c.summary()
    assert s["samples"] == 2
    assert s["sm_mhz"] == (2070 + 2055) / 2
    assert s["sm_max_mhz"] == 2070
    assert s["reasons"] == ["sw_power_cap"]
    c.skip = len(c.lines)
    assert c.summary()["samples"] == 0


def test_layout_bytes_charge_the_claim_sweep_only_to_bitmap_steps():
    n = 1 << 20
    W4 = 4 * (n // 32)
    small = dict(kind="td", edges=n >> 3, count=100)
    big = dict(kind="td", edges=(n >> 3) + 1, count=100)
    assert bench.step_layout_bytes(n, big, 10) - bench.step_layout_bytes(n, small, 10) == \
        4 * 1 + 2 * W4
    assert bench.step_alg_bytes(n, big, 10) - bench.step_alg_bytes(n, small, 10) == 8


class _Stats:
    def __init__(self, trace):
        self.trace = trace


class _FakeBinding:
    """Stands in for gbbfs.DOBFS: fills the depth array from a table."""

    def __init__(self, depths, traces):
        self.depths, self.traces = depths, traces

    def DOBFS(self, g, s, depth=True, stats=True, parent_out=None, depth_out=None):
        depth_out[:] = self.depths[s]
        return parent_out, depth_out, _Stats(self.traces[s])


class _G:
    n = 4


def test_check_parity_against_a_fixture():
    depths = {5: np.array([1, 0, 2, -1], np.int32), 7: np.array([0, 1, 1, 2], np.int32)}
    traces = {5: [("td", 1), ("td", 2)], 7: [("td", 3)]}
    fixture = {"flags": ["-g", "2"], "trials": [
        {"source": 5, "trace": [["td", 1], ["td", 2]],
         "depth_sha256": hashlib.sha256(depths[5].tobytes()).hexdigest()},
        {"source": 7, "trace": [["td", 3]],
         "depth_sha256": hashlib.sha256(depths[7].tobytes()).hexdigest()}]}
    r = bench.check_parity(_FakeBinding(depths, traces), _G(), [5, 7, 9], fixture)
    assert r["ok"] and r["sources_checked"] == 2 and r["sources_without_fixture"] == 1
    bad = dict(depths)
    bad[7] = np.array([0, 1, 2, 2], np.int32)
    r = bench.check_parity(_FakeBinding(bad, traces), _G(), [5, 7], fixture)
    assert not r["ok"] and r["depth_sha256_equal"] == 1 and r["trace_equal"] == 2
    assert bench.check_parity(None, _G(), [5], None) == {"fixture": None, "ok": None}
