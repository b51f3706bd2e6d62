"""The query server's batching policy (csrc/serve_policy.h), on the CPU:
the C++ functions the server runs, compiled into a small driver, against a
plain Python statement of the rule."""
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "dist_mem_gapbs_gb300", "csrc")

KGROUP_WINDOW = 4
KPLAIN_BUSY = 3


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("no g++")
    exe = str(tmp_path_factory.mktemp("policy") / "serve_policy_driver")
    subprocess.run([cxx, "-O2", "-std=c++17", "-I", CSRC,
                    os.path.join(ROOT, "tests", "serve_policy_driver.cc"), "-o", exe], check=True)

    def run(lines):
        out = subprocess.run([exe], input="\n".join(lines) + "\n", capture_output=True,
                             text=True, check=True).stdout
        return out.splitlines()
    return run


def python_pick(keys, lanes):
    """The rule: a window that fits goes whole; else, in stable key order,
    the run of `lanes` holding the oldest query (position 0) with the
    smallest key spread, the earliest such run on ties."""
    w = len(keys)
    if w <= lanes:
        return list(range(w))
    order = sorted(range(w), key=lambda i: (keys[i], i))
    p = order.index(0)
    best = None
    for s in range(max(0, p - lanes + 1), min(p, w - lanes) + 1):
        spread = keys[order[s + lanes - 1]] - keys[order[s]]
        if best is None or spread < best[0]:
            best = (spread, s)
    return sorted(order[best[1]:best[1] + lanes])


def test_pick_group_matches_rule(driver):
    rng = np.random.default_rng(11)
    cases = []
    for _ in range(400):
        lanes = int(rng.choice([1, 2, 3, 8, 32]))
        w = int(rng.integers(1, KGROUP_WINDOW * lanes + 1))
        hi = int(rng.choice([1, 3, 50, 65535]))     # many ties, some, few
        keys = [int(x) for x in rng.integers(0, hi + 1, size=w)]
        cases.append((lanes, keys))
    got = driver(["pick %d %d %s" % (l, len(k), " ".join(map(str, k))) for l, k in cases])
    assert len(got) == len(cases)
    for (lanes, keys), line in zip(cases, got):
        chosen = [int(x) for x in line.split()]
        assert chosen == python_pick(keys, lanes), (lanes, keys)
        assert 0 in chosen and len(chosen) == min(lanes, len(keys))


def test_pick_group_hand_cases(driver):
    got = driver([
        "pick 2 4 5 1 1 9",      # runs {1, 5} and {5, 9} tie at spread 4: the earlier
        "pick 2 4 5 1 4 9",      # {4, 5} is the tighter run holding the oldest
        "pick 2 4 9 1 1 5",      # the oldest has the largest key
        "pick 3 3 7 7 7",        # fits: all
        "pick 2 5 4 4 4 4 4",    # all tied: the oldest and the next in arrival order
    ])
    assert got == ["0 2", "0 2", "0 3", "0 1 2", "0 1"]


def test_oldest_query_never_starves(driver):
    """Repeated launches from a queue the policy keeps reordering: every query
    leaves within as many launches as there were queries ahead of it."""
    rng = np.random.default_rng(3)
    lanes = 4
    queue = [(i, int(k)) for i, k in enumerate(rng.integers(0, 6, size=60))]
    launched_at = {}
    launch = 0
    while queue:
        window = queue[:KGROUP_WINDOW * lanes]
        chosen = [int(x) for x in driver(["pick %d %d %s" % (
            lanes, len(window), " ".join(str(k) for _, k in window))])[0].split()]
        for pos in chosen:
            launched_at[window[pos][0]] = launch
        keep = set(chosen)
        queue = [q for pos, q in enumerate(window) if pos not in keep] + queue[len(window):]
        launch += 1
    for qid, at in launched_at.items():
        assert at <= qid


def test_plain_is_cheaper(driver):
    cases = [(1, 0.5, 6.0, 0), (12, 0.5, 6.0, 0), (11, 0.5, 6.0, 0), (1, 0.5, 6.0, KPLAIN_BUSY),
             (1, 0.5, 6.0, KPLAIN_BUSY - 1), (1, -1, 6.0, 0), (1, 0.5, -1, 0), (4, 2.0, 8.0, 0)]
    got = driver(["plain %d %g %g %d" % c for c in cases])
    want = [int(b < KPLAIN_BUSY and p > 0 and t > 0 and k * p < t) for k, p, t, b in cases]
    assert [int(x) for x in got] == want
    assert want == [1, 0, 1, 0, 1, 0, 0, 0]
