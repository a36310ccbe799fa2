"""Host planner of the batched launch (host/fc_batch_plan.cpp), through the
C++ harness tests/replay/batch_plan_replay.cpp: group sizes within the block
budget and the per-problem caps, larger problems never get fewer blocks,
and the greedy plan's makespan equals the best over all allocations (brute
force on small cases)."""
import itertools
import os
import shutil
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
HOST = os.path.join(ROOT, "freecappuccino-dev_gb300", "host")


@pytest.fixture(scope="module")
def planner(tmp_path_factory):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not available")
    exe = str(tmp_path_factory.mktemp("plan") / "batch_plan_replay")
    subprocess.run([gxx, "-std=c++17", "-O2", "-I", HOST, os.path.join(HERE, "replay", "batch_plan_replay.cpp"),
                    os.path.join(HOST, "fc_batch_plan.cpp"), "-o", exe], check=True)

    def run(budget, gmax, min_rows, probs):
        txt = f"{budget} {gmax} {min_rows} {len(probs)}\n" + "".join(f"{r} {l} {w}\n" for r, l, w in probs)
        out = subprocess.run([exe], input=txt, capture_output=True, text=True, check=True).stdout.splitlines()
        tiles = [int(v) for v in out[0].split()] if out[0].strip() else []
        iters = np.array([[float(v) for v in line.split()] for line in out[2:]])
        return tiles, float(out[1]), iters
    return run


def makespan(iters_fn, probs, g):
    return max(w * iters_fn(p, t) for p, ((r, l, w), t) in enumerate(zip(probs, g)))


def test_plan_respects_budget_and_caps(planner):
    rng = np.random.default_rng(44)
    ns = rng.integers(20, 81, 64)
    probs = [(int(n) ** 3, 3 * int(n), 1.0) for n in ns]
    tiles, span, _ = planner(152, 152, 1024, probs)
    assert len(tiles) == 64 and min(tiles) >= 1 and sum(tiles) <= 152
    for (r, _, _), t in zip(probs, tiles):
        assert t <= max(1, r // 1024)
    # a larger problem (same weight, more rows and levels) never gets fewer
    # blocks (equal sizes may differ by the last block handed out)
    for i in range(64):
        for j in range(64):
            if ns[i] < ns[j]:
                assert tiles[i] <= tiles[j], (ns[i], ns[j], tiles[i], tiles[j])
    assert span > 0


def test_more_problems_than_blocks(planner):
    tiles, span, _ = planner(4, 4, 1, [(1000, 10, 1.0)] * 5)
    assert tiles == [] and span < 0


def test_weights_move_blocks(planner):
    same = [(200000, 100, 1.0), (200000, 100, 1.0)]
    t_eq, _, _ = planner(20, 152, 1024, same)
    assert t_eq[0] == t_eq[1]
    t_w, _, _ = planner(20, 152, 1024, [(200000, 100, 4.0), (200000, 100, 1.0)])
    assert t_w[0] > t_w[1]


@pytest.mark.parametrize("seed", [1, 2, 3, 4])
def test_greedy_matches_brute_force(planner, seed):
    rng = np.random.default_rng(seed)
    probs = [(int(rng.integers(2000, 400000)), int(rng.integers(10, 300)), float(rng.uniform(0.5, 3.0)))
             for _ in range(3)]
    budget = 9
    tiles, span, iters = planner(budget, budget, 1, probs)

    def it(p, g):
        # the model is a + b / g: recover a, b from g = 1, 2
        a = 2 * iters[p, 1] - iters[p, 0]
        b = iters[p, 0] - a
        return a + b / g
    best = min(makespan(it, probs, g) for g in itertools.product(range(1, budget + 1), repeat=3) if sum(g) <= budget)
    assert span == pytest.approx(best, rel=1e-12)
    assert makespan(it, probs, tiles) == pytest.approx(span, rel=1e-12)
