"""Host logic of the schedule-ordered sweeps: the C++ replay in
tests/replay/schedule_replay.cpp rebuilds the ordered structure with the
library's own builder (host/fc_schedule.cpp) and replays the sweeps with the
kernel's ring and exchange rules against plain substitution, bit for bit."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
HOST = os.path.join(ROOT, "freecappuccino-dev_gb300", "host")


@pytest.fixture(scope="module")
def replay(tmp_path_factory):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not available")
    exe = str(tmp_path_factory.mktemp("replay") / "schedule_replay")
    subprocess.run([gxx, "-std=c++17", "-O2", "-I", HOST, os.path.join(HERE, "replay", "schedule_replay.cpp"),
                    os.path.join(HOST, "fc_schedule.cpp"), "-o", exe], check=True)
    return exe


# nx ny nz tiles [random couplings] [ring depth] [stage depth] [rows per step cap]
CASES = [
    "12 10 8 16",          # structured, coordinate tiles
    "16 16 16 152",        # more tiles than chains per tile
    "30 30 30 152 0 4",    # one tile per SM of the GPU
    "20 7 5 40 1",         # long-range and one-sided couplings, overflow entries, graph tiles
    "9 9 9 3 1 2",         # ring depth 2: most dependencies through the exchange
    "7 3 1 2 1",
    "5 1 1 3",             # a single chain
    "1 1 1 1",             # one row
    "30 30 30 152 0 4 4 3",  # steps capped at 3 rows: wide levels split into consecutive steps
    "16 16 16 4 0 4 2 5",    # few wide tiles, ring depth 4, stage depth 2, steps of at most 5 rows
    "20 7 5 40 1 4 4 4",     # capped steps with long-range couplings and overflow entries
]


@pytest.mark.parametrize("args", CASES)
def test_ordered_sweep_replay_matches_substitution(replay, args):
    out = subprocess.run([replay] + args.split(), capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.strip().endswith("OK"), out.stdout


@pytest.fixture(scope="module")
def pick_tiles(tmp_path_factory):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not available")
    exe = str(tmp_path_factory.mktemp("pick") / "pick_tiles_replay")
    subprocess.run([gxx, "-std=c++17", "-O2", "-pthread", "-I", HOST,
                    os.path.join(HERE, "replay", "pick_tiles_replay.cpp"), os.path.join(HOST, "fc_schedule.cpp"),
                    "-o", exe], check=True)
    return exe


@pytest.mark.parametrize("case", ["40 30 20 152", "7 5 3 152", "30 30 30 16 0", "3 1 1 4", "64 64 64 152"])
def test_concurrent_tile_choice_matches_sequential(pick_tiles, case):
    """The pattern analysis builds its candidate tile counts concurrently
    (pick_sweep_tiles); the choice and its estimate equal building them one
    after another."""
    out = subprocess.run([pick_tiles] + case.split(), capture_output=True, text=True, check=True).stdout.split()
    assert out[0] == out[2] and out[1] == out[3], out
