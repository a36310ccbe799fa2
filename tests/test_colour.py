"""Host logic of the multicolour FP32 inner solve: the C++ replay in
tests/replay/colour_replay.cpp builds the layout with the library's own
builder (host/fc_colour.cpp), checks the colouring and every stored index,
and replays the kernel's phase sequence (reads only of values written before
a grid barrier) through a converging PCG."""
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
    exe = str(tmp_path_factory.mktemp("creplay") / "colour_replay")
    subprocess.run([gxx, "-std=c++17", "-O2", "-I", HOST, os.path.join(HERE, "replay", "colour_replay.cpp"),
                    os.path.join(HOST, "fc_colour.cpp"), "-o", exe], check=True)
    return exe


# nx ny nz [random couplings]
CASES = ["12 10 8", "40 40 40", "20 7 5 1", "9 9 9 1", "5 1 1", "1 1 1", "33 1 1"]


@pytest.mark.parametrize("args", CASES)
def test_coloured_layout_and_phase_replay(replay, args):
    out = subprocess.run([replay] + args.split(), capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.strip().endswith("OK"), out.stdout
