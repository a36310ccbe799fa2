"""Node-based Green-Gauss gradients (grad_node_based_gauss, gradients.f90:
1491-1602; weights of node_interpolation.f90) on the CPU: the oracle's
restatement against the library's weight builder (host/fc_node_interp.cpp)
plus the per-node and per-cell code the CUDA kernels run
(csrc/fc_nodegrad.cuh), replayed on the host by
tests/replay/nodegrad_replay.cpp, bit for bit, for both cell-to-node methods
on perturbed hex and tet meshes; and the linear-field property.

The pseudo-Laplacian weights of a node on a box edge (boundary faces in two
planes) all evaluate to 0 or nearly: the reference's normalisation then
divides 0 by 0 and those nodes' cells get NaN gradients.  That is the
reference's arithmetic; the comparisons treat NaN as equal at equal places."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import load_fcgpu
from test_limiters import cell_faces

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
PKG = os.path.join(ROOT, "freecappuccino-dev_gb300")


@pytest.fixture(scope="module")
def replay(tmp_path_factory):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not available")
    exe = str(tmp_path_factory.mktemp("ng") / "nodegrad_replay")
    subprocess.run([gxx, "-std=c++17", "-O2", "-ffp-contract=off", "-I", os.path.join(PKG, "csrc"), "-I",
                    os.path.join(PKG, "host"), os.path.join(HERE, "replay", "nodegrad_replay.cpp"),
                    os.path.join(PKG, "host", "fc_node_interp.cpp"), "-o", exe], check=True)
    return exe


def make_case(oracle, tets, perturb=0.2, seed=4, n=(6, 5, 4)):
    fc = load_fcgpu()
    m = fc.Mesh.box(*n, 1.0, 1.1, 0.9, perturb=perturb, seed=seed, tets=tets)
    a = m.arrays()
    return a, oracle.Case(a)


def run_replay(exe, a, oc, phi, method, tmp_path):
    nN, nC, nI, nF, nT = len(a["x"]), oc.numCells, oc.numInnerFaces, oc.numFaces, oc.numTotal
    cfp, cff = cell_faces(oc)
    inp, out = tmp_path / f"ng{method}.bin", tmp_path / f"ngo{method}.bin"
    nodes = np.asarray(a["nodes"], np.int32).reshape(nF, 6) - 1
    nodes[nodes < 0] = 0
    with open(inp, "wb") as f:
        np.array([method, nN, nC, nI, nF, nT, len(cff)], np.int32).tofile(f)
        for v in (np.asarray(a["owner"]) - 1, np.asarray(a["neighbour"]) - 1, a["nnodes"], nodes, cfp, cff):
            np.asarray(v, np.int32).ravel().tofile(f)
        for v in (a["x"], a["y"], a["z"]):
            np.asarray(v, np.float64).tofile(f)
        for nm in ("xc", "yc", "zc", "xf", "yf", "zf", "arx", "ary", "arz", "vol"):
            oc.get(nm).tofile(f)
        np.asarray(phi, np.float64).tofile(f)
    subprocess.run([exe, str(inp), str(out)], check=True)
    return np.fromfile(out, np.float64).reshape(3, nT).T.ravel()


@pytest.mark.parametrize("tets", [False, True])
@pytest.mark.parametrize("method", [0, 1])
def test_device_node_gradient_code_matches_oracle(oracle, replay, tmp_path, tets, method):
    a, oc = make_case(oracle, tets)
    phi = np.random.default_rng(8).standard_normal(oc.numTotal)
    oc.param("c2n", method)
    go = oc.grad(3, phi)
    got = run_replay(replay, a, oc, phi, method, tmp_path)
    nC = oc.numCells
    # NaN where the reference's pseudo-Laplacian weights of a node all come
    # out 0 (nodes on a box edge: 0/0 in the normalisation), at the same places
    assert np.array_equal(got[:3 * nC], go[:3 * nC], equal_nan=True)
    assert not np.array_equal(go[:3 * nC], oc.grad(0, phi)[:3 * nC])


def test_linear_field_is_exact_away_from_the_boundary(oracle):
    """On a uniform hex mesh the pseudo-Laplacian weights of an interior node
    are 1/8 each, so a linear field is interpolated exactly and the
    gradient of cells not touching the boundary is exact."""
    a, oc = make_case(oracle, False, perturb=0.0, n=(6, 6, 6))
    xc, yc, zc = oc.get("xc"), oc.get("yc"), oc.get("zc")
    xf, yf, zf = oc.get("xf"), oc.get("yf"), oc.get("zf")
    nI = oc.numInnerFaces
    lin = lambda x, y, z: 0.3 + 2.0 * x - 1.5 * y + 0.7 * z  # noqa: E731
    phi = np.concatenate([lin(xc, yc, zc), lin(xf, yf, zf)[nI:]])
    oc.param("c2n", 0)
    g = oc.grad(3, phi).reshape(-1, 3)[:oc.numCells]
    inner = (xc > 1 / 6) & (xc < 5 / 6) & (yc > 1.1 / 6) & (yc < 1.1 * 5 / 6) & (zc > 0.9 / 6) & (zc < 0.9 * 5 / 6)
    assert inner.sum() == 64
    np.testing.assert_allclose(g[inner], np.tile([2.0, -1.5, 0.7], (64, 1)), atol=1e-10)
