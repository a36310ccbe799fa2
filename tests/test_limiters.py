"""Slope limiters of the cell gradients (gradients.f90:141-656) on the CPU:
the oracle's restatement against the per-cell code the CUDA kernels run
(csrc/fc_limiter.cuh, replayed on the host by tests/replay/limiter_replay.cpp,
-ffp-contract=off as the kernels are built without FMA), bit for bit, for the
four limiters on Gauss and least-squares gradients of perturbed hex and tet
meshes; plus properties of the limited gradients."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import load_fcgpu

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(ROOT, "freecappuccino-dev_gb300", "csrc")


@pytest.fixture(scope="module")
def replay(tmp_path_factory):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not available")
    exe = str(tmp_path_factory.mktemp("lim") / "limiter_replay")
    subprocess.run([gxx, "-std=c++17", "-O2", "-ffp-contract=off", "-I", CSRC,
                    os.path.join(HERE, "replay", "limiter_replay.cpp"), "-o", exe], check=True)
    return exe


def case(oracle, tets, seed=3):
    fc = load_fcgpu()
    m = fc.Mesh.box(7, 6, 5, 1.0, 1.2, 0.8, perturb=0.2, seed=seed, tets=tets)
    oc = oracle.Case(m.arrays())
    rng = np.random.default_rng(seed)
    nT = oc.numTotal
    xc = np.concatenate([oc.get("xc"), rng.uniform(0, 1, nT - oc.numCells)])
    # a steep front plus noise: overshoots for every limiter
    phi = np.tanh((xc - 0.5) / 0.08) + 0.05 * rng.standard_normal(nT)
    return oc, phi


def cell_faces(oc):
    nC, nI, nF = oc.numCells, oc.numInnerFaces, oc.numFaces
    own = oc.get_int("owner") - 1
    nb = oc.get_int("neighbour") - 1
    lists = [[] for _ in range(nC)]
    for f in range(nF):
        lists[own[f]].append(f)
        if f < nI:
            lists[nb[f]].append(f)
    ptr = np.zeros(nC + 1, np.int32)
    ptr[1:] = np.cumsum([len(v) for v in lists])
    return ptr, np.array([f for v in lists for f in v], np.int32)


def run_replay(exe, oc, phi, g_aos, kind, tmp_path):
    nC, nI, nF, nT = oc.numCells, oc.numInnerFaces, oc.numFaces, oc.numTotal
    ia, ja, dg = oc.get_int("ia") - 1, oc.get_int("ja") - 1, oc.get_int("diag") - 1
    cfp, cff = cell_faces(oc)
    g_soa = g_aos.reshape(nT, 3).T.copy()
    inp, out = tmp_path / f"in{kind}.bin", tmp_path / f"out{kind}.bin"
    with open(inp, "wb") as f:
        np.array([kind, nC, nI, nF, nT, len(ja), len(cff)], np.int32).tofile(f)
        for v in (ia, ja, dg, cfp, cff):
            np.asarray(v, np.int32).tofile(f)
        for nm in ("xc", "yc", "zc", "xf", "yf", "zf"):
            oc.get(nm).tofile(f)
        np.asarray(phi, np.float64).tofile(f)
        g_soa.tofile(f)
    subprocess.run([exe, str(inp), str(out)], check=True)
    return np.fromfile(out, np.float64).reshape(3, nT).T.ravel()


@pytest.mark.parametrize("tets", [False, True])
@pytest.mark.parametrize("scheme", [0, 1])
@pytest.mark.parametrize("kind", [1, 2, 3, 4])
def test_device_limiter_code_matches_oracle(oracle, replay, tmp_path, tets, scheme, kind):
    oc, phi = case(oracle, tets)
    if scheme:
        oc.L.orc_prepare_lsq(oc.h, scheme)
    oc.param("limiter", 0)
    g0 = oc.grad(scheme, phi)
    oc.param("limiter", kind)
    gk = oc.grad(scheme, phi)
    nC = oc.numCells
    assert not np.array_equal(gk[:3 * nC], g0[:3 * nC])  # the front is limited somewhere
    got = run_replay(replay, oc, phi, g0, kind, tmp_path)
    assert np.array_equal(got[:3 * nC], gk[:3 * nC])


@pytest.mark.parametrize("kind", [1, 2, 3])
def test_scaling_limiters_scale_by_at_most_one(oracle, kind):
    oc, phi = case(oracle, False, seed=5)
    g0 = oc.grad(0, phi).reshape(-1, 3)[:oc.numCells]
    oc.param("limiter", kind)
    gk = oc.grad(0, phi).reshape(-1, 3)[:oc.numCells]
    n0 = np.linalg.norm(g0, axis=1)
    s = np.linalg.norm(gk, axis=1) / np.where(n0 > 0, n0, 1.0)
    assert s.min() >= 0.0 and s.max() <= 1.0 + 1e-15
    # each cell's gradient keeps its direction
    dots = (g0 * gk).sum(axis=1)
    assert (dots >= -1e-300).all()


def test_barth_jespersen_bounds_the_neighbour_extrapolations(oracle):
    """Barth-Jespersen: phi_c + g.(x_n - x_c) stays within the global
    extremes of phi over the cells (where |g.d| >= 1e-6)."""
    oc, phi = case(oracle, False, seed=9)
    oc.param("limiter", 1)
    g = oc.grad(0, phi).reshape(-1, 3)
    nC = oc.numCells
    lo, hi = phi[:nC].min(), phi[:nC].max()
    ia, ja, dg = oc.get_int("ia") - 1, oc.get_int("ja") - 1, oc.get_int("diag") - 1
    x = np.stack([oc.get("xc"), oc.get("yc"), oc.get("zc")], axis=1)
    for c in range(nC):
        for k in range(ia[c], ia[c + 1]):
            if k == dg[c]:
                continue
            v = phi[c] + g[c] @ (x[ja[k]] - x[c])
            assert lo - 1e-12 <= v <= hi + 1e-12


def test_limiter_none_is_identity(oracle):
    oc, phi = case(oracle, True)
    g0 = oc.grad(1, phi)
    oc.param("limiter", 0)
    assert np.array_equal(oc.grad(1, phi), g0)
