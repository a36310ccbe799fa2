"""The FP32 inner BiCGStab of the mixed-precision solves against its CPU
replay (tests/replay/bicgstab32_replay.cpp: the reference's DILU-BiCGStab,
linear_solvers.f90:548-786, with FP32 matrix, factors and vectors and FP64
dots, the device's precision split), on problem 11 of the batched
convection-diffusion configuration (72^3 cells, cell Peclet 0.55):

  - the iterates after k = 1..6 iterations from dx = 0, single solve
    (fc_csrsolve in FC_PREC_MIXED with the inner solve capped at k) and
    batched (fc_batch_solve), agree with the replay's to FP32 rounding;
  - the first inner solve to the relative tolerance 1e-4 takes the
    replay's iteration count, single and batched;
  - the whole FP64 refinement to 1e-6 takes the replay's refinement steps
    and inner iterations.  FP32 BiCGStab as the reference writes it stalls
    on the second refinement system of this problem (its recurrence
    residual stays near 5e-4 of the inner right-hand side, while the FP64
    residual is already at 1e-7): the replay and the device both end such an
    inner solve by the same stagnation rule (STALL_WINDOW)."""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

from cd_cases import cd_batch_sizes, cd_batch_system
from conftest import load_fcgpu

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
PROBLEM = 11
ITERATE_TOL = 1e-4     # max |x_gpu - x_replay| / max |x_replay| after k FP32 iterations
COUNT_SLACK = 2        # iterations to 1e-4: FP32 rounding of the dot partners only
STALL_WINDOW = 32      # the device's inner-solve stagnation stop (FC_INNER_STALL_WINDOW)


@pytest.fixture(scope="module")
def replay(tmp_path_factory):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not available")
    so = str(tmp_path_factory.mktemp("bicg32") / "libbicgstab32_replay.so")
    subprocess.run([gxx, "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-shared",
                    os.path.join(HERE, "replay", "bicgstab32_replay.cpp"), "-o", so], check=True)
    L = C.CDLL(so)
    fp = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
    ip = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
    dp = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
    L.bicgstab32.restype = C.c_int
    L.bicgstab32.argtypes = [C.c_int, ip, ip, fp, ip, fp, fp, C.c_int, C.c_double, C.c_int, dp]

    def run(ia, ja, a, dg, b, itr_max, tol_rel, stall_window=STALL_WINDOW):
        x = np.zeros(len(dg), np.float32)
        hist = np.zeros(itr_max + 1)
        used = L.bicgstab32(len(dg), ia.astype(np.int32), ja.astype(np.int32), a.astype(np.float32),
                            dg.astype(np.int32), x, b.astype(np.float32), itr_max, tol_rel, stall_window, hist)
        return x.astype(np.float64), used, hist
    return run


@pytest.fixture(scope="module")
def problem():
    fc = load_fcgpu()
    ns, pe = cd_batch_sizes(64)
    gen = fc.Context(0)
    try:
        pr = cd_batch_system(fc, gen, int(ns[PROBLEM]), float(pe[PROBLEM]), 42 + PROBLEM)
    finally:
        gen.close()
    return pr


def gpu_single(fc, ctx, pr, itr_max, inner_tol, tol_rel):
    ia, ja, dg, a, b, _ = pr
    ctx.set_precision(fc.FC_PREC_MIXED, inner_tol, itr_max)
    try:
        x, _, info, st = ctx.csrsolve("bicgstab", ia, ja, a, dg, np.zeros(len(dg)), b, itr_max, 0.0, tol_rel)
    finally:
        ctx.set_precision(fc.FC_PREC_FP64)
    return x, info


def gpu_batched(fc, ctx, pr, itr_max, inner_tol, tol_rel):
    ia, ja, dg, a, b, xyz = pr
    ctx.set_precision(fc.FC_PREC_MIXED, inner_tol, itr_max)
    B = fc.Batch(ctx)
    try:
        B.add(ia, ja, dg, xyz)
        B.plan()
        xs, infos, st = B.solve([a], [np.zeros(len(dg))], [b], itr_max, 0.0, tol_rel, raise_on_error=False)
    finally:
        B.close()
        ctx.set_precision(fc.FC_PREC_FP64)
    return xs[0], infos[0]


@pytest.mark.parametrize("path", ["single", "batched"])
def test_fp32_bicgstab_iterates_match_replay(ctx, fc, replay, problem, path):
    ia, ja, dg, a, b, _ = problem
    run = gpu_single if path == "single" else gpu_batched
    for k in range(1, 7):
        x_ref, used, _ = replay(ia, ja, a, dg, b, k, 1e-30)
        assert used == k
        # one refinement step whose inner solve stops after k iterations: x = dx_k
        x, info = run(fc, ctx, problem, k, 1e-30, 1e-30)
        assert info.itr_used == k, (path, k, info.itr_used)
        err = np.abs(x - x_ref).max() / np.abs(x_ref).max()
        assert err <= ITERATE_TOL, f"{path}: after {k} FP32 iterations max rel diff {err:.3e}"


@pytest.mark.parametrize("path", ["single", "batched"])
def test_fp32_bicgstab_inner_count_matches_replay(ctx, fc, replay, problem, path):
    ia, ja, dg, a, b, _ = problem
    _, used, hist = replay(ia, ja, a, dg, b, 1000, 1e-4)
    run = gpu_single if path == "single" else gpu_batched
    # outer tolerance 0.5: the refinement loop stops after the first inner solve
    x, info = run(fc, ctx, problem, 1000, 1e-4, 0.5)
    assert info.outer_iterations == 1, info.outer_iterations
    assert abs(info.itr_used - used) <= COUNT_SLACK, f"{path}: GPU {info.itr_used} iterations, replay {used}"


def replay_refinement(replay, pr, inner_tol, tol_rel, itr_max=4000, max_outer=64):
    """The mixed solve's FP64 refinement around the FP32 replay: r = b - A x
    in FP64, inner FP32 solve of A dx = (float) r from dx = 0 to inner_tol,
    x += dx, until L1(r) / L1(r_0) < tol_rel.  Returns (inner counts, x)."""
    import scipy.sparse as sp
    ia, ja, dg, a, b, _ = pr
    n = len(dg)
    A = sp.csr_matrix((a, ja - 1, ia - 1), shape=(n, n))
    x = np.zeros(n)
    counts, res0 = [], None
    for _ in range(max_outer):
        r = b - A @ x
        resl = np.abs(r).sum()
        if res0 is None:
            res0 = resl
        elif resl / (res0 + 1e-20) < tol_rel:
            break
        dx, used, _ = replay(ia, ja, a, dg, r, itr_max, inner_tol)
        counts.append(used)
        x += dx
    return counts, x


@pytest.mark.parametrize("path", ["single", "batched"])
def test_fp32_bicgstab_refinement_matches_replay(ctx, fc, replay, problem, path):
    """The whole refinement to 1e-6 (inner solves to 1e-4): the same number
    of refinement steps and inner iterations as the replay (the device's FP32
    path follows its own algorithm)."""
    counts, x_ref = replay_refinement(replay, problem, 1e-4, 1e-6)
    ia, ja, dg, a, b, _ = problem
    ctx.set_precision(fc.FC_PREC_MIXED, 1e-4, 0)
    try:
        if path == "single":
            x, _, info, st = ctx.csrsolve("bicgstab", ia, ja, a, dg, np.zeros(len(dg)), b, 4000, 0.0, 1e-6)
        else:
            B = fc.Batch(ctx)
            B.add(ia, ja, dg, problem[5])
            B.plan()
            xs, infos, st = B.solve([a], [np.zeros(len(dg))], [b], 4000, 0.0, 1e-6)
            B.close()
            x, info = xs[0], infos[0]
    finally:
        ctx.set_precision(fc.FC_PREC_FP64)
    assert info.status == 0
    assert info.outer_iterations == len(counts), (path, info.outer_iterations, counts)
    assert abs(info.itr_used - sum(counts)) <= COUNT_SLACK * len(counts), (path, info.itr_used, counts)
    assert np.abs(x - x_ref).max() <= 1e-5 * np.abs(x_ref).max()
