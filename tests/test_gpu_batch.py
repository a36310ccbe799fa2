"""Batched solves (fc_batch_*) on the GPU, on small problems of the batched
convection-diffusion configuration (tests/cd_cases.py).

- FP64: each problem's iterates in a batch are those of the same problem
  solved alone with the same tile count (bit for bit: the group runs the
  single-problem kernel code on its own blocks, barrier and reductions), and
  the solutions agree with sparse direct solves.
- Mixed (FP32 inner BiCGStab inside FP64 refinement, per problem): every
  problem reaches the FP64 stopping test and the direct solution.
- A failing problem (NaN right-hand side) reports its error alone; the others
  are unchanged bit for bit.
- Planner and tuner: plans stay within the resident blocks, tuning leaves x0
  alone and its plan solves to the same answers."""
import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from cd_cases import cd_batch_system
from conftest import load_fcgpu

pytestmark = pytest.mark.gpu

# cells per side, cell Peclet number
SIZES = [(12, 0.5), (16, 2.0), (10, 1.0), (14, 4.0)]
TILES = [3, 5, 2, 4]
TOL = 1e-9


@pytest.fixture(scope="module")
def bctx():
    fc = load_fcgpu()
    c = fc.Context(0)
    yield fc, c
    c.close()


@pytest.fixture(scope="module")
def problems(bctx):
    fc, c = bctx
    return [cd_batch_system(fc, c, n, pe, seed=100 + k) for k, (n, pe) in enumerate(SIZES)]


def direct(pr):
    ia, ja, dg, a, b, _ = pr
    n = len(dg)
    A = sp.csr_matrix((a, ja - 1, ia - 1), shape=(n, n))
    return spla.spsolve(A.tocsc(), b)


def make_batch(fc, c, probs, tiles):
    B = fc.Batch(c)
    for ia, ja, dg, a, b, xyz in probs:
        B.add(ia, ja, dg, xyz)
    B.plan(tiles)
    return B


def solve(B, probs, rhs=None, itr=2000, tol=TOL, raise_on_error=True):
    a = [p[3] for p in probs]
    b = rhs if rhs is not None else [p[4] for p in probs]
    x0 = [np.zeros(len(p[2])) for p in probs]
    return B.solve(a, x0, b, itr, 0.0, tol, raise_on_error=raise_on_error)


def test_fp64_batch_equals_single_groups_and_direct(bctx, problems):
    fc, c = bctx
    c.set_precision(fc.FC_PREC_FP64)
    B = make_batch(fc, c, problems, TILES)
    assert list(B.tiles()) == TILES
    xs, infos, st = solve(B, problems)
    assert st == 0
    for k, pr in enumerate(problems):
        assert infos[k].status == 0 and infos[k].resl / infos[k].res0_l1 < TOL
        B1 = make_batch(fc, c, [pr], [TILES[k]])
        x1, i1, _ = solve(B1, [pr])
        assert np.array_equal(xs[k], x1[0]), k
        assert (infos[k].itr_used, infos[k].resl, infos[k].res0_l1) == (i1[0].itr_used, i1[0].resl, i1[0].res0_l1)
        xd = direct(pr)
        assert np.abs(xs[k] - xd).max() <= 1e-6 * np.abs(xd).max(), k
        B1.close()
    # deterministic from run to run
    xs2, _, _ = solve(B, problems)
    assert all(np.array_equal(u, v) for u, v in zip(xs, xs2))
    B.close()


def test_fp64_batch_matches_csrsolve(bctx, problems):
    fc, c = bctx
    c.set_precision(fc.FC_PREC_FP64)
    B = make_batch(fc, c, problems, None)
    xs, infos, _ = solve(B, problems)
    for k, (ia, ja, dg, a, b, _) in enumerate(problems):
        x, _, info, st = c.csrsolve("bicgstab", ia, ja, a, dg, np.zeros(len(dg)), b, 2000, 0.0, TOL)
        assert st == 0
        assert np.abs(xs[k] - x).max() <= 1e-7 * np.abs(x).max(), k
    B.close()


def test_mixed_batch_reaches_fp64_tolerance(bctx, problems):
    fc, c = bctx
    c.set_precision(fc.FC_PREC_MIXED, 1e-4, 0)
    try:
        B = make_batch(fc, c, problems, TILES)
        xs, infos, st = solve(B, problems)
        assert st == 0
        for k, pr in enumerate(problems):
            assert infos[k].status == 0, k
            assert infos[k].outer_iterations >= 2
            assert infos[k].resl / infos[k].res0_l1 < TOL
            xd = direct(pr)
            assert np.abs(xs[k] - xd).max() <= 1e-6 * np.abs(xd).max(), k
        B.close()
    finally:
        c.set_precision(fc.FC_PREC_FP64)


@pytest.mark.parametrize("mode", ["fp64", "mixed"])
def test_failing_problem_is_isolated(bctx, problems, mode):
    fc, c = bctx
    c.set_precision(fc.FC_PREC_FP64 if mode == "fp64" else fc.FC_PREC_MIXED, 1e-4, 0)
    try:
        B = make_batch(fc, c, problems, TILES)
        good, _, _ = solve(B, problems)
        rhs = [p[4].copy() for p in problems]
        rhs[1][7] = np.nan
        xs, infos, st = solve(B, problems, rhs=rhs, raise_on_error=False)
        assert st == fc.FC_ERR_NAN
        assert infos[1].status == fc.FC_ERR_NAN
        for k in (0, 2, 3):
            assert infos[k].status == 0
            assert np.array_equal(xs[k], good[k]), k
        B.close()
    finally:
        c.set_precision(fc.FC_PREC_FP64)


def test_plan_and_tune(bctx, problems):
    fc, c = bctx
    c.set_precision(fc.FC_PREC_FP64)
    B = make_batch(fc, c, problems, None)
    t_model = B.tiles()
    assert t_model.min() >= 1
    a = [p[3] for p in problems]
    b = [p[4] for p in problems]
    x0 = [np.full(len(p[2]), 0.25) for p in problems]
    keep = [v.copy() for v in x0]
    tiles, ms = B.tune(a, x0, b, 2000, 0.0, TOL, rounds=3)
    assert ms > 0 and tiles.min() >= 1
    assert all(np.array_equal(u, v) for u, v in zip(x0, keep))
    xs, infos, st = B.solve(a, x0, b, 2000, 0.0, TOL)
    assert st == 0
    for k, pr in enumerate(problems):
        xd = direct(pr)
        assert np.abs(xs[k] - xd).max() <= 1e-6 * np.abs(xd).max(), k
    # the tuned plan is cached for these sizes: a new batch plans to it
    B2 = make_batch(fc, c, problems, None)
    assert list(B2.tiles()) == list(tiles)
    B.close()
    B2.close()


def test_plan_rejects_more_blocks_than_resident(bctx, problems):
    fc, c = bctx
    B = fc.Batch(c)
    for ia, ja, dg, a, b, xyz in problems[:2]:
        B.add(ia, ja, dg, xyz)
    with pytest.raises(fc.FcError) as e:
        B.plan([100000, 1])
    assert e.value.code == fc.FC_ERR_UNSUPPORTED
    B.close()
