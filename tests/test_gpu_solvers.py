"""GPU solvers vs the oracle (the CPU restatement of linear_solvers.f90).

Tolerances: the DIC/DILU factors, the ILU(0) factors, A^T x and the
Gauss-Seidel sweep follow the reference's recurrences operation by operation
without FMA contraction, so they are compared bit for bit.  The triangular
sweeps of the preconditioner application accumulate with FMA (same order of
terms), so z = M^-1 q agrees to a few ulps.  Solver results
differ only through the order of the FP64 dot/norm reductions and FMA in
A*x: iterates agree to 1e-9 relative after tens of iterations and the
converged fields to 1e-8 relative (the required bar).
"""
import json

import numpy as np
import pytest

from conftest import golden_path
from gpu_cases import laplacian_system, mesh_case, nonsymmetric_values

pytestmark = pytest.mark.gpu
KAT = json.load(open(golden_path("spsolve_5x5.json")))


@pytest.mark.parametrize("system,solver", [("nonsymmetric", "bicgstab"), ("spd", "iccg"), ("spd", "dpcg"),
                                           ("spd", "gauss-seidel")])
def test_reference_5x5_systems(ctx, oracle, system, solver):
    s = KAT[system]
    itr = KAT["itr_max_gauss_seidel"] if solver == "gauss-seidel" else KAT["itr_max"]
    args = (s["ia"], s["ja"], s["a"], s["diag"], np.zeros(5), s["b"], itr, KAT["tol_abs"], KAT["tol_rel"])
    xo, r0o, info_o, _ = oracle.solve(solver, *args)
    x, r0, info, st = ctx.csrsolve(solver, *args)
    assert st >= 0
    np.testing.assert_allclose(x, xo, rtol=1e-9, atol=1e-12)
    assert info.itr_used == int(info_o[0])
    np.testing.assert_allclose(x, s["x_expected"], atol=0.006)
    assert r0 == pytest.approx(r0o, rel=1e-12)


def test_reference_5x5_gmres_as_written(ctx, oracle):
    """pmgmres_ilu on the nonsymmetric 5x5 system: with a full pattern the
    ILU(0) is the exact LU, the Arnoldi process breaks down after one step
    and the reference's unnormalised start vector (rho taken before the
    preconditioner, linear_solvers.f90:970-978) leaves the answer to
    rounding noise.  Both the oracle and the GPU reproduce that: neither
    reaches the printed solution, and both report the same first residual."""
    s = KAT["nonsymmetric"]
    args = (s["ia"], s["ja"], s["a"], s["diag"], np.zeros(5), s["b"], KAT["itr_max"], KAT["tol_abs"], KAT["tol_rel"])
    xo, r0o, info_o, _ = oracle.solve("pmgmres", *args)
    x, r0, info, st = ctx.csrsolve("pmgmres", *args)
    assert st >= 0 and np.all(np.isfinite(x))
    assert np.abs(x - np.array(s["x_expected"])).max() > 1.0
    assert np.abs(xo - np.array(s["x_expected"])).max() > 1.0
    assert info.res0_l1 == pytest.approx(info_o[1], rel=1e-12)


@pytest.mark.parametrize("mesh", ["hex", "tet"])
@pytest.mark.parametrize("kind", ["dic", "dilu"])
def test_preconditioner_factors_bit_exact(ctx, oracle, mesh, kind):
    m, a, oc = mesh_case(mesh, 9, 7, 6, tets=(mesh == "tet"))
    if kind == "dic":
        ia, ja, av, dg, b = laplacian_system(oc, mask=0b1)
    else:
        ia, ja, av, dg = nonsymmetric_values(oc)
        b = np.random.default_rng(9).standard_normal(len(dg))
    d_gpu = ctx.precond_setup(kind, ia, ja, av, dg)
    d_ref = oracle.dic_setup(ia, ja, av, dg, dilu=(kind == "dilu"))
    assert np.array_equal(d_gpu, d_ref)
    z_gpu = ctx.precond_apply(kind, ia, ja, av, dg, b)
    z_ref = oracle.precond_apply(ia, ja, av, dg, d_ref, b)
    np.testing.assert_allclose(z_gpu, z_ref, rtol=1e-13, atol=1e-13 * np.abs(z_ref).max())


def test_spmv_and_transpose(ctx, oracle):
    m, a, oc = mesh_case("hex", 9, 7, 6)
    ia, ja, av, dg = nonsymmetric_values(oc)
    x = np.random.default_rng(1).standard_normal(len(dg))
    y = ctx.spmv(ia, ja, av, dg, x)
    np.testing.assert_allclose(y, oracle.spmv(ia, ja, av, x), rtol=1e-14, atol=1e-14)
    yt = ctx.spmv(ia, ja, av, dg, x, transpose=True)
    assert np.array_equal(yt, oracle.spmv(ia, ja, av, x, transpose=True))


def test_ilu0_factors_bit_exact(ctx, oracle):
    m, a, oc = mesh_case("hex", 9, 7, 6)
    ia, ja, av, dg = nonsymmetric_values(oc)
    l_gpu = ctx.ilu0(ia, ja, av, dg)
    l_ref = np.zeros(len(ja))
    L = oracle.lib()
    assert L.orc_ilu0(len(dg), oracle._i32(ia), oracle._i32(ja), oracle._f64(av), oracle._i32(dg), l_ref,
                      np.zeros(len(dg), np.int32)) == 0
    assert np.array_equal(l_gpu, l_ref)


@pytest.mark.parametrize("solver,itr", [("iccg", 30), ("dpcg", 30), ("gauss-seidel", 25), ("bicgstab", 15),
                                        ("pmgmres", 6)])
def test_solver_iterates_match_oracle(ctx, oracle, solver, itr):
    m, a, oc = mesh_case("hex", 9, 7, 6)
    if solver in ("iccg", "dpcg", "gauss-seidel"):
        ia, ja, av, dg, b = laplacian_system(oc, mask=0b1)
    else:
        ia, ja, av, dg = nonsymmetric_values(oc)
        b = np.random.default_rng(3).standard_normal(len(dg))
    x0 = np.random.default_rng(4).standard_normal(len(dg)) * 0.1
    args = (ia, ja, av, dg, x0, b, itr, 1e-30, 1e-30)
    xo, r0o, info_o, _ = oracle.solve(solver, *args)
    x, r0, info, st = ctx.csrsolve(solver, *args)
    assert st >= 0
    assert info.itr_used == int(info_o[0])
    np.testing.assert_allclose(x, xo, rtol=1e-9, atol=1e-9 * np.abs(xo).max())
    assert r0 == pytest.approx(r0o, rel=1e-12)


@pytest.mark.parametrize("mesh", ["hex", "tet"])
def test_converged_iccg_and_bicgstab_fields(ctx, oracle, mesh):
    """Converged fields agree to 1e-8 relative.  Both sides are converged well
    below that (1e-12 relative L1 residual): at 1e-10 the solution itself is
    only defined to about cond(A)*1e-10, so two correct rounding paths may
    already differ by ~1e-8."""
    m, a, oc = mesh_case(mesh + "c", 12, 10, 9, tets=(mesh == "tet"))
    ia, ja, av, dg, b = laplacian_system(oc, mask=0b1)
    for solver in ("iccg", "bicgstab"):
        xo, _, info_o, _ = oracle.solve(solver, ia, ja, av, dg, np.zeros(len(dg)), b, 4000, 0.0, 1e-12)
        x, _, info, st = ctx.csrsolve(solver, ia, ja, av, dg, np.zeros(len(dg)), b, 4000, 0.0, 1e-12)
        assert st == 0
        # BiCGStab's iteration count near 1e-12 follows the rounding; the
        # converged fields are what must agree
        if solver == "iccg":
            assert abs(info.itr_used - int(info_o[0])) <= max(2, int(0.05 * info_o[0]))
        assert np.abs(x - xo).max() <= 1e-8 * np.abs(xo).max()


def test_mixed_precision_reaches_fp64_tolerance(ctx, oracle):
    m, a, oc = mesh_case("hexm", 14, 12, 10)
    ia, ja, av, dg, b = laplacian_system(oc, mask=0b1)
    xo, _, _, _ = oracle.solve("iccg", ia, ja, av, dg, np.zeros(len(dg)), b, 5000, 0.0, 1e-10)
    ctx.set_precision(1, 1e-4, 0)
    try:
        x, _, info, st = ctx.csrsolve("iccg", ia, ja, av, dg, np.zeros(len(dg)), b, 5000, 0.0, 1e-10)
    finally:
        ctx.set_precision(0)
    assert st == 0 and info.outer_iterations >= 2
    # reached the reference's stopping criterion in FP64
    r = b - oracle.spmv(ia, ja, av, x)
    assert np.abs(r).sum() / info.res0_l1 < 1e-10
    assert np.abs(x - xo).max() <= 1e-7 * np.abs(xo).max()


@pytest.mark.parametrize("mode", ["mixed", "fp64"])
@pytest.mark.parametrize("case", ["hex", "tet"])
def test_mixed_coloured_reaches_fp64_tolerance(ctx, oracle, fc, case, mode):
    """FC_PREC_MIXED_COLOURED: the FP32 inner ICCG runs on the multicolour
    ordering (2 colours on hexes, more on tets); the FP64 refinement still
    stops on the reference's criterion, so the answer is the FP64 one.
    FC_PREC_COLOURED_FP64 runs the same inner solve in FP64."""
    if case == "hex":
        m, a, oc = mesh_case("hexm", 14, 12, 10)
    else:
        m, a, oc = mesh_case("tetm", 7, 6, 5, tets=True)
    ia, ja, av, dg, b = laplacian_system(oc, mask=0b1)
    xo, _, _, _ = oracle.solve("iccg", ia, ja, av, dg, np.zeros(len(dg)), b, 5000, 0.0, 1e-10)
    ctx.set_precision(fc.FC_PREC_MIXED_COLOURED if mode == "mixed" else fc.FC_PREC_COLOURED_FP64, 1e-5, 0)
    try:
        x, _, info, st = ctx.csrsolve("iccg", ia, ja, av, dg, np.zeros(len(dg)), b, 5000, 0.0, 1e-10)
        # same pattern, new values: the colour-ordered factor is rebuilt
        av2 = av * 1.7
        av2[dg - 1] += 0.05
        x2, _, info2, st2 = ctx.csrsolve("iccg", ia, ja, av2, dg, np.zeros(len(dg)), b, 5000, 0.0, 1e-10)
    finally:
        ctx.set_precision(0)
    assert st == 0 and info.outer_iterations >= 2
    r = b - oracle.spmv(ia, ja, av, x)
    assert np.abs(r).sum() / info.res0_l1 < 1e-10
    assert np.abs(x - xo).max() <= 1e-7 * np.abs(xo).max()
    assert st2 == 0
    r2 = b - oracle.spmv(ia, ja, av2, x2)
    assert np.abs(r2).sum() / info2.res0_l1 < 1e-10


@pytest.mark.parametrize("solver", ["iccg", "bicgstab", "gauss-seidel"])
def test_capped_sweep_steps_keep_the_preconditioner(ctx, oracle, fc, solver):
    """Sweep steps capped at 3 rows (levels split into consecutive steps, the
    path wide tetrahedral meshes take): same iterations and fields as the
    oracle."""
    m, a, oc = mesh_case("hexcap", 9, 8, 7)
    ia, ja, av, dg, b = laplacian_system(oc, mask=0b1)
    if solver == "bicgstab":
        _, _, av, _ = nonsymmetric_values(oc)
    itr = 40
    xo, _, info_o, _ = oracle.solve(solver, ia, ja, av, dg, np.zeros(len(dg)), b, itr, 0.0, 1e-30)
    ctx.set_sweep_cap(3)
    ctx.pattern_forget()
    try:
        x, _, info, st = ctx.csrsolve(solver, ia, ja, av, dg, np.zeros(len(dg)), b, itr, 0.0, 1e-30,
                                      raise_on_error=False)
        assert ctx.sweep_stats(1)["max_width"] <= 3
    finally:
        ctx.set_sweep_cap(0)
        ctx.pattern_forget()
    assert st >= 0 and info.itr_used == int(info_o[0])
    assert np.abs(x - xo).max() <= 1e-9 * np.abs(xo).max()


def test_failure_detection_nan_rhs(ctx, fc):
    m, a, oc = mesh_case("hex", 9, 7, 6)
    ia, ja, av, dg, b = laplacian_system(oc, mask=0b1)
    b = b.copy()
    b[5] = np.nan
    x, r0, info, st = ctx.csrsolve("iccg", ia, ja, av, dg, np.zeros(len(dg)), b, 50, 0.0, 1e-8,
                                   raise_on_error=False)
    assert st == fc.FC_ERR_NAN
    # the context stays usable afterwards
    ia, ja, av, dg, b = laplacian_system(oc, mask=0b1)
    x, r0, info, st = ctx.csrsolve("iccg", ia, ja, av, dg, np.zeros(len(dg)), b, 50, 0.0, 1e-8)
    assert st >= 0


def test_failure_detection_bad_pattern_and_zero_pivot(ctx, fc):
    ia = np.array([1, 2, 3], np.int32)
    ja = np.array([1, 3], np.int32)  # column out of range
    with pytest.raises(fc.FcError) as e:
        ctx.csrsolve("iccg", ia, ja, [1.0, 1.0], np.array([1, 2], np.int32), np.zeros(2), np.ones(2), 5, 0, 1e-6)
    assert e.value.code == fc.FC_ERR_BAD_INPUT
    ia = np.array([1, 3, 5], np.int32)
    ja = np.array([1, 2, 1, 2], np.int32)
    with pytest.raises(fc.FcError) as e:
        ctx.ilu0(ia, ja, [0.0, 1.0, 1.0, 1.0], np.array([1, 4], np.int32))
    assert e.value.code == fc.FC_ERR_ZERO_PIVOT
