"""Steps wider than the rows the stage buffers hold.  A step then stages its
first rows only and reads the others (row and coefficient records,
right-hand side and extra row values, push targets) from global memory, the
path wide tetrahedral meshes take instead of splitting their levels.  Forced
here with 8 staged rows on small meshes cut into few tiles, whose widest
steps have several times as many rows, against the oracle: the DIC and DILU factors bit for
bit, the iterates of the ordered-sweep solvers, the FP32 mixed ICCG."""
import numpy as np
import pytest

from gpu_cases import laplacian_system, mesh_case, nonsymmetric_values

pytestmark = pytest.mark.gpu

STAGED = 8


# few tiles, so that the steps of these small meshes are wider than STAGED
TILES = {"hex": 2, "tet": 8}


@pytest.fixture
def staged(ctx):
    ctx.set_sweep_stage_rows(STAGED)
    ctx.pattern_forget()
    try:
        yield ctx
    finally:
        ctx.set_sweep_stage_rows(0)
        ctx.set_sweep_tiles(0)
        ctx.pattern_forget()


@pytest.mark.parametrize("mesh", ["hex", "tet"])
@pytest.mark.parametrize("kind", ["dic", "dilu"])
def test_factors_with_unstaged_rows(staged, oracle, mesh, kind):
    ctx = staged
    ctx.set_sweep_tiles(TILES[mesh])
    m, a, oc = mesh_case(mesh, 9, 7, 6, tets=(mesh == "tet"))
    if kind == "dic":
        ia, ja, av, dg, b = laplacian_system(oc, mask=0b1)
    else:
        ia, ja, av, dg = nonsymmetric_values(oc)
        b = np.random.default_rng(9).standard_normal(len(dg))
    d_gpu = ctx.precond_setup(kind, ia, ja, av, dg)
    st = ctx.sweep_stats(1)
    assert st["staged_rows"] == STAGED and st["max_width"] > STAGED
    d_ref = oracle.dic_setup(ia, ja, av, dg, dilu=(kind == "dilu"))
    assert np.array_equal(d_gpu, d_ref)
    z_gpu = ctx.precond_apply(kind, ia, ja, av, dg, b)
    z_ref = oracle.precond_apply(ia, ja, av, dg, d_ref, b)
    np.testing.assert_allclose(z_gpu, z_ref, rtol=1e-13, atol=1e-13 * np.abs(z_ref).max())


@pytest.mark.parametrize("solver,itr", [("iccg", 30), ("gauss-seidel", 25), ("bicgstab", 15)])
@pytest.mark.parametrize("mesh", ["hex", "tet"])
def test_iterates_with_unstaged_rows(staged, oracle, solver, itr, mesh):
    ctx = staged
    ctx.set_sweep_tiles(TILES[mesh])
    m, a, oc = mesh_case(mesh, 9, 7, 6, tets=(mesh == "tet"))
    if solver in ("iccg", "gauss-seidel"):
        ia, ja, av, dg, b = laplacian_system(oc, mask=0b1)
    else:
        ia, ja, av, dg = nonsymmetric_values(oc)
        b = np.random.default_rng(3).standard_normal(len(dg))
    x0 = np.random.default_rng(4).standard_normal(len(dg)) * 0.1
    args = (ia, ja, av, dg, x0, b, itr, 1e-30, 1e-30)
    xo, r0o, info_o, _ = oracle.solve(solver, *args)
    x, r0, info, st = ctx.csrsolve(solver, *args)
    assert ctx.sweep_stats(1)["staged_rows"] == STAGED
    assert st >= 0 and info.itr_used == int(info_o[0])
    np.testing.assert_allclose(x, xo, rtol=1e-9, atol=1e-9 * np.abs(xo).max())
    assert r0 == pytest.approx(r0o, rel=1e-12)


def test_mixed_iccg_with_unstaged_rows(staged, oracle, fc):
    ctx = staged
    ctx.set_sweep_tiles(TILES["tet"])
    m, a, oc = mesh_case("hexm", 14, 12, 10)
    ia, ja, av, dg, b = laplacian_system(oc, mask=0b1)
    xo, _, _, _ = oracle.solve("iccg", ia, ja, av, dg, np.zeros(len(dg)), b, 5000, 0.0, 1e-10)
    ctx.set_precision(fc.FC_PREC_MIXED, 1e-4, 0)
    try:
        x, _, info, st = ctx.csrsolve("iccg", ia, ja, av, dg, np.zeros(len(dg)), b, 5000, 0.0, 1e-10)
    finally:
        ctx.set_precision(fc.FC_PREC_FP64)
    assert st == 0 and ctx.sweep_stats(1)["staged_rows"] == STAGED
    assert np.abs(x - xo).max() <= 1e-7 * np.abs(xo).max()
