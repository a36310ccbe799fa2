"""Every device allocation filled with 0xFF bytes (NaN as float and double)
before it is used (fc_debug_fill_allocations): a kernel that reads memory
nothing has written then produces NaN or a breakdown.  On a fresh context
the solvers, the coloured mixed-precision ICCG in both precisions, a batched
mixed solve and SIMPLE with the temperature equation must give the same
answers as on ordinary memory."""
import numpy as np
import pytest

from gpu_cases import laplacian_system, mesh_case, nonsymmetric_values

pytestmark = pytest.mark.gpu


@pytest.fixture
def poisoned(fc):
    fc.debug_fill_allocations(0xFF)
    c = fc.Context(0)
    try:
        yield c
    finally:
        c.close()
        fc.debug_fill_allocations(-1)


def test_solvers_on_poisoned_memory(poisoned, fc, oracle):
    ctx = poisoned
    for key, dims in (("hexm", (14, 12, 10)), ("tetm", (7, 6, 5))):
        m, a, oc = mesh_case(key, *dims, tets=key.startswith("tet"))
        ia, ja, av, dg, b = laplacian_system(oc, mask=0b1)
        xo, _, _, _ = oracle.solve("iccg", ia, ja, av, dg, np.zeros(len(dg)), b, 5000, 0.0, 1e-10)
        for mode in (fc.FC_PREC_FP64, fc.FC_PREC_MIXED, fc.FC_PREC_MIXED_COLOURED, fc.FC_PREC_COLOURED_FP64):
            ctx.set_precision(mode, 1e-5, 0)
            try:
                x, _, info, st = ctx.csrsolve("iccg", ia, ja, av, dg, np.zeros(len(dg)), b, 5000, 0.0, 1e-10)
            finally:
                ctx.set_precision(fc.FC_PREC_FP64)
            assert st == 0, (key, mode)
            assert np.abs(x - xo).max() <= 1e-7 * np.abs(xo).max(), (key, mode)
        nia, nja, nav, ndg = nonsymmetric_values(oc)
        rhs = np.random.default_rng(3).standard_normal(len(ndg))
        for solver in ("bicgstab", "pmgmres", "gauss-seidel", "dpcg"):
            A = (ia, ja, av, dg) if solver in ("gauss-seidel", "dpcg") else (nia, nja, nav, ndg)
            bb = b if solver in ("gauss-seidel", "dpcg") else rhs
            xo, _, info_o, _ = oracle.solve(solver, *A, np.zeros(len(dg)), bb, 12, 1e-30, 1e-30)
            x, _, info, st = ctx.csrsolve(solver, *A, np.zeros(len(dg)), bb, 12, 1e-30, 1e-30)
            assert st >= 0 and info.itr_used == int(info_o[0]), (key, solver)
            assert np.abs(x - xo).max() <= 1e-9 * np.abs(xo).max(), (key, solver)
        ctx.pattern_forget()


def _cavity_run(fc, ctx, n=8, iters=3):
    """SIMPLE iterations of the n^3 lid-driven cavity with the temperature
    equation (hot lid) on ctx: the fields after the last iteration."""
    m = fc.Mesh.box(n, n, n, 1.0, 1.0, 1.0, perturb=0.15, seed=42)
    a = m.arrays()
    nC, nT, nI = m.numCells, m.numTotal, m.numInnerFaces
    lid = 3
    s0 = a["startFace"][lid] - nI
    u, t = np.zeros(nT), np.zeros(nT)
    u[nC + s0:nC + s0 + a["nfaces"][lid]] = 1.0
    t[nC + s0:nC + s0 + a["nfaces"][lid]] = 1.0
    nwal = int(sum(nf for ty, nf in zip(a["bctype"], a["nfaces"]) if ty == 1))
    ctx.set_mesh(m)
    zero = np.zeros(nT)
    for k, v in dict(u=u, v=zero, w=zero, p=zero, pp=zero, den=np.ones(nT), vis=np.full(nT, 0.01), t=t).items():
        ctx.field_set(k, v)
    ctx.field_set("visw", np.full(nwal, 0.01))
    for k in ("flmass", "a", "dUdxi", "dVdxi", "dWdxi", "dPdxi", "dTdxi"):
        ctx.field_fill(k, 0.0)
    ctx.simple_params(fc.SimpleParams.cavity(viscos=0.01))
    bcdf = np.zeros(len(a["bctype"]))
    bcdf[lid] = 1.0
    ctx.temperature_params(fc.TemperatureParams.defaults(), bcdf)
    ctx.init_flmass()
    for _ in range(iters):
        ctx.simple_iteration()
        ctx.calculate_temperature()
    return {k: ctx.field_get(k) for k in ("u", "v", "w", "p", "t", "flmass")}


def test_simple_and_temperature_on_poisoned_memory(ctx, fc):
    ref = _cavity_run(fc, ctx)  # ordinary memory
    fc.debug_fill_allocations(0xFF)
    c = fc.Context(0)
    try:
        got = _cavity_run(fc, c)
    finally:
        c.close()
        fc.debug_fill_allocations(-1)
    for k, v in ref.items():
        assert np.array_equal(got[k], v), k
