"""The Poisson manufactured solution of the reference's Poisson application
(tests/mms_cases.py) on the GPU: the device Laplacian and ICCG give the
oracle's solution (converged fields within FIELD_RTOL) and the same
second-order fall of the L_inf error."""
import numpy as np
import pytest

from mms_cases import EDGES, ITR_MAX, TOL_REL, mms_mesh, oracle_solve, source, exact

pytestmark = pytest.mark.gpu

FIELD_RTOL = 1e-8
ORDER_RATIO = (3.5, 4.5)


def test_poisson_mms_on_the_gpu(ctx, oracle):
    errs = []
    for n in (16, 32):
        m = mms_mesh(n)
        ctx.set_mesh(m)
        nC, nT = m.numCells, m.numTotal
        xc, yc, vol = ctx.geometry("xc"), ctx.geometry("yc"), ctx.geometry("vol")
        ctx.field_set("su", source(xc, yc, vol))
        ctx.laplacian(-np.ones(nC), np.zeros(nT), EDGES)
        ctx.field_fill("pp", 0.0)
        _, _, st = ctx.solve_field("iccg", "pp", "su", ITR_MAX, 0.0, TOL_REL)
        assert st == 0
        x = ctx.field_get("pp")[:nC]
        xo, _, _ = oracle_solve(oracle, n)
        assert np.abs(x - xo).max() <= FIELD_RTOL * np.abs(xo).max()
        errs.append(np.abs(x - exact(xc, yc)).max())
    assert ORDER_RATIO[0] < errs[0] / errs[1] < ORDER_RATIO[1], errs
