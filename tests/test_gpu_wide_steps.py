"""Sweep steps as wide as the staging of the solves allows, on 60^3 x 6
tetrahedra (1,296,000 cells).  The factor setups and applications stage
two of the widest steps in shared memory, the Gauss-Seidel sweep (which
stages the upper triangle as well) does not.
ICCG and BiCGStab therefore run on the unsplit levels, and the first
Gauss-Seidel solve analyses the pattern again for a staging that suits it
(fewer staged rows per step, the further rows read from global memory, or
narrower steps).  Iterates agree with the oracle in every case."""
import numpy as np
import pytest

from gpu_cases import laplacian_system, mesh_case

pytestmark = pytest.mark.gpu

FIELD_RTOL = 1e-9


def test_wide_steps_and_gauss_seidel_reanalysis(ctx, oracle):
    m, a, oc = mesh_case("tet60", 60, 60, 60, tets=True)
    ctx.set_mesh(m)  # the csrsolve pattern below is the mesh's: its tiles are cut with the cell centroids
    ia, ja, av, dg, b = laplacian_system(oc, mask=0b1)
    ctx.pattern_forget()
    # 640 staged rows leave the setups and applications two stage buffers
    # each but not the Gauss-Seidel sweep, whose solve then re-analyses
    ctx.set_sweep_stage_rows(640)
    widths = {}
    try:
        runs = _runs(ctx, oracle, ia, ja, av, dg, b)
    finally:
        ctx.set_sweep_stage_rows(0)
    for solver, st in runs:
        widths.setdefault(solver, []).append(st)
    ctx.pattern_forget()
    assert widths["bicgstab"][0] == widths["iccg"][0]
    # the Gauss-Seidel solve left a structure with less staged per step
    # (narrower steps, or fewer staged rows of the widest ones) behind, which
    # later solves keep
    (w0, s0), (wg, sg) = widths["iccg"][0], widths["gauss-seidel"][0]
    assert wg < w0 or 0 < sg < (s0 or w0)
    assert widths["iccg"][1] == widths["gauss-seidel"][0]


def _runs(ctx, oracle, ia, ja, av, dg, b):
    out = []
    for solver, itr in (("iccg", 20), ("bicgstab", 6), ("gauss-seidel", 4), ("iccg", 20)):
        xo, r0o, info_o, _ = oracle.solve(solver, ia, ja, av, dg, np.zeros(len(dg)), b, itr, 0.0, 1e-30)
        x, r0, info, st = ctx.csrsolve(solver, ia, ja, av, dg, np.zeros(len(dg)), b, itr, 0.0, 1e-30)
        assert st >= 0, solver
        assert info.itr_used == int(info_o[0]), solver
        assert np.abs(x - xo).max() <= FIELD_RTOL * np.abs(xo).max(), solver
        assert r0 == pytest.approx(r0o, rel=1e-12), solver
        st = ctx.sweep_stats(1)
        out.append((solver, (st["max_width"], st["staged_rows"])))
    return out
