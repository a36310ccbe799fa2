"""Temperature transport on the GPU vs the oracle restatement of
calculate_temperature (ScalarEqns/temperature.f90 with facefluxsc,
scalar_fluxes.f90:32-141 and :256-337, and updateBoundary).

The assembly (matrix, su, sp, dTdxi and the boundary values an adiabatic wall
copies) is bit-exact: face kernel + cell gather in the reference's face order,
no FMA.  The solved field agrees to 1e-9 relative (the Krylov dot products are
reduced in a different order).  The patch layout puts an adiabatic wall before
the isothermal ones, so the isothermal walls read srdw at the wall counter the
reference computes (it counts isothermal wall faces only)."""
import numpy as np
import pytest

from gpu_cases import mesh_case

pytestmark = pytest.mark.gpu

SMALL = float(np.float32(1e-20))


def setup_temperature(ctx, fc, key, sides, bcdf, n=(7, 6, 5), tets=False, seed=11, tneg=False, **kw):
    m, a, oc = mesh_case(key, *n, tets=tets, sides=sides)
    ctx.set_mesh(m)
    nC, nT, nF = m.numCells, m.numTotal, m.numFaces
    rng = np.random.default_rng(seed)
    T = rng.random(nT) + (-0.8 if tneg else 0.5)
    vis = 0.01 + 0.02 * rng.random(nT)
    fm = 0.05 * rng.standard_normal(nF)
    for k, v in (("t", T), ("vis", vis), ("flmass", fm)):
        ctx.field_set(k, v)
        oc.set(k, v)
    ctx.field_fill("dTdxi", 0.0)
    oc.set("dTdxi", np.zeros(3 * nT))
    prm = fc.TemperatureParams.defaults(**kw)
    ctx.temperature_params(prm, np.asarray(bcdf, dtype=np.float64))
    for ib, v in enumerate(bcdf, start=1):
        oc.set_bcdfrac_t(ib, v)
    for name in ("viscos", "pranl", "sigt", "urfT", "gdsT", "cSchemeT", "maxiterT", "tolAbsT", "tolRelT"):
        oc.param(name, getattr(prm, name))
    oc.param("gradScheme", prm.gradScheme)
    if prm.gradScheme:
        oc.L.orc_prepare_lsq(oc.h, prm.gradScheme)
    oc.solver("T", prm.lSolverT.decode())
    return m, oc


# xmin, xmax, ymin, ymax, zmin, zmax
SIDES_FLOW = ["inlet", "outlet", "wall", "wall", "wall", "symmetry"]
BCDF_FLOW = [0, 0, 0, 1, 1, 0]          # ymin adiabatic before two isothermal walls
SIDES_PRESS = ["wall", "pressure", "wall", "wall", "empty", "wall"]
BCDF_PRESS = [1, 0, 0, 1, 0, 0.5]        # 0.5: a wall without a temperature condition

ASSEMBLY_CASES = {
    "hex_lupw": dict(sides=SIDES_FLOW, bcdf=BCDF_FLOW),
    "hex_cds": dict(sides=SIDES_FLOW, bcdf=BCDF_FLOW, scheme=0),
    "hex_central_lsq": dict(sides=SIDES_FLOW, bcdf=BCDF_FLOW, scheme=1, grad=1),
    "hex_muscl_lsqdm": dict(sides=SIDES_FLOW, bcdf=BCDF_FLOW, scheme=10, grad=2),
    "hex_pressure_empty": dict(sides=SIDES_PRESS, bcdf=BCDF_PRESS, gdsT=0.7, sigt=0.9, urfT=0.8),
    "tet": dict(sides=SIDES_FLOW, bcdf=BCDF_FLOW, n=(4, 4, 3), tets=True),
}


@pytest.mark.parametrize("case", list(ASSEMBLY_CASES))
def test_temperature_assembly_bit_exact(ctx, fc, case):
    kw = dict(ASSEMBLY_CASES[case])
    m, oc = setup_temperature(ctx, fc, "sc_" + case + ("_t" if kw.get("tets") else ""), **kw)
    ctx.calculate_temperature(solve=False)
    assert oc.calculate_temperature(solve=False) == 0
    for k in ("a", "su", "sp", "dTdxi", "t"):
        assert np.array_equal(ctx.field_get(k), oc.get(k)), k


@pytest.mark.parametrize("solver", ["bicgstab", "pmgmres", "gauss-seidel"])
def test_temperature_solve_tracks_oracle(ctx, fc, solver):
    m, oc = setup_temperature(ctx, fc, "sc_solve", SIDES_FLOW, BCDF_FLOW, solver=solver, maxiterT=30,
                              tolRelT=1e-6)
    res_g, res_o = [], []
    for it in range(3):
        res_g.append(ctx.calculate_temperature())
        assert oc.calculate_temperature() >= 0
        res_o.append(oc.scalar("resor7"))
    np.testing.assert_allclose(res_g, res_o, rtol=1e-7)
    g, o = ctx.field_get("t"), oc.get("t")
    assert np.abs(g - o).max() <= 1e-9 * np.abs(o).max()
    # updateBoundary: outlet and symmetry faces hold their owners' values
    a = m.arrays()
    own = a["owner"] - 1
    nC, nI = m.numCells, m.numInnerFaces
    for ib in (1, 5):
        st = a["startFace"][ib] - nI
        faces = np.arange(st, st + a["nfaces"][ib])
        assert np.array_equal(g[nC + faces], g[own[faces + nI]]), ib


def test_temperature_clip_to_small(ctx, fc):
    m, oc = setup_temperature(ctx, fc, "sc_clip", SIDES_FLOW, BCDF_FLOW, tneg=True, maxiterT=40, tolRelT=1e-8)
    ctx.calculate_temperature()
    assert oc.calculate_temperature() >= 0
    g, o = ctx.field_get("t"), oc.get("t")
    nC = m.numCells
    assert (o[:nC] == SMALL).any() and (o[:nC] != SMALL).any(), "case does not exercise the clip"
    assert np.array_equal(g[:nC] == SMALL, o[:nC] == SMALL)
    mask = o[:nC] != SMALL
    assert np.abs(g[:nC][mask] - o[:nC][mask]).max() <= 1e-9 * np.abs(o[:nC]).max()


def test_temperature_requires_params_for_current_mesh(ctx, fc):
    m, a, oc = mesh_case("sc_state", 3, 3, 3)
    ctx.set_mesh(m)
    with pytest.raises(fc.FcError):
        ctx.calculate_temperature()
