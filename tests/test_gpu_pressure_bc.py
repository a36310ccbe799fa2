"""Pressure boundaries in the SIMPLE path on the GPU against the oracle, on
a channel with a velocity inlet and a p = 0 outlet (tests/channel_cases.py):
the pressure-correction matrix with the pressure faces' diagonal terms
(facefluxmassPressBnd, faceflux_mass.f90:765-830) bit for bit, the fields and
mass fluxes after calcp_simple (the solve, facefluxmassCorrPressBnd :699-762
and p' = 0 as the reference value) to the solvers' reduction-order rounding,
and eight SIMPLE iterations tracking the oracle; the PISO corrector still
rejects pressure patches."""
import numpy as np
import pytest

from channel_cases import channel, patch_flux

pytestmark = pytest.mark.gpu


def test_calcp_simple_with_pressure_outlet(ctx, fc, oracle):
    m, a, oc, prm = channel(oracle, ctx=ctx)
    ctx.calcuvw()
    assert oc.L.orc_calcuvw(oc.h) >= 0
    for k in ("u", "v", "w"):
        oc.set(k, ctx.field_get(k))
    r4 = ctx.calcp_simple()
    assert oc.L.orc_calcp_simple(oc.h) >= 0
    assert np.array_equal(ctx.field_get("a"), oc.get("a"))
    for k in ("pp", "p", "u", "v", "w", "flmass"):
        g, o = ctx.field_get(k), oc.get(k)
        assert np.abs(g - o).max() <= 1e-9 * max(1e-300, np.abs(o).max()), k
    nC, nI = m.numCells, m.numInnerFaces
    b1 = a["startFace"][1] - nI
    assert np.all(ctx.field_get("pp")[nC + b1:nC + b1 + a["nfaces"][1]] == 0.0)
    assert r4 == pytest.approx(oc.scalar("resor4"), rel=1e-6)


def test_simple_iterations_with_pressure_outlet_track_oracle(ctx, fc, oracle):
    m, a, oc, prm = channel(oracle, dims=(12, 6, 5), ctx=ctx)
    res_g, res_o = [], []
    for _ in range(8):
        res_g.append(ctx.simple_iteration())
        res_o.append(oc.simple_iteration()[1])
    res_g, res_o = np.array(res_g), np.array(res_o)
    mask = np.abs(res_o) > 1e-12
    np.testing.assert_allclose(res_g[mask], res_o[mask], rtol=1e-7)
    for k in ("u", "v", "w", "p"):
        g, o = ctx.field_get(k), oc.get(k)
        assert np.abs(g - o).max() <= 1e-8 * np.abs(o).max(), k
    fm = ctx.field_get("flmass")
    assert abs(patch_flux(a, fm, 0) + patch_flux(a, fm, 1)) < 1e-3


def test_piso_rejects_pressure_patches(ctx, fc, oracle):
    channel(oracle, dims=(6, 4, 4), ctx=ctx)
    ctx.transient_params(0.01, fc.FC_TIME_BDF, 1, 2)
    try:
        with pytest.raises(fc.FcError) as e:
            ctx.piso_iteration()
    finally:
        ctx.transient_params(1.0, fc.FC_TIME_STEADY, 0, 1)  # the shared context back to steady SIMPLE
    assert e.value.code == fc.FC_ERR_UNSUPPORTED and "PISO" in str(e.value)
