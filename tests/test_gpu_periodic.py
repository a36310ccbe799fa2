"""Periodic boundaries on the GPU against the oracle, on a channel periodic
in x and z between a resting and a moving wall (tests/periodic_cases.py),
with the twin patches listed before and after their periodic patches:

  - the mesh after face_mapping (geometry.f90:1848-1997): the twin faces'
    centres and area vectors, the CSR pattern with the pairs and the slot
    maps (sparse_matrix.f90:136-165, :262-292), bit for bit;
  - calcuvw with facefluxuvw_periodic (velocity.f90:393-430, :1038-1179):
    the matrix, sources and diagonals bit for bit, the solved fields to the
    solvers' reduction-order rounding;
  - calcp_simple with facefluxmass2_periodic (calcp_simple.f90:185-225,
    faceflux_mass.f90:313-384) and the pairs' flux correction (:322-342):
    the matrix bit for bit, fields and mass fluxes (the twin faces take the
    periodic faces' fluxes) to the solvers' rounding;
  - calculate_temperature with facefluxsc_periodic (temperature.f90:262-313,
    scalar_fluxes.f90:147-251) and updateBoundary's pair means, bit for bit
    before the solve;
  - SIMPLE iterations and PISO time steps (calcp_piso.f90:248-289,
    :437-456) tracking the oracle."""
import numpy as np
import pytest

from periodic_cases import SIDES, SIDES_TWIN_AFTER, pair_faces, periodic_channel

pytestmark = pytest.mark.gpu

LAYOUTS = {"twin_first": SIDES, "twin_after": SIDES_TWIN_AFTER}
FIELD_TOL = 1e-9
TRACK_RESOR_RTOL = 1e-7
TRACK_FIELD_TOL = 1e-8


@pytest.mark.parametrize("layout", list(LAYOUTS))
def test_periodic_mesh_matches_oracle(ctx, fc, oracle, layout):
    m, a, oc, _ = periodic_channel(oracle, sides=LAYOUTS[layout], ctx=ctx)
    for k in ("xf", "yf", "zf", "arx", "ary", "arz", "xc", "yc", "zc", "vol", "facint", "Df"):
        assert np.array_equal(ctx.geometry(k), oc.get(k)), k
    ia, ja, dg, ijk, jik = ctx.csr_pattern()
    assert len(ja) == oc.nnz == 2 * (oc.numInnerFaces + oc.numPeriodic) + oc.numCells
    for k, v in (("ia", ia), ("ja", ja), ("diag", dg), ("ijk", ijk), ("jik", jik)):
        assert np.array_equal(v, oc.get_int(k)), k


@pytest.mark.parametrize("layout", list(LAYOUTS))
def test_calcuvw_with_periodic_pairs_bit_exact(ctx, fc, oracle, layout):
    m, a, oc, _ = periodic_channel(oracle, sides=LAYOUTS[layout], ctx=ctx)
    r = ctx.calcuvw()
    assert oc.L.orc_calcuvw(oc.h) >= 0
    for k in ("spu", "spv", "sp", "apu", "apv", "apw", "su", "sv", "sw", "a", "dUdxi", "dVdxi", "dWdxi"):
        assert np.array_equal(ctx.field_get(k), oc.get(k)), k
    for k in ("u", "v", "w"):
        g, o = ctx.field_get(k), oc.get(k)
        assert np.abs(g - o).max() <= FIELD_TOL * np.abs(o).max(), k
    np.testing.assert_allclose(r, [oc.scalar("resor1"), oc.scalar("resor2"), oc.scalar("resor3")], rtol=1e-12)


@pytest.mark.parametrize("layout", list(LAYOUTS))
def test_calcp_simple_with_periodic_pairs(ctx, fc, oracle, layout):
    m, a, oc, _ = periodic_channel(oracle, sides=LAYOUTS[layout], ctx=ctx)
    ctx.calcuvw()
    assert oc.L.orc_calcuvw(oc.h) >= 0
    for k in ("u", "v", "w"):
        oc.set(k, ctx.field_get(k))
    r4 = ctx.calcp_simple()
    assert oc.L.orc_calcp_simple(oc.h) >= 0
    assert np.array_equal(ctx.field_get("a"), oc.get("a"))
    for k in ("pp", "p", "u", "v", "w", "flmass"):
        g, o = ctx.field_get(k), oc.get(k)
        assert np.abs(g - o).max() <= FIELD_TOL * max(1e-300, np.abs(o).max()), k
    pf, tf = pair_faces(a)
    fm = ctx.field_get("flmass")
    assert np.array_equal(fm[tf], fm[pf]) and np.abs(fm[pf]).max() > 0
    assert r4 == pytest.approx(oc.scalar("resor4"), rel=1e-6)


@pytest.mark.parametrize("layout", list(LAYOUTS))
def test_temperature_with_periodic_pairs(ctx, fc, oracle, layout):
    m, a, oc, _ = periodic_channel(oracle, sides=LAYOUTS[layout], ctx=ctx)
    for _ in range(2):  # non-trivial mass fluxes through the pairs
        ctx.simple_iteration()
        oc.simple_iteration()
    for k in ("u", "v", "w", "p", "flmass"):
        oc.set(k, ctx.field_get(k))
    rng = np.random.default_rng(11)
    t = rng.random(m.numTotal)
    ctx.field_set("t", t)
    oc.set("t", t)
    tp = fc.TemperatureParams.defaults()
    ctx.temperature_params(tp, np.zeros(len(a["bctype"])))
    for name in ("viscos", "pranl", "sigt", "urfT", "gdsT", "cSchemeT", "maxiterT", "tolAbsT", "tolRelT"):
        oc.param(name, getattr(tp, name))
    oc.solver("T", tp.lSolverT.decode())
    ctx.calculate_temperature(solve=False)
    oc.calculate_temperature(solve=False)
    for k in ("a", "su", "sp", "dTdxi"):
        assert np.array_equal(ctx.field_get(k), oc.get(k)), k
    ctx.field_set("t", t)
    oc.set("t", t)
    ctx.calculate_temperature(solve=True)
    oc.calculate_temperature(solve=True)
    g, o = ctx.field_get("t"), oc.get("t")
    assert np.abs(g - o).max() <= FIELD_TOL * np.abs(o).max()
    # updateBoundary: a periodic face holds its pair's mean; the twin face the
    # mean too when its patch comes first, its owner's value when after
    pf, tf = pair_faces(a)
    nC, nI = m.numCells, m.numInnerFaces
    for faces in (pf, tf):
        assert np.abs(g[nC + faces - nI] - o[nC + faces - nI]).max() <= FIELD_TOL * np.abs(o).max()
    same = np.array_equal(g[nC + tf - nI], g[nC + pf - nI])
    assert same == (layout == "twin_first")


def test_simple_iterations_with_periodic_pairs_track_oracle(ctx, fc, oracle):
    m, a, oc, _ = periodic_channel(oracle, dims=(12, 8, 6), ctx=ctx)
    res_g, res_o = [], []
    for _ in range(8):
        res_g.append(ctx.simple_iteration())
        res_o.append(oc.simple_iteration()[1])
    res_g, res_o = np.array(res_g), np.array(res_o)
    mask = np.abs(res_o) > 1e-12
    np.testing.assert_allclose(res_g[mask], res_o[mask], rtol=TRACK_RESOR_RTOL)
    for k in ("u", "v", "w", "p"):
        g, o = ctx.field_get(k), oc.get(k)
        assert np.abs(g - o).max() <= TRACK_FIELD_TOL * np.abs(o).max(), k


def test_piso_steps_with_periodic_pairs_track_oracle(ctx, fc, oracle):
    m, a, oc, _ = periodic_channel(oracle, dims=(10, 6, 5), ctx=ctx)
    dt = 0.02
    ctx.transient_params(dt, fc.FC_TIME_BDF, 1, 2)
    try:
        oc.param("timestep", dt)
        oc.param("tscheme", fc.FC_TIME_BDF)
        oc.param("piso", 1)
        oc.param("ncorr", 2)
        for _ in range(3):
            ctx.time_shift()
            oc.time_shift()
            rg = ctx.piso_iteration()
            ro = oc.piso_iteration()[1]
            np.testing.assert_allclose(rg[:3], np.asarray(ro)[:3], rtol=TRACK_RESOR_RTOL)
        for k in ("u", "v", "w", "p", "flmass"):
            g, o = ctx.field_get(k), oc.get(k)
            assert np.abs(g - o).max() <= TRACK_FIELD_TOL * np.abs(o).max(), k
    finally:
        ctx.transient_params(1.0, fc.FC_TIME_STEADY, 0, 1)


def test_node_gradient_rejects_periodic_meshes(ctx, fc, oracle):
    m, _, _, _ = periodic_channel(oracle, dims=(6, 4, 4), ctx=ctx)
    with pytest.raises(fc.FcError) as e:
        ctx.grad(fc.FC_GRAD_NODE_GAUSS, np.ones(m.numTotal))
    assert e.value.code == fc.FC_ERR_UNSUPPORTED
