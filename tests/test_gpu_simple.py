"""SIMPLE path on the GPU vs the oracle restatement of calcuvw, calcp_simple
and gradp_and_sources on a lid-driven cavity (moving y=1 wall, u=(1,0,0)).

Assembly is bit-exact (face kernels + cell gathers in the reference's face
order, no FMA); fields after Krylov solves agree to 1e-9 relative (the solves'
dot products are reduced in a different order)."""
import numpy as np
import pytest

from gpu_cases import mesh_case

pytestmark = pytest.mark.gpu

LID = 3  # patch index of ymax in the box generator (xmin, xmax, ymin, ymax, zmin, zmax)


def setup_cavity(ctx, fc, key, nx, ny, nz, tets=False, sym=False, perturb=0.15, **kw):
    sides = ["wall"] * 6
    if sym:
        sides[4] = sides[5] = "symmetry"
    m, a, oc = mesh_case(key, nx, ny, nz, perturb=perturb, tets=tets, sides=sides)
    ctx.set_mesh(m)
    nC, nT = m.numCells, m.numTotal
    u = np.zeros(nT)
    st = a["startFace"][LID] - m.numInnerFaces
    u[nC + st:nC + st + a["nfaces"][LID]] = 1.0
    zero = np.zeros(nT)
    nwal = int(sum(nf for t, nf in zip(a["bctype"], a["nfaces"]) if t == 1))
    fields = dict(u=u, v=zero, w=zero, p=zero, pp=zero, den=np.ones(nT), vis=np.full(nT, kw.get("viscos", 0.01)))
    for k, v in fields.items():
        ctx.field_set(k, v)
        oc.set(k, v)
    ctx.field_set("visw", np.full(max(nwal, 1), 0.01)[:max(nwal, 1)])
    if nwal:
        oc.set("visw", np.full(nwal, 0.01))
    for k in ("flmass", "a"):
        ctx.field_fill(k, 0.0)
        oc.set(k, np.zeros(oc._len(k)))
    for k in ("dUdxi", "dVdxi", "dWdxi", "dPdxi"):
        ctx.field_fill(k, 0.0)
        oc.set(k, np.zeros(3 * nT))
    prm = fc.SimpleParams.cavity(**kw)
    ctx.simple_params(prm)
    for name in ("viscos", "densit", "urfP", "gdsU"):
        oc.param(name, getattr(prm, name))
    for i in range(3):
        oc.param(f"urfU{i + 1}", prm.urfU[i])
    for name in ("cSchemeU", "pscheme", "maxiterU", "maxiterP", "npcor", "pRefCell", "tolAbsU", "tolRelU",
                 "tolAbsP", "tolRelP"):
        oc.param(name, getattr(prm, name))
    oc.param("gradScheme", prm.gradScheme)
    if prm.gradScheme:
        oc.L.orc_prepare_lsq(oc.h, prm.gradScheme)
    oc.solver("U", prm.lSolverU.decode())
    oc.solver("P", prm.lSolverP.decode())
    ctx.init_flmass()
    oc.L.orc_init_flmass(oc.h)
    return m, oc


@pytest.mark.parametrize("pscheme", [0, 1, 2])
def test_gradp_and_sources_bit_exact(ctx, fc, pscheme):
    m, oc = setup_cavity(ctx, fc, "cav_gp", 8, 7, 6, pscheme=pscheme)
    rng = np.random.default_rng(21)
    p = rng.standard_normal(m.numTotal)
    apu = rng.random(m.numCells) + 0.5
    ctx.field_set("p", p); oc.set("p", p)
    ctx.field_set("apu", apu); oc.set("apu", apu)
    ctx.gradp_and_sources("p")
    oc.L.orc_gradp_and_sources(oc.h, 0)
    for k in ("su", "sv", "sw", "dPdxi", "p"):
        assert np.array_equal(ctx.field_get(k), oc.get(k)), k


@pytest.mark.parametrize("case", ["hex", "tet", "hex_sym", "lsq", "blu"])
def test_calcuvw_assembly_bit_exact_and_solves(ctx, fc, case):
    kw = {}
    tets = case == "tet"
    if case == "lsq":
        kw["grad"] = 1
    if case == "blu":
        kw["scheme"] = 19  # boundedLinearUpwind
    m, oc = setup_cavity(ctx, fc, "cav_" + case, 7 if not tets else 4, 6 if not tets else 4, 5 if not tets else 3,
                         tets=tets, sym=(case == "hex_sym"), **kw)
    # one iteration first so that the fields are not trivial, then compare
    r = ctx.calcuvw()
    assert oc.L.orc_calcuvw(oc.h) >= 0
    for k in ("spu", "spv", "sp", "apu", "apv", "apw", "sv", "sw", "su", "a", "dUdxi", "dVdxi", "dWdxi"):
        assert np.array_equal(ctx.field_get(k), oc.get(k)), k
    for k in ("u", "v", "w"):
        g, o = ctx.field_get(k), oc.get(k)
        assert np.abs(g - o).max() <= 1e-9 * max(1e-300, np.abs(o).max()), k
    np.testing.assert_allclose(r, [oc.scalar("resor1"), oc.scalar("resor2"), oc.scalar("resor3")], rtol=1e-12)


def test_calcp_simple_assembly_bit_exact(ctx, fc):
    m, oc = setup_cavity(ctx, fc, "cav_p", 8, 7, 6, npcor=2)
    ctx.calcuvw()
    assert oc.L.orc_calcuvw(oc.h) >= 0
    # give both sides the same momentum state, then compare the pressure step
    for k in ("u", "v", "w"):
        oc.set(k, ctx.field_get(k))
    r4 = ctx.calcp_simple()
    assert oc.L.orc_calcp_simple(oc.h) >= 0
    assert np.array_equal(ctx.field_get("a"), oc.get("a"))
    for k in ("pp", "p", "u", "v", "w", "flmass"):
        g, o = ctx.field_get(k), oc.get(k)
        assert np.abs(g - o).max() <= 1e-9 * max(1e-300, np.abs(o).max()), k
    assert r4 == pytest.approx(oc.scalar("resor4"), rel=1e-6)


def test_simple_iterations_batched_momentum_track_oracle(ctx, fc):
    """U, V, W solved in one batched launch (three block groups) follow the
    oracle's sequential solves as closely as the sequential GPU path does."""
    m, oc = setup_cavity(ctx, fc, "cav_itb", 10, 10, 10)
    ctx.simple_batched_momentum(True)
    try:
        res_g, res_o = [], []
        for it in range(8):
            res_g.append(ctx.simple_iteration())
            res_o.append(oc.simple_iteration()[1])
    finally:
        ctx.simple_batched_momentum(False)
    np.testing.assert_allclose(np.array(res_g), np.array(res_o), rtol=1e-7)
    for k in ("u", "v", "w", "p"):
        g, o = ctx.field_get(k), oc.get(k)
        assert np.abs(g - o).max() <= 1e-8 * np.abs(o).max(), k


@pytest.mark.parametrize("tets", [False, True])
def test_simple_iterations_track_oracle(ctx, fc, tets):
    n = (4, 4, 3) if tets else (10, 10, 10)
    m, oc = setup_cavity(ctx, fc, "cav_it" + str(tets), *n, tets=tets)
    res_g, res_o = [], []
    for it in range(8):
        r = ctx.simple_iteration()
        st, ro, _ = oc.simple_iteration()
        res_g.append(r)
        res_o.append(ro)
    np.testing.assert_allclose(np.array(res_g), np.array(res_o), rtol=1e-7)
    for k in ("u", "v", "w", "p"):
        g, o = ctx.field_get(k), oc.get(k)
        assert np.abs(g - o).max() <= 1e-8 * np.abs(o).max(), k
