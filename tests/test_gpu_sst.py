"""The k-omega SST model on the GPU against the oracle's restatement of
k_omega_SST.f90 (calcsc, modify_mu_eff), calc_strain_and_vorticity.f90 and
wall_distance.f90, on the channel periodic in x and z between a resting and a
moving wall (tests/periodic_cases.py): wall functions on both walls,
periodic pairs in both directions.

The assembly restates the reference's FP64 formulas without contraction, as
the oracle does; tanh (the blending functions) and log (the wall law) come
from CUDA's and the C library's maths, which may differ in the last bit, so
the comparisons after them allow ASSEMBLY_RTOL.  The solved fields agree to
the solvers' reduction-order rounding (FIELD_RTOL)."""
import numpy as np
import pytest

from periodic_cases import periodic_channel

pytestmark = pytest.mark.gpu

ASSEMBLY_RTOL = 1e-12
FIELD_RTOL = 1e-8
FIRST_RESOR_RTOL = 1e-4
TURB = ("te", "ed")


def rel(g, o):
    return float(np.abs(g - o).max() / max(np.abs(o).max(), 1e-300))


def setup(ctx, fc, oracle, maxiter=10, iters=2):
    m, a, oc, prm = periodic_channel(oracle, dims=(10, 12, 6), ctx=ctx)
    nT = m.numTotal
    for k, v in (("te", 1e-3), ("ed", 1.0)):
        ctx.field_set(k, np.full(nT, v))
        oc.set(k, np.full(nT, v))
    kp = fc.TurbulenceParams.defaults(k=fc.TurbScalar.defaults(maxiter=maxiter),
                                      omega=fc.TurbScalar.defaults(maxiter=maxiter))
    ctx.turbulence_params(kp)
    for eq in ("K", "W"):
        oc.param("maxiter" + eq, maxiter)
    for _ in range(iters):  # a developed velocity field, the same on both sides
        ctx.simple_iteration()
    for k in ("u", "v", "w", "p", "flmass", "vis"):
        oc.set(k, ctx.field_get(k))
    return m, a, oc


def test_wall_distance_matches_oracle(ctx, fc, oracle):
    m, a, oc = setup(ctx, fc, oracle, iters=0)
    ctx.wall_distance()
    assert oc.wall_distance() == 0
    g, o = ctx.field_get("walldist"), oc.get("walldist")
    assert rel(g, o) <= FIELD_RTOL
    assert o.min() > 0


def test_kw_sst_assembly_matches_oracle(ctx, fc, oracle):
    """No linear-solver iterations (maxiter 0): the k and omega systems, the
    blending function, the wall functions and the eddy viscosity from the
    same state on both sides."""
    m, a, oc = setup(ctx, fc, oracle, maxiter=0)
    ctx.wall_distance()
    oc.wall_distance()
    oc.set("walldist", ctx.field_get("walldist"))
    ctx.kw_sst()
    assert oc.kw_sst() >= 0
    for k in ("magStrain", "gen", "dUdxi", "dVdxi", "dWdxi"):
        assert np.array_equal(ctx.field_get(k), oc.get(k)), k
    # the omega system left in the global matrix, the fields and wall values
    for k in ("a", "su", "sp", "fsst", "te", "ed", "vis", "visw", "ypl", "tau", "dTEdxi", "dEDdxi"):
        assert rel(ctx.field_get(k), oc.get(k)) <= ASSEMBLY_RTOL, k


def test_kw_sst_with_simple_iterations_tracks_oracle(ctx, fc, oracle):
    """Four SIMPLE iterations each followed by the SST update, the oracle
    taking the GPU's state before each update (lockstep): the update's
    residuals and fields.  The first update starts from uniform k and omega,
    where the normalised residual resor(5) divides rounding noise by rounding
    noise, so its residuals are compared loosely (FIRST_RESOR_RTOL)."""
    m, a, oc = setup(ctx, fc, oracle)
    ctx.wall_distance()
    oc.wall_distance()
    oc.set("walldist", ctx.field_get("walldist"))
    for it in range(4):
        ctx.simple_iteration()
        for k in ("u", "v", "w", "p", "flmass", "vis", "te", "ed", "fsst", "visw"):
            oc.set(k, ctx.field_get(k))
        r = ctx.kw_sst()
        assert oc.kw_sst() >= 0
        np.testing.assert_allclose(r, [oc.scalar("resor5"), oc.scalar("resor6")],
                                   rtol=FIRST_RESOR_RTOL if it == 0 else 1e-6)
        for k in ("te", "ed", "vis", "fsst", "visw"):
            assert rel(ctx.field_get(k), oc.get(k)) <= FIELD_RTOL, (it, k)
