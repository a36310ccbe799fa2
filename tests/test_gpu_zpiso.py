"""Transient momentum and PISO on the GPU against the oracle (velocity.f90:
226-290, :565-570; calcp_piso.f90; time_shift.f90): time steps of a
lid-driven cavity with PISO (Euler) and with transient SIMPLE iterations
(BDF2, BDF3), residuals and fields tracking the oracle; the combinations the
reference cannot run (PISO with BDF2/BDF3) are rejected."""
import numpy as np
import pytest

from test_gpu_simple import setup_cavity

pytestmark = pytest.mark.gpu

KW = dict(urfU=1.0, urfP=1.0, maxiterU=50, maxiterP=200, tolRelU=1e-9, tolRelP=1e-9)


def transient(ctx, oc, dt, scheme, piso, ncorr=2):
    ctx.transient_params(dt, scheme, piso, ncorr)
    for k, v in dict(timestep=dt, tscheme=scheme, piso=piso, ncorr=ncorr).items():
        oc.param(k, v)


def steady(ctx, oc):
    ctx.transient_params(1.0, 0, 0, 1)
    oc.param("tscheme", 0)
    oc.param("piso", 0)


def compare_fields(ctx, oc):
    for k in ("u", "v", "w", "p"):
        g, o = ctx.field_get(k), oc.get(k)
        assert np.abs(g - o).max() <= 1e-8 * max(np.abs(o).max(), 1e-30), k


@pytest.mark.parametrize("npcor", [1, 2])
def test_piso_time_steps_track_oracle(ctx, fc, npcor):
    m, oc = setup_cavity(ctx, fc, "piso" + str(npcor), 8, 8, 8, npcor=npcor, **KW)
    oc.param("npcor", npcor)
    transient(ctx, oc, 0.01, fc.FC_TIME_BDF, 1)
    try:
        rg, ro = [], []
        for step in range(4):
            ctx.time_shift()
            oc.time_shift()
            rg.append(ctx.piso_iteration())
            ro.append(oc.piso_iteration()[1])
        np.testing.assert_allclose(np.array(rg), np.array(ro), rtol=1e-7)
        compare_fields(ctx, oc)
        assert np.abs(ctx.field_get("rU") - oc.get("rU")).max() <= 1e-8 * np.abs(oc.get("rU")).max()
    finally:
        steady(ctx, oc)


@pytest.mark.parametrize("scheme", [2, 3])
def test_transient_simple_tracks_oracle(ctx, fc, scheme):
    m, oc = setup_cavity(ctx, fc, "tsimple" + str(scheme), 8, 8, 8, **dict(KW, urfU=0.8, urfP=0.3))
    transient(ctx, oc, 0.02, scheme, 0)
    try:
        rg, ro = [], []
        for step in range(3):
            ctx.time_shift()
            oc.time_shift()
            for it in range(2):
                rg.append(ctx.simple_iteration())
                ro.append(oc.simple_iteration()[1])
        np.testing.assert_allclose(np.array(rg), np.array(ro), rtol=1e-7)
        compare_fields(ctx, oc)
    finally:
        steady(ctx, oc)


def test_unsupported_combinations_are_rejected(ctx, fc):
    with pytest.raises(fc.FcError) as e:
        ctx.transient_params(0.01, fc.FC_TIME_BDF2, 1, 2)
    assert e.value.code == fc.FC_ERR_UNSUPPORTED
    with pytest.raises(fc.FcError):
        ctx.transient_params(0.0, fc.FC_TIME_BDF, 0, 1)


def oracle_run(oc, numstep, maxit, tolerance, transient, piso):
    """main.f90:132-267 driven from Python on the oracle."""
    steps = iters = 0
    r = None
    for itime in range(numstep):
        if transient:
            oc.time_shift()
        steps += 1
        done = False
        for it in range(maxit):
            r = oc.piso_iteration()[1] if piso else oc.simple_iteration()[1]
            iters += 1
            if max(r[:3]) < tolerance:
                done = not transient
                break
        if done:
            break
    return steps, iters, r


def test_run_loops_track_oracle(ctx, fc):
    """fc_run: steady SIMPLE to a tolerance, then PISO time steps with up to
    two iterations each, against the same loops on the oracle."""
    m, oc = setup_cavity(ctx, fc, "run", 6, 6, 6, **dict(KW, urfU=0.8, urfP=0.3))
    sg, ig, rg = ctx.run(1, 40, 1e-2)
    so, io, ro = oracle_run(oc, 1, 40, 1e-2, False, False)
    assert (sg, ig) == (so, io)
    np.testing.assert_allclose(rg, ro, rtol=1e-7)
    compare_fields(ctx, oc)
    transient(ctx, oc, 0.01, fc.FC_TIME_BDF, 1)
    try:
        sg, ig, rg = ctx.run(3, 2, 1e-12)
        so, io, ro = oracle_run(oc, 3, 2, 1e-12, True, True)
        assert (sg, ig) == (so, io) == (3, 6)
        np.testing.assert_allclose(rg, ro, rtol=1e-7)
        compare_fields(ctx, oc)
    finally:
        steady(ctx, oc)
