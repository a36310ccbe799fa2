"""The oracle's transient momentum and PISO (velocity.f90:226-290, :565-570;
calcp_piso.f90; time_shift.f90) on the CPU: time_shift moves the velocity
levels as written; after calcp_piso with one pressure solve per corrector
the inner-face mass fluxes are conservative to the pressure solve's
tolerance (the flux correction makes div(flmass) the solve's residual); a
transient lid-driven cavity develops from rest toward the lid velocity."""
import numpy as np
import pytest

from conftest import load_fcgpu

LID = 3


def cavity(oracle, n=8, dt=0.01, scheme=1, piso=1, ncorr=2, npcor=1, tolp=1e-10):
    fc = load_fcgpu()
    m = fc.Mesh.box(n, n, n, 1.0, 1.0, 1.0, perturb=0.15, seed=42)
    a = m.arrays()
    oc = oracle.Case(a)
    nC, nT = m.numCells, m.numTotal
    u = np.zeros(nT)
    st = a["startFace"][LID] - m.numInnerFaces
    u[nC + st:nC + st + a["nfaces"][LID]] = 1.0
    z = np.zeros(nT)
    for k, v in dict(u=u, v=z, w=z, p=z, pp=z, den=np.ones(nT), vis=np.full(nT, 0.01)).items():
        oc.set(k, v)
    nwal = int(sum(nf for t, nf in zip(a["bctype"], a["nfaces"]) if t == 1))
    oc.set("visw", np.full(nwal, 0.01))
    prm = dict(viscos=0.01, densit=1.0, urfP=1.0, gdsU=1.0, cSchemeU=1, pscheme=0, maxiterU=50, maxiterP=200,
               npcor=npcor, pRefCell=1, tolAbsU=1e-15, tolRelU=1e-8, tolAbsP=1e-15, tolRelP=tolp, urfU1=1.0,
               urfU2=1.0, urfU3=1.0, tscheme=scheme, piso=piso, ncorr=ncorr, timestep=dt)
    for k, v in prm.items():
        oc.param(k, v)
    oc.solver("U", "bicgstab")
    oc.solver("P", "iccg")
    oc.L.orc_init_flmass(oc.h)
    return m, a, oc


def divergence(m, a, oc):
    nC, nI = m.numCells, m.numInnerFaces
    own, nb = np.asarray(a["owner"]) - 1, np.asarray(a["neighbour"]) - 1
    fl = oc.get("flmass")
    div = np.zeros(nC)
    np.add.at(div, own[:nI], fl[:nI])
    np.subtract.at(div, nb, fl[:nI])
    return div, fl


@pytest.mark.parametrize("scheme", [1, 2, 3])
def test_time_shift_moves_the_levels(oracle, scheme):
    m, a, oc = cavity(oracle, n=4, scheme=scheme, piso=0)
    rng = np.random.default_rng(1)
    vals = {k: rng.standard_normal(m.numTotal) for k in ("u", "uo", "uoo", "uooo")}
    for k, v in vals.items():
        oc.set(k, v)
    oc.time_shift()
    assert np.array_equal(oc.get("uo"), vals["u"])
    assert np.array_equal(oc.get("uoo"), vals["uo"] if scheme >= 2 else vals["uoo"])
    assert np.array_equal(oc.get("uooo"), vals["uoo"] if scheme == 3 else vals["uooo"])


def test_piso_fluxes_are_conservative(oracle):
    m, a, oc = cavity(oracle, npcor=1, tolp=1e-12)
    for step in range(3):
        oc.time_shift()
        st, r = oc.piso_iteration()
        assert st == 0
        div, fl = divergence(m, a, oc)
        # inner cells: no inlet/outlet; walls carry no mass flux
        assert np.abs(div).max() <= 1e-9 * np.abs(fl).max(), step


def test_transient_cavity_develops(oracle):
    m, a, oc = cavity(oracle)
    umax = []
    for step in range(4):
        oc.time_shift()
        st, r = oc.piso_iteration()
        assert st == 0 and np.isfinite(r).all()
        umax.append(oc.get("u")[:m.numCells].max())
    assert all(b > a_ for a_, b in zip(umax, umax[1:])) and umax[-1] < 1.0
    # rU is kept from calcuvw: the explicit part of the U equation
    assert np.abs(oc.get("rU")).max() > 0
