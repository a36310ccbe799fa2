"""A channel with a velocity inlet at x = 0, a pressure boundary (p = 0) at
x = lx and walls elsewhere, set up identically on the oracle and (optionally)
on the GPU context: the inputs of the pressure-boundary tests."""
import numpy as np

from conftest import load_fcgpu

SIDES = ["inlet", "pressure", "wall", "wall", "wall", "wall"]
VISC = 0.05


def channel(oracle, dims=(16, 6, 6), size=(2.0, 1.0, 1.0), perturb=0.1, seed=3, ctx=None):
    """(mesh, arrays, oracle case, SimpleParams); with ctx the GPU context
    gets the same mesh, fields and parameters.  Inlet u = 1 and its mass
    fluxes den u.S; inner mass fluxes from init_flmass."""
    fc = load_fcgpu()
    m = fc.Mesh.box(*dims, *size, perturb=perturb, seed=seed, sides=SIDES)
    a = m.arrays()
    oc = oracle.Case(a)
    nC, nT, nI = m.numCells, m.numTotal, m.numInnerFaces
    u = np.zeros(nT)
    s0 = a["startFace"][0] - nI
    u[nC + s0:nC + s0 + a["nfaces"][0]] = 1.0
    nwal = int(sum(nf for t, nf in zip(a["bctype"], a["nfaces"]) if t == 1))
    zero = np.zeros(nT)
    fields = dict(u=u, v=zero, w=zero, p=zero, pp=zero, den=np.ones(nT), vis=np.full(nT, VISC))
    prm = fc.SimpleParams.cavity(viscos=VISC)
    for k, v in fields.items():
        oc.set(k, v)
    oc.set("visw", np.full(nwal, VISC))
    oc.set("flmass", np.zeros(oc._len("flmass")))
    oc.set("a", np.zeros(oc._len("a")))
    for k in ("dUdxi", "dVdxi", "dWdxi", "dPdxi"):
        oc.set(k, np.zeros(3 * nT))
    for name in ("viscos", "densit", "urfP", "gdsU", "cSchemeU", "pscheme", "maxiterU", "maxiterP", "npcor",
                 "pRefCell", "tolAbsU", "tolRelU", "tolAbsP", "tolRelP", "gradScheme"):
        oc.param(name, getattr(prm, name))
    for i in range(3):
        oc.param(f"urfU{i + 1}", prm.urfU[i])
    oc.solver("U", prm.lSolverU.decode())
    oc.solver("P", prm.lSolverP.decode())
    oc.L.orc_init_flmass(oc.h)
    fm = oc.get("flmass")
    f0, n0 = a["startFace"][0], a["nfaces"][0]
    fm[f0:f0 + n0] = oc.get("arx")[f0:f0 + n0]  # den = 1, u = (1, 0, 0)
    oc.set("flmass", fm)
    if ctx is not None:
        ctx.set_mesh(m)
        for k, v in fields.items():
            ctx.field_set(k, v)
        ctx.field_set("visw", np.full(nwal, VISC))
        for k in ("a", "dUdxi", "dVdxi", "dWdxi", "dPdxi"):
            ctx.field_fill(k, 0.0)
        ctx.simple_params(prm)
        ctx.field_set("flmass", fm)
    return m, a, oc, prm


def patch_flux(a, flmass, ib):
    f0, n = a["startFace"][ib], a["nfaces"][ib]
    return float(np.sum(flmass[f0:f0 + n]))
