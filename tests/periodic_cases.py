"""A channel periodic in x and z between two walls (y = 0 at rest, y = ly
moving at u = 1), set up identically on the oracle and (optionally) on the
GPU context: the inputs of the periodic-boundary tests.

The box generator pairs a periodic side with the opposite side, typed
'empty', as the reference's boundary files do (the twin patch is listed
first in SIDES, last in SIDES_TWIN_AFTER, which changes what updateBoundary
leaves on the twin faces)."""
import numpy as np

from conftest import load_fcgpu

SIDES = ["empty", "periodic", "wall", "wall", "empty", "periodic"]
SIDES_TWIN_AFTER = ["periodic", "empty", "wall", "wall", "periodic", "empty"]
LID = 3  # ymax
VISC = 0.02


def periodic_channel(oracle, dims=(10, 6, 5), size=(2.0, 1.0, 1.0), perturb=0.1, seed=7, sides=SIDES, ctx=None,
                     noise=0.05):
    """(mesh, arrays, oracle case, SimpleParams).  Cell velocities start as
    seeded noise of amplitude `noise` (so that no component is trivial), the
    lid moves at u = 1, inner mass fluxes come from init_flmass and the
    periodic faces start at zero flux, as in the reference."""
    fc = load_fcgpu()
    m = fc.Mesh.box(*dims, *size, perturb=perturb, seed=seed, sides=sides)
    a = m.arrays()
    oc = oracle.Case(a)
    nC, nT, nI = m.numCells, m.numTotal, m.numInnerFaces
    rng = np.random.default_rng(seed)
    u, v, w = (np.zeros(nT) for _ in range(3))
    for f in (u, v, w):
        f[:nC] = noise * rng.standard_normal(nC)
    s0 = a["startFace"][LID] - nI
    u[nC + s0:nC + s0 + a["nfaces"][LID]] = 1.0
    nwal = int(sum(nf for t, nf in zip(a["bctype"], a["nfaces"]) if t == 1))
    zero = np.zeros(nT)
    fields = dict(u=u, v=v, w=w, p=zero, pp=zero, den=np.ones(nT), vis=np.full(nT, VISC))
    prm = fc.SimpleParams.cavity(viscos=VISC)
    for k, val in fields.items():
        oc.set(k, val)
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
    if ctx is not None:
        ctx.set_mesh(m)
        for k, val in fields.items():
            ctx.field_set(k, val)
        ctx.field_set("visw", np.full(max(nwal, 1), VISC))
        for k in ("a", "flmass", "dUdxi", "dVdxi", "dWdxi", "dPdxi"):
            ctx.field_fill(k, 0.0)
        ctx.simple_params(prm)
        ctx.init_flmass()
    return m, a, oc, prm


def pair_faces(a):
    """(periodic faces, twin faces) in the order of the pair loops."""
    pf, tf = [], []
    for b, t in enumerate(a["bctype"]):
        if t == 7:
            n = a["nfaces"][b]
            pf.extend(range(a["startFace"][b], a["startFace"][b] + n))
            tf.extend(range(a["startFaceTwin"][b], a["startFaceTwin"][b] + n))
    return np.array(pf), np.array(tf)
