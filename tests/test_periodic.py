"""Periodic boundaries without a GPU: the mesh records (twins from the box
generator, the native and OpenFOAM readers and writers, OpenFOAM's cyclic
pairs, validation), and the oracle's restatement of face_mapping
(geometry.f90:1848-1997), of the periodic CSR pairs (sparse_matrix.f90:
136-165, :262-292) and of the periodic branches of the SIMPLE path, checked
through properties the reference's formulas guarantee: a permuted twin
patch is put back in pair order, the pattern stays symmetric, uniform flow
through a fully periodic box is a fixed point, and the flow between a
moving and a resting wall, periodic in x and z, converges to the linear
Couette profile."""
import os

import numpy as np
import pytest

import oracle_lib
from conftest import load_fcgpu
from periodic_cases import SIDES, pair_faces

FC = None


def fc():
    global FC
    if FC is None:
        FC = load_fcgpu()
    return FC


def test_box_periodic_sides_name_their_twins():
    m = fc().Mesh.box(5, 4, 3, sides=SIDES)
    a = m.arrays()
    sf = a["startFace"]
    assert list(a["startFaceTwin"]) == [-1, sf[0], -1, -1, -1, sf[4]]


@pytest.mark.parametrize("sides", [["wall", "periodic", "wall", "wall", "wall", "wall"],
                                   ["periodic", "periodic", "wall", "wall", "wall", "wall"]])
def test_periodic_twin_must_be_an_empty_patch(sides):
    with pytest.raises(fc().FcError):
        fc().Mesh.box(5, 4, 3, sides=sides)


@pytest.mark.parametrize("fmt", ["native", "openfoam"])
def test_readers_and_writers_keep_twins(tmp_path, fmt):
    m = fc().Mesh.box(5, 4, 3, perturb=0.1, sides=SIDES)
    d = str(tmp_path / fmt)
    os.makedirs(d, exist_ok=True)
    getattr(m, "write_" + fmt)(d)
    line = [l for l in open(os.path.join(d, "boundary")).read().splitlines() if " periodic " in l][0]
    assert len(line.split()) == 5  # name type nFaces startFace startFaceTwin
    r = getattr(fc().Mesh, "read_" + fmt)(d).arrays()
    a = m.arrays()
    for k in ("bctype", "nfaces", "startFace", "startFaceTwin"):
        assert np.array_equal(r[k], a[k]), k


def test_openfoam_cyclic_pair_becomes_empty_twin_and_periodic(tmp_path):
    m = fc().Mesh.box(5, 4, 3, sides=["wall"] * 6)
    d = str(tmp_path)
    m.write_openfoam(d)
    a = m.arrays()
    names = ["left", "right", "bottom", "top", "back", "front"]
    types = ["cyclic", "cyclic", "wall", "wall", "wall", "wall"]
    body = ["FoamFile\n{\n    version 2.0;\n    format ascii;\n    class polyBoundaryMesh;\n    object boundary;\n}\n",
            "6\n("]
    for b in range(6):
        extra = ""
        if types[b] == "cyclic":
            extra = f" neighbourPatch {names[1 - b]};"
        body.append(f"{names[b]} {{ type {types[b]}; nFaces {a['nfaces'][b]}; startFace {a['startFace'][b]};{extra} }}")
    body.append(")\n")
    open(os.path.join(d, "boundary"), "w").write("\n".join(body))
    r = fc().Mesh.read_openfoam(d).arrays()
    assert list(r["bctype"][:2]) == [fc().BC["empty"], fc().BC["periodic"]]
    assert r["startFaceTwin"][1] == a["startFace"][0]


def test_arrays_with_twins_round_trip():
    a = fc().Mesh.box(5, 4, 3, perturb=0.1, sides=SIDES).arrays()
    r = fc().Mesh.from_arrays(a).arrays()
    assert np.array_equal(r["startFaceTwin"], a["startFaceTwin"])


def reversed_twin_patch(a, b):
    """The arrays with the faces of patch b in reverse order."""
    r = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in a.items()}
    s, n = a["startFace"][b], a["nfaces"][b]
    idx = np.arange(s, s + n)[::-1]
    r["owner"][s:s + n] = a["owner"][idx]
    nodes = a["nodes"].reshape(-1, 6)
    rn = nodes.copy()
    rn[s:s + n] = nodes[idx]
    r["nodes"] = rn.reshape(-1)
    r["nnodes"][s:s + n] = a["nnodes"][idx]
    return r


def test_oracle_face_mapping_puts_a_permuted_twin_patch_back_in_pair_order():
    a = fc().Mesh.box(6, 5, 4, 2.0, 1.0, 1.0, perturb=0.12, seed=3, sides=SIDES).arrays()
    ref = oracle_lib.Case(a)
    r = reversed_twin_patch(a, 0)
    assert not np.array_equal(r["owner"], a["owner"])
    perm = oracle_lib.Case(r)
    assert np.array_equal(perm.get_int("owner"), ref.get_int("owner"))
    for k in ("xf", "yf", "zf", "arx", "ary", "arz", "xc", "vol"):
        assert np.array_equal(perm.get(k), ref.get(k)), k
    for k in ("ia", "ja", "ijk", "jik"):
        assert np.array_equal(perm.get_int(k), ref.get_int(k)), k


def test_oracle_periodic_pattern_and_slot_maps():
    a = fc().Mesh.box(6, 5, 4, perturb=0.1, sides=SIDES).arrays()
    oc = oracle_lib.Case(a)
    pf, tf = pair_faces(a)
    assert oc.numPeriodic == len(pf)
    assert oc.nnz == 2 * (oc.numInnerFaces + oc.numPeriodic) + oc.numCells
    ia, ja = oc.get_int("ia") - 1, oc.get_int("ja") - 1
    rows = np.repeat(np.arange(oc.numCells), np.diff(ia))
    pairs = set(zip(rows.tolist(), ja.tolist()))
    assert all((j, i) in pairs for i, j in pairs)
    own = oc.get_int("owner") - 1
    ijk, jik = oc.get_int("ijk") - 1, oc.get_int("jik") - 1
    nI = oc.numInnerFaces
    for q, (f, t) in enumerate(zip(pf, tf)):
        ijp, ijn = own[f], own[t]
        assert (rows[ijk[nI + q]], ja[ijk[nI + q]]) == (ijp, ijn)
        assert (rows[jik[nI + q]], ja[jik[nI + q]]) == (ijn, ijp)


def setup_flow(a, u0, viscos=0.02, lid=None):
    oc = oracle_lib.Case(a)
    nC, nT = oc.numCells, oc.numTotal
    prm = fc().SimpleParams.cavity(viscos=viscos)
    u = np.zeros(nT)
    v, w = np.zeros(nT), np.zeros(nT)
    u[:nC], v[:nC], w[:nC] = u0
    if lid is not None:
        s, n = a["startFace"][lid] - oc.numInnerFaces, a["nfaces"][lid]
        u[nC + s:nC + s + n] = 1.0
    for k, val in dict(u=u, v=v, w=w, p=np.zeros(nT), pp=np.zeros(nT), den=np.ones(nT),
                       vis=np.full(nT, viscos)).items():
        oc.set(k, val)
    if oc.nwal:
        oc.set("visw", np.full(oc.nwal, viscos))
    for name in ("viscos", "densit", "urfP", "gdsU", "cSchemeU", "pscheme", "maxiterU", "maxiterP", "npcor",
                 "pRefCell", "tolAbsU", "tolRelU", "tolAbsP", "tolRelP", "gradScheme"):
        oc.param(name, getattr(prm, name))
    for i in range(3):
        oc.param(f"urfU{i + 1}", prm.urfU[i])
    oc.solver("U", prm.lSolverU.decode())
    oc.solver("P", prm.lSolverP.decode())
    oc.L.orc_init_flmass(oc.h)
    return oc


def test_oracle_uniform_flow_through_a_fully_periodic_box_is_a_fixed_point():
    sides = ["empty", "periodic"] * 3
    a = fc().Mesh.box(6, 5, 4, 1.0, 1.0, 1.0, perturb=0.1, seed=5, sides=sides).arrays()
    oc = setup_flow(a, (1.0, 0.5, -0.25))
    for _ in range(3):
        oc.simple_iteration()
    nC = oc.numCells
    for k, val in (("u", 1.0), ("v", 0.5), ("w", -0.25)):
        assert np.abs(oc.get(k)[:nC] - val).max() < 1e-9, k


def test_oracle_periodic_couette_flow_reaches_the_linear_profile():
    """Periodic in x and z, y walls with the lid at u = 1: the converged
    velocity is u = y / ly, v = w = 0 (central differences are exact for a
    linear profile on this uniform mesh)."""
    a = fc().Mesh.box(4, 8, 3, 1.0, 1.0, 1.0, perturb=0.0, sides=SIDES).arrays()
    oc = setup_flow(a, (0.0, 0.0, 0.0), viscos=0.05, lid=3)
    for _ in range(200):  # U's residual falls below 1e-15 by iteration 180
        oc.simple_iteration()
    nC = oc.numCells
    y = oc.get("yc")
    u = oc.get("u")[:nC]
    assert np.abs(u - y).max() < 1e-6, np.abs(u - y).max()
    assert np.abs(oc.get("v")[:nC]).max() < 1e-6 and np.abs(oc.get("w")[:nC]).max() < 1e-6
