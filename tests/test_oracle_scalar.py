"""The oracle's restatement of calculate_temperature (ScalarEqns/temperature.f90)
checked against properties of the discretisation that hold exactly: steady
conduction between two isothermal walls of an orthogonal box is linear in x,
the clip of temperature.f90:381 and updateBoundary's copy to outlet faces.
No GPU is used."""
import numpy as np
import pytest

from conftest import load_fcgpu

SMALL = float(np.float32(1e-20))  # parameters.f90: small = 1e-20 (single literal)


def box_case(oracle, nx, ny, nz, sides, bcdf):
    fc = load_fcgpu()
    m = fc.Mesh.box(nx, ny, nz, 1.0, 1.0, 1.0, perturb=0.0, sides=sides)
    a = m.arrays()
    oc = oracle.Case(a)
    for ib, v in enumerate(bcdf, start=1):
        oc.set_bcdfrac_t(ib, v)
    nT = oc.numTotal
    oc.set("vis", np.full(nT, 0.01))
    oc.param("viscos", 0.01)
    oc.param("pranl", 0.7)
    oc.set("flmass", np.zeros(oc.numFaces))
    return m, a, oc


def patch_slice(a, nC, nI, ib):
    st = a["startFace"][ib] - nI
    return slice(nC + st, nC + st + a["nfaces"][ib])


def test_conduction_between_isothermal_walls_is_linear(oracle):
    # xmin at T=1 and xmax at T=0 (isothermal), the other walls adiabatic
    m, a, oc = box_case(oracle, 8, 3, 3, ["wall"] * 6, [1, 1, 0, 0, 0, 0])
    nC, nI = oc.numCells, oc.numInnerFaces
    T = np.zeros(oc.numTotal)
    T[patch_slice(a, nC, nI, 0)] = 1.0
    oc.set("t", T)
    oc.param("urfT", 1.0)
    oc.param("maxiterT", 400)
    oc.param("tolAbsT", 1e-300)
    oc.param("tolRelT", 1e-14)
    oc.solver("T", "iccg")
    assert oc.calculate_temperature() == 0
    t = oc.get("t")
    xc = oc.get("xc")
    assert np.abs(t[:nC] - (1.0 - xc)).max() < 1e-10
    # adiabatic walls copied their owners' values during the assembly
    own = oc.get_int("owner") - 1
    for ib in (2, 3, 4, 5):
        sl = patch_slice(a, nC, nI, ib)
        faces = np.arange(sl.start - nC, sl.stop - nC) + nI
        assert np.array_equal(t[sl], T[own[faces]]), ib


def test_negative_solution_is_clipped_to_small(oracle):
    m, a, oc = box_case(oracle, 6, 3, 3, ["wall"] * 6, [1, 1, 0, 0, 0, 0])
    nC, nI = oc.numCells, oc.numInnerFaces
    T = np.zeros(oc.numTotal)
    T[patch_slice(a, nC, nI, 0)] = -1.0
    oc.set("t", T)
    oc.param("urfT", 1.0)
    oc.param("maxiterT", 200)
    oc.param("tolRelT", 1e-12)
    oc.solver("T", "bicgstab")
    assert oc.calculate_temperature() == 0
    assert np.all(oc.get("t")[:nC] == SMALL)


def test_outlet_faces_take_owner_values(oracle):
    sides = ["inlet", "outlet", "wall", "wall", "symmetry", "empty"]
    m, a, oc = box_case(oracle, 6, 4, 3, sides, [0] * 6)
    nC, nI = oc.numCells, oc.numInnerFaces
    rng = np.random.default_rng(3)
    oc.set("t", rng.random(oc.numTotal) + 0.5)
    # uniform flow in +x: inner x-faces and the inlet/outlet carry the flux
    arx = oc.get("arx")
    oc.set("flmass", 0.3 * arx)
    oc.solver("T", "bicgstab")
    assert oc.calculate_temperature() == 0
    t = oc.get("t")
    own = oc.get_int("owner") - 1
    for ib in (1, 4, 5):  # outlet, symmetry, empty
        sl = patch_slice(a, nC, nI, ib)
        faces = np.arange(sl.start - nC, sl.stop - nC) + nI
        assert np.array_equal(t[sl], t[own[faces]]), ib
    assert oc.scalar("resor7") > 0


def test_assembly_rows_of_pure_upwind_transport(oracle):
    """With gds = 0 and no diffusion (viscos -> tiny), the assembled row of an
    inner cell is the first-order upwind operator: a(diag) = sum of outflows
    and off-diagonals -inflow, so each row sums to the net outflow (zero for a
    divergence-free flux)."""
    sides = ["inlet", "outlet", "wall", "wall", "wall", "wall"]
    m, a, oc = box_case(oracle, 6, 3, 3, sides, [0] * 6)
    oc.param("gdsT", 0.0)
    oc.param("urfT", 1.0)
    oc.param("viscos", 0.0)
    oc.set("vis", np.zeros(oc.numTotal))
    arx = oc.get("arx")
    oc.set("flmass", 0.3 * arx)
    assert oc.calculate_temperature(solve=False) == 0
    A = oc.get("a")
    ia = oc.get_int("ia")
    dg = oc.get_int("diag")
    nC = oc.numCells
    rows = np.array([A[ia[i] - 1:ia[i + 1] - 1].sum() for i in range(nC)])
    # outflow through the outlet appears on the diagonal through sp = -can = cp
    assert np.abs(rows).max() < 1e-15 + 0.3 * (1.0 / 9) * 1.0001
    interior = [i for i in range(nC) if ia[i + 1] - ia[i] == 7]
    assert interior and np.abs(rows[interior]).max() == 0.0
    assert np.all(A[dg[:nC] - 1] >= 0)
