"""The Poisson manufactured-solution case of the reference's Poisson
application (applications/Poisson/poisson.f90:62-104), set up identically on
the oracle and (optionally) on the GPU context.

-div(grad p) = 8 pi^2 sin(2 pi x) sin(2 pi y) on the unit square (one cell
layer in z, no flux through the z faces), p = 0 on the four edges; exact
solution p = sin(2 pi x) sin(2 pi y).  As there, the source is the cell
value times the cell volume, the Laplacian is assembled with the
coefficient -1 (sv = -1) and Dirichlet values p = 0 on the edge patches, and
ICCG solves it (sor = 1e-16 there; a relative 1e-12 here)."""
import numpy as np

from conftest import load_fcgpu

EDGES = 0b001111  # Dirichlet on xmin, xmax, ymin, ymax; the z patches carry no flux
TOL_REL = 1e-12
ITR_MAX = 5000


def mms_mesh(n):
    fc = load_fcgpu()
    return fc.Mesh.box(n, n, 1, 1.0, 1.0, 1.0 / n, perturb=0.0, sides=["wall"] * 6)


def exact(xc, yc):
    return np.sin(2 * np.pi * xc) * np.sin(2 * np.pi * yc)


def source(xc, yc, vol):
    return 8 * np.pi ** 2 * np.sin(2 * np.pi * xc) * np.sin(2 * np.pi * yc) * vol


def oracle_solve(oracle, n):
    """(cell solution, exact cell values, oracle case) from the oracle."""
    m = mms_mesh(n)
    oc = oracle.Case(m.arrays())
    nC, nT = m.numCells, m.numTotal
    xc, yc, vol = oc.get("xc"), oc.get("yc"), oc.get("vol")
    oc.set("su", source(xc, yc, vol))
    oc.laplacian(-np.ones(nC), np.zeros(nT), EDGES)
    x, _, info, _ = oracle.solve("iccg", oc.get_int("ia"), oc.get_int("ja"), oc.get("a"), oc.get_int("diag"),
                                 np.zeros(nC), oc.get("su"), ITR_MAX, 0.0, TOL_REL)
    return x, exact(xc, yc), oc
