"""The oracle's discrete adjoint of the implicit convection-diffusion operator
(cd_assemble / cd_gradient) checked against central finite differences, with
exact sparse direct solves.  No GPU is used."""
import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from cd_cases import TWO_PI, cd_inputs, cd_objective, cd_source, cell_centres
from conftest import load_fcgpu


def csr_of(oc):
    ia, ja, a = oc.get_int("ia") - 1, oc.get_int("ja") - 1, oc.get("a")
    n = oc.numCells
    return sp.csr_matrix((a, ja, ia), shape=(n, n))


@pytest.fixture(scope="module")
def cd(oracle):
    fc = load_fcgpu()
    m = fc.Mesh.box(8, 7, 6, TWO_PI, TWO_PI, TWO_PI, perturb=0.15, seed=42)
    a, fm, gamma = cd_inputs(fc, m)
    oc = oracle.Case(a)
    oc.set("flmass", fm)
    xc, yc, zc = cell_centres(oc)
    src = cd_source(xc, yc, zc)
    return oc, gamma, src, xc


def solve_J(oc, gamma, src, xc):
    oc.cd_assemble(gamma, src)
    A = csr_of(oc)
    phi = spla.spsolve(A.tocsc(), oc.get("su"))
    J, g = cd_objective(phi, oc.get("vol"), xc)
    return J, g, phi, A


def test_stream_function_fluxes_are_divergence_free(cd):
    oc, gamma, src, xc = cd
    fm = oc.get("flmass")
    own, nb = oc.get_int("owner") - 1, oc.get_int("neighbour") - 1
    div = np.zeros(oc.numCells)
    np.add.at(div, own, fm)
    np.add.at(div, nb, -fm[:len(nb)])
    assert np.abs(div).max() < 1e-12 * np.abs(fm).max()
    # tangential on the box walls
    assert np.abs(fm[oc.numInnerFaces:]).max() < 1e-12 * np.abs(fm).max()


def test_adjoint_gradient_matches_central_differences(cd):
    oc, gamma, src, xc = cd
    J, g, phi, A = solve_J(oc, gamma, src, xc)
    lam = spla.spsolve(A.T.tocsc(), g)
    grad = oc.cd_gradient(phi, lam)
    cells = np.random.default_rng(47).choice(oc.numCells, 8, replace=False)
    for c in cells:
        h = 1e-6 * gamma[c]
        gp, gm = gamma.copy(), gamma.copy()
        gp[c] += h
        gm[c] -= h
        fd = (solve_J(oc, gp, src, xc)[0] - solve_J(oc, gm, src, xc)[0]) / (2 * h)
        assert fd == pytest.approx(grad[c], rel=1e-5, abs=1e-9 * np.abs(grad).max()), c


def test_assembly_rows_and_m_matrix(cd):
    """Off-diagonals are <= 0 (upwind, positive diffusivity), and every row
    sums to its boundary coefficient sp >= 0."""
    oc, gamma, src, xc = cd
    oc.cd_assemble(gamma, src)
    A = csr_of(oc)
    off = A - sp.diags(A.diagonal())
    assert off.data.max() <= 0.0
    rows = np.asarray(A.sum(axis=1)).ravel()
    assert rows.min() >= -1e-12 * np.abs(A.diagonal()).max()
