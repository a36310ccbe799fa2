"""Discrete adjoint of steady convection-diffusion on the GPU (fc_cd_assemble,
fc_cd_solve, fc_cd_adjoint) against the oracle (cd_assemble, cd_gradient)
with exact sparse direct solves, and against central finite differences.

The assembly and the reverse face loop are bit-exact (no FMA, the oracle's
order); the solved fields agree to the BiCGStab tolerance.  BiCGStab as the
reference writes it stalls near a relative L1 residual of 5e-11 on these
systems (the oracle identically), so the solves stop at 1e-9; the central
differences are taken as perturbation solves (cd_cases.cd_fd_perturbation),
which keeps them accurate to that tolerance relative to the perturbation."""
import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from cd_cases import TWO_PI, cd_fd_perturbation, cd_inputs, cd_objective, cd_source, cell_centres
from conftest import load_fcgpu

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def case(oracle):
    fc = load_fcgpu()
    m = fc.Mesh.box(10, 9, 8, TWO_PI, TWO_PI, TWO_PI, perturb=0.15, seed=42)
    a, fm, gamma = cd_inputs(fc, m)
    oc = oracle.Case(a)
    oc.set("flmass", fm)
    xc, yc, zc = cell_centres(oc)
    return m, oc, fm, gamma, cd_source(xc, yc, zc), xc


def setup(ctx, case):
    m, oc, fm, gamma, src, xc = case
    ctx.set_mesh(m)
    ctx.field_set("flmass", fm)
    return m, oc, fm, gamma, src, xc


def direct(oc, gamma, src, xc):
    oc.cd_assemble(gamma, src)
    n = oc.numCells
    A = sp.csr_matrix((oc.get("a"), oc.get_int("ja") - 1, oc.get_int("ia") - 1), shape=(n, n))
    phi = spla.spsolve(A.tocsc(), oc.get("su"))
    J, g = cd_objective(phi, oc.get("vol"), xc)
    lam = spla.spsolve(A.T.tocsc(), g)
    return A, phi, J, g, lam


def test_cd_assembly_bit_exact(ctx, case):
    m, oc, fm, gamma, src, xc = setup(ctx, case)
    ctx.cd_assemble(gamma, src)
    oc.cd_assemble(gamma, src)
    assert np.array_equal(ctx.field_get("a"), oc.get("a"))
    assert np.array_equal(ctx.field_get("su"), oc.get("su"))


def test_cd_forward_adjoint_and_gradient(ctx, case):
    m, oc, fm, gamma, src, xc = setup(ctx, case)
    A, phi_d, J_d, g_d, lam_d = direct(oc, gamma, src, xc)
    ctx.cd_assemble(gamma, src)
    phi, info = ctx.cd_solve(itr_max=500, tol_rel=1e-9)
    assert info.status == 0
    assert np.abs(phi - phi_d).max() <= 1e-8 * np.abs(phi_d).max()
    J, g = cd_objective(phi, oc.get("vol"), xc)
    lam, grad, info2 = ctx.cd_adjoint(g, itr_max=500, tol_rel=1e-9)
    assert info2.status == 0
    assert np.abs(lam - lam_d).max() <= 1e-7 * np.abs(lam_d).max()
    # the reverse face loop is the oracle's, bit for bit, on the same fields
    assert np.array_equal(grad, oc.cd_gradient(phi, lam))
    grad_d = oc.cd_gradient(phi_d, lam_d)
    assert np.abs(grad - grad_d).max() <= 1e-6 * np.abs(grad_d).max()


def test_cd_gradient_matches_central_differences(ctx, case):
    m, oc, fm, gamma, src, xc = setup(ctx, case)
    vol = oc.get("vol")
    ctx.cd_assemble(gamma, src)
    phi, info = ctx.cd_solve(itr_max=500, tol_rel=1e-9)
    J, g = cd_objective(phi, vol, xc)
    _, grad, info = ctx.cd_adjoint(g, itr_max=500, tol_rel=1e-9)
    assert info.status == 0
    for c in np.random.default_rng(47).choice(m.numCells, 6, replace=False):
        fd = cd_fd_perturbation(ctx, gamma, src, phi, vol, xc, c, 1e-3 * gamma[c])
        assert fd == pytest.approx(grad[c], rel=1e-3, abs=1e-5 * np.abs(grad).max()), c
