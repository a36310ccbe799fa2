"""Inputs of the convection-diffusion adjoint cases (the C4 configuration
scaled down): [0, 2 pi]^3 perturbed hex mesh, u = 0.5 (sin x cos y,
-cos x sin y, 0) as face fluxes of the stream function 0.5 sin x sin y,
lognormal diffusivity (mu = -4, sigma = 0.5), a Gaussian source blob at
(pi, pi, pi) with sigma 0.5, J = volume-weighted mean of phi^2 over x > pi."""
import numpy as np

TWO_PI = 2.0 * np.pi


def cd_inputs(fc, m, seed_gamma=46):
    a = m.arrays()
    fm = fc.stream_function_fluxes(a, lambda x, y, z: 0.5 * np.sin(x) * np.sin(y))
    nC = m.numCells
    gamma = np.exp(np.random.default_rng(seed_gamma).normal(-4.0, 0.5, nC))
    return a, fm, gamma


def cell_centres(oc):
    return oc.get("xc"), oc.get("yc"), oc.get("zc")


def cd_source(xc, yc, zc, sigma=0.5):
    r2 = (xc - np.pi) ** 2 + (yc - np.pi) ** 2 + (zc - np.pi) ** 2
    return np.exp(-r2 / (2.0 * sigma * sigma))


def cd_objective(phi, vol, xc):
    """J and dJ/dphi."""
    mask = xc > np.pi
    vt = vol[mask].sum()
    J = float((vol[mask] * phi[mask] ** 2).sum() / vt)
    g = np.where(mask, 2.0 * vol * phi / vt, 0.0)
    return J, g


def cd_fd_perturbation(ctx, gamma, src, phi, vol, xc, c, h, itr_max=500, tol_rel=1e-9):
    """Central difference of J with respect to gamma_c, each side computed as
    a perturbation solve: A(gamma +- h e_c) dphi = -(A(gamma +- h e_c) -
    A(gamma)) phi, J(+-) - J = sum V (2 phi dphi + dphi^2) / V over x > pi.
    The same finite difference as re-solving and subtracting, without the
    cancellation (the solver's residual, relative to dphi, stays small where
    relative to phi it would swamp a one-cell perturbation)."""
    import scipy.sparse as sp
    ia, ja, dg, _, _ = ctx.csr_pattern()
    n = len(dg)
    ctx.cd_assemble(gamma, src)
    a0 = ctx.field_get("a")
    mask = xc > np.pi
    vt = vol[mask].sum()
    dJ = []
    for sgn in (1.0, -1.0):
        gp = gamma.copy()
        gp[c] += sgn * h
        ctx.cd_assemble(gp, src)
        dA = sp.csr_matrix((ctx.field_get("a") - a0, ja - 1, ia - 1), shape=(n, n))
        ctx.field_set("su", -(dA @ phi))
        dphi, info = ctx.cd_solve(itr_max=itr_max, tol_rel=tol_rel)
        dJ.append(float((vol[mask] * (2.0 * phi[mask] * dphi[mask] + dphi[mask] ** 2)).sum() / vt))
    ctx.cd_assemble(gamma, src)
    return (dJ[0] - dJ[1]) / (2.0 * h)


def cd_batch_sizes(count=64, lo=20, hi=80, seed_n=44, seed_pe=45):
    """Cells per side ~ U{lo..hi} (seed 44) and cell Peclet numbers
    Pe_h = U h / gamma ~ lognormal(0, 1) (seed 45) of the batched
    convection-diffusion configuration."""
    ns = np.random.default_rng(seed_n).integers(lo, hi + 1, count)
    pe = np.random.default_rng(seed_pe).lognormal(0.0, 1.0, count)
    return ns, pe


def cd_batch_system(fc, ctx, n, pe_cell, seed):
    """One problem of the batched configuration on ctx: the n^3 perturbed hex
    mesh of [0, 2 pi]^3 (interior vertices moved by up to 0.15 h, seed), the
    velocity above, uniform gamma = U h / pe_cell with U = 0.5, h = 2 pi / n,
    the Gaussian source.  Returns (ia, ja, diag, a, b, xyz): 1-based CSR
    pattern, values, right-hand side and cell centres (x..., y..., z...)."""
    m = fc.Mesh.box(n, n, n, TWO_PI, TWO_PI, TWO_PI, perturb=0.15, seed=seed)
    ctx.set_mesh(m)
    _, fm, _ = cd_inputs(fc, m)
    ctx.field_set("flmass", fm)
    xc, yc, zc = ctx.geometry("xc"), ctx.geometry("yc"), ctx.geometry("zc")
    gamma = np.full(m.numCells, 0.5 * (TWO_PI / n) / pe_cell)
    ctx.cd_assemble(gamma, cd_source(xc, yc, zc))
    ia, ja, dg, _, _ = ctx.csr_pattern()
    return ia, ja, dg, ctx.field_get("a"), ctx.field_get("su"), np.concatenate([xc, yc, zc])
