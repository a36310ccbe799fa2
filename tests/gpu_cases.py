"""Shared inputs of the GPU parity tests: seeded meshes, matrices and fields
built by the library's own mesh generator and fed identically to the oracle
and to the GPU."""
import numpy as np

from conftest import load_fcgpu

_cache = {}


def mesh_case(key, nx, ny, nz, perturb=0.15, seed=42, tets=False, sides=None):
    """(fc.Mesh, arrays dict, oracle.Case) for a box mesh, cached per key."""
    if key in _cache:
        return _cache[key]
    import oracle_lib
    fc = load_fcgpu()
    m = fc.Mesh.box(nx, ny, nz, 1.0, 1.0, 1.0, perturb=perturb, seed=seed, tets=tets, sides=sides)
    a = m.arrays()
    oc = oracle_lib.Case(a)
    _cache[key] = (m, a, oc)
    return _cache[key]


def laplacian_system(oc, mask, seed=43):
    """The implicit Laplacian matrix of the oracle case with a zero-mean N(0,1)
    right-hand side: (ia, ja, a, diag, rhs), 1-based CSR."""
    oc.set("su", np.zeros(oc.numCells))
    oc.laplacian(np.ones(oc.numCells), np.zeros(oc.numTotal), mask)
    rng = np.random.default_rng(seed)
    b = rng.standard_normal(oc.numCells)
    b -= b.mean()
    return oc.get_int("ia"), oc.get_int("ja"), oc.get("a"), oc.get_int("diag"), b


def nonsymmetric_values(oc, seed=5):
    """Convection-diffusion-like values on the mesh pattern: off-diagonals
    -1 - U(0,1) per slot (not symmetric), a diagonally dominant diagonal."""
    ia, ja, dg = oc.get_int("ia"), oc.get_int("ja"), oc.get_int("diag")
    rng = np.random.default_rng(seed)
    a = -1.0 - rng.random(len(ja))
    rows = np.repeat(np.arange(len(ia) - 1), np.diff(ia))
    off = np.bincount(rows, weights=a, minlength=len(ia) - 1) - a[dg - 1]
    a[dg - 1] = -off * 1.05 + 0.1
    return ia, ja, a, dg
