"""Device mesh setup and finite-volume operators vs the oracle.

The geometry, the CSR pattern and face -> slot maps, the gradients and the
Laplacian coefficients are computed on the device in the reference's
accumulation order without FMA contraction and compared bit for bit."""
import numpy as np
import pytest

from conftest import polymesh_arrays
from gpu_cases import mesh_case

pytestmark = pytest.mark.gpu

GEO = ("arx", "ary", "arz", "xf", "yf", "zf", "xc", "yc", "zc", "vol", "facint", "Df")
MESHES = {"hex": dict(nx=9, ny=7, nz=6), "tet": dict(nx=5, ny=4, nz=3, tets=True)}


def _setup(ctx, key):
    kw = dict(MESHES[key])
    m, a, oc = mesh_case("geo_" + key, kw.pop("nx"), kw.pop("ny"), kw.pop("nz"), **kw)
    ctx.set_mesh(m)
    return m, a, oc


@pytest.mark.parametrize("key", ["hex", "tet"])
def test_geometry_bit_exact(ctx, key):
    m, a, oc = _setup(ctx, key)
    for name in GEO:
        assert np.array_equal(ctx.geometry(name), oc.get(name)), name


@pytest.mark.parametrize("key", ["hex", "tet"])
def test_csr_pattern_and_slot_maps_bit_exact(ctx, key):
    m, a, oc = _setup(ctx, key)
    ia, ja, dg, ijk, jik = ctx.csr_pattern()
    for name, v in (("ia", ia), ("ja", ja), ("diag", dg), ("ijk", ijk), ("jik", jik)):
        assert np.array_equal(v, oc.get_int(name)), name


@pytest.mark.parametrize("key,dims", [("csr_hex", dict(nx=40, ny=30, nz=20)),
                                      ("csr_tet", dict(nx=14, ny=12, nz=10, tets=True))])
def test_csr_pattern_across_scan_blocks(ctx, key, dims):
    """24,000 hexes and 10,080 tetrahedra: the row-length scan of the device
    CSR build spans many blocks of 1024 rows."""
    kw = dict(dims)
    m, a, oc = mesh_case(key, kw.pop("nx"), kw.pop("ny"), kw.pop("nz"), **kw)
    ctx.set_mesh(m)
    ia, ja, dg, ijk, jik = ctx.csr_pattern()
    for name, v in (("ia", ia), ("ja", ja), ("diag", dg), ("ijk", ijk), ("jik", jik)):
        assert np.array_equal(v, oc.get_int(name)), name
    t = ctx.setup_times()
    assert set(t) == set(ctx.SETUP_PHASES) and min(t.values()) >= 0.0
    assert t["csr"] > 0.0 and t["tiling"] > 0.0 and t["schedule"] > 0.0


def test_cells_coupled_twice_are_rejected(ctx, fc):
    """Two cells across x, periodic in x: the inner face and the periodic
    pair couple the same two cells, which would repeat a CSR column."""
    from periodic_cases import SIDES
    m = fc.Mesh.box(2, 3, 3, 1.0, 1.0, 1.0, perturb=0.0, sides=SIDES)
    with pytest.raises(fc.FcError, match="coupled twice"):
        ctx.set_mesh(m)


@pytest.mark.parametrize("key", ["hex", "tet"])
@pytest.mark.parametrize("scheme", [0, 1, 2, 4, 5])
def test_gradients_bit_exact(ctx, key, scheme):
    m, a, oc = _setup(ctx, key)
    rng = np.random.default_rng(11)
    phi = rng.standard_normal(m.numTotal)
    assert np.array_equal(ctx.grad(scheme, phi), oc.grad(scheme, phi))


@pytest.mark.parametrize("mask", [(1 << 64) - 1, 0b1, 0])
def test_laplacian_bit_exact(ctx, mask):
    m, a, oc = _setup(ctx, "hex")
    rng = np.random.default_rng(12)
    mu = np.exp(rng.standard_normal(m.numCells) * 0.5)
    phi = rng.standard_normal(m.numTotal)
    su0 = rng.standard_normal(m.numCells)
    oc.set("su", su0)
    oc.laplacian(mu, phi, mask)
    ctx.field_set("su", su0)
    ctx.laplacian(mu, phi, mask)
    assert np.array_equal(ctx.field_get("a"), oc.get("a"))
    assert np.array_equal(ctx.field_get("su"), oc.get("su"))


def test_linear_field_gradient_on_reference_test_mesh(ctx, fc):
    """testFieldOperations.f90:133-160 on its own polyMesh: grad(x+y+z) = (1,1,1)."""
    m = fc.Mesh.from_arrays(polymesh_arrays())
    ctx.set_mesh(m)
    xc, yc, zc = ctx.geometry("xc"), ctx.geometry("yc"), ctx.geometry("zc")
    xf, yf, zf = ctx.geometry("xf"), ctx.geometry("yf"), ctx.geometry("zf")
    phi = np.concatenate([xc + yc + zc, (xf + yf + zf)[m.numInnerFaces:]])
    g = ctx.grad(0, phi).reshape(-1, 3)[:m.numCells]
    np.testing.assert_allclose(g, 1.0, atol=1e-12)


@pytest.mark.parametrize("key", ["hex", "tet"])
@pytest.mark.parametrize("scheme", [4, 5])
def test_exact_lsq_gradient_of_linear_field(ctx, key, scheme):
    """FC_GRAD_LSQ_EXACT / _DM_EXACT reproduce the gradient of a linear field
    in every cell (cell values at centroids, boundary values at face
    centres); the reference's schemes 1 and 2 miss its y component."""
    m, a, oc = _setup(ctx, key)
    xc, yc, zc = ctx.geometry("xc"), ctx.geometry("yc"), ctx.geometry("zc")
    xf, yf, zf = ctx.geometry("xf"), ctx.geometry("yf"), ctx.geometry("zf")
    lin = lambda x, y, z: 0.5 + 2.0 * x - 3.0 * y + 1.5 * z  # noqa: E731
    nI = m.numInnerFaces
    phi = np.concatenate([lin(xc, yc, zc), lin(xf[nI:], yf[nI:], zf[nI:])])
    g = ctx.grad(scheme, phi).reshape(-1, 3)[:m.numCells]
    np.testing.assert_allclose(g, np.tile([2.0, -3.0, 1.5], (m.numCells, 1)), atol=1e-9)
    gq = ctx.grad(scheme - 3, phi).reshape(-1, 3)[:m.numCells]
    assert np.abs(gq[:, 1] + 3.0).max() > 1e-3


def test_poisson_solve_on_global_matrix(ctx, oracle):
    """The pressure-Poisson setup of the 128^3 benchmark at a small size:
    perturbed hexes, Laplacian with one Dirichlet patch, N(0,1) zero-mean
    RHS, ICCG to 1e-10 on the mesh's global matrix."""
    m, a, oc = mesh_case("poisson", 16, 16, 16)
    ctx.set_mesh(m)
    rng = np.random.default_rng(43)
    b = rng.standard_normal(m.numCells)
    b -= b.mean()
    ctx.field_set("su", b)
    ctx.laplacian(np.ones(m.numCells), np.zeros(m.numTotal), 0b1)
    ctx.field_fill("pp", 0.0)
    r0, info, st = ctx.solve_field("iccg", "pp", "su", 5000, 0.0, 1e-10)
    assert st == 0
    oc.set("su", b)
    oc.laplacian(np.ones(m.numCells), np.zeros(m.numTotal), 0b1)
    xo, r0o, info_o, _ = oracle.solve("iccg", oc.get_int("ia"), oc.get_int("ja"), oc.get("a"),
                                      oc.get_int("diag"), np.zeros(m.numCells), oc.get("su"), 5000, 0.0, 1e-10)
    x = ctx.field_get("pp")[:m.numCells]
    assert abs(info.itr_used - int(info_o[0])) <= 1
    assert np.abs(x - xo).max() <= 1e-8 * np.abs(xo).max()
    assert r0 == pytest.approx(r0o, rel=1e-12)
