"""The least-squares gradients with the correct 3x3 solve (schemes 4 and 5,
no reference counterpart) in the oracle: exact for linear fields on
perturbed hex and tet meshes, where the reference's grad_lsq / grad_lsq_dm
(schemes 1 and 2, y row b1*D4 - b2*D5 - b3*D6 of gradients.f90:887,1480)
are not; x and z rows are the reference's own."""
import numpy as np
import pytest

from conftest import load_fcgpu


@pytest.mark.parametrize("tets", [False, True])
@pytest.mark.parametrize("scheme", [4, 5])
def test_exact_lsq_linear_field(oracle, tets, scheme):
    fc = load_fcgpu()
    m = fc.Mesh.box(6, 5, 4, 1.0, 1.2, 0.8, perturb=0.2, seed=9, tets=tets)
    oc = oracle.Case(m.arrays())
    xc, yc, zc = oc.get("xc"), oc.get("yc"), oc.get("zc")
    xf, yf, zf = oc.get("xf"), oc.get("yf"), oc.get("zf")
    nI = m.numInnerFaces
    lin = lambda x, y, z: -1.0 + 0.7 * x + 2.5 * y - 4.0 * z  # noqa: E731
    phi = np.concatenate([lin(xc, yc, zc), lin(xf[nI:], yf[nI:], zf[nI:])])
    g = oc.grad(scheme, phi).reshape(-1, 3)[:m.numCells]
    np.testing.assert_allclose(g, np.tile([0.7, 2.5, -4.0], (m.numCells, 1)), atol=1e-10)
    q = oc.grad(scheme - 3, phi).reshape(-1, 3)[:m.numCells]
    # the reference's rows x and z agree with the exact solve where the
    # boundary weights agree (everywhere for scheme 1); y does not
    if scheme == 4:
        assert np.array_equal(q[:, 0], g[:, 0]) and np.array_equal(q[:, 2], g[:, 2])
    assert np.abs(q[:, 1] - 2.5).max() > 1e-3
