"""Gradient options on the GPU against the oracle:
- slope limiters (fc_set_gradient_limiter; gradients.f90:141-656): limited
  Gauss and least-squares gradients bit for bit on perturbed hex and tet
  meshes, and SIMPLE iterations with a limiter on every velocity gradient;
- node-based Gauss gradients (FC_GRAD_NODE_GAUSS; gradients.f90:1491-1602,
  node_interpolation.f90) with both cell-to-node methods, bit for bit (NaN
  at the same places where the reference's pseudo-Laplacian normalisation
  divides 0 by 0), and SIMPLE iterations on them.
The per-cell code is also replayed on the CPU against the oracle
(tests/test_limiters.py, tests/test_node_gradient.py)."""
import numpy as np
import pytest

from gpu_cases import mesh_case
from test_gpu_simple import setup_cavity

pytestmark = pytest.mark.gpu


def front(m, oc, seed):
    rng = np.random.default_rng(seed)
    xc = np.concatenate([oc.get("xc"), rng.uniform(0, 1, m.numTotal - m.numCells)])
    return np.tanh((xc - 0.5) / 0.08) + 0.05 * rng.standard_normal(m.numTotal)


@pytest.mark.parametrize("tets", [False, True])
@pytest.mark.parametrize("scheme", [0, 1, 2])
@pytest.mark.parametrize("kind", [1, 2, 3, 4])
def test_limited_gradients_bit_exact(ctx, fc, tets, scheme, kind):
    m, a, oc = mesh_case("lim" + str(tets), 9, 8, 7, tets=tets)
    ctx.set_mesh(m)
    phi = front(m, oc, 21 + kind)
    try:
        oc.param("limiter", kind)
        ctx.set_gradient_limiter(kind)
        g = ctx.grad(scheme, phi)
        go = oc.grad(scheme, phi)
    finally:
        oc.param("limiter", 0)
        ctx.set_gradient_limiter(fc.FC_LIMITER_NONE)
    nC = m.numCells
    assert np.array_equal(g[:3 * nC], go[:3 * nC])
    assert not np.array_equal(g[:3 * nC], ctx.grad(scheme, phi)[:3 * nC])  # the limiter acted


def test_unknown_limiter_is_rejected(ctx, fc):
    with pytest.raises(fc.FcError):
        ctx.set_gradient_limiter(9)


@pytest.mark.parametrize("kind", [1, 4])
def test_simple_iterations_with_limiter_track_oracle(ctx, fc, kind):
    m, oc = setup_cavity(ctx, fc, "cav_lim" + str(kind), 10, 10, 10)
    oc.param("limiter", kind)
    ctx.set_gradient_limiter(kind)
    try:
        res_g, res_o = [], []
        for it in range(6):
            res_g.append(ctx.simple_iteration())
            res_o.append(oc.simple_iteration()[1])
    finally:
        oc.param("limiter", 0)
        ctx.set_gradient_limiter(fc.FC_LIMITER_NONE)
    np.testing.assert_allclose(np.array(res_g), np.array(res_o), rtol=1e-7)
    for k in ("u", "v", "w", "p"):
        g, o = ctx.field_get(k), oc.get(k)
        assert np.abs(g - o).max() <= 1e-8 * np.abs(o).max(), k


@pytest.mark.parametrize("tets", [False, True])
@pytest.mark.parametrize("method", [0, 1])
def test_node_gradients_bit_exact(ctx, fc, tets, method):
    m, a, oc = mesh_case("ng" + str(tets), 8, 7, 6, tets=tets)
    ctx.set_mesh(m)
    phi = np.random.default_rng(31).standard_normal(m.numTotal)
    try:
        oc.param("c2n", method)
        ctx.set_node_interpolation(method)
        g = ctx.grad(fc.FC_GRAD_NODE_GAUSS, phi)
        go = oc.grad(3, phi)
    finally:
        oc.param("c2n", 0)
        ctx.set_node_interpolation(fc.FC_C2N_PSL)
    nC = m.numCells
    assert np.array_equal(g[:3 * nC], go[:3 * nC], equal_nan=True)


def test_simple_iterations_node_gradients_track_oracle(ctx, fc):
    """Inverse-distance node values (the pseudo-Laplacian ones are NaN at
    box edges, as in the reference)."""
    m, oc = setup_cavity(ctx, fc, "cav_ng", 8, 8, 8, grad=3)
    oc.param("c2n", 1)
    ctx.set_node_interpolation(fc.FC_C2N_IDS)
    try:
        res_g, res_o = [], []
        for it in range(6):
            res_g.append(ctx.simple_iteration())
            res_o.append(oc.simple_iteration()[1])
    finally:
        oc.param("c2n", 0)
        ctx.set_node_interpolation(fc.FC_C2N_PSL)
    np.testing.assert_allclose(np.array(res_g), np.array(res_o), rtol=1e-7)
    for k in ("u", "v", "w", "p"):
        g, o = ctx.field_get(k), oc.get(k)
        assert np.abs(g - o).max() <= 1e-8 * np.abs(o).max(), k
