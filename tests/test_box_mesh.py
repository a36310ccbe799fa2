"""The numpy box generator used by the CPU arm of the benchmark gives the
library's fc_mesh_box mesh array for array (no GPU needed: the mesh
generator is host code)."""
import numpy as np
import pytest

from box_mesh import hex_box
from conftest import load_fcgpu


@pytest.mark.parametrize("dims,perturb,seed", [((3, 4, 5), 0.0, 42), ((6, 5, 4), 0.15, 42), ((9, 7, 8), 0.15, 7)])
def test_hex_box_matches_library_generator(dims, perturb, seed):
    fc = load_fcgpu()
    m = fc.Mesh.box(*dims, 1.0, 1.0, 1.0, perturb=perturb, seed=seed)
    ref = m.arrays()
    got = hex_box(*dims, perturb=perturb, seed=seed)
    for k in ("numNodes", "numCells", "numInnerFaces", "numBoundaryFaces"):
        assert got[k] == ref[k], k
    for k in ("x", "y", "z", "nnodes", "nodes", "owner", "neighbour", "bctype", "nfaces", "startFace"):
        assert np.array_equal(np.asarray(got[k]), np.asarray(ref[k])), k
