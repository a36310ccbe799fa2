import importlib.util
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "freecappuccino-dev_gb300")
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def load_fcgpu():
    spec = importlib.util.spec_from_file_location("fcgpu", os.path.join(PKG, "fcgpu.py"))
    mod = sys.modules.get("fcgpu")
    if mod is None:
        mod = importlib.util.module_from_spec(spec)
        sys.modules["fcgpu"] = mod
        spec.loader.exec_module(mod)
    return mod


@pytest.fixture(scope="session")
def fc():
    return load_fcgpu()


@pytest.fixture(scope="session")
def oracle():
    import oracle_lib
    return oracle_lib


@pytest.fixture(scope="session")
def ctx(fc):
    c = fc.Context(0)
    yield c
    c.close()


def golden_path(name):
    return os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", name)


def polymesh_arrays():
    """The 20x20x1 cavity polyMesh of the reference's testFieldOperations."""
    m = np.load(golden_path("cavity20_polymesh.npz"))
    return dict(numNodes=len(m["points"]), numCells=int(m["owner"].max()), numInnerFaces=len(m["neighbour"]),
                numBoundaryFaces=len(m["owner"]) - len(m["neighbour"]), x=m["points"][:, 0].copy(),
                y=m["points"][:, 1].copy(), z=m["points"][:, 2].copy(), nnodes=m["nnodes"],
                nodes=m["nodes"].ravel().copy(), owner=m["owner"], neighbour=m["neighbour"], bctype=m["bctype"],
                nfaces=m["nfaces"], startFace=m["startFace"])
