"""Generate the golden fixtures of this directory from the reference's own tests.

Run in a checkout that has the reference tree available (path given as the
first argument or in FC_REFERENCE_DIR).  It reads, as text:

  test/test_linear_solvers_spsolve.f90
      the two 5x5 known-answer systems (nonsymmetric: BiCGStab/GMRES; SPD:
      ICCG/DPCG/Gauss-Seidel), their right-hand sides, the printed analytic
      solutions and the solver settings.  The Fortran literals there are
      default REAL (single precision) assigned to real(dp) arrays, so they are
      rounded to float32 and widened, which is what the reference program
      feeds its solvers.
  test/testFieldOperations/polyMesh/{points,faces,owner,neighbour,boundary}
      the 20x20x1 OpenFOAM-format cavity mesh used by testFieldOperations.f90
      (read_mesh_openfoam turns its 0-based labels into 1-based ones).

and writes spsolve_5x5.json and cavity20_polymesh.npz next to this script.
"""
import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def _f32(values):
    return [float(np.float32(v)) for v in values]


def _array_after(src, name, start=0):
    """Return the numbers of the first `name = (/ ... /)` constructor after start."""
    m = re.compile(r"\b" + name + r"\s*=\s*\(/(.*?)/\)", re.S).search(src, start)
    body = re.sub(r"&", " ", m.group(1))
    return [float(t) for t in re.findall(r"[-+]?\d*\.?\d+(?:[eEdD][-+]?\d+)?", body)], m.end()


def spsolve_fixture(ref):
    path = os.path.join(ref, "test", "test_linear_solvers_spsolve.f90")
    src = open(path).read()
    itr_max = int(re.search(r"itr_max\s*=\s*(\d+)", src).group(1))
    tol_rel = float(re.search(r"tol_rel\s*=\s*([-+\deE.]+)", src).group(1))
    tol_abs = float(re.search(r"tol_abs\s*=\s*([-+\deE.]+)", src).group(1))
    a1, pos = _array_after(src, "a")
    b1, pos = _array_after(src, "b", pos)
    ja, pos = _array_after(src, "ja", pos)
    ioffset, pos = _array_after(src, "ioffset", pos)
    diag, pos = _array_after(src, "diag", pos)
    xa1, pos = _array_after(src, "xa", pos)
    a2, pos = _array_after(src, "a", pos)
    b2, pos = _array_after(src, "b", pos)
    xa2, pos = _array_after(src, "xa", pos)
    gs_itr = int(re.search(r"spsolve\('gauss-seidel',\s*x,\s*b,\s*res0,\s*(\d+)", src).group(1))
    common = {
        "n": 5,
        "ia": [int(v) for v in ioffset],
        "ja": [int(v) for v in ja],
        "diag": [int(v) for v in diag],
    }
    return {
        "source": "test/test_linear_solvers_spsolve.f90",
        "itr_max": itr_max,
        "itr_max_gauss_seidel": gs_itr,
        "tol_rel": float(np.float32(tol_rel)),
        "tol_abs": float(np.float32(tol_abs)),
        "nonsymmetric": dict(common, a=_f32(a1), b=_f32(b1), x_expected=xa1,
                             solvers=["bicgstab", "pmgmres"]),
        "spd": dict(common, a=_f32(a2), b=_f32(b2), x_expected=xa2,
                    solvers=["iccg", "dpcg", "gauss-seidel"]),
    }


def _foam_list(path):
    txt = open(path).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    txt = re.sub(r"//[^\n]*", "", txt)
    txt = re.sub(r"FoamFile\s*\{.*?\}", "", txt, flags=re.S)
    m = re.search(r"(\d+)\s*\((.*)\)", txt, re.S)
    return int(m.group(1)), m.group(2)


def polymesh_fixture(ref):
    d = os.path.join(ref, "test", "testFieldOperations", "polyMesh")
    n, body = _foam_list(os.path.join(d, "points"))
    pts = np.array([[float(v) for v in t.split()] for t in re.findall(r"\(([^()]*)\)", body)])
    assert pts.shape == (n, 3)
    n, body = _foam_list(os.path.join(d, "faces"))
    faces = [[int(v) for v in t.split()] for t in re.findall(r"\d+\(([^()]*)\)", body)]
    assert len(faces) == n
    nomax = 6
    nnodes = np.array([len(f) for f in faces], dtype=np.int32)
    nodes = np.zeros((n, nomax), dtype=np.int32)
    for i, f in enumerate(faces):
        nodes[i, :len(f)] = np.array(f) + 1
    n, body = _foam_list(os.path.join(d, "owner"))
    owner = np.array(body.split(), dtype=np.int32) + 1
    n2, body = _foam_list(os.path.join(d, "neighbour"))
    neighbour = np.array(body.split(), dtype=np.int32) + 1
    types = {"wall": 1, "inlet": 2, "outlet": 3, "symmetry": 4, "pressure": 5, "empty": 6}
    bctype, nfaces, start = [], [], []
    for line in open(os.path.join(d, "boundary")):
        line = line.strip()
        if not line or line.startswith("#"):
            continue
        name, t, nf, sf = line.split()[:4]
        bctype.append(types[t])
        nfaces.append(int(nf))
        start.append(int(sf))
    return dict(points=pts, nnodes=nnodes, nodes=nodes, owner=owner, neighbour=neighbour,
                bctype=np.array(bctype, np.int32), nfaces=np.array(nfaces, np.int32),
                startFace=np.array(start, np.int32))


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("FC_REFERENCE_DIR", "/root/reference")
    fx = spsolve_fixture(ref)
    with open(os.path.join(HERE, "spsolve_5x5.json"), "w") as f:
        json.dump(fx, f, indent=1)
    pm = polymesh_fixture(ref)
    np.savez_compressed(os.path.join(HERE, "cavity20_polymesh.npz"), **pm)
    print("wrote spsolve_5x5.json and cavity20_polymesh.npz")


if __name__ == "__main__":
    main()
