"""C-ABI library: it builds, loads and exports every declared entry point;
host-side mesh logic (no GPU needed)."""
import ctypes as C
import os
import tempfile

import numpy as np
import pytest


def test_library_exports_every_declared_symbol(fc):
    L = fc.lib()
    names = fc.declared_symbols()
    assert "fc_csrsolve" in names and "fc_set_mesh" in names
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_no_gpu_calls_fail_cleanly_without_device(fc):
    # fc_init must either succeed (GPU present) or return an error code
    h = C.c_void_p()
    st = fc.lib().fc_init(0, C.byref(h))
    if st == 0:
        fc.lib().fc_finalize(h)
    else:
        assert st < 0


@pytest.mark.parametrize("n,tets", [((3, 2, 2), False), ((2, 2, 2), True), ((5, 4, 3), False)])
def test_box_mesh_counts_and_orientation(fc, n, tets):
    nx, ny, nz = n
    m = fc.Mesh.box(nx, ny, nz, 1.0, 1.0, 1.0, perturb=0.1, seed=7, tets=tets)
    a = m.arrays()
    ncell = nx * ny * nz * (6 if tets else 1)
    assert m.numCells == ncell
    if not tets:
        assert m.numInnerFaces == (nx - 1) * ny * nz + nx * (ny - 1) * nz + nx * ny * (nz - 1)
        assert m.numBoundaryFaces == 2 * (nx * ny + ny * nz + nx * nz)
    else:
        assert 4 * ncell == 2 * m.numInnerFaces + m.numBoundaryFaces
        assert m.numBoundaryFaces == 4 * (nx * ny + ny * nz + nx * nz)
    own, nb = a["owner"], a["neighbour"]
    assert np.all(own[:m.numInnerFaces] < nb)
    key = own[:m.numInnerFaces].astype(np.int64) * (ncell + 1) + nb
    assert np.all(np.diff(key) > 0), "inner faces sorted by (owner, neighbour)"
    assert list(a["startFace"]) == list(np.cumsum([m.numInnerFaces] + list(a["nfaces"][:-1])))


def test_native_format_roundtrip(fc):
    m = fc.Mesh.box(3, 3, 2, 2.0, 1.0, 1.0, perturb=0.15, seed=3, sides=["wall", "outlet", "wall", "wall",
                                                                           "symmetry", "symmetry"])
    with tempfile.TemporaryDirectory() as d:
        m.write_native(d)
        assert sorted(os.listdir(d)) == ["boundary", "faces", "neighbour", "owner", "points", "size"]
        m2 = fc.Mesh.read_native(d)
    a, b = m.arrays(), m2.arrays()
    for k in ("x", "y", "z", "nnodes", "nodes", "owner", "neighbour", "bctype", "nfaces", "startFace"):
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)


def test_perturbation_is_seeded(fc):
    a = fc.Mesh.box(4, 4, 4, perturb=0.15, seed=42).arrays()
    b = fc.Mesh.box(4, 4, 4, perturb=0.15, seed=42).arrays()
    c = fc.Mesh.box(4, 4, 4, perturb=0.15, seed=43).arrays()
    np.testing.assert_array_equal(a["x"], b["x"])
    assert np.abs(a["x"] - c["x"]).max() > 0


def test_mesh_rejects_bad_input(fc):
    m = fc.Mesh.box(2, 2, 2).arrays()
    bad = dict(m)
    bad["owner"] = m["owner"].copy()
    bad["owner"][0] = 999
    with pytest.raises(fc.FcError):
        fc.Mesh.from_arrays(bad)


def test_noalloc_size_limit_is_host_side(fc):
    """fc_dpcg_noalloc rejects n > FC_NOALLOC_MAX_N before touching the
    device (the arrays here are host dummies and are never read)."""
    import ctypes as C
    L = fc.lib()
    dummy_i = np.zeros(4, dtype=np.int32)
    dummy_d = np.zeros(4)
    err = C.create_string_buffer(256)
    info = fc.SolveInfo()
    n = fc.FC_NOALLOC_MAX_N + 1
    p = lambda arr: arr.ctypes.data_as(C.c_void_p)  # noqa: E731
    st = L.fc_dpcg_noalloc(None, n, n, p(dummy_i), p(dummy_i), p(dummy_d), p(dummy_i), p(dummy_d), p(dummy_d),
                           10, 0.0, 1e-8, C.byref(info), C.cast(err, C.c_void_p), 256)
    assert st == fc.FC_ERR_BAD_INPUT
    assert b"FC_NOALLOC_MAX_N" in err.value


@pytest.mark.parametrize("tets", [False, True])
def test_openfoam_format_roundtrip(fc, tets):
    """fc_mesh_write_openfoam / fc_mesh_read_openfoam (read_mesh_openfoam,
    geometry.f90:846-1400): FoamFile headers, 0-based lists, the owner
    file's note line; the mesh comes back unchanged."""
    m = fc.Mesh.box(3, 2, 2, 2.0, 1.0, 1.0, perturb=0.15, seed=5, tets=tets,
                    sides=["inlet", "outlet", "wall", "wall", "symmetry", "symmetry"])
    with tempfile.TemporaryDirectory() as d:
        m.write_openfoam(d)
        owner = open(os.path.join(d, "owner")).read()
        assert "FoamFile" in owner and "nInternalFaces:" in owner
        m2 = fc.Mesh.read_openfoam(d)
    a, b = m.arrays(), m2.arrays()
    for k in ("x", "y", "z", "nnodes", "nodes", "owner", "neighbour", "bctype", "nfaces", "startFace"):
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)


def test_openfoam_reader_parses_comments_and_checks_sizes(fc):
    """Comments and compact lists are read; a list whose own size disagrees
    with the owner file's note is rejected, as the reference stops there."""
    m = fc.Mesh.box(2, 2, 1, sides=["wall"] * 6)
    with tempfile.TemporaryDirectory() as d:
        m.write_openfoam(d)
        p = os.path.join(d, "points")
        txt = open(p).read()
        head, body = txt.split("\n\n", 1)
        n, rest = body.split("\n", 1)
        open(p, "w").write("/* generated */\n" + head + "\n// the points\n" + n + rest)
        m2 = fc.Mesh.read_openfoam(d)
        np.testing.assert_array_equal(m.arrays()["x"], m2.arrays()["x"])
        nb = os.path.join(d, "neighbour")
        t = open(nb).read().split("\n\n", 1)
        cnt, rest = t[1].split("\n", 1)
        open(nb, "w").write(t[0] + "\n\n" + str(int(cnt) + 1) + "\n" + rest)
        with pytest.raises(fc.FcError):
            fc.Mesh.read_openfoam(d)


def test_struct_layouts_match_the_header(fc, tmp_path):
    """The ctypes mirrors of the header's structs have the C layout: sizes
    and field offsets from a C program compiled against include/fc_gpu.h."""
    import ctypes as C
    import shutil
    import subprocess
    gcc = shutil.which("gcc")
    if not gcc:
        pytest.skip("gcc not available")
    structs = {"fc_solve_info": fc.SolveInfo, "fc_simple_params": fc.SimpleParams,
               "fc_temperature_params": fc.TemperatureParams, "fc_transient_params": fc.TransientParams,
               "fc_run_params": fc.RunParams, "fc_case_settings": fc.CaseSettings,
               "fc_turb_scalar": fc.TurbScalar, "fc_turbulence_params": fc.TurbulenceParams}
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "fc_gpu.h"', "int main(void) {"]
    for cname, py in structs.items():
        lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        for f in py._fields_:
            lines.append(f'  printf("{cname} {f[0]} %zu\\n", offsetof({cname}, {f[0]}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")
    subprocess.run([gcc, "-I", inc, str(src), "-o", str(exe)], check=True)
    got = {}
    for line in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.splitlines():
        name, field, val = line.split()
        got[(name, field)] = int(val)
    for cname, py in structs.items():
        assert got[(cname, "size")] == C.sizeof(py), cname
        for f in py._fields_:
            assert got[(cname, f[0])] == getattr(py, f[0]).offset, (cname, f[0])


def test_openfoam_dictionary_boundary(fc):
    """OpenFOAM's own boundary dictionary: roles from the patch type, or
    from the name of a generic patch."""
    m = fc.Mesh.box(3, 2, 2, sides=["inlet", "outlet", "wall", "wall", "symmetry", "symmetry"])
    a = m.arrays()
    with tempfile.TemporaryDirectory() as d:
        m.write_openfoam(d)
        kinds = {fc.BC["wall"]: "wall", fc.BC["symmetry"]: "symmetryPlane"}
        names = ["inlet", "outlet", "bottom", "top", "front", "back"]
        body = "".join(
            f"    {nm}\n    {{\n        type {kinds.get(int(t), 'patch')};\n        inGroups 1(x);\n"
            f"        nFaces {int(nf)};\n        startFace {int(sf)};\n    }}\n"
            for nm, t, nf, sf in zip(names, a["bctype"], a["nfaces"], a["startFace"]))
        open(os.path.join(d, "boundary"), "w").write(
            "FoamFile\n{\n    version 2.0;\n    format ascii;\n    class polyBoundaryMesh;\n    object boundary;\n}\n"
            f"// patches\n{len(names)}\n(\n{body})\n")
        m2 = fc.Mesh.read_openfoam(d)
    b = m2.arrays()
    for k in ("bctype", "nfaces", "startFace", "owner", "neighbour"):
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)


def test_setup_phase_names_match_the_header(fc):
    """Context.setup_times() names the values of fc_get_setup_times in the
    order of the header's FC_SETUP_* indices."""
    import re
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "fc_gpu.h")
    idx = {m.group(1).lower(): int(m.group(2)) for m in re.finditer(r"#define FC_SETUP_(\w+) (\d+)", open(inc).read())}
    assert idx.pop("phases") == len(fc.Context.SETUP_PHASES)
    assert {name: k for k, name in enumerate(fc.Context.SETUP_PHASES)} == idx
