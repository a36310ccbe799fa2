"""The case namelist reader (fc_namelist_read; read_input.f90:28-227) on the
CPU: values, module defaults (with the reference's default-real literals),
Fortran array and case rules, comments and quotes, the gradient and time
scheme selection, and the rejected options."""
import os
import tempfile

import pytest

from conftest import load_fcgpu

CASE = """! a test case
&input_parameters
  title = 'Box with a lid! not a comment'
  mesh_format = 'foamMesh'        ! OpenFOAM files
  urfU = 0.6, 0.5
  cSchemeU = 'boundedCentral'
  maxiterU = 8, tolRelU = 1d-3
  urfP = 0.25
  pscheme = 'weighted'
  densit = 1.2, viscos = 1.5e-5
  calcT = T
  pranl = 0.71, sigt = 0.85
  ltransient = .true.  bdf = F  bdf2 = T
  LSTSQ_DM = T
  limiter = 'Venkatakrishnan'
  SIMPLE = T, PISO = F
  npcor = 2
  NUMSTEP = 10, MAXIT = 3, tolerance = 1e-4, timestep = 0.005
  CoNumFix = F                    ! a key this path does not use
/
"""


def read(fc, text):
    with tempfile.NamedTemporaryFile("w", suffix=".nml", delete=False) as f:
        f.write(text)
        path = f.name
    try:
        return fc.read_namelist(path)
    finally:
        os.unlink(path)


def f32(x):
    import numpy as np
    return float(np.float32(x))


def test_values_and_defaults():
    fc = load_fcgpu()
    c = read(fc, CASE)
    s = c.simple
    assert c.title.decode() == "Box with a lid! not a comment" and c.mesh_foam == 1
    # a list shorter than the array leaves the rest at the default (0.7, a default-real literal)
    assert list(s.urfU) == [0.6, 0.5, f32(0.7)]
    assert s.cSchemeU == 21 and s.maxiterU == 8 and s.tolRelU == 1e-3 and s.urfP == 0.25 and s.pscheme == 2
    assert s.densit == 1.2 and s.viscos == 1.5e-5
    # untouched keys keep the module defaults
    assert s.maxiterP == 30 and s.tolAbsU == f32(1e-13) and s.lSolverP.decode() == "iccg" and s.gdsU == 1.0
    assert c.calcT == 1 and c.temperature.pranl == 0.71 and c.temperature.sigt == 0.85
    assert c.temperature.urfT == 0.9 and c.temperature.maxiterT == 10
    assert s.gradScheme == fc.FC_GRAD_LSQ_DM and c.temperature.gradScheme == fc.FC_GRAD_LSQ_DM
    assert c.limiter == fc.FC_LIMITER_VENKAT
    assert c.transient.scheme == fc.FC_TIME_BDF2 and c.transient.piso == 0 and c.transient.timestep == 0.005
    assert s.npcor == 2 and (c.run.numstep, c.run.maxit, c.run.tolerance, c.run.temperature) == (10, 3, 1e-4, 1)


def test_element_assignment_and_steady_default():
    fc = load_fcgpu()
    c = read(fc, "&input_parameters\n urfU(2) = 0.4\n PISO = T\n ncorr = 3\n node_gauss = T\n/\n")
    assert list(c.simple.urfU) == [f32(0.7), 0.4, f32(0.7)]
    assert c.transient.scheme == fc.FC_TIME_STEADY and c.transient.piso == 1 and c.transient.ncorr == 3
    assert c.simple.gradScheme == fc.FC_GRAD_NODE_GAUSS


@pytest.mark.parametrize("bad", ["lstsq_qr = T", "CN = T", "ltransient = T", "cSchemeU = 'nosuch'",
                                 "compressible = T", "const_mflux = T", "maxiterU = 'x'"])
def test_rejected(bad):
    fc = load_fcgpu()
    with pytest.raises(fc.FcError):
        read(fc, "&input_parameters\n " + bad + "\n/\n")


def test_missing_group_or_terminator():
    fc = load_fcgpu()
    with pytest.raises(fc.FcError):
        read(fc, "title = 'x'\n")
    with pytest.raises(fc.FcError):
        read(fc, "&input_parameters\n title = 'x'\n")
