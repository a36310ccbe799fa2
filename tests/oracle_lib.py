"""ctypes view of the C++ oracle (oracle/), for tests and the CPU-baseline leg.

The oracle is test infrastructure: a CPU restatement of the reference Fortran
routines.  This module only loads it (building it with `make` when the shared
library is missing) and converts numpy arrays at the boundary.
"""
import ctypes as C
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")

_libs = {}


def build():
    subprocess.run(["make", "-s", "-C", ORACLE_DIR], check=True)


def lib(fast=False):
    name = "liboracle_fast.so" if fast else "liboracle.so"
    if name in _libs:
        return _libs[name]
    path = os.path.join(ORACLE_DIR, "build", name)
    if not os.path.exists(path):
        build()
    L = C.CDLL(path)
    dp = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
    ip = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
    L.orc_case_new.restype = C.c_void_p
    L.orc_case_new.argtypes = [C.c_int] * 4 + [dp, dp, dp, ip, ip, ip, ip, C.c_int, ip, ip, ip, ip]
    L.orc_case_free.argtypes = [C.c_void_p]
    L.orc_case_sizes.argtypes = [C.c_void_p, ip]
    for f in ("orc_case_get", "orc_case_set"):
        getattr(L, f).argtypes = [C.c_void_p, C.c_char_p, dp]
    L.orc_case_get_int.argtypes = [C.c_void_p, C.c_char_p, ip]
    L.orc_case_set_param.argtypes = [C.c_void_p, C.c_char_p, C.c_double]
    L.orc_case_set_solver.argtypes = [C.c_void_p, C.c_char_p, C.c_char_p]
    L.orc_case_get_scalar.restype = C.c_double
    L.orc_case_get_scalar.argtypes = [C.c_void_p, C.c_char_p]
    L.orc_grad.argtypes = [C.c_void_p, C.c_int, dp, dp]
    L.orc_prepare_lsq.argtypes = [C.c_void_p, C.c_int]
    L.orc_laplacian.argtypes = [C.c_void_p, dp, dp, C.c_ulonglong]
    L.orc_gradp_and_sources.argtypes = [C.c_void_p, C.c_int]
    for f in ("orc_init_flmass", "orc_update_velocity_at_boundary", "orc_calcuvw", "orc_calcp_simple",
              "orc_wall_distance", "orc_calc_strain", "orc_modify_mu_eff_sst", "orc_kw_sst"):
        getattr(L, f).argtypes = [C.c_void_p]
    L.orc_calcsc_sst.argtypes = [C.c_void_p, C.c_int]
    L.orc_simple_iteration.argtypes = [C.c_void_p, dp, dp]
    L.orc_time_shift.argtypes = [C.c_void_p]
    L.orc_piso_iteration.argtypes = [C.c_void_p, dp]
    L.orc_case_set_bcdfrac_t.argtypes = [C.c_void_p, C.c_int, C.c_double]
    L.orc_calculate_temperature.argtypes = [C.c_void_p, C.c_int]
    L.orc_cd_assemble.argtypes = [C.c_void_p, dp, dp]
    L.orc_cd_gradient.argtypes = [C.c_void_p, dp, dp, dp]
    L.orc_solve.argtypes = [C.c_char_p, C.c_int, C.c_int, ip, ip, dp, ip, dp, dp, dp, C.c_int, C.c_double,
                            C.c_double, dp]
    L.orc_dic_setup.argtypes = [C.c_int, ip, ip, dp, ip, dp, C.c_int]
    L.orc_precond_apply.argtypes = [C.c_int, ip, ip, dp, ip, dp, dp, dp]
    L.orc_spmv.argtypes = [C.c_int, ip, ip, dp, dp, dp, C.c_int]
    L.orc_ilu0.argtypes = [C.c_int, ip, ip, dp, ip, dp, ip]
    _libs[name] = L
    return L


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


class Case:
    """Reference-layout state (mesh, geometry, CSR, fields) held by the oracle."""

    def __init__(self, mesh, fast=False):
        self.L = lib(fast)
        m = mesh
        self.h = self.L.orc_case_new(m["numNodes"], m["numCells"], m["numInnerFaces"], m["numBoundaryFaces"],
                                     _f64(m["x"]), _f64(m["y"]), _f64(m["z"]), _i32(m["nnodes"]),
                                     _i32(m["nodes"]), _i32(m["owner"]), _i32(m["neighbour"]),
                                     len(m["bctype"]), _i32(m["bctype"]), _i32(m["nfaces"]), _i32(m["startFace"]),
                                     _i32(m.get("startFaceTwin", np.full(len(m["bctype"]), -1))))
        s = np.zeros(9, np.int32)
        self.L.orc_case_sizes(self.h, s)
        (self.numCells, self.numInnerFaces, self.numBoundaryFaces, self.numFaces, self.numTotal, self.nnz,
         self.nwal, self.nsym, self.numPeriodic) = [int(v) for v in s]

    def __del__(self):
        try:
            self.L.orc_case_free(self.h)
        except Exception:
            pass

    _lens = None

    def _len(self, name):
        faces = ("arx", "ary", "arz", "xf", "yf", "zf", "flmass")
        cells = ("xc", "yc", "zc", "vol", "su", "sv", "sw", "spu", "spv", "sp", "apu", "apv", "apw", "d",
                 "rU", "rV", "rW", "gen", "magStrain", "walldist")
        total = ("u", "v", "w", "p", "pp", "vis", "den", "t", "uo", "vo", "wo", "uoo", "voo", "woo", "uooo",
                 "vooo", "wooo", "te", "ed", "fsst")
        if name in faces:
            return self.numFaces
        if name in cells:
            return self.numCells
        if name in total:
            return self.numTotal
        if name in ("ijk", "jik"):
            return self.numInnerFaces + self.numPeriodic
        if name in ("facint", "Df", "neighbour"):
            return self.numInnerFaces
        if name in ("dUdxi", "dVdxi", "dWdxi", "dPdxi", "dTdxi", "dTEdxi", "dEDdxi"):
            return 3 * self.numTotal
        if name == "Dmat":
            return 9 * self.numCells
        if name in ("a", "ja"):
            return self.nnz
        if name == "ia":
            return self.numCells + 1
        if name == "diag":
            return self.numCells
        if name in ("dnw", "srdw", "visw", "tau", "ypl"):
            return self.nwal
        if name in ("dns", "srds"):
            return self.nsym
        if name == "owner":
            return self.numFaces
        raise KeyError(name)

    def get(self, name):
        out = np.zeros(self._len(name), np.float64)
        if self.L.orc_case_get(self.h, name.encode(), out) < 0:
            raise KeyError(name)
        return out

    def set(self, name, values):
        v = _f64(values)
        assert v.size == self._len(name), (name, v.size)
        if self.L.orc_case_set(self.h, name.encode(), v) < 0:
            raise KeyError(name)

    def get_int(self, name):
        out = np.zeros(self._len(name), np.int32)
        if self.L.orc_case_get_int(self.h, name.encode(), out) < 0:
            raise KeyError(name)
        return out

    def param(self, name, value):
        assert self.L.orc_case_set_param(self.h, name.encode(), float(value)) == 0, name

    def solver(self, which, name):
        self.L.orc_case_set_solver(self.h, which.encode(), name.encode())

    def scalar(self, name):
        return self.L.orc_case_get_scalar(self.h, name.encode())

    def grad(self, scheme, phi):
        out = np.zeros(3 * self.numTotal, np.float64)
        self.L.orc_grad(self.h, scheme, _f64(phi), out)
        return out

    def laplacian(self, mu, phi, mask=(1 << 64) - 1):
        self.L.orc_laplacian(self.h, _f64(mu), _f64(phi), mask)

    def set_bcdfrac_t(self, ib, value):
        """bcDFraction(7, ib) of the temperature equation (ib 1-based)."""
        assert self.L.orc_case_set_bcdfrac_t(self.h, int(ib), float(value)) == 0

    def calculate_temperature(self, solve=True):
        return self.L.orc_calculate_temperature(self.h, 1 if solve else 0)

    def cd_assemble(self, gamma, source):
        """Implicit convection-diffusion operator into a, source*vol into su."""
        self.L.orc_cd_assemble(self.h, _f64(gamma), _f64(source))

    def cd_gradient(self, phi, lam):
        out = np.zeros(self.numCells)
        self.L.orc_cd_gradient(self.h, _f64(phi), _f64(lam), out)
        return out

    def wall_distance(self):
        return self.L.orc_wall_distance(self.h)

    def kw_sst(self):
        """One modify_viscosity_turbulence with the k-omega SST model."""
        return self.L.orc_kw_sst(self.h)

    def time_shift(self):
        self.L.orc_time_shift(self.h)

    def piso_iteration(self):
        r = np.zeros(4)
        st = self.L.orc_piso_iteration(self.h, r)
        return st, r

    def simple_iteration(self):
        r = np.zeros(4)
        t = np.zeros(1)
        st = self.L.orc_simple_iteration(self.h, r, t)
        return st, r, float(t[0])


def solve(solver, ia, ja, a, diag, fi, rhs, itr_max, tol_abs, tol_rel, fast=False):
    """Standalone reference solver; returns (x, res0, info[itr, res0_l1, resl, factor], status)."""
    L = lib(fast)
    x = _f64(fi).copy()
    r0 = np.zeros(1)
    info = np.zeros(4)
    n = len(ia) - 1
    st = L.orc_solve(solver.encode(), n, len(ja), _i32(ia), _i32(ja), _f64(a), _i32(diag), x, _f64(rhs), r0,
                     int(itr_max), float(tol_abs), float(tol_rel), info)
    return x, float(r0[0]), info, st


def dic_setup(ia, ja, a, diag, dilu=False):
    n = len(ia) - 1
    d = np.zeros(n)
    lib().orc_dic_setup(n, _i32(ia), _i32(ja), _f64(a), _i32(diag), d, int(dilu))
    return d


def precond_apply(ia, ja, a, diag, d, r):
    n = len(ia) - 1
    z = np.zeros(n)
    lib().orc_precond_apply(n, _i32(ia), _i32(ja), _f64(a), _i32(diag), _f64(d), _f64(r), z)
    return z


def spmv(ia, ja, a, x, transpose=False):
    n = len(ia) - 1
    y = np.zeros(n)
    lib().orc_spmv(n, _i32(ia), _i32(ja), _f64(a), _f64(x), y, int(transpose))
    return y
