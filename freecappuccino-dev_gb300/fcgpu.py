"""Python view of libfcgpu.so (the C ABI declared in include/fc_gpu.h).

A thin ctypes layer used by the tests and bench.py; every call goes straight
to the CUDA library.  There is no CPU fallback: if the library is missing or
no GPU is present, the calls fail with an error.

Array arguments may be numpy arrays (host memory, copied by the library) or
objects exposing data_ptr() (device memory used in place, e.g. torch CUDA
tensors), or raw integer device addresses.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libfcgpu.so")

FC_OK = 0
FC_WARN_MAXITER = 1
FC_ERR_BAD_INPUT = -1
FC_ERR_CUDA = -2
FC_ERR_NAN = -3
FC_ERR_BREAKDOWN = -4
FC_ERR_TIMEOUT = -5
FC_ERR_STATE = -6
FC_ERR_UNSUPPORTED = -7
FC_ERR_ZERO_PIVOT = -8

BC = {"wall": 1, "inlet": 2, "outlet": 3, "symmetry": 4, "pressure": 5, "empty": 6, "periodic": 7}
FC_GRAD_GAUSS, FC_GRAD_LSQ, FC_GRAD_LSQ_DM, FC_GRAD_NODE_GAUSS = 0, 1, 2, 3
FC_GRAD_LSQ_EXACT, FC_GRAD_LSQ_DM_EXACT = 4, 5  # correct 3x3 least-squares solve (no reference counterpart)
FC_C2N_PSL, FC_C2N_IDS = 0, 1
FC_LIMITER_NONE, FC_LIMITER_BJ, FC_LIMITER_VENKAT, FC_LIMITER_R, FC_LIMITER_MD = 0, 1, 2, 3, 4
FC_TIME_STEADY, FC_TIME_BDF, FC_TIME_BDF2, FC_TIME_BDF3 = 0, 1, 2, 3
FC_PREC_FP64 = 0
FC_PREC_MIXED = 1
FC_PREC_MIXED_COLOURED = 2
FC_PREC_COLOURED_FP64 = 3  # the coloured inner ICCG in FP64 (diagnostic)
FC_NOALLOC_MAX_N = 1 << 20  # rows of fc_dpcg_noalloc's static scratch
GRAD = {"gauss": 0, "lstsq": 1, "lstsq_dm": 2}
NOMAX = 6


class FcError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"fc error {code}: {msg}")
        self.code = code


class SolveInfo(C.Structure):
    _fields_ = [("status", C.c_int), ("itr_used", C.c_int), ("outer_iterations", C.c_int),
                ("early_exit", C.c_int), ("res0_l1", C.c_double), ("resor", C.c_double),
                ("resl", C.c_double), ("factor", C.c_double), ("ms", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_lib = None


def lib():
    """Load libfcgpu.so (building it first if it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        import importlib.util
        spec = importlib.util.spec_from_file_location("fc_build", os.path.join(HERE, "build.py"))
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        mod.build()
    L = C.CDLL(LIB_PATH)
    vp, ip, i, d, cp = C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_char_p
    sig = {
        "fc_mesh_box": (i, [i, i, i, d, d, d, d, C.c_ulonglong, i, vp, C.POINTER(vp)]),
        "fc_mesh_from_arrays": (i, [i, i, i, i, vp, vp, vp, vp, vp, vp, vp, i, vp, vp, vp, C.POINTER(vp)]),
        "fc_mesh_read_native": (i, [cp, C.POINTER(vp)]),
        "fc_mesh_write_native": (i, [vp, cp]),
        "fc_mesh_read_openfoam": (i, [cp, C.POINTER(vp)]),
        "fc_mesh_write_openfoam": (i, [vp, cp]),
        "fc_mesh_info": (i, [vp, vp]),
        "fc_mesh_export": (i, [vp] + [vp] * 10),
        "fc_mesh_set_twin": (i, [vp, i, i]),
        "fc_mesh_twins": (i, [vp, vp]),
        "fc_mesh_free": (None, [vp]),
        "fc_init": (i, [i, C.POINTER(vp)]),
        "fc_finalize": (None, [vp]),
        "fc_last_error": (cp, [vp]),
        "fc_set_verbosity": (i, [vp, i]),
        "fc_set_precision": (i, [vp, i, d, i]),
        "fc_kernel_launches": (C.c_longlong, [vp]),
        "fc_device_alloc_count": (C.c_longlong, []),
        "fc_debug_fill_allocations": (i, [i]),
        "fc_stream_sync": (i, [vp]),
        "fc_stream": (vp, [vp]),
        "fc_event_record": (i, [vp, i]),
        "fc_event_elapsed_ms": (i, [vp, C.POINTER(C.c_float)]),
        "fc_csrsolve": (i, [vp, cp, i, i, vp, vp, vp, vp, vp, vp, vp, i, d, d, cp, i, C.POINTER(SolveInfo)]),
        "fc_csr_pattern_forget": (i, [vp]),
        "fc_precond_setup": (i, [vp, cp, i, i, vp, vp, vp, vp, vp]),
        "fc_precond_apply": (i, [vp, cp, i, i, vp, vp, vp, vp, vp, vp]),
        "fc_spmv": (i, [vp, i, i, vp, vp, vp, vp, vp, vp, i]),
        "fc_ilu0": (i, [vp, i, i, vp, vp, vp, vp, vp]),
        "fc_dpcg_noalloc": (i, [vp, i, i, vp, vp, vp, vp, vp, vp, i, d, d, C.POINTER(SolveInfo), vp, i]),
        "fc_set_mesh": (i, [vp, vp]),
        "fc_get_geometry": (i, [vp, cp, vp]),
        "fc_get_csr_pattern": (i, [vp, vp, vp, vp, vp, vp, vp, vp]),
        "fc_get_setup_times": (i, [vp, vp]),
        "fc_field_set": (i, [vp, cp, vp, C.c_longlong]),
        "fc_field_get": (i, [vp, cp, vp, C.c_longlong]),
        "fc_field_fill": (i, [vp, cp, d]),
        "fc_field_ptr": (vp, [vp, cp]),
        "fc_grad": (i, [vp, i, vp, vp]),
        "fc_laplacian": (i, [vp, vp, vp, C.c_ulonglong]),
        "fc_solve_field": (i, [vp, cp, cp, cp, vp, i, d, d, cp, C.POINTER(SolveInfo)]),
        "fc_simple_set_params": (i, [vp, vp]),
        "fc_sweep_stats": (i, [vp, i, vp]),
        "fc_mixed_colours": (i, [vp, i, vp]),
        "fc_set_sweep_cap": (i, [vp, i]),
        "fc_set_sweep_tiles": (i, [vp, i]),
        "fc_set_sweep_stage_rows": (i, [vp, i]),
        "fc_set_tracing": (i, [vp, i]),
        "fc_trace_get": (i, [vp, vp, vp]),
        "fc_init_flmass": (i, [vp]),
        "fc_update_velocity_at_boundary": (i, [vp]),
        "fc_gradp_and_sources": (i, [vp, cp]),
        "fc_calcuvw": (i, [vp, vp]),
        "fc_calcp_simple": (i, [vp, vp]),
        "fc_simple_iteration": (i, [vp, vp]),
        "fc_temperature_set_params": (i, [vp, vp, vp]),
        "fc_turbulence_set_params": (i, [vp, vp]),
        "fc_wall_distance": (i, [vp]),
        "fc_kw_sst": (i, [vp, vp]),
        "fc_calculate_temperature": (i, [vp, i, vp]),
        "fc_cd_assemble": (i, [vp, vp, vp]),
        "fc_cd_solve": (i, [vp, vp, i, d, C.POINTER(SolveInfo)]),
        "fc_cd_adjoint": (i, [vp, vp, vp, vp, i, d, C.POINTER(SolveInfo)]),
        "fc_simple_set_batched_momentum": (i, [vp, i]),
        "fc_set_solve_log": (i, [vp, cp]),
        "fc_set_gradient_limiter": (i, [vp, i]),
        "fc_set_node_interpolation": (i, [vp, i]),
        "fc_transient_set_params": (i, [vp, vp]),
        "fc_time_shift": (i, [vp]),
        "fc_calcp_piso": (i, [vp, vp]),
        "fc_piso_iteration": (i, [vp, vp]),
        "fc_run": (i, [vp, vp, vp, vp, vp]),
        "fc_namelist_read": (i, [cp, vp, vp, i]),
        "fc_apply_settings": (i, [vp, vp]),
        "fc_download_fields": (i, [vp, i, vp, vp, vp]),
        "fc_batch_create": (i, [vp, vp]),
        "fc_batch_destroy": (i, [vp]),
        "fc_batch_add": (i, [vp, i, i, vp, vp, vp, vp]),
        "fc_batch_plan": (i, [vp, vp]),
        "fc_batch_tiles": (i, [vp, vp]),
        "fc_batch_solve": (i, [vp, cp, vp, vp, vp, i, d, d, C.POINTER(SolveInfo)]),
        "fc_batch_tune": (i, [vp, cp, vp, vp, vp, i, d, d, i, vp]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def device_alloc_count():
    """Device allocations plus frees the library has made so far."""
    return int(lib().fc_device_alloc_count())


def debug_fill_allocations(byte):
    """Fill every later device allocation with `byte` (-1: off); 0xFF makes
    uninitialised floats and doubles NaN (fc_debug_fill_allocations)."""
    st = lib().fc_debug_fill_allocations(int(byte))
    if st < 0:
        raise FcError(st, "fc_debug_fill_allocations")


def declared_symbols(header=None):
    """Names of the functions declared in include/fc_gpu.h."""
    import re
    header = header or os.path.join(os.path.dirname(HERE), "include", "fc_gpu.h")
    txt = open(header).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(fc_[a-z0-9_]+)\s*\(", txt)))


def _ptr(x):
    if x is None:
        return None
    if isinstance(x, np.ndarray):
        assert x.flags.c_contiguous
        return x.ctypes.data_as(C.c_void_p)
    if hasattr(x, "data_ptr"):
        return C.c_void_p(x.data_ptr())
    if isinstance(x, int):
        return C.c_void_p(x)
    raise TypeError(type(x))


def _f64(x):
    if hasattr(x, "data_ptr") or isinstance(x, int):
        return x
    return np.ascontiguousarray(x, dtype=np.float64)


def _i32(x):
    if hasattr(x, "data_ptr") or isinstance(x, int):
        return x
    return np.ascontiguousarray(x, dtype=np.int32)


def stream_function_fluxes(arrays, psi):
    """Face volume fluxes of the velocity curl(psi(x, y, z) e_z) through every
    face of a mesh given by Mesh.arrays(): by Stokes' theorem the flux through
    a face is the circulation of psi e_z around its edges, here with psi
    linear along each edge, in the face's node order (which orients its area
    vector).  Every edge is shared by the faces around it with opposite
    orientations, so the fluxes of every cell sum to zero up to rounding."""
    x, y, z = arrays["x"], arrays["y"], arrays["z"]
    nn = np.asarray(arrays["nnodes"])
    nodes = np.asarray(arrays["nodes"]).reshape(-1, NOMAX) - 1
    ps = psi(x, y, z)
    flux = np.zeros(len(nn))
    for k in range(NOMAX):
        on = k < nn
        a = nodes[:, k]
        b = np.where(k + 1 < nn, nodes[:, (k + 1) % NOMAX], nodes[:, 0])
        a = np.where(on, a, 0)
        b = np.where(on, b, 0)
        flux += np.where(on, 0.5 * (ps[a] + ps[b]) * (z[b] - z[a]), 0.0)
    return flux


class SimpleParams(C.Structure):
    """fc_simple_params: namelist parameters of the SIMPLE path."""
    _fields_ = [("densit", C.c_double), ("viscos", C.c_double), ("urfU", C.c_double * 3), ("gdsU", C.c_double),
                ("urfP", C.c_double), ("cSchemeU", C.c_int), ("gradScheme", C.c_int), ("pscheme", C.c_int),
                ("maxiterU", C.c_int), ("maxiterP", C.c_int), ("npcor", C.c_int), ("pRefCell", C.c_int),
                ("tolAbsU", C.c_double), ("tolRelU", C.c_double), ("tolAbsP", C.c_double), ("tolRelP", C.c_double),
                ("lSolverU", C.c_char * 16), ("lSolverP", C.c_char * 16), ("flomas", C.c_double)]

    @classmethod
    def cavity(cls, **kw):
        """Settings of examples/cavity/input.nml (urfU 0.8, urfP 0.3, central
        scheme, gds 1, BiCGStab U / ICCG p, maxiter 5 / 20, tolRel 0.01 / 0.025)."""
        p = cls()
        p.densit, p.viscos = kw.get("densit", 1.0), kw.get("viscos", 0.01)
        for i in range(3):
            p.urfU[i] = kw.get("urfU", 0.8)
        p.gdsU, p.urfP = kw.get("gdsU", 1.0), kw.get("urfP", 0.3)
        p.cSchemeU = kw.get("scheme", 1)
        p.gradScheme = kw.get("grad", 0)
        p.pscheme = kw.get("pscheme", 0)
        p.maxiterU, p.maxiterP = kw.get("maxiterU", 5), kw.get("maxiterP", 20)
        p.npcor, p.pRefCell = kw.get("npcor", 1), kw.get("pRefCell", 1)
        p.tolAbsU, p.tolRelU = kw.get("tolAbsU", 1e-15), kw.get("tolRelU", 0.01)
        p.tolAbsP, p.tolRelP = kw.get("tolAbsP", 1e-15), kw.get("tolRelP", 0.025)
        p.lSolverU = kw.get("solverU", "bicgstab").encode()
        p.lSolverP = kw.get("solverP", "iccg").encode()
        p.flomas = kw.get("flomas", 0.0)
        return p


class RunParams(C.Structure):
    """fc_run_params: the outer loops of main.f90."""
    _fields_ = [("numstep", C.c_int), ("maxit", C.c_int), ("tolerance", C.c_double), ("temperature", C.c_int)]


class TransientParams(C.Structure):
    """fc_transient_params: unsteady momentum term and PISO."""
    _fields_ = [("timestep", C.c_double), ("scheme", C.c_int), ("piso", C.c_int), ("ncorr", C.c_int)]


class TemperatureParams(C.Structure):
    """fc_temperature_params: namelist parameters of calculate_temperature."""
    _fields_ = [("viscos", C.c_double), ("pranl", C.c_double), ("sigt", C.c_double), ("urfT", C.c_double),
                ("gdsT", C.c_double), ("cSchemeT", C.c_int), ("gradScheme", C.c_int), ("maxiterT", C.c_int),
                ("tolAbsT", C.c_double), ("tolRelT", C.c_double), ("lSolverT", C.c_char * 16)]

    @classmethod
    def defaults(cls, **kw):
        """The reference's defaults (temperature.f90:14-25): urfT 0.9, gdsT 1,
        linearUpwind, BiCGStab with maxiter 10, tolAbs 1e-13, tolRel 0.02,
        sigt 1; pranl 0.7 (air) and viscos 0.01 unless given."""
        p = cls()
        p.viscos, p.pranl, p.sigt = kw.get("viscos", 0.01), kw.get("pranl", 0.7), kw.get("sigt", 1.0)
        p.urfT, p.gdsT = kw.get("urfT", 0.9), kw.get("gdsT", 1.0)
        p.cSchemeT = kw.get("scheme", 2)
        p.gradScheme = kw.get("grad", 0)
        p.maxiterT = kw.get("maxiterT", 10)
        p.tolAbsT, p.tolRelT = kw.get("tolAbsT", 1e-13), kw.get("tolRelT", 0.02)
        p.lSolverT = kw.get("solver", "bicgstab").encode()
        return p


class TurbScalar(C.Structure):
    """fc_turb_scalar: settings of one turbulence scalar (TurbModelData.f90)."""
    _fields_ = [("urf", C.c_double), ("gds", C.c_double), ("cScheme", C.c_int), ("lSolver", C.c_char * 16),
                ("maxiter", C.c_int), ("tolAbs", C.c_double), ("tolRel", C.c_double)]

    @classmethod
    def defaults(cls, **kw):
        """TurbModelData.f90's defaults: urf 0.7, gds 1, linearUpwind,
        BiCGStab, maxiter 10, tolAbs 1e-10 (a default-real literal), tolRel 0.01."""
        t = cls()
        t.urf, t.gds = kw.get("urf", 0.7), kw.get("gds", 1.0)
        t.cScheme = kw.get("scheme", 2)
        t.lSolver = kw.get("solver", "bicgstab").encode()
        t.maxiter = kw.get("maxiter", 10)
        t.tolAbs, t.tolRel = kw.get("tolAbs", float(np.float32(1e-10))), kw.get("tolRel", 0.01)
        return t


class TurbulenceParams(C.Structure):
    """fc_turbulence_params: the k-omega SST model's settings."""
    _fields_ = [("k", TurbScalar), ("omega", TurbScalar), ("urfVis", C.c_double), ("gradScheme", C.c_int)]

    @classmethod
    def defaults(cls, k=None, omega=None, urfVis=1.0, grad=0):
        p = cls()
        p.k = k or TurbScalar.defaults()
        p.omega = omega or TurbScalar.defaults()
        p.urfVis, p.gradScheme = urfVis, grad
        return p


class CaseSettings(C.Structure):
    """fc_case_settings: the case namelist as the path uses it."""
    _fields_ = [("simple", SimpleParams), ("temperature", TemperatureParams), ("transient", TransientParams),
                ("run", RunParams), ("limiter", C.c_int), ("calcU", C.c_int), ("calcP", C.c_int),
                ("calcT", C.c_int), ("mesh_foam", C.c_int), ("title", C.c_char * 72)]


def read_namelist(path):
    """fc_namelist_read: CaseSettings of a namelist file (no GPU needed)."""
    out = CaseSettings()
    err = C.create_string_buffer(256)
    st = lib().fc_namelist_read(path.encode(), C.byref(out), err, 256)
    if st != 0:
        raise FcError(st, err.value.decode())
    return out

class Mesh:
    """Host mesh in the reference's native layout (1-based indices)."""

    def __init__(self, handle):
        self.h = handle
        info = np.zeros(6, np.int32)
        lib().fc_mesh_info(self.h, _ptr(info))
        (self.numNodes, self.numCells, self.numInnerFaces, self.numBoundaryFaces, self.numFaces,
         self.numBoundaries) = [int(v) for v in info]
        self.numTotal = self.numCells + self.numBoundaryFaces

    @classmethod
    def box(cls, nx, ny, nz, lx=1.0, ly=1.0, lz=1.0, perturb=0.0, seed=42, tets=False, sides=None):
        sides = np.array([BC[s] if isinstance(s, str) else s for s in (sides or ["wall"] * 6)], np.int32)
        h = C.c_void_p()
        st = lib().fc_mesh_box(nx, ny, nz, lx, ly, lz, perturb, seed, int(tets), _ptr(sides), C.byref(h))
        if st != 0:
            raise FcError(st, "fc_mesh_box")
        return cls(h)

    @classmethod
    def from_arrays(cls, a):
        h = C.c_void_p()
        arrs = [_f64(a["x"]), _f64(a["y"]), _f64(a["z"]), _i32(a["nnodes"]), _i32(a["nodes"]), _i32(a["owner"]),
                _i32(a["neighbour"]), _i32(a["bctype"]), _i32(a["nfaces"]), _i32(a["startFace"])]
        st = lib().fc_mesh_from_arrays(a["numNodes"], a["numCells"], a["numInnerFaces"], a["numBoundaryFaces"],
                                       *[_ptr(v) for v in arrs[:7]], len(a["bctype"]),
                                       *[_ptr(v) for v in arrs[7:]], C.byref(h))
        if st != 0:
            raise FcError(st, "fc_mesh_from_arrays")
        m = cls(h)
        twin = a.get("startFaceTwin")
        if twin is not None:
            for b, t in enumerate(np.asarray(twin)):
                if a["bctype"][b] == BC["periodic"]:
                    st = lib().fc_mesh_set_twin(m.h, b, int(t))
                    if st != 0:
                        raise FcError(st, "fc_mesh_set_twin")
        return m

    @classmethod
    def read_native(cls, d):
        h = C.c_void_p()
        st = lib().fc_mesh_read_native(d.encode(), C.byref(h))
        if st != 0:
            raise FcError(st, "fc_mesh_read_native")
        return cls(h)

    @classmethod
    def read_openfoam(cls, d):
        h = C.c_void_p()
        st = lib().fc_mesh_read_openfoam(d.encode(), C.byref(h))
        if st != 0:
            raise FcError(st, "fc_mesh_read_openfoam")
        return cls(h)

    def write_openfoam(self, d):
        st = lib().fc_mesh_write_openfoam(self.h, d.encode())
        if st != 0:
            raise FcError(st, "fc_mesh_write_openfoam")

    def write_native(self, d):
        os.makedirs(d, exist_ok=True)
        st = lib().fc_mesh_write_native(self.h, d.encode())
        if st != 0:
            raise FcError(st, "fc_mesh_write_native")

    def arrays(self):
        nN, nF, nI, nB = self.numNodes, self.numFaces, self.numInnerFaces, self.numBoundaries
        out = dict(x=np.zeros(nN), y=np.zeros(nN), z=np.zeros(nN), nnodes=np.zeros(nF, np.int32),
                   nodes=np.zeros(nF * NOMAX, np.int32), owner=np.zeros(nF, np.int32),
                   neighbour=np.zeros(max(nI, 1), np.int32), bctype=np.zeros(nB, np.int32),
                   nfaces=np.zeros(nB, np.int32), startFace=np.zeros(nB, np.int32))
        lib().fc_mesh_export(self.h, *[_ptr(out[k]) for k in ("x", "y", "z", "nnodes", "nodes", "owner",
                                                              "neighbour", "bctype", "nfaces", "startFace")])
        out["neighbour"] = out["neighbour"][:nI]
        out["startFaceTwin"] = np.zeros(nB, np.int32)
        lib().fc_mesh_twins(self.h, _ptr(out["startFaceTwin"]))
        out.update(numNodes=nN, numCells=self.numCells, numInnerFaces=nI, numBoundaryFaces=self.numBoundaryFaces)
        return out

    def __del__(self):
        try:
            lib().fc_mesh_free(self.h)
        except Exception:
            pass


class Context:
    """One GPU context (fc_ctx): a stream, the mesh, its matrix and fields."""

    def __init__(self, device=0):
        self.L = lib()
        h = C.c_void_p()
        st = self.L.fc_init(device, C.byref(h))
        if st != 0:
            raise FcError(st, "fc_init (is a GPU present?)")
        self.h = h
        self.mesh = None

    def close(self):
        if self.h:
            self.L.fc_finalize(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st, what):
        if st < 0:
            raise FcError(st, f"{what}: {self.L.fc_last_error(self.h).decode()}")
        return st

    def error(self):
        return self.L.fc_last_error(self.h).decode()

    def set_verbosity(self, level):
        self.L.fc_set_verbosity(self.h, level)

    def set_precision(self, mode, inner_tol=0.0, inner_itmax=0):
        self._check(self.L.fc_set_precision(self.h, mode, inner_tol, inner_itmax), "fc_set_precision")

    def kernel_launches(self):
        return int(self.L.fc_kernel_launches(self.h))

    def sync(self):
        self._check(self.L.fc_stream_sync(self.h), "sync")

    def stream(self):
        return self.L.fc_stream(self.h)

    def event(self, which):
        self._check(self.L.fc_event_record(self.h, which), "event")

    def elapsed_ms(self):
        ms = C.c_float()
        self._check(self.L.fc_event_elapsed_ms(self.h, C.byref(ms)), "elapsed")
        return float(ms.value)

    # --------------------------------------------------------------- solvers
    def csrsolve(self, solver, ia, ja, a, diag, fi, rhs, itr_max, tol_abs, tol_rel, chvar="x", verbose=0,
                 raise_on_error=True):
        """Returns (x, res0, info, status); fi is not modified when it is a numpy array."""
        ia, ja, diag = _i32(ia), _i32(ja), _i32(diag)
        a, rhs = _f64(a), _f64(rhs)
        x = _f64(fi).copy() if isinstance(fi, np.ndarray) or not hasattr(fi, "data_ptr") else fi
        n = len(ia) - 1 if isinstance(ia, np.ndarray) else None
        nnz = len(ja) if isinstance(ja, np.ndarray) else None
        self._keep = (ia, ja, diag)  # pattern cache is keyed by these addresses
        r0 = np.zeros(1)
        info = SolveInfo()
        st = self.L.fc_csrsolve(self.h, solver.encode(), n, nnz, _ptr(ia), _ptr(ja), _ptr(a), _ptr(diag), _ptr(x),
                                _ptr(rhs), _ptr(r0), int(itr_max), float(tol_abs), float(tol_rel), chvar.encode(),
                                int(verbose), C.byref(info))
        if raise_on_error:
            self._check(st, "fc_csrsolve")
        return x, float(r0[0]), info, st

    def csrsolve_sized(self, solver, n, nnz, ia, ja, a, diag, x, rhs, itr_max, tol_abs, tol_rel, chvar="x"):
        """Same call with explicit sizes (device arrays); x is updated in place."""
        r0 = np.zeros(1)
        info = SolveInfo()
        st = self.L.fc_csrsolve(self.h, solver.encode(), n, nnz, _ptr(ia), _ptr(ja), _ptr(a), _ptr(diag), _ptr(x),
                                _ptr(rhs), _ptr(r0), int(itr_max), float(tol_abs), float(tol_rel), chvar.encode(),
                                0, C.byref(info))
        self._check(st, "fc_csrsolve")
        return float(r0[0]), info, st

    def dpcg_noalloc(self, n, nnz, ia, ja, a, diag, x, b, itr_max, tol_abs, tol_rel, stream=None):
        """fc_dpcg_noalloc on device arrays (0-based ia/ja/diag; x updated in
        place); stream defaults to this context's stream.  Returns (status,
        info); raises on an error status with the call's own message."""
        info = SolveInfo()
        err = C.create_string_buffer(256)
        st = self.L.fc_dpcg_noalloc(stream if stream is not None else self.L.fc_stream(self.h), int(n), int(nnz),
                                    _ptr(ia), _ptr(ja), _ptr(a), _ptr(diag), _ptr(x), _ptr(b), int(itr_max),
                                    float(tol_abs), float(tol_rel), C.byref(info), C.cast(err, C.c_void_p), 256)
        if st < 0:
            raise FcError(st, err.value.decode())
        return st, info

    def pattern_forget(self):
        self.L.fc_csr_pattern_forget(self.h)

    def precond_setup(self, kind, ia, ja, a, diag):
        ia, ja, diag, a = _i32(ia), _i32(ja), _i32(diag), _f64(a)
        self._keep = (ia, ja, diag)
        d = np.zeros(len(ia) - 1)
        self._check(self.L.fc_precond_setup(self.h, kind.encode(), len(ia) - 1, len(ja), _ptr(ia), _ptr(ja), _ptr(a),
                                            _ptr(diag), _ptr(d)), "fc_precond_setup")
        return d

    def precond_apply(self, kind, ia, ja, a, diag, q):
        ia, ja, diag, a, q = _i32(ia), _i32(ja), _i32(diag), _f64(a), _f64(q)
        self._keep = (ia, ja, diag)
        z = np.zeros(len(ia) - 1)
        self._check(self.L.fc_precond_apply(self.h, kind.encode(), len(ia) - 1, len(ja), _ptr(ia), _ptr(ja), _ptr(a),
                                            _ptr(diag), _ptr(q), _ptr(z)), "fc_precond_apply")
        return z

    def spmv(self, ia, ja, a, diag, x, transpose=False):
        ia, ja, diag, a, x = _i32(ia), _i32(ja), _i32(diag), _f64(a), _f64(x)
        self._keep = (ia, ja, diag)
        y = np.zeros(len(ia) - 1)
        self._check(self.L.fc_spmv(self.h, len(ia) - 1, len(ja), _ptr(ia), _ptr(ja), _ptr(a), _ptr(diag), _ptr(x),
                                   _ptr(y), int(transpose)), "fc_spmv")
        return y

    def ilu0(self, ia, ja, a, diag):
        ia, ja, diag, a = _i32(ia), _i32(ja), _i32(diag), _f64(a)
        self._keep = (ia, ja, diag)
        l = np.zeros(len(ja))
        self._check(self.L.fc_ilu0(self.h, len(ia) - 1, len(ja), _ptr(ia), _ptr(ja), _ptr(a), _ptr(diag), _ptr(l)),
                    "fc_ilu0")
        return l

    # ------------------------------------------------------- mesh and fields
    def set_mesh(self, mesh):
        self._check(self.L.fc_set_mesh(self.h, mesh.h), "fc_set_mesh")
        self.mesh = mesh

    def geometry(self, name):
        m = self.mesh
        n = {"arx": m.numFaces, "ary": m.numFaces, "arz": m.numFaces, "xf": m.numFaces, "yf": m.numFaces,
             "zf": m.numFaces, "xc": m.numCells, "yc": m.numCells, "zc": m.numCells, "vol": m.numCells,
             "facint": m.numInnerFaces, "Df": m.numInnerFaces}[name]
        out = np.zeros(n)
        self._check(self.L.fc_get_geometry(self.h, name.encode(), _ptr(out)), "fc_get_geometry")
        return out

    def csr_pattern(self):
        """(ia, ja, diag, ijk, jik), 1-based; the slot maps hold the inner
        faces, then the periodic pairs."""
        m = self.mesh
        n, nnz = C.c_int(0), C.c_int(0)
        self._check(self.L.fc_get_csr_pattern(self.h, C.byref(n), C.byref(nnz), None, None, None, None, None),
                    "fc_get_csr_pattern")
        nl = (nnz.value - n.value) // 2  # numInnerFaces + numPeriodic
        ia = np.zeros(m.numCells + 1, np.int32)
        ja = np.zeros(nnz.value, np.int32)
        dg = np.zeros(m.numCells, np.int32)
        ijk = np.zeros(max(1, nl), np.int32)
        jik = np.zeros(max(1, nl), np.int32)
        self._check(self.L.fc_get_csr_pattern(self.h, None, None, _ptr(ia), _ptr(ja), _ptr(dg), _ptr(ijk), _ptr(jik)),
                    "fc_get_csr_pattern")
        return ia, ja, dg, ijk[:nl], jik[:nl]

    SETUP_PHASES = ("topology", "geometry", "periodic", "csr", "tiling", "schedule", "analysis", "fields")

    def setup_times(self):
        """Seconds of the phases of the last set_mesh (fc_get_setup_times)."""
        t = np.zeros(len(self.SETUP_PHASES))
        self._check(self.L.fc_get_setup_times(self.h, _ptr(t)), "fc_get_setup_times")
        return dict(zip(self.SETUP_PHASES, t.tolist()))

    def field_len(self, name):
        m = self.mesh
        if name in ("u", "v", "w", "p", "pp", "vis", "den", "t", "uo", "vo", "wo", "uoo", "voo", "woo", "uooo",
                    "vooo", "wooo", "te", "ed", "fsst"):
            return m.numTotal
        if name in ("gen", "magStrain", "walldist"):
            return m.numCells
        if name in ("tau", "ypl"):
            return self._nwal()
        if name in ("rU", "rV", "rW"):
            return m.numCells
        if name == "flmass":
            return m.numFaces
        if name in ("su", "sv", "sw", "spu", "spv", "sp", "apu", "apv", "apw"):
            return m.numCells
        if name in ("dUdxi", "dVdxi", "dWdxi", "dPdxi", "dTdxi", "dTEdxi", "dEDdxi"):
            return 3 * m.numTotal
        if name == "a":  # nnz: 2 (numInnerFaces + numPeriodic) + numCells
            n, nnz = C.c_int(0), C.c_int(0)
            self._check(self.L.fc_get_csr_pattern(self.h, C.byref(n), C.byref(nnz), None, None, None, None, None),
                        "fc_get_csr_pattern")
            return nnz.value
        if name == "visw":
            return self._nwal()
        raise KeyError(name)

    def _nwal(self):
        a = self.mesh.arrays()
        n = int(sum(nf for t, nf in zip(a["bctype"], a["nfaces"]) if t == BC["wall"]))
        return max(n, 1)

    def field_set(self, name, values):
        v = _f64(values)
        n = self.field_len(name)
        if isinstance(v, np.ndarray):
            assert v.size == n, (name, v.size, n)
        self._check(self.L.fc_field_set(self.h, name.encode(), _ptr(v), n), f"fc_field_set({name})")

    def field_get(self, name):
        n = self.field_len(name)
        out = np.zeros(n)
        self._check(self.L.fc_field_get(self.h, name.encode(), _ptr(out), n), f"fc_field_get({name})")
        return out

    def field_fill(self, name, value):
        self._check(self.L.fc_field_fill(self.h, name.encode(), float(value)), f"fc_field_fill({name})")

    def field_ptr(self, name):
        return self.L.fc_field_ptr(self.h, name.encode())

    def grad(self, scheme, phi):
        out = np.zeros(3 * self.mesh.numTotal)
        s = GRAD[scheme] if isinstance(scheme, str) else scheme
        self._check(self.L.fc_grad(self.h, s, _ptr(_f64(phi)), _ptr(out)), "fc_grad")
        return out

    def laplacian(self, mu, phi, mask=(1 << 64) - 1):
        self._check(self.L.fc_laplacian(self.h, _ptr(_f64(mu)), _ptr(_f64(phi)), mask), "fc_laplacian")

    def solve_field(self, solver, x_field, rhs_field, itr_max, tol_abs, tol_rel, chvar="x"):
        r0 = np.zeros(1)
        info = SolveInfo()
        st = self.L.fc_solve_field(self.h, solver.encode(), x_field.encode(), rhs_field.encode(), _ptr(r0),
                                   int(itr_max), float(tol_abs), float(tol_rel), chvar.encode(), C.byref(info))
        self._check(st, "fc_solve_field")
        return float(r0[0]), info, st

    def sweep_stats(self, which=0):
        out = np.zeros(11)
        self._check(self.L.fc_sweep_stats(self.h, which, _ptr(out)), "fc_sweep_stats")
        keys = ("tiles", "levels", "max_width", "ring_depth", "est_sweep_us", "ring_entries", "pushed_entries",
                "cross_tile_entries", "stages", "max_tile_steps", "staged_rows")
        return dict(zip(keys, [float(v) for v in out]))

    def set_sweep_stage_rows(self, rows):
        """Rows of a step held in the stage buffers in the pattern analyses that follow (0: the default)."""
        self._check(self.L.fc_set_sweep_stage_rows(self.h, int(rows)), "fc_set_sweep_stage_rows")

    def set_sweep_tiles(self, tiles):
        """Tile count of the pattern analyses that follow (0: the default)."""
        self._check(self.L.fc_set_sweep_tiles(self.h, int(tiles)), "fc_set_sweep_tiles")

    def set_sweep_cap(self, rows):
        """Rows per sweep step cap of the next pattern analyses (0: default)."""
        self._check(self.L.fc_set_sweep_cap(self.h, int(rows)), "fc_set_sweep_cap")

    def mixed_colours(self, which=0):
        """Colours of the multicolour ordering of FC_PREC_MIXED_COLOURED."""
        out = np.zeros(1, np.int32)
        self._check(self.L.fc_mixed_colours(self.h, which, _ptr(out)), "fc_mixed_colours")
        return int(out[0])

    def set_tracing(self, on=True):
        self._check(self.L.fc_set_tracing(self.h, int(on)), "fc_set_tracing")

    def trace(self, timeline=False):
        """Phase cycles of the last traced ICCG solve: (dict phase -> cycles
        summed over blocks, blocks); with timeline=True also the step stamps
        as a uint64 array [sweep(fwd, bwd)][tile][step][8]: step start,
        stage buffer landed, staging started (clock64), step start
        (globaltimer), then thread 0's next-step loads issued, dependency
        values ready, value computed, stores issued (clock64)."""
        out = np.zeros(11)
        self._check(self.L.fc_trace_get(self.h, _ptr(out), None), "fc_trace_get")
        keys = ("setup", "fwd_sweep", "sweep_barrier", "bwd_sweep", "dot", "p_update", "spmv", "xr_update")
        res = (dict(zip(keys, out[:8].tolist())), int(out[8]))
        if not timeline:
            return res
        nb, cap = int(out[9]), int(out[10])
        tl = np.zeros((2, nb, cap, 8), dtype=np.uint64)
        self._check(self.L.fc_trace_get(self.h, _ptr(out), _ptr(tl)), "fc_trace_get")
        return res + (tl,)

    # ------------------------------------------------------------ SIMPLE
    def simple_params(self, prm):
        self._prm = prm
        self._check(self.L.fc_simple_set_params(self.h, C.byref(prm)), "fc_simple_set_params")

    def init_flmass(self):
        self._check(self.L.fc_init_flmass(self.h), "fc_init_flmass")

    def gradp_and_sources(self, field="p"):
        self._check(self.L.fc_gradp_and_sources(self.h, field.encode()), "fc_gradp_and_sources")

    def calcuvw(self):
        r = np.zeros(3)
        self._check(self.L.fc_calcuvw(self.h, _ptr(r)), "fc_calcuvw")
        return r

    def calcp_simple(self):
        r = np.zeros(1)
        self._check(self.L.fc_calcp_simple(self.h, _ptr(r)), "fc_calcp_simple")
        return float(r[0])

    def simple_iteration(self):
        r = np.zeros(4)
        self._check(self.L.fc_simple_iteration(self.h, _ptr(r)), "fc_simple_iteration")
        return r

    # ------------------------------------------ convection-diffusion adjoint
    def cd_assemble(self, gamma, source):
        self._check(self.L.fc_cd_assemble(self.h, _ptr(_f64(gamma)), _ptr(_f64(source))), "fc_cd_assemble")

    def cd_solve(self, itr_max=2000, tol_rel=1e-12):
        """Returns (phi, info)."""
        phi = np.zeros(self.mesh.numCells)
        info = SolveInfo()
        st = self.L.fc_cd_solve(self.h, _ptr(phi), int(itr_max), float(tol_rel), C.byref(info))
        self._check(st, "fc_cd_solve")
        return phi, info

    def cd_adjoint(self, dJdphi, itr_max=2000, tol_rel=1e-12):
        """Returns (lambda, dJ/dgamma, info)."""
        n = self.mesh.numCells
        lam, grad = np.zeros(n), np.zeros(n)
        info = SolveInfo()
        st = self.L.fc_cd_adjoint(self.h, _ptr(_f64(dJdphi)), _ptr(lam), _ptr(grad), int(itr_max), float(tol_rel),
                                  C.byref(info))
        self._check(st, "fc_cd_adjoint")
        return lam, grad, info

    def set_node_interpolation(self, method):
        """FC_C2N_PSL (0) or FC_C2N_IDS (1) for node-based gradients."""
        self._check(self.L.fc_set_node_interpolation(self.h, int(method)), "fc_set_node_interpolation")

    def set_gradient_limiter(self, kind):
        """FC_LIMITER_* for every gradient of the context (0: none)."""
        self._check(self.L.fc_set_gradient_limiter(self.h, int(kind)), "fc_set_gradient_limiter")

    def set_solve_log(self, path):
        """JSON line per solve appended to path (None: stop)."""
        self._check(self.L.fc_set_solve_log(self.h, path.encode() if path else None), "fc_set_solve_log")

    def download_fields(self, names):
        """{name: numpy array} of several fields, one synchronisation."""
        outs = [np.zeros(self.field_len(nm)) for nm in names]
        cn = (C.c_char_p * len(names))(*[nm.encode() for nm in names])
        po = (C.c_void_p * len(names))(*[o.ctypes.data for o in outs])
        cnt = (C.c_longlong * len(names))(*[len(o) for o in outs])
        self._check(self.L.fc_download_fields(self.h, len(names), cn, po, cnt), "fc_download_fields")
        return dict(zip(names, outs))

    def transient_params(self, timestep, scheme, piso=0, ncorr=1):
        prm = TransientParams(float(timestep), int(scheme), int(piso), int(ncorr))
        self._check(self.L.fc_transient_set_params(self.h, C.byref(prm)), "fc_transient_set_params")

    def run(self, numstep, maxit, tolerance, temperature=False):
        """main.f90's time and iteration loops; returns (steps, iterations, resor[4])."""
        p = RunParams(int(numstep), int(maxit), float(tolerance), int(bool(temperature)))
        steps, iters = C.c_int(0), C.c_int(0)
        r = np.zeros(4)
        self._check(self.L.fc_run(self.h, C.byref(p), C.byref(steps), C.byref(iters), _ptr(r)), "fc_run")
        return steps.value, iters.value, r

    def apply_settings(self, settings):
        """fc_apply_settings: simple, transient, limiter and temperature settings."""
        self._check(self.L.fc_apply_settings(self.h, C.byref(settings)), "fc_apply_settings")

    def time_shift(self):
        self._check(self.L.fc_time_shift(self.h), "fc_time_shift")

    def piso_iteration(self):
        r = np.zeros(4)
        self._check(self.L.fc_piso_iteration(self.h, _ptr(r)), "fc_piso_iteration")
        return r

    def simple_batched_momentum(self, on=True):
        """calcuvw solves U, V, W in one batched launch (bicgstab only)."""
        self._check(self.L.fc_simple_set_batched_momentum(self.h, int(bool(on))), "fc_simple_set_batched_momentum")

    # ------------------------------------------------------- temperature
    def temperature_params(self, prm, bc_dfraction=None):
        """prm: TemperatureParams; bc_dfraction: bcDFraction(7,:) per patch
        (1 isothermal wall, 0 adiabatic wall) or None for all 0."""
        self._tprm = prm
        fr = None if bc_dfraction is None else _f64(bc_dfraction)
        self._check(self.L.fc_temperature_set_params(self.h, C.byref(prm), _ptr(fr) if fr is not None else None),
                    "fc_temperature_set_params")

    def turbulence_params(self, prm):
        """prm: TurbulenceParams of the k-omega SST model."""
        self._kprm = prm
        self._check(self.L.fc_turbulence_set_params(self.h, C.byref(prm)), "fc_turbulence_set_params")

    def wall_distance(self):
        """wall_distance_poisson into the field "walldist"."""
        self._check(self.L.fc_wall_distance(self.h), "fc_wall_distance")

    def kw_sst(self):
        """One modify_viscosity_turbulence with the k-omega SST model; returns resor(5:6)."""
        r = np.zeros(2)
        self._check(self.L.fc_kw_sst(self.h, _ptr(r)), "fc_kw_sst")
        return r

    def calculate_temperature(self, solve=True):
        """One calculate_temperature; returns resor(7)."""
        r = np.zeros(1)
        self._check(self.L.fc_calculate_temperature(self.h, int(bool(solve)), _ptr(r)), "fc_calculate_temperature")
        return float(r[0])


class Batch:
    """Independent sparse systems solved in one batched launch (fc_batch_*).
    Problems are added as 1-based CSR patterns (numpy or device arrays);
    solve() takes per-problem lists of values, solutions and right-hand
    sides.  numpy solutions are copied and returned, device ones updated in
    place."""

    def __init__(self, ctx):
        self.ctx = ctx
        self.L = ctx.L
        h = C.c_void_p()
        ctx._check(self.L.fc_batch_create(ctx.h, C.byref(h)), "fc_batch_create")
        self.h = h
        self.sizes = []

    def close(self):
        if self.h:
            self.L.fc_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add(self, ia, ja, diag, xyz=None):
        ia, ja, diag = _i32(ia), _i32(ja), _i32(diag)
        n, nnz = len(ia) - 1, len(ja)
        xyz = None if xyz is None else _f64(xyz)
        k = self.L.fc_batch_add(self.h, n, nnz, _ptr(ia), _ptr(ja), _ptr(diag), _ptr(xyz))
        self.ctx._check(k, "fc_batch_add")
        self.sizes.append((n, nnz))
        return k

    def plan(self, tiles=None):
        t = None if tiles is None else np.ascontiguousarray(tiles, dtype=np.int32)
        self.ctx._check(self.L.fc_batch_plan(self.h, _ptr(t)), "fc_batch_plan")
        return self.tiles()

    def tiles(self):
        t = np.zeros(len(self.sizes), dtype=np.int32)
        self.ctx._check(self.L.fc_batch_tiles(self.h, _ptr(t)), "fc_batch_tiles")
        return t

    @staticmethod
    def _ptrs(arrays):
        v = (C.c_void_p * len(arrays))()
        for k, a in enumerate(arrays):
            v[k] = _ptr(a).value
        return v

    def solve(self, a, x, rhs, itr_max, tol_abs, tol_rel, solver="bicgstab", raise_on_error=True):
        """Returns (x list, [SolveInfo], status)."""
        a = [_f64(v) for v in a]
        rhs = [_f64(v) for v in rhs]
        x = [_f64(v).copy() if isinstance(v, np.ndarray) or not hasattr(v, "data_ptr") else v for v in x]
        infos = (SolveInfo * len(a))()
        st = self.L.fc_batch_solve(self.h, solver.encode(), self._ptrs(a), self._ptrs(x), self._ptrs(rhs),
                                   int(itr_max), float(tol_abs), float(tol_rel), infos)
        if raise_on_error:
            self.ctx._check(st, "fc_batch_solve")
        return x, list(infos), st

    def tune(self, a, x0, rhs, itr_max, tol_abs, tol_rel, rounds=3, solver="bicgstab"):
        """Measured re-planning; returns (tiles, best ms)."""
        a = [_f64(v) for v in a]
        rhs = [_f64(v) for v in rhs]
        x0 = [_f64(v) for v in x0]
        best = np.zeros(1)
        self.ctx._check(self.L.fc_batch_tune(self.h, solver.encode(), self._ptrs(a), self._ptrs(x0),
                                             self._ptrs(rhs), int(itr_max), float(tol_abs), float(tol_rel),
                                             int(rounds), _ptr(best)), "fc_batch_tune")
        return self.tiles(), float(best[0])
