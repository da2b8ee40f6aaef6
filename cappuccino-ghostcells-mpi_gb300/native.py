"""ctypes binding of libcappgpu.so -- the host-side mirror of the reference's
routine interface.

Every method maps to one C-ABI entry point of include/cappgpu.h and keeps
the reference routine's name and argument meaning (field arrays are passed
by name, like the Fortran module arrays they stand for).  The library is
CUDA-only: if it is missing or no GPU is present, loading fails loudly --
there is no CPU fallback.
"""
import ctypes
import pathlib

import numpy as np

from .params import FIELD, FIELD_NAMES, BC, Params, SolveReport, SOLVER

PKG = pathlib.Path(__file__).resolve().parent
LIB_PATH = PKG / "_build" / "libcappgpu.so"

_INT = ctypes.c_int
_DP = ctypes.POINTER(ctypes.c_double)
_REP = ctypes.POINTER(SolveReport)

# (name, argtypes) of every exported entry point
SIGNATURES = {
    "cappgpu_init": [_INT, _INT, _INT],
    "cappgpu_finalize": [],
    "cappgpu_last_error": [],
    "cappgpu_field_name": [_INT],
    "cappgpu_field_id": [ctypes.c_char_p],
    "cappgpu_set_field": [_INT, _DP, ctypes.c_int64],
    "cappgpu_get_field": [_INT, _DP, ctypes.c_int64],
    "cappgpu_set_bc": [_INT, ctypes.POINTER(ctypes.c_int), ctypes.c_int64],
    "cappgpu_set_params": [ctypes.POINTER(Params)],
    "cappgpu_get_params": [ctypes.POINTER(Params)],
    "cappgpu_register": [_INT, _DP],
    "cappgpu_unregister_all": [],
    "cappgpu_build_geometry": [_INT],
    "cappgpu_find_intersection_point": [_DP, _DP],
    "cappgpu_get_index_maps": [ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)],
    "cappgpu_ijkpr": [],
    "cappgpu_update_values_at_ghostcells": [],
    "cappgpu_exchange": [_INT],
    "cappgpu_global_sum": [_DP],
    "cappgpu_global_max": [_DP],
    "cappgpu_grad_gauss": [_INT, _INT, _INT, _INT],
    "cappgpu_grad_gauss_h": [_DP, _DP, _DP, _DP],
    "cappgpu_sipsol": [_INT, _INT, _REP],
    "cappgpu_pcgsip": [_INT, _INT, _REP],
    "cappgpu_iccg": [_INT, _INT, _REP],
    "cappgpu_cgstab": [_INT, _INT, _REP],
    "cappgpu_cgstab_sip": [_INT, _INT, _REP],
    "cappgpu_dpcg": [_INT, _INT, _REP],
    "cappgpu_sipsol_h": [_DP, _INT],
    "cappgpu_pcgsip_h": [_DP, _INT],
    "cappgpu_iccg_h": [_DP, _INT],
    "cappgpu_cgstab_h": [_DP, _INT],
    "cappgpu_cgstab_sip_h": [_DP, _INT],
    "cappgpu_dpcg_h": [_DP, _INT],
    "cappgpu_spmv": [_INT, _INT, _DP],
    "cappgpu_spmv_noalloc": [_INT, _INT, _DP],
    "cappgpu_precision": [_INT],
    "cappgpu_learn_reset": [_INT, ctypes.c_ulonglong],
    "cappgpu_learn_collect": [_INT],
    "cappgpu_learn_windows": [_INT, _INT],
    "cappgpu_learn_train": [_INT, _INT, ctypes.c_double, _DP],
    "cappgpu_learn_params": [ctypes.POINTER(ctypes.c_float), _INT, _INT],
    "cappgpu_learn_stats": [ctypes.POINTER(_INT), ctypes.POINTER(_INT), ctypes.POINTER(_INT), _DP],
    "cappgpu_learn_fit": [_DP, _DP],
    "cappgpu_find_strain_rate": [],
    "cappgpu_calc_vis_les": [],
    "cappgpu_const_massflux_correction": [],
    "cappgpu_learn_check": [ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float), _INT, _INT, _INT,
                            ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float), _DP],
    "cappgpu_learn_check_loss": [_INT, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float),
                                 ctypes.POINTER(ctypes.c_float), _INT, _INT, _INT, ctypes.POINTER(ctypes.c_float),
                                 ctypes.POINTER(ctypes.c_float), _DP],
    "cappgpu_learn_sample": [_INT, ctypes.POINTER(ctypes.c_float), ctypes.c_longlong],
    "cappgpu_sweep_stats": [_DP, ctypes.POINTER(ctypes.c_longlong), _INT],
    "cappgpu_fluxuvw": [_INT] * 10,
    "cappgpu_calcuvw": [_REP],
    "cappgpu_piso_assemble_pressure_eq": [_INT] * 12,
    "cappgpu_assemble_pressure_eq": [_INT] * 10,
    "cappgpu_piso_gethbya": [],
    "cappgpu_bpres": [_INT],
    "cappgpu_piso_multiple_correction": [_REP],
    "cappgpu_fluxmass": [_INT] * 10,
    "cappgpu_calcp": [_REP],
    "cappgpu_outbc": [],
    "cappgpu_correct_boundary_conditions": [],
    "cappgpu_courant": [],
    "cappgpu_continuity_errors": [],
    "cappgpu_piso_steps": [_INT, _REP],
    "cappgpu_simple_iters": [_INT, _REP],
    "cappgpu_timer_start": [],
    "cappgpu_timer_stop": [_DP],
    "cappgpu_get_stats": [ctypes.c_void_p],
    "cappgpu_host_alloc": [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int64],
    "cappgpu_host_free": [ctypes.c_void_p],
    "cappgpu_profile_kernel": [_INT, _INT, _DP, _DP],
    "cappgpu_set_option": [ctypes.c_char_p, _INT],
    # host-pointer drop-ins of the assembly routines (hostcall.cu)
    "cappgpu_register_vec3": [_INT, _DP],
    "cappgpu_update_values_at_ghostcells_h": [],
    "cappgpu_bpres_h": [_DP],
    "cappgpu_exchange_h": [_DP],
    "cappgpu_fluxuvw_h": [_INT, _INT, _INT] + [_DP] * 7,
    "cappgpu_piso_assemble_pressure_eq_h": [_INT, _INT, _INT] + [_DP] * 7 + [_INT, _DP],
    "cappgpu_assemble_pressure_eq_h": [_INT, _INT, _INT] + [_DP] * 7,
    "cappgpu_calcuvw_h": [_REP],
    "cappgpu_piso_gethbya_h": [],
    "cappgpu_piso_multiple_correction_h": [_REP],
    "cappgpu_last_report": [ctypes.POINTER(_INT), ctypes.POINTER(_INT), _REP],
    "cappgpu_calcscm": [_INT, _REP],
    "cappgpu_modvis": [],
    "cappgpu_calcscm_h": [_DP, _DP, _INT],
    "cappgpu_modvis_h": [],
    "cappgpu_solver_report_line": [_INT, _INT, _REP, _INT, _INT, ctypes.c_char_p, _INT],
}
RESTYPES = {"cappgpu_last_error": ctypes.c_char_p, "cappgpu_field_name": ctypes.c_char_p}


class CappError(RuntimeError):
    pass


class Stats(ctypes.Structure):
    """Mirror of ``cappgpu_stats``."""
    _fields_ = [("launches", ctypes.c_longlong), ("p_solve_ms", ctypes.c_double),
                ("p_report", SolveReport)]


def load_library(path=None):
    """Load libcappgpu.so (raises if it has not been built)."""
    p = pathlib.Path(path) if path else LIB_PATH
    if not p.exists():
        raise CappError(f"native library {p} is missing: run build() first")
    lib = ctypes.CDLL(str(p))
    for name, args in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = RESTYPES.get(name, ctypes.c_int)
    return lib


def _dp(a):
    return a.ctypes.data_as(_DP)


def fid(name):
    return FIELD[name] if isinstance(name, str) else int(name)


class Library:
    """The reference's module state on the GPU plus its routines."""

    def __init__(self, path=None):
        self.lib = load_library(path)
        self.dims = None

    # ---------------------------------------------------------------- errors
    def _check(self, rc, what, allow_not_converged=True):
        if rc < 0:
            msg = self.lib.cappgpu_last_error().decode(errors="replace")
            raise CappError(f"{what} failed ({rc}): {msg}")
        if rc > 0 and not allow_not_converged:
            raise CappError(f"{what} returned {rc}")
        return rc

    # ------------------------------------------------------------- lifecycle
    def init(self, ni, nj, nk):
        self._check(self.lib.cappgpu_init(ni, nj, nk), "init")
        self.dims = (ni, nj, nk)
        return self

    def finalize(self):
        self.lib.cappgpu_finalize()
        self.dims = None

    @property
    def nijk(self):
        ni, nj, nk = self.dims
        return ni * nj * nk

    def set_field(self, name, arr):
        a = np.ascontiguousarray(arr, dtype=np.float64)
        self._check(self.lib.cappgpu_set_field(fid(name), _dp(a), a.size), f"set_field({name})")

    def get_field(self, name, out=None):
        """The field as a new array, or copied into `out` (a contiguous
        float64 array of nijk elements, e.g. one from pinned())."""
        if out is None:
            out = np.empty(self.nijk, np.float64)
        elif out.dtype != np.float64 or out.size != self.nijk or not out.flags.c_contiguous:
            raise ValueError(f"get_field({name}): out must be a contiguous float64 array of {self.nijk}")
        self._check(self.lib.cappgpu_get_field(fid(name), _dp(out), out.size), f"get_field({name})")
        return out

    def set_bc(self, face, codes):
        a = np.ascontiguousarray(codes, dtype=np.int32)
        f = BC[face] if isinstance(face, str) else face
        self._check(self.lib.cappgpu_set_bc(f, a.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), a.size),
                    f"set_bc({face})")

    def set_params(self, p):
        if isinstance(p, dict):
            p = Params().update(p)
        self._check(self.lib.cappgpu_set_params(ctypes.byref(p)), "set_params")

    def get_params(self):
        p = Params()
        self._check(self.lib.cappgpu_get_params(ctypes.byref(p)), "get_params")
        return p

    def build_geometry(self, orient=1):
        self._check(self.lib.cappgpu_build_geometry(orient), "build_geometry")

    def load_case(self, case, geometry_orient=1, build_geometry=True):
        """Create the context for a Case, upload its arrays, compute the
        face areas/interpolation factors on the device and the case's
        geometry-dependent initial data."""
        from .cases import finalize_case
        self.init(case.ni, case.nj, case.nk)
        for name, arr in case.fields.items():
            self.set_field(name, arr)
        for face, codes in case.bc.items():
            self.set_bc(face, codes)
        self.set_params(case.params)
        if build_geometry:
            self.build_geometry(geometry_orient)
            for name in ("ar1x", "ar1y", "ar1z", "ar2x", "ar2y", "ar2z", "ar3x", "ar3y", "ar3z",
                         "fx", "fy", "fz"):
                case.fields[name] = self.get_field(name)
            before = set(case.fields)
            finalize_case(case)
            for name in case.fields:
                if name in ("f1", "f2", "f3") or name not in before:
                    self.set_field(name, case.fields[name])
        return self

    def set_option(self, key, value):
        self._check(self.lib.cappgpu_set_option(key.encode(), int(value)), f"set_option({key})")

    def index_maps(self):
        ni, nj, nk = self.dims
        li = np.empty(ni, np.int32)
        lk = np.empty(nk, np.int32)
        self._check(self.lib.cappgpu_get_index_maps(li.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                                    lk.ctypes.data_as(ctypes.POINTER(ctypes.c_int))), "index_maps")
        return li, lk

    # ---------------------------------------------------------- routines
    def update_values_at_ghostcells(self):
        self._check(self.lib.cappgpu_update_values_at_ghostcells(), "update_values_at_ghostcells")

    def grad_gauss(self, u, dudx, dudy, dudz):
        self._check(self.lib.cappgpu_grad_gauss(fid(u), fid(dudx), fid(dudy), fid(dudz)), "grad_gauss")

    def bpres(self, p="p"):
        self._check(self.lib.cappgpu_bpres(fid(p)), "bpres")

    def solve(self, solver, fi, ifi):
        rep = SolveReport()
        fn = getattr(self.lib, "cappgpu_" + solver)
        self._check(fn(fid(fi), ifi, ctypes.byref(rep)), solver)
        return rep

    def sipsol(self, fi, ifi):
        return self.solve("sipsol", fi, ifi)

    def pcgsip(self, fi, ifi):
        return self.solve("pcgsip", fi, ifi)

    def iccg(self, fi, ifi):
        return self.solve("iccg", fi, ifi)

    def cgstab(self, fi, ifi):
        return self.solve("cgstab", fi, ifi)

    def cgstab_sip(self, fi, ifi):
        return self.solve("cgstab_sip", fi, ifi)

    def dpcg(self, fi, ifi):
        return self.solve("dpcg", fi, ifi)

    def precision(self, mode):
        """0 = FP64 plain (reference arithmetic), 1 = FP32 preconditioned CG in FP64 refinement."""
        self._check(self.lib.cappgpu_precision(int(mode)), "precision")

    # ------------------------------------------------ learned initial guess
    def learn_reset(self, max_samples, seed=0):
        self._check(self.lib.cappgpu_learn_reset(int(max_samples), int(seed)), "learn_reset")

    def learn_windows(self, block, per_solve):
        """Record random block^3 windows of each solve (per_solve of them)
        instead of the whole interior; clears the recorded pairs."""
        self._check(self.lib.cappgpu_learn_windows(int(block), int(per_solve)), "learn_windows")

    def learn_collect(self, on=True):
        self._check(self.lib.cappgpu_learn_collect(1 if on else 0), "learn_collect")

    def learn_train(self, epochs, block=32, lr=1e-3):
        loss = ctypes.c_double()
        self._check(self.lib.cappgpu_learn_train(int(epochs), int(block), float(lr), ctypes.byref(loss)), "learn_train")
        return loss.value

    def learn_params(self, values=None):
        fp = ctypes.POINTER(ctypes.c_float)
        n = self.lib.cappgpu_learn_params(ctypes.cast(None, fp), 0, 0)
        self._check(n, "learn_params")
        if values is None:
            out = np.empty(n, np.float32)
            self._check(self.lib.cappgpu_learn_params(out.ctypes.data_as(fp), n, 0), "learn_params")
            return out
        a = np.ascontiguousarray(values, dtype=np.float32)
        self._check(self.lib.cappgpu_learn_params(a.ctypes.data_as(fp), a.size, 1), "learn_params")

    def learn_stats(self):
        s, g, f, r = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_double()
        self._check(self.lib.cappgpu_learn_stats(ctypes.byref(s), ctypes.byref(g), ctypes.byref(f), ctypes.byref(r)),
                    "learn_stats")
        a, b = ctypes.c_double(), ctypes.c_double()
        self._check(self.lib.cappgpu_learn_fit(ctypes.byref(a), ctypes.byref(b)), "learn_fit")
        return {"samples": s.value, "guesses": g.value, "fallbacks": f.value, "last_ratio": r.value,
                "last_alpha": a.value, "last_beta": b.value}

    def learn_check(self, rhs, coef, target=None, kind=0):
        """One forward + backward pass of a training loss on a (D, H, W)
        normalised residual and its (7, D, H, W) window operator (planes xp,
        xm, yp, ym, zp, zm, diag): kind 0 the residual norm, 1 supervised and
        2 energy norm against `target` (D, H, W).  Returns output, parameter
        gradients, loss."""
        fp = ctypes.POINTER(ctypes.c_float)
        rhs = np.ascontiguousarray(rhs, np.float32)
        coef = np.ascontiguousarray(coef, np.float32)
        D, H, W = rhs.shape
        if coef.shape != (7, D, H, W):
            raise ValueError("coef must have shape (7, D, H, W)")
        tp = ctypes.cast(None, fp)
        if target is not None:
            target = np.ascontiguousarray(target, np.float32)
            if target.shape != rhs.shape:
                raise ValueError("target must have the shape of rhs")
            tp = target.ctypes.data_as(fp)
        out = np.empty_like(rhs)
        n = self.lib.cappgpu_learn_params(ctypes.cast(None, fp), 0, 0)
        grad = np.empty(n, np.float32)
        loss = ctypes.c_double()
        self._check(self.lib.cappgpu_learn_check_loss(int(kind), rhs.ctypes.data_as(fp), coef.ctypes.data_as(fp), tp,
                                                      D, H, W, out.ctypes.data_as(fp), grad.ctypes.data_as(fp),
                                                      ctypes.byref(loss)),
                    "learn_check")
        return out, grad, loss.value

    def sweep_stats(self, reset=True):
        """(summed ms, count) of the FP64 pcgsip forward substitutions timed
        with option sweep_timing since the last reset."""
        ms, n = ctypes.c_double(), ctypes.c_longlong()
        self._check(self.lib.cappgpu_sweep_stats(ctypes.byref(ms), ctypes.byref(n), 1 if reset else 0),
                    "sweep_stats")
        return ms.value, n.value

    def learn_sample(self, index, shape):
        """Recorded pair `index` as (9, *shape) float32 planes: r^, A^ (xp, xm,
        yp, ym, zp, zm, diag), the converged correction t^; `shape` is the
        sample's (D, H, W) = (k, i, j) extent."""
        a = np.empty((9,) + tuple(shape), np.float32)
        self._check(self.lib.cappgpu_learn_sample(int(index), a.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                                  a.size), "learn_sample")
        return a

    def spmv(self, pk, zk):
        dot = ctypes.c_double()
        self._check(self.lib.cappgpu_spmv(fid(pk), fid(zk), ctypes.byref(dot)), "spmv")
        return dot.value

    def fluxuvw(self, idew, idns, idtb, arvx, arvy, arvz, fif, acfe, acfw, fcf):
        self._check(self.lib.cappgpu_fluxuvw(idew, idns, idtb, *map(fid, (arvx, arvy, arvz, fif, acfe, acfw, fcf))),
                    "fluxuvw")

    def calcuvw(self):
        reps = (SolveReport * 3)()
        self._check(self.lib.cappgpu_calcuvw(reps), "calcuvw")
        return list(reps)

    def piso_assemble_pressure_eq(self, idew, idns, idtb, arvx, arvy, arvz, fif, acfe, acfw, fcf, ipc, bp):
        self._check(self.lib.cappgpu_piso_assemble_pressure_eq(
            idew, idns, idtb, *map(fid, (arvx, arvy, arvz, fif, acfe, acfw, fcf)), ipc, fid(bp)),
            "piso_assemble_pressure_eq")

    def assemble_pressure_eq(self, idew, idns, idtb, arvx, arvy, arvz, fif, acfe, acfw, fcf):
        self._check(self.lib.cappgpu_assemble_pressure_eq(
            idew, idns, idtb, *map(fid, (arvx, arvy, arvz, fif, acfe, acfw, fcf))), "assemble_pressure_eq")

    def piso_gethbya(self):
        self._check(self.lib.cappgpu_piso_gethbya(), "piso_gethbya")

    def piso_multiple_correction(self, nreports=64):
        reps = (SolveReport * nreports)()
        self._check(self.lib.cappgpu_piso_multiple_correction(reps), "piso_multiple_correction")
        return list(reps)

    def fluxmass(self, idew, idns, idtb, arvx, arvy, arvz, fif, acfe, acfw, fcf):
        self._check(self.lib.cappgpu_fluxmass(idew, idns, idtb, *map(fid, (arvx, arvy, arvz, fif, acfe, acfw, fcf))),
                    "fluxmass")

    def calcp(self, nreports=64):
        reps = (SolveReport * nreports)()
        self._check(self.lib.cappgpu_calcp(reps), "calcp")
        return list(reps)

    def correct_boundary_conditions(self):
        self._check(self.lib.cappgpu_correct_boundary_conditions(), "correctBoundaryConditions")

    def outbc(self):
        self._check(self.lib.cappgpu_outbc(), "outbc")

    def courant(self):
        self._check(self.lib.cappgpu_courant(), "courant")

    def find_strain_rate(self):
        self._check(self.lib.cappgpu_find_strain_rate(), "find_strain_rate")

    def calc_vis_les(self):
        self._check(self.lib.cappgpu_calc_vis_les(), "calc_vis_les")

    def calcscm(self, ifi):
        """calcscm(fi, gradfi, ifi) for ifi = ite (te) or ied (ed), SST"""
        rep = SolveReport()
        self._check(self.lib.cappgpu_calcscm(int(ifi), ctypes.byref(rep)), "calcscm")
        return rep

    def modvis(self):
        self._check(self.lib.cappgpu_modvis(), "modvis")

    def const_massflux_correction(self):
        self._check(self.lib.cappgpu_const_massflux_correction(), "const_massflux_correction")

    def continuity_errors(self):
        self._check(self.lib.cappgpu_continuity_errors(), "continuity_errors")

    def piso_steps(self, n):
        rep = SolveReport()
        self._check(self.lib.cappgpu_piso_steps(n, ctypes.byref(rep)), "piso_steps")
        return rep

    def simple_iters(self, n):
        rep = SolveReport()
        self._check(self.lib.cappgpu_simple_iters(n, ctypes.byref(rep)), "simple_iters")
        return rep

    # ---------------------------------------------------------- instrumentation
    def timer_start(self):
        self._check(self.lib.cappgpu_timer_start(), "timer_start")

    def timer_stop(self):
        ms = ctypes.c_double()
        self._check(self.lib.cappgpu_timer_stop(ctypes.byref(ms)), "timer_stop")
        return ms.value

    def stats(self):
        s = Stats()
        self._check(self.lib.cappgpu_get_stats(ctypes.byref(s)), "get_stats")
        return s

    def pinned(self, n):
        """A page-locked float64 host array of n elements (freed with free_pinned)."""
        p = ctypes.c_void_p()
        self._check(self.lib.cappgpu_host_alloc(ctypes.byref(p), 8 * n), "host_alloc")
        arr = np.ctypeslib.as_array(ctypes.cast(p, _DP), shape=(n,))
        self._pinned = getattr(self, "_pinned", []) + [p]
        return arr

    def free_pinned(self):
        for p in getattr(self, "_pinned", []):
            self.lib.cappgpu_host_free(p)
        self._pinned = []

    def profile_kernel(self, which, reps=5):
        ms, b = ctypes.c_double(), ctypes.c_double()
        self._check(self.lib.cappgpu_profile_kernel(which, reps, ctypes.byref(ms), ctypes.byref(b)),
                    "profile_kernel")
        return ms.value, b.value

    def find_intersection_point(self, pts):
        p = np.ascontiguousarray(pts, np.float64).reshape(15)
        out = np.empty(3)
        self._check(self.lib.cappgpu_find_intersection_point(_dp(p), _dp(out)), "find_intersection_point")
        return out
