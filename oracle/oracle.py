"""ctypes wrapper of the CPU oracle (TEST INFRASTRUCTURE ONLY).

The oracle (oracle_*.c) restates the reference's hot-path routines line by
line on the same full-extent module arrays as the GPU library; tests run
a routine on both from identical state and compare every array it writes.
Parity status: see oracle.h (pinned bit for bit against the reference's
own Fortran routines, run from their source by tests/golden/f90exec.py;
find_intersection_point also by the reference's known-answer test).
"""
import ctypes
import pathlib
import subprocess

import numpy as np

import cappgpu
from cappgpu import Params, SolveReport

HERE = pathlib.Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "liboracle.so"

_VP = ctypes.c_void_p
_INT = ctypes.c_int
_DP = ctypes.POINTER(ctypes.c_double)
_REP = ctypes.POINTER(SolveReport)

_SIGS = {
    "cap_new": ([_INT, _INT, _INT], _VP),
    "cap_free": ([_VP], None),
    "cap_field": ([_VP, _INT], _DP),
    "cap_bc": ([_VP, _INT], ctypes.POINTER(ctypes.c_int)),
    "cap_params": ([_VP], ctypes.POINTER(Params)),
    "cap_li": ([_VP], ctypes.POINTER(ctypes.c_int)),
    "cap_lk": ([_VP], ctypes.POINTER(ctypes.c_int)),
    "cap_nijk": ([_VP], _INT),
    "cap_face_areas": ([_VP], None),
    "cap_intfac_all": ([_VP], None),
    "cap_find_intersection_point": ([_DP, _DP], None),
    "cap_update_values_at_ghostcells": ([_VP], None),
    "cap_grad_gauss": ([_VP, _INT, _INT, _INT, _INT], None),
    "cap_bpres": ([_VP, _INT], None),
    "cap_sipsol": ([_VP, _INT, _INT, _REP], _INT),
    "cap_pcgsip": ([_VP, _INT, _INT, _REP], _INT),
    "cap_iccg": ([_VP, _INT, _INT, _REP], _INT),
    "cap_cgstab": ([_VP, _INT, _INT, _REP], _INT),
    "cap_cgstab_sip": ([_VP, _INT, _INT, _REP], _INT),
    "cap_dpcg": ([_VP, _INT, _INT, _REP], _INT),
    "cap_spmv": ([_VP, _INT, _INT], ctypes.c_double),
    "cap_fluxuvw": ([_VP] + [_INT] * 10, None),
    "cap_calcuvw": ([_VP, _REP], _INT),
    "cap_piso_assemble_pressure_eq": ([_VP] + [_INT] * 12, None),
    "cap_assemble_pressure_eq": ([_VP] + [_INT] * 10, None),
    "cap_piso_gethbya": ([_VP], None),
    "cap_piso_multiple_correction": ([_VP, _REP], _INT),
    "cap_fluxmass": ([_VP] + [_INT] * 10, None),
    "cap_calcp": ([_VP, _REP], _INT),
    "cap_outbc": ([_VP], None),
    "cap_correct_boundary_conditions": ([_VP], None),
    "cap_courant": ([_VP], None),
    "cap_continuity_errors": ([_VP], None),
    "cap_find_strain_rate": ([_VP], None),
    "cap_calc_vis_les": ([_VP], None),
    "cap_const_massflux_correction": ([_VP], None),
    "cap_calculate_stuff_for_sst": ([_VP], None),
    "cap_fluxscm": ([_VP] + [_INT] * 13, None),
    "cap_calcscm": ([_VP, _INT, _REP], _INT),
    "cap_modvis": ([_VP], None),
    "cap_piso_steps": ([_VP, _INT, _REP], _INT),
    "cap_simple_iters": ([_VP, _INT, _REP], _INT),
}

_lib = None


def build():
    """Compile the oracle with its Makefile (gcc, -ffp-contract=off)."""
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            build()
        L = ctypes.CDLL(str(LIB_PATH))
        for name, (args, res) in _SIGS.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _lib = L
    return _lib


def find_intersection_point(pts):
    p = np.ascontiguousarray(pts, np.float64).reshape(15)
    out = np.empty(3)
    lib().cap_find_intersection_point(p.ctypes.data_as(_DP), out.ctypes.data_as(_DP))
    return out


def fid(name):
    return cappgpu.FIELD[name] if isinstance(name, str) else int(name)


class State:
    """The reference's module arrays and scalars on the host."""

    def __init__(self, ni, nj, nk):
        self.L = lib()
        self.ptr = self.L.cap_new(ni, nj, nk)
        self.dims = (ni, nj, nk)
        self.nijk = ni * nj * nk

    def __del__(self):
        try:
            if self.ptr:
                self.L.cap_free(self.ptr)
                self.ptr = None
        except Exception:
            pass

    # -- data ------------------------------------------------------------
    def field(self, name):
        """numpy view (no copy) of a module array."""
        p = self.L.cap_field(self.ptr, fid(name))
        return np.ctypeslib.as_array(p, shape=(self.nijk,))

    def set_field(self, name, arr):
        self.field(name)[:] = np.asarray(arr, np.float64)

    def bc(self, face):
        ni, nj, nk = self.dims
        n = {"lbw": nj * nk, "lbe": nj * nk, "lbs": ni * nk, "lbn": ni * nk, "lbb": ni * nj, "lbt": ni * nj}[face]
        p = self.L.cap_bc(self.ptr, cappgpu.params.BC[face])
        return np.ctypeslib.as_array(p, shape=(n,))

    @property
    def params(self):
        return self.L.cap_params(self.ptr).contents

    def li(self):
        return np.ctypeslib.as_array(self.L.cap_li(self.ptr), shape=(self.dims[0] + 1,))[1:].copy()

    def lk(self):
        return np.ctypeslib.as_array(self.L.cap_lk(self.ptr), shape=(self.dims[2] + 1,))[1:].copy()

    def snapshot(self):
        return {n: self.field(n).copy() for n in cappgpu.FIELD_NAMES}

    def copy_from(self, other):
        for n in cappgpu.FIELD_NAMES:
            self.field(n)[:] = other.field(n)

    @classmethod
    def from_case(cls, case, geometry_orient=1):
        """State with the case's arrays; face areas and interpolation
        factors recomputed from the nodes by the oracle (init.f90:54-144),
        north/top areas negated for geometry_orient=1 (see
        cappgpu_build_geometry)."""
        s = cls(case.ni, case.nj, case.nk)
        for name, arr in case.fields.items():
            s.set_field(name, arr)
        for face, codes in case.bc.items():
            s.bc(face)[:] = codes
        s.params.update(case.params)
        s.geometry(geometry_orient)
        return s

    def geometry(self, orient=1):
        self.L.cap_face_areas(self.ptr)
        if orient:
            for n in ("ar2x", "ar2y", "ar2z", "ar3x", "ar3y", "ar3z"):
                f = self.field(n)
                f *= -1.0
        self.L.cap_intfac_all(self.ptr)

    # -- routines --------------------------------------------------------
    def update_values_at_ghostcells(self):
        self.L.cap_update_values_at_ghostcells(self.ptr)

    def grad_gauss(self, u, dx, dy, dz):
        self.L.cap_grad_gauss(self.ptr, fid(u), fid(dx), fid(dy), fid(dz))

    def bpres(self, p="p"):
        self.L.cap_bpres(self.ptr, fid(p))

    def solve(self, solver, fi, ifi):
        rep = SolveReport()
        rc = getattr(self.L, "cap_" + solver)(self.ptr, fid(fi), ifi, ctypes.byref(rep))
        if rc < 0:
            raise RuntimeError(f"oracle {solver} failed ({rc})")
        return rep

    def spmv(self, pk, zk):
        return self.L.cap_spmv(self.ptr, fid(pk), fid(zk))

    def fluxuvw(self, idew, idns, idtb, *names):
        self.L.cap_fluxuvw(self.ptr, idew, idns, idtb, *map(fid, names))

    def calcuvw(self):
        reps = (SolveReport * 3)()
        rc = self.L.cap_calcuvw(self.ptr, reps)
        if rc < 0:
            raise RuntimeError(f"oracle calcuvw failed ({rc})")
        return list(reps)

    def piso_assemble_pressure_eq(self, idew, idns, idtb, arvx, arvy, arvz, fif, acfe, acfw, fcf, ipc, bp):
        self.L.cap_piso_assemble_pressure_eq(self.ptr, idew, idns, idtb,
                                             *map(fid, (arvx, arvy, arvz, fif, acfe, acfw, fcf)), ipc, fid(bp))

    def assemble_pressure_eq(self, idew, idns, idtb, *names):
        self.L.cap_assemble_pressure_eq(self.ptr, idew, idns, idtb, *map(fid, names))

    def piso_gethbya(self):
        self.L.cap_piso_gethbya(self.ptr)

    def piso_multiple_correction(self, nreports=64):
        reps = (SolveReport * nreports)()
        rc = self.L.cap_piso_multiple_correction(self.ptr, reps)
        if rc < 0:
            raise RuntimeError(f"oracle PISO failed ({rc})")
        return list(reps)

    def fluxmass(self, idew, idns, idtb, *names):
        self.L.cap_fluxmass(self.ptr, idew, idns, idtb, *map(fid, names))

    def calcp(self, nreports=64):
        reps = (SolveReport * nreports)()
        rc = self.L.cap_calcp(self.ptr, reps)
        if rc < 0:
            raise RuntimeError(f"oracle calcp failed ({rc})")
        return list(reps)

    def correct_boundary_conditions(self):
        self.L.cap_correct_boundary_conditions(self.ptr)

    def outbc(self):
        self.L.cap_outbc(self.ptr)

    def courant(self):
        self.L.cap_courant(self.ptr)

    def continuity_errors(self):
        self.L.cap_continuity_errors(self.ptr)

    def find_strain_rate(self):
        self.L.cap_find_strain_rate(self.ptr)

    def calc_vis_les(self):
        self.L.cap_calc_vis_les(self.ptr)

    def const_massflux_correction(self):
        self.L.cap_const_massflux_correction(self.ptr)

    def calculate_stuff_for_sst(self):
        self.L.cap_calculate_stuff_for_sst(self.ptr)

    def fluxscm(self, idew, idns, idtb, fi, gx, ifi, *names):
        self.L.cap_fluxscm(self.ptr, idew, idns, idtb, fid(fi), fid(gx), ifi, *(fid(n) for n in names))

    def calcscm(self, ifi):
        rep = SolveReport()
        rc = self.L.cap_calcscm(self.ptr, ifi, ctypes.byref(rep))
        assert rc >= 0, rc
        return rep

    def modvis(self):
        self.L.cap_modvis(self.ptr)

    def piso_steps(self, n):
        rep = SolveReport()
        rc = self.L.cap_piso_steps(self.ptr, n, ctypes.byref(rep))
        if rc < 0:
            raise RuntimeError(f"oracle piso_steps failed ({rc})")
        return rep

    def simple_iters(self, n):
        rep = SolveReport()
        rc = self.L.cap_simple_iters(self.ptr, n, ctypes.byref(rep))
        if rc < 0:
            raise RuntimeError(f"oracle simple_iters failed ({rc})")
        return rep
