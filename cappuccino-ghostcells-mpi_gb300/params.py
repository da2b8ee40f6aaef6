"""ctypes mirror of the C ABI structures declared in include/cappgpu.h.

The field and BC-face identifiers follow the reference's Fortran module
arrays (modules_allocatable.f90:147-398); the parameter block carries the
module scalars the hot path reads or writes (read_input.f90:28-59,
init.f90:164-344).
"""
import ctypes

NPHI = 10
IU, IV, IW, IP, ITE, IED, IEN, IVIS, IVART, ICON = range(1, 11)

FIELD_NAMES = [
    "x", "y", "z", "xc", "yc", "zc", "vol", "fx", "fy", "fz",
    "ar1x", "ar1y", "ar1z", "ar2x", "ar2y", "ar2z", "ar3x", "ar3y", "ar3z", "walldist",
    "u", "v", "w", "p", "pp", "f1", "f2", "f3", "vis", "den", "te", "ed", "t", "strain",
    "uo", "vo", "wo", "uoo", "voo", "woo",
    "ae", "aw", "an", "as", "at", "ab", "ap", "sp", "spv", "su", "sv", "sw", "res",
    "apu", "apv", "apw",
    "bb", "bs", "bw", "bp", "bn", "be", "bt",
    "he", "hw", "hn", "hs", "ht", "hb",
    "gradu_x", "gradu_y", "gradu_z", "gradv_x", "gradv_y", "gradv_z",
    "gradw_x", "gradw_y", "gradw_z", "gradp_x", "gradp_y", "gradp_z",
    "gradte_x", "gradte_y", "gradte_z", "graded_x", "graded_y", "graded_z",
    "gen", "alphasst", "bettasst", "domega", "prtinv_te", "prtinv_ed",
    "teo", "edo", "teoo", "edoo",
]
FIELD = {n: i for i, n in enumerate(FIELD_NAMES)}
NFIELDS = len(FIELD_NAMES)

BC_NAMES = ["lbw", "lbe", "lbs", "lbn", "lbb", "lbt"]
BC = {n: i for i, n in enumerate(BC_NAMES)}

# geometry computed from the nodes (init.f90:54-144)
GEOMETRY_DERIVED = ["ar1x", "ar1y", "ar1z", "ar2x", "ar2y", "ar2z",
                    "ar3x", "ar3y", "ar3z", "fx", "fy", "fz"]

SOLVER = {"sipsol": 1, "cgstab": 2, "iccg": 3, "pcgsip": 4, "cgstab_sip": 5, "dpcg": 6}

OK, NOT_CONVERGED = 0, 1


class Params(ctypes.Structure):
    """Mirror of ``cappgpu_params`` (include/cappgpu.h)."""
    _fields_ = [
        ("alfa", ctypes.c_double),
        ("densit", ctypes.c_double), ("viscos", ctypes.c_double),
        ("timestep", ctypes.c_double), ("btime", ctypes.c_double), ("time", ctypes.c_double),
        ("uin", ctypes.c_double), ("vin", ctypes.c_double), ("win", ctypes.c_double),
        ("tein", ctypes.c_double), ("edin", ctypes.c_double), ("tin", ctypes.c_double),
        ("flowin", ctypes.c_double), ("zero", ctypes.c_double),
        ("cappa", ctypes.c_double), ("elog", ctypes.c_double),
        ("gradpcmf", ctypes.c_double),
        ("gravx", ctypes.c_double), ("gravy", ctypes.c_double), ("gravz", ctypes.c_double),
        ("beta", ctypes.c_double), ("tref", ctypes.c_double),
        ("conumfixvalue", ctypes.c_double), ("conum", ctypes.c_double), ("meanconum", ctypes.c_double),
        ("localconterr", ctypes.c_double), ("sumlocalconterr", ctypes.c_double),
        ("globalconterr", ctypes.c_double), ("cumulativeconterr", ctypes.c_double),
        ("sor", ctypes.c_double * NPHI), ("resor", ctypes.c_double * NPHI),
        ("snorin", ctypes.c_double * NPHI),
        ("urf", ctypes.c_double * NPHI), ("gds", ctypes.c_double * NPHI),
        ("nsw", ctypes.c_int * NPHI),
        ("lcal", ctypes.c_int * NPHI),
        ("ipr", ctypes.c_int), ("jpr", ctypes.c_int), ("kpr", ctypes.c_int),
        ("ncorr", ctypes.c_int), ("npcor", ctypes.c_int), ("icorr", ctypes.c_int), ("ipcorr", ctypes.c_int),
        ("bdf", ctypes.c_int), ("cn", ctypes.c_int),
        ("lcds", ctypes.c_int), ("lluds", ctypes.c_int), ("lquds", ctypes.c_int), ("lsmart", ctypes.c_int),
        ("lavl", ctypes.c_int), ("lmuscl", ctypes.c_int), ("lumist", ctypes.c_int), ("lgamma", ctypes.c_int),
        ("lcds4", ctypes.c_int),
        ("flux_limiter", ctypes.c_int),
        ("const_mflux", ctypes.c_int), ("lbuoy", ctypes.c_int), ("boussinesq", ctypes.c_int),
        ("lout", ctypes.c_int), ("ltransient", ctypes.c_int), ("lles", ctypes.c_int),
        ("periodic", ctypes.c_int),
        ("conumfix", ctypes.c_int),
        ("isol_p", ctypes.c_int),
        ("piso_solver", ctypes.c_int),
        ("low", ctypes.c_int), ("loe", ctypes.c_int), ("los", ctypes.c_int),
        ("lon", ctypes.c_int), ("lob", ctypes.c_int), ("lot", ctypes.c_int),
        ("sst", ctypes.c_int),
        ("cmu", ctypes.c_double),
        ("top_plane", ctypes.c_int),
        ("pad_", ctypes.c_int),
    ]

    def update(self, d):
        """Set fields from a dict; list values fill the per-variable arrays."""
        for k, val in d.items():
            cur = getattr(self, k)
            if isinstance(cur, ctypes.Array):
                for q, x in enumerate(val):
                    cur[q] = x
            else:
                setattr(self, k, val)
        return self

    def as_dict(self):
        out = {}
        for name, _ in self._fields_:
            cur = getattr(self, name)
            out[name] = list(cur) if isinstance(cur, ctypes.Array) else cur
        return out


class SolveReport(ctypes.Structure):
    """Mirror of ``cappgpu_solve_report`` (the reference's unit-66 solver line)."""
    _fields_ = [("res0", ctypes.c_double), ("resl", ctypes.c_double),
                ("iters", ctypes.c_int), ("status", ctypes.c_int)]

    def __repr__(self):
        return (f"SolveReport(res0={self.res0:.3e}, resl={self.resl:.3e}, "
                f"iters={self.iters}, status={self.status})")
