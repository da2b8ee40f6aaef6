"""The reference's on-disk formats: grid files (read_grid.f90:126-161) and
restart files (writefiles.f90:30-71, readfiles.f90:39-63), so that grids and
restarts written by the Fortran code load into the library and the
library's state can be written back for it.

Both are Fortran unformatted sequential files: every record is a 4-byte
little-endian byte count, the payload, and the count again.  Integers and
logicals are 4 bytes (default kinds), reals 8 bytes (prec = dp,
modules_allocatable.f90:8-11).  Records of 2**31 bytes or more (gfortran
splits them into sub-records) are refused.

Grid file records, in order: ni, nj, nk | nij, nik, njk, nijk, ijs, iks, jks,
ijks, lbw(njk), lbe(njk), lbs(nik), lbn(nik), lbb(nij), lbt(nij), low, loe,
los, lon, lob, lot, lout (logical), lthermbc, lconbc (integer) | then one
record each of x, y, z, xc, yc, zc, vol, fx, fy, fz, ar1x, ar1y, ar1z, ar2x,
ar2y, ar2z, ar3x, ar3y, ar3z (nijk reals).  The reference opens
'<grid_file>-<rank+1>' (read_grid.f90:29-34).

Restart file records: itime, time | gradpcmf (only with const_mflux) | f1,
f2, f3, u, v, w, p, te, ed, t, vis, uu, vv, ww, uv, uw, vw, uo, vo, wo, teo,
edo (nijk reals each).  writefiles writes to 'restart_file', readfiles reads
'<restart_file>-<rank+1>'.  The Reynolds stresses uu..vw have no device
field here: they are written as zeros and skipped on reading.
"""
import struct

import numpy as np

GRID_FIELDS = ("x", "y", "z", "xc", "yc", "zc", "vol", "fx", "fy", "fz",
               "ar1x", "ar1y", "ar1z", "ar2x", "ar2y", "ar2z", "ar3x", "ar3y", "ar3z")
RESTART_FIELDS = ("f1", "f2", "f3", "u", "v", "w", "p", "te", "ed", "t", "vis",
                  "uu", "vv", "ww", "uv", "uw", "vw", "uo", "vo", "wo", "teo", "edo")
_NO_FIELD = {"uu", "vv", "ww", "uv", "uw", "vw"}
BC_FACES = ("lbw", "lbe", "lbs", "lbn", "lbb", "lbt")


class FortranFileError(ValueError):
    pass


def _write_record(f, payload):
    n = len(payload)
    if n >= 2 ** 31:
        raise FortranFileError(f"record of {n} bytes needs sub-records")
    f.write(struct.pack("<i", n))
    f.write(payload)
    f.write(struct.pack("<i", n))


def _read_record(f):
    head = f.read(4)
    if len(head) < 4:
        raise FortranFileError("unexpected end of file")
    (n,) = struct.unpack("<i", head)
    if n < 0:
        raise FortranFileError("sub-records are not supported")
    payload = f.read(n)
    tail = f.read(4)
    if len(payload) < n or len(tail) < 4 or struct.unpack("<i", tail)[0] != n:
        raise FortranFileError("record markers do not match")
    return payload


def _reals(a, n=None):
    a = np.ascontiguousarray(a, dtype="<f8").reshape(-1)
    if n is not None and a.size != n:
        raise FortranFileError(f"array of {a.size} values, expected {n}")
    return a.tobytes()


def write_grid(path, case, source=None, low=False, loe=False, los=False, lon=False, lob=False, lot=False,
               lout=False, lthermbc=0, lconbc=0):
    """Grid file of a Case: its dimensions and BC code arrays, and the
    geometry arrays x..ar3z from `source` -- any object with get_field (the
    Library after load_case, which computes the face areas and interpolation
    factors, or an oracle state) -- or from case.fields."""
    ni, nj, nk = case.ni, case.nj, case.nk
    nij, nik, njk, nijk = ni * nj, ni * nk, nj * nk, ni * nj * nk
    bc = {n: np.ascontiguousarray(case.bc[n], dtype="<i4").reshape(-1) for n in BC_FACES}
    sizes = {"lbw": njk, "lbe": njk, "lbs": nik, "lbn": nik, "lbb": nij, "lbt": nij}
    for n in BC_FACES:
        if bc[n].size != sizes[n]:
            raise FortranFileError(f"{n}: {bc[n].size} codes, expected {sizes[n]}")
    with open(path, "wb") as f:
        _write_record(f, struct.pack("<3i", ni, nj, nk))
        head = struct.pack("<8i", nij, nik, njk, nijk, 0, 0, 0, 0)
        flags = struct.pack("<7i2i", *(int(bool(v)) for v in (low, loe, los, lon, lob, lot, lout)),
                            int(lthermbc), int(lconbc))
        _write_record(f, head + b"".join(bc[n].tobytes() for n in BC_FACES) + flags)
        for n in GRID_FIELDS:
            a = source.get_field(n) if source is not None else case.fields[n]
            _write_record(f, _reals(a, nijk))


def read_grid(path):
    """A Case with the grid file's dimensions, geometry and BC codes (the
    solver parameters are the defaults; set them before use).  The boundary
    logicals and flags go to case.meta; the outlet logicals low..lot and
    lout also to case.params, where outbc reads them."""
    from .cases import Case, _base_params, _common_fields
    with open(path, "rb") as f:
        ni, nj, nk = struct.unpack("<3i", _read_record(f))
        rec = _read_record(f)
        nij, nik, njk, nijk = struct.unpack("<4i", rec[:16])
        if (nij, nik, njk, nijk) != (ni * nj, ni * nk, nj * nk, ni * nj * nk):
            raise FortranFileError("index sums do not match ni, nj, nk")
        o = 32
        bc = {}
        for n, m in zip(BC_FACES, (njk, njk, nik, nik, nij, nij)):
            bc[n] = np.frombuffer(rec, "<i4", m, o).astype(np.int32)
            o += 4 * m
        if len(rec) != o + 36:
            raise FortranFileError("second record has an unexpected length")
        flags = struct.unpack("<9i", rec[o:o + 36])
        fields = {}
        for n in GRID_FIELDS:
            a = np.frombuffer(_read_record(f), "<f8")
            if a.size != nijk:
                raise FortranFileError(f"{n}: {a.size} values, expected {nijk}")
            fields[n] = a.astype(np.float64)
    case = Case("grid", ni, nj, nk, fields=fields, params=_base_params())
    case.bc = bc
    _common_fields(case, nijk)
    names = ("low", "loe", "los", "lon", "lob", "lot", "lout")
    case.meta.update(dict(zip(names, (bool(v) for v in flags[:7]))),
                     lthermbc=flags[7], lconbc=flags[8], grid_file=str(path))
    case.params.update(dict(zip(names, (int(bool(v)) for v in flags[:7]))))   # outbc reads them
    return case


def write_restart(path, lib, itime, time, const_mflux=False, gradpcmf=0.0):
    """Restart file of the library's state (fields read from the device)."""
    nijk = lib.nijk
    with open(path, "wb") as f:
        _write_record(f, struct.pack("<id", int(itime), float(time)))
        if const_mflux:
            _write_record(f, struct.pack("<d", float(gradpcmf)))
        for n in RESTART_FIELDS:
            a = np.zeros(nijk) if n in _NO_FIELD else lib.get_field(n)
            _write_record(f, _reals(a, nijk))


def read_restart(path, lib, const_mflux=False):
    """Load a restart file into the library; returns (itime, time, gradpcmf)."""
    nijk = lib.nijk
    gradpcmf = None
    with open(path, "rb") as f:
        itime, time = struct.unpack("<id", _read_record(f))
        if const_mflux:
            (gradpcmf,) = struct.unpack("<d", _read_record(f))
        for n in RESTART_FIELDS:
            a = np.frombuffer(_read_record(f), "<f8")
            if a.size != nijk:
                raise FortranFileError(f"{n}: {a.size} values, expected {nijk}")
            if n not in _NO_FIELD:
                lib.set_field(n, a.astype(np.float64))
    return itime, time, gradpcmf
