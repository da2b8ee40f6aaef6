"""The reference's grid and restart file formats (read_grid.f90:126-161,
writefiles.f90:30-71, readfiles.f90:39-63): byte layout of Fortran
unformatted sequential records, round trips, and refusal of damaged files."""
import struct

import numpy as np
import pytest

import cappgpu
fortio = cappgpu.fortio


def _geometry(oracle_mod, case):
    """The case's full geometry (areas, interpolation factors) from the oracle."""
    return oracle_mod.State.from_case(case)


class _Fields:
    def __init__(self, st):
        self.st = st

    def get_field(self, n):
        return self.st.field(n).copy()


def test_grid_round_trip_and_byte_layout(tmp_path, oracle_mod):
    case = cappgpu.cases.cavity(N=(5, 4, 6))
    geo = _Fields(_geometry(oracle_mod, case))
    path = tmp_path / "grid-1"
    fortio.write_grid(path, case, geo, lout=True, lthermbc=2)
    raw = path.read_bytes()
    ni, nj, nk = case.ni, case.nj, case.nk
    nijk = ni * nj * nk
    # first record: 4-byte count 12, three integers, count again
    assert raw[:20] == struct.pack("<i3ii", 12, ni, nj, nk, 12)
    # second record: 8 integers, the six code arrays, 7 logicals, 2 integers
    n2 = 4 * (8 + 2 * (nj * nk + ni * nk + ni * nj) + 9)
    assert struct.unpack("<i", raw[20:24])[0] == n2
    # then 19 records of nijk reals
    assert len(raw) == 20 + (8 + n2) + 19 * (8 + 8 * nijk)
    back = fortio.read_grid(path)
    assert (back.ni, back.nj, back.nk) == (ni, nj, nk)
    for n in fortio.GRID_FIELDS:
        np.testing.assert_array_equal(back.fields[n], geo.get_field(n))
    for n in fortio.BC_FACES:
        np.testing.assert_array_equal(back.bc[n], case.bc[n])
    assert back.meta["lout"] is True and back.meta["lthermbc"] == 2 and back.meta["low"] is False


class _HostLib:
    """Stand-in for Library: fields in host memory."""

    def __init__(self, nijk, rng):
        self.nijk = nijk
        self.f = {n: rng.standard_normal(nijk) for n in cappgpu.FIELD_NAMES}

    def get_field(self, n):
        return self.f[n].copy()

    def set_field(self, n, a):
        self.f[n] = np.array(a, dtype=np.float64)


@pytest.mark.parametrize("const_mflux", [False, True])
def test_restart_round_trip(tmp_path, const_mflux):
    rng = np.random.default_rng(1)
    src = _HostLib(60, rng)
    path = tmp_path / "restart"
    fortio.write_restart(path, src, itime=17, time=0.125, const_mflux=const_mflux, gradpcmf=3.5)
    raw = path.read_bytes()
    assert raw[:20] == struct.pack("<iidi", 12, 17, 0.125, 12)
    dst = _HostLib(60, np.random.default_rng(2))
    itime, time, g = fortio.read_restart(path, dst, const_mflux=const_mflux)
    assert (itime, time) == (17, 0.125)
    assert g == (3.5 if const_mflux else None)
    for n in fortio.RESTART_FIELDS:
        if n in cappgpu.FIELD_NAMES:
            np.testing.assert_array_equal(dst.f[n], src.f[n])
    # 22 field records of nijk reals after the header records
    assert len(raw) == 20 + (16 if const_mflux else 0) + 22 * (8 + 8 * 60)


def test_damaged_files_are_refused(tmp_path, oracle_mod):
    case = cappgpu.cases.cavity(N=(4, 4, 4))
    path = tmp_path / "grid-1"
    fortio.write_grid(path, case, _Fields(_geometry(oracle_mod, case)))
    raw = bytearray(path.read_bytes())
    raw[-1] ^= 0xFF                      # trailing record marker
    bad = tmp_path / "bad-1"
    bad.write_bytes(bytes(raw))
    with pytest.raises(fortio.FortranFileError):
        fortio.read_grid(bad)
    (tmp_path / "short-1").write_bytes(bytes(raw[:100]))
    with pytest.raises(fortio.FortranFileError):
        fortio.read_grid(tmp_path / "short-1")
    src = _HostLib(30, np.random.default_rng(3))
    fortio.write_restart(tmp_path / "r", src, 1, 0.0)
    with pytest.raises(fortio.FortranFileError):
        fortio.read_restart(tmp_path / "r", _HostLib(31, np.random.default_rng(4)))
