"""Restart round trip through the device: the reference's restart file
(writefiles.f90:30-71) written from the library's fields after some PISO
steps of the channel, read back (readfiles.f90:35-70) into a fresh context,
and the run continued.

The file holds f1..f3, u, v, w, p, te, ed, t, vis, uo, vo, wo and itime,
time and (with constant mass flux) gradpcmf.  The rest of the module state
is not in it -- in the reference either: the SIP factor arrays, for one,
keep in their ghost layers what the pressure assembly stored there
(PISO_assemble_pressure_eq.f90:194 writes its source into the bp argument,
be/bn/bt), and the next factorisation reads those layers
(pcg-sip.f90:72-84).  So the continued run is compared with the
uninterrupted one with that remaining state carried over by hand: it must
then be bit-identical, which shows the file carries its fields exactly.
The time step size comes from the input deck in the reference (rescaled to
the fixed Courant number, CourantNo.h:58-64) and is handed over the same
way."""
import numpy as np
import pytest

import cappgpu
from cappgpu import fortio

pytestmark = pytest.mark.gpu
CHECK = ("u", "v", "w", "p", "f1", "f2", "f3", "vis")


def test_restart_write_read_continue_is_bit_identical(gpu_lib, tmp_path):
    case = cappgpu.cases.channel(N=(16, 12, 20))
    gpu_lib.load_case(case)
    gpu_lib.piso_steps(3)
    pr = gpu_lib.get_params()
    assert pr.const_mflux == 1
    path = tmp_path / "restart_file-1"
    fortio.write_restart(path, gpu_lib, itime=3, time=pr.time, const_mflux=True, gradpcmf=pr.gradpcmf)
    at3 = {n: gpu_lib.get_field(n) for n in cappgpu.FIELD_NAMES}
    dt, time, gradpcmf = pr.timestep, pr.time, pr.gradpcmf
    gpu_lib.piso_steps(4)
    straight = {n: gpu_lib.get_field(n) for n in CHECK}
    t_straight = gpu_lib.get_params().time

    gpu_lib.load_case(case)   # fresh context: the initial fields of the case
    in_file = [n for n in fortio.RESTART_FIELDS if n in cappgpu.FIELD_NAMES]
    for n in cappgpu.FIELD_NAMES:   # the state the file does not carry
        if n not in in_file:
            gpu_lib.set_field(n, at3[n])
    itime, t, g = fortio.read_restart(path, gpu_lib, const_mflux=True)
    assert (itime, t, g) == (3, time, gradpcmf)
    for n in in_file:   # the file's fields reached the device unchanged
        np.testing.assert_array_equal(gpu_lib.get_field(n), at3[n], err_msg=n)
    pr2 = gpu_lib.get_params()
    pr2.time, pr2.gradpcmf, pr2.timestep = t, g, dt
    gpu_lib.set_params(pr2)
    gpu_lib.piso_steps(4)
    for n in CHECK:
        np.testing.assert_array_equal(gpu_lib.get_field(n), straight[n], err_msg=n)
    assert gpu_lib.get_params().time == t_straight
