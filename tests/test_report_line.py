"""The reference's unit-66 solver report lines, formatted by the library
(cappgpu_solver_report_line; no GPU needed): the exact text of the
reference's write statements, including Fortran's 1PE10.3 edit descriptor
(three-digit exponents drop the E) and the loop index it prints (nsw + 1
when the solver did not converge)."""
import ctypes

import pytest

import cappgpu
from cappgpu import SOLVER, SolveReport


@pytest.fixture(scope="module")
def L():
    return cappgpu.load_library()


def line(L, solver, ifi, res0, resl, iters, status=0, icorr=0, ipcorr=0):
    rep = SolveReport(res0=res0, resl=resl, iters=iters, status=status)
    buf = ctypes.create_string_buffer(256)
    assert L.cappgpu_solver_report_line(SOLVER[solver], ifi, ctypes.byref(rep), icorr, ipcorr, buf, 256) == 0
    return buf.value.decode()


def test_pcgsip_line(L):
    # pcg-sip.f90:195-197, the reference's own spelling "fFinal" included
    assert line(L, "pcgsip", 4, 1.25e-3, 6.5e-10, 140) == (
        "PCG(SIP):  Solving for p, Initial residual =  1.250E-03, fFinal residual =  6.500E-10, No Iterations 140")


def test_sipsol_line_not_converged_prints_nsw_plus_one(L):
    # sipsol.f90:101-103; the DO loop ran out, so N = NSW + 1
    assert line(L, "sipsol", 1, 0.5, 2.0e-4, 20, status=1) == (
        "SIP:  Solving for U, Initial residual =  5.000E-01, Final residual =  2.000E-04, No Iterations 21")


def test_cgstab_sip_line_and_three_digit_exponent(L):
    # cgstab_sip.f90:273-275; 1PE10.3 of 1e-100 is " 1.000-100"
    assert line(L, "cgstab_sip", 4, 1.0, 1e-100, 5, icorr=1, ipcorr=2) == (
        "BiCGStab(SIP):  Solving for p(icorr=1,npcor=2), Initial residual =  1.000E+00, "
        "Final residual =  1.000-100, No Iterations 5")


def test_other_solver_lines(L):
    assert line(L, "iccg", 3, -3.0, 0.0, 7) == (
        "PCG(IC0):  Solving for W, Initial residual = -3.000E+00, Final residual =  0.000E+00, No Iterations 7")
    assert line(L, "cgstab", 2, 2.5e5, 1.5e-7, 12) == (
        "BiCGStab(ILU(0)):  Solving for V, Initial residual =  2.500E+05, Final residual =  1.500E-07, "
        "No Iterations 12")
    assert line(L, "dpcg", 8, 1e300, 1e-300, 1) == (
        "PCG(Jacobi):  Solving for Visc, Initial residual =  1.000+300, Final residual =  1.000-300, "
        "No Iterations 1")
