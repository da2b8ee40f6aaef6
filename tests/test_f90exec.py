"""The Fortran-subset executor that runs the reference's routines for the
golden fixture (tests/golden/f90exec.py), on small programs of its own:
each test pins one rule of Fortran arithmetic or control flow that the
reference's routines rely on.  (CPU only; no reference files needed.)"""
import pathlib
import sys

import numpy as np
import pytest

sys.path.insert(0, str(pathlib.Path(__file__).resolve().parent / "golden"))

import f90exec as F  # noqa: E402

MODULES = """
module types
  integer, parameter :: dp = kind(1.0d0)
  integer, parameter :: prec = dp
end module types
module parameters
  use types
  integer, parameter :: nphi=10
  integer :: nxyza
  real(prec), parameter :: small = 1e-30
  real(prec), dimension(nphi) :: sor, resor
  logical :: ltest
end module parameters
module coef
  use types
  real(prec), dimension(:), allocatable :: ae, res
  integer, dimension(:), allocatable :: li
end module coef
"""


def run(body, name="t", args=(), dims=(4, 4, 4)):
    prog = F.Program(MODULES)
    prog.add_source(body)
    prog.compile()
    ns = prog.namespace(dims)
    out = ns.call(name, *args)
    return ns, out


def test_default_real_literals_are_single_precision():
    ns, out = run("""
subroutine t(a, b, c, d)
  use types
  use parameters
  real(prec) :: a, b, c, d
  a = 1e-30
  b = 1.0d0/3.0d0
  c = 1./3.
  d = small
end subroutine""", args=(0.0, 0.0, 0.0, 0.0))
    a, b, c, d = out
    assert a == float(np.float32(1e-30)) and a != 1e-30
    assert b == 1.0 / 3.0
    assert c == float(np.float32(1.0) / np.float32(3.0))      # the division itself in single precision
    assert d == float(np.float32(1e-30))


def test_mixed_kinds_promote_to_double():
    ns, out = run("""
subroutine t(x, y)
  use types
  real(prec) :: x, y
  y = 1./(x + 0.1)
end subroutine""", args=(F.F8(0.25), 0.0))
    assert out[1] == 1.0 / (0.25 + float(np.float32(0.1)))


def test_integer_division_truncates_towards_zero():
    ns, out = run("""
subroutine t(a, b, c)
  integer :: a, b, c
  a = -7/2
  b = 7/2
  c = (-7)/(-2)
end subroutine""", args=(0, 0, 0))
    assert out == (-3, 3, 3)


def test_integer_powers_are_products():
    x = F.F8(1.0000001234567)
    ns, out = run("""
subroutine t(x, a, b, c)
  use types
  real(prec) :: x, a, b, c
  a = x**2
  b = x**3
  c = x**4
end subroutine""", args=(x, 0.0, 0.0, 0.0))
    assert out[1] == x * x and out[2] == x * x * x and out[3] == (x * x) * (x * x)


def test_do_index_after_the_loop():
    ns, out = run("""
subroutine t(n, last, stop)
  integer :: n, last, stop, l
  do l=1,n
  end do
  last = l
  do l=1,n
    if (l.eq.3) exit
  end do
  stop = l
  do l=n,1,-2
  end do
  n = l
end subroutine""", args=(5, 0, 0))
    assert out == (-1, 6, 3)     # 5,3,1 then -1; 1..5 then 6; exit at 3


def test_zero_trip_loop_leaves_the_start_value():
    ns, out = run("""
subroutine t(k, m)
  integer :: k, m, i
  m = 0
  do i=3,2
    m = m + 1
  end do
  k = i
end subroutine""", args=(0, 0))
    assert out == (3, 0)


def test_if_blocks_and_logical_operators():
    ns, out = run("""
subroutine t(a, b, r)
  integer :: a, b, r
  if (a.gt.2.and.b.lt.5) then
    r = 1
  else if (a == 2 .or. .not. (b /= 9)) then
    r = 2
  elseif (a.le.0) then
    r = 3
  else
    r = 4
  endif
end subroutine""", args=(2, 9, 0))
    assert out[2] == 2
    for (a, b), r in {(3, 4): 1, (1, 9): 2, (0, 1): 3, (1, 1): 4}.items():
        assert run("""
subroutine t(a, b, r)
  integer :: a, b, r
  if (a.gt.2.and.b.lt.5) then
    r = 1
  else if (a == 2 .or. .not. (b /= 9)) then
    r = 2
  elseif (a.le.0) then
    r = 3
  else
    r = 4
  endif
end subroutine""", args=(a, b, 0))[1][2] == r


def test_module_arrays_and_whole_array_assignment():
    ns, out = run("""
subroutine t(n)
  use types
  use parameters
  use coef
  integer :: n, i
  real(prec), dimension(nxyza) :: w
  res = 0.0_dp
  do i=1,n
    li(i) = (i-1)*4
    ae(i) = dble(i)*0.5d0
    w(i) = ae(i) + 1
  end do
  res(2) = w(3)
end subroutine""", args=(5,))
    assert list(ns.get("li")[1:6]) == [0, 4, 8, 12, 16]
    assert ns.get("ae")[3] == 1.5 and ns.get("res")[2] == 2.5


def test_scalar_arguments_are_passed_by_reference():
    prog = F.Program(MODULES)
    prog.add_source("""
subroutine inner(x, k)
  use types
  real(prec) :: x
  integer :: k
  x = x*2.0d0
  k = k + 1
end subroutine
subroutine outer(y, m)
  use types
  real(prec) :: y
  integer :: m
  call inner(y, m)
  call inner(y, m)
end subroutine""")
    prog.compile()
    ns = prog.namespace((4, 4, 4))
    assert ns.call("outer", F.F8(1.5), 0) == (6.0, 2)


def test_calls_outside_the_set_fail():
    prog = F.Program(MODULES)
    prog.add_source("subroutine t\n  call nowhere(1)\nend subroutine\n")
    with pytest.raises(NameError):
        prog.compile()
    prog = F.Program(MODULES)
    prog.add_source("subroutine t\n  call nowhere(1)\nend subroutine\n")
    prog.compile(stubs=["nowhere"])
    with pytest.raises(RuntimeError):
        prog.namespace((4, 4, 4)).call("t")


def test_unsupported_statements_raise():
    prog = F.Program(MODULES)
    prog.add_source("subroutine t\n  goto 10\nend subroutine\n")
    with pytest.raises(NotImplementedError):
        prog.compile()


def test_formatted_write_of_a_solver_line():
    ns, _ = run("""
subroutine t(r0, r1, n)
  use types
  real(prec) :: r0, r1
  integer :: n
  write(66,'(3a,1pe10.3,a,1pe10.3,a,i0)') 'SIP:  Solving for ','p', &
  ', Initial residual = ',r0,', Final residual = ',r1,', No Iterations ',n
  write(66,'(20X,"FI=",A3,"  SWEEP=",I4)') ' U',7
end subroutine""", args=(F.F8(1.25e-3), F.F8(-6.5e-120), 140))
    assert ns.units[66] == [
        "SIP:  Solving for p, Initial residual =  1.250E-03, Final residual = -6.500-120, No Iterations 140",
        " " * 20 + "FI=  U  SWEEP=   7"]      # A3 right-justifies a shorter string


def test_exact_single_rounding_of_decimal_literals():
    for text in ("0.1", "1e-30", "1.e20", "3.4028235e38", "0.92", "1.17549435e-38"):
        f = F.exact_f32(text)
        from fractions import Fraction
        v = Fraction(text)
        with np.errstate(over="ignore"):
            nb = [np.nextafter(f, np.float32(-np.inf)), np.nextafter(f, np.float32(np.inf))]
        for c in nb:
            if np.isfinite(c):
                assert abs(Fraction(float(f)) - v) <= abs(Fraction(float(c)) - v)


def test_module_functions_return_their_result_variable():
    prog = F.Program(MODULES)
    prog.add_source("""
module stuff
contains
  pure function wsum(a, n) result(s)
  use types
  real(prec), dimension(nxyza), intent(in) :: a
  integer, intent(in) :: n
  real(prec) :: s
  integer :: i
  s = 0.0_dp
  do i=1,n
    s = s + a(i)*2
  end do
  end function
  subroutine noisy
  call random_number(x)
  end subroutine
end module
subroutine t(n, r)
  use types
  use coef
  integer :: n
  real(prec) :: r
  r = wsum(ae, n) + 1
end subroutine""", only={"wsum", "t"})
    prog.compile()
    ns = prog.namespace((4, 4, 4))
    ns.get("ae")[1:4] = [0.5, 1.25, 2.0]
    assert ns.call("t", 3, F.F8(0)) == (3, 2 * (0.5 + 1.25 + 2.0) + 1)
