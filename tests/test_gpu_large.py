"""The pressure solve at the largest configured storage extent: 516 x 260 x
260 = 34.9 M cells, the grid of the 512 x 256 x 256 RANS channel config.

A seeded symmetric, diagonally dominant 7-diagonal system is solved with
PCG-SIP in the FP64 plain form and in the FP32 + FP64-refinement form; the
final residual is recomputed independently on the host with numpy in the
reference's formula (res = su + sum a_nb phi_nb - ap phi over the interior,
pcg-sip.f90:161-175, sipsol.f90:66-69).  At this size the hyperplane layout
has 129 M slots, so the test covers the 32-bit index arithmetic of the
layout, of the compact cell walk and of the wavefront at the top of the
configured range."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
IP = 4
DIMS = (516, 260, 260)
SOR = 1e-8


def _system(gpu_lib, rng):
    ni, nj, nk = DIMS
    n = ni * nj * nk
    v = lambda a: a.reshape(nk, ni, nj)
    a = {q: rng.uniform(0.05, 1.0, n) for q in ("ae", "an", "at")}
    # symmetric: aw(i+1) = ae(i), as(j+1) = an(j), ab(k+1) = at(k)
    for west, east, ax in (("aw", "ae", 1), ("as", "an", 2), ("ab", "at", 0)):
        w = np.full(n, 0.5)
        src, dst = [slice(None)] * 3, [slice(None)] * 3
        src[ax], dst[ax] = slice(None, -1), slice(1, None)
        v(w)[tuple(dst)] = v(a[east])[tuple(src)]
        a[west] = w
    ap = (a["ae"] + a["aw"] + a["an"] + a["as"] + a["at"] + a["ab"]) * 1.5
    su = rng.uniform(-1.0, 1.0, n)
    for q, arr in a.items():
        gpu_lib.set_field(q, arr)
    gpu_lib.set_field("ap", ap)
    gpu_lib.set_field("su", su)
    gpu_lib.set_field("p", np.zeros(n))
    gpu_lib.set_field("res", np.zeros(n))
    return a, ap, su


def _true_residual_l1(a, ap, su, phi):
    ni, nj, nk = DIMS
    v = lambda x: x.reshape(nk, ni, nj)
    f = v(phi)
    I = (slice(2, nk - 2), slice(2, ni - 2), slice(2, nj - 2))
    sh = lambda dk, di, dj: f[2 + dk:nk - 2 + dk, 2 + di:ni - 2 + di, 2 + dj:nj - 2 + dj]
    r = (v(su)[I] + v(a["ae"])[I] * sh(0, 1, 0) + v(a["aw"])[I] * sh(0, -1, 0)
         + v(a["an"])[I] * sh(0, 0, 1) + v(a["as"])[I] * sh(0, 0, -1)
         + v(a["at"])[I] * sh(1, 0, 0) + v(a["ab"])[I] * sh(-1, 0, 0) - v(ap)[I] * f[I])
    return float(np.abs(r).sum()), float(np.abs(v(su)[I]).sum())


@pytest.mark.parametrize("mode", [0, 1])
def test_pressure_solve_at_the_largest_extent(gpu_lib, mode):
    gpu_lib.init(*DIMS)
    p = gpu_lib.get_params()
    p.update(dict(alfa=0.92, sor=[SOR] * 10, nsw=[500] * 10, ipr=3, jpr=3, kpr=3))
    gpu_lib.set_params(p)
    a, ap, su = _system(gpu_lib, np.random.default_rng(12 + mode))
    gpu_lib.precision(mode)
    try:
        rep = gpu_lib.pcgsip("p", IP)
    finally:
        gpu_lib.precision(0)
    assert rep.status == 0, rep
    res_l1, su_l1 = _true_residual_l1(a, ap, su, gpu_lib.get_field("p"))
    # the solve starts from p = 0: its initial residual is |su| over the interior
    assert rep.res0 == pytest.approx(su_l1, rel=1e-10)
    # the tolerance holds for the residual recomputed from the solution
    assert res_l1 / su_l1 < 2 * SOR, (res_l1 / su_l1, rep)
    if mode == 1:   # the refinement form's exit test is on this FP64 residual
        assert rep.resl == pytest.approx(res_l1, rel=1e-8)
