"""The skewed-grid pressure-correction system of the standalone Poisson
configuration, GPU against the oracle, at a size the oracle solves in
seconds.

Both sides assemble the system the same way: a seeded non-zero pressure
field and its Gauss gradient, piso_assemble_pressure_eq in the three
directions with ipc = 1 (PISO_assemble_pressure_eq.f90:3-257), so the
explicit non-orthogonal source (:165-194, added back to the neighbours at
:241-253) is non-zero; then the Neumann boundary (links to ghost cells
removed), ap = the sum of the links, su = the assembled source minus the
divergence of a seeded Gaussian face-velocity field (mean removed) and the
reference cell pinned (PISO_multiple_correction.f90:117-129).  The GPU's
assembled matrix must equal the oracle's bit for bit; PCG-SIP in FP64 from
p = 0 must reach the oracle's solution to 1e-10 in as many iterations; the
FP32 refinement form must satisfy the same FP64 exit test and lie within
the distance the 1e-6 tolerance allows."""
import numpy as np
import pytest

import cappgpu
from helpers import compare, push

pytestmark = pytest.mark.gpu
IP = 4
N = (48, 44, 40)
TOL = 1e-6


class OracleSide:
    def __init__(self, st):
        self.st = st

    def get_field(self, n):
        return self.st.field(n).copy()

    def set_field(self, n, a):
        self.st.set_field(n, a)

    def ref_cell(self):
        p = self.st.params
        return p.kpr - 1, p.ipr - 1, p.jpr - 1

    def grad_gauss(self, *names):
        self.st.grad_gauss(*names)

    def piso_assemble_pressure_eq(self, *args):
        self.st.piso_assemble_pressure_eq(*args)


class GpuSide(OracleSide):
    def __init__(self, lib):
        self.lib = lib

    def get_field(self, n):
        return self.lib.get_field(n)

    def set_field(self, n, a):
        self.lib.set_field(n, a)

    def ref_cell(self):
        p = self.lib.get_params()
        return p.kpr - 1, p.ipr - 1, p.jpr - 1

    def grad_gauss(self, *names):
        self.lib.grad_gauss(*names)

    def piso_assemble_pressure_eq(self, *args):
        self.lib.piso_assemble_pressure_eq(*args)


def assemble(side, case, seed):
    ni, nj, nk = case.ni, case.nj, case.nk
    nij, n = ni * nj, ni * nj * nk
    rng = np.random.default_rng(seed)
    for c in "uvw":
        side.set_field(c, rng.standard_normal(n))
    side.set_field("p", rng.standard_normal(n))
    side.grad_gauss("p", "gradp_x", "gradp_y", "gradp_z")
    for g in ("gradu", "gradv", "gradw"):
        for c in "xyz":
            side.set_field(f"{g}_{c}", np.zeros(n))
    side.set_field("su", np.zeros(n))
    for idew, idns, idtb, ar, fif, ae, aw, f, bp in (
            (nj, 1, nij, "ar1", "fx", "ae", "aw", "f1", "be"),
            (1, nij, nj, "ar2", "fy", "an", "as", "f2", "bn"),
            (nij, nj, 1, "ar3", "fz", "at", "ab", "f3", "bt")):
        side.piso_assemble_pressure_eq(idew, idns, idtb, ar + "x", ar + "y", ar + "z", fif, ae, aw, f, 1, bp)
    v = lambda name: side.get_field(name).reshape(nk, ni, nj)
    I = (slice(2, nk - 2), slice(2, ni - 2), slice(2, nj - 2))
    a = {name: v(name) for name in ("ae", "aw", "an", "as", "at", "ab")}
    a["aw"][:, 2, :] = 0.0
    a["ae"][:, ni - 3, :] = 0.0
    a["as"][:, :, 2] = 0.0
    a["an"][:, :, nj - 3] = 0.0
    a["ab"][2, :, :] = 0.0
    a["at"][nk - 3, :, :] = 0.0
    f1, f2, f3 = v("f1"), v("f2"), v("f3")
    f1[:, 1, :] = 0.0
    f1[:, ni - 3, :] = 0.0
    f2[:, :, 1] = 0.0
    f2[:, :, nj - 3] = 0.0
    f3[1, :, :] = 0.0
    f3[nk - 3, :, :] = 0.0
    div = (f1[I] - f1[2:nk - 2, 1:ni - 3, 2:nj - 2] + f2[I] - f2[2:nk - 2, 2:ni - 2, 1:nj - 3]
           + f3[I] - f3[1:nk - 3, 2:ni - 2, 2:nj - 2])
    su = v("su")
    nonorth = float(np.abs(su[I]).sum())
    su[I] = su[I] - (div - div.mean())
    ap = np.zeros((nk, ni, nj))
    ap[I] = sum(a[name][I] for name in a)
    kp, ip, jp = side.ref_cell()
    for name in a:
        a[name][kp, ip, jp] = 0.0
    ap[kp, ip, jp] = 1.0
    su[kp, ip, jp] = 0.0
    for name, arr in a.items():
        side.set_field(name, arr.reshape(-1))
    side.set_field("ap", ap.reshape(-1))
    side.set_field("su", su.reshape(-1))
    side.set_field("p", np.zeros(n))
    return nonorth


def level_free_diff(case, p, ref):
    I = (slice(2, case.nk - 2), slice(2, case.ni - 2), slice(2, case.nj - 2))
    a = case.view(p)[I]
    b = case.view(ref)[I]
    a = a - a.mean()
    b = b - b.mean()
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_skewed_poisson_system_and_solves_match_the_oracle(gpu_lib, oracle_mod):
    case = cappgpu.cases.poisson(N=N)
    st = oracle_mod.State.from_case(case)
    push(gpu_lib, st)
    ng = assemble(GpuSide(gpu_lib), case, seed=21)
    no = assemble(OracleSide(st), case, seed=21)
    assert ng > 0 and ng == no   # the explicit non-orthogonal source is present and equal
    compare(gpu_lib, st, exact=["ae", "aw", "an", "as", "at", "ab", "ap", "su", "be", "bn", "bt",
                                "gradp_x", "gradp_y", "gradp_z", "f1", "f2", "f3"])
    ro = st.solve("pcgsip", "p", IP)
    rg = gpu_lib.pcgsip("p", IP)
    assert ro.status == 0 and ro.resl / ro.res0 < TOL
    assert rg.iters == ro.iters, (rg, ro)
    assert rg.res0 == pytest.approx(ro.res0, rel=1e-12)
    compare(gpu_lib, st, rtol=1e-10, names=["p"])
    # the converged residual is tiny: compare it on the scale of the start
    r = compare(gpu_lib, st, names=["res"])
    assert r["res"][0] <= 1e-9 * ro.res0 / (N[0] * N[1] * N[2]) + 1e-16
    # FP32 refinement form from the same start: the reference's exit test on
    # the FP64 residual, and a solution within the tolerance's reach
    gpu_lib.set_field("p", np.zeros(gpu_lib.nijk))
    gpu_lib.precision(1)
    try:
        r32 = gpu_lib.pcgsip("p", IP)
    finally:
        gpu_lib.precision(0)
    assert r32.status == 0 and r32.resl / r32.res0 < TOL
    assert r32.res0 == pytest.approx(ro.res0, rel=1e-12)
    d32 = level_free_diff(case, gpu_lib.get_field("p"), st.field("p"))
    print(f"skewed Poisson {N}: oracle {ro.iters} it, GPU FP64 {rg.iters} it, FP32+IR {r32.iters} it "
          f"(level-free diff to the oracle {d32:.2e})")
    assert d32 < 1e-4
