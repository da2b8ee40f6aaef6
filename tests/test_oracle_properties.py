"""Analytic and cross-solver checks of the CPU oracle (no GPU).

These pin the restatement where the reference has no tests of its own:
index maps (setind.f90), exact Green-Gauss gradients of linear fields on
uniform grids, symmetry of the assembled pressure operator, and agreement
of the six linear solvers on the same system."""
import numpy as np
import pytest

import cappgpu
from helpers import diag_dominant_matrix, with_fluxes


def test_index_maps(oracle_mod):
    ni, nj, nk = 9, 8, 7
    st = oracle_mod.State(ni, nj, nk)
    np.testing.assert_array_equal(st.li(), (np.arange(1, ni + 1) - 1) * nj)   # setind.f90:34-36
    np.testing.assert_array_equal(st.lk(), (np.arange(1, nk + 1) - 1) * ni * nj)  # setind.f90:38-40


def test_uniform_volumes_and_orientation(oracle_mod):
    case = cappgpu.cases.cavity(N=(6, 5, 4))
    st = oracle_mod.State.from_case(case, geometry_orient=1)
    v = case.view(st.field("vol"))
    np.testing.assert_allclose(v[2:-2, 2:-2, 2:-2], (1 / 6) * (1 / 5) * (1 / 4), rtol=1e-12)
    # all three face area vectors point towards increasing index
    for n, comp in (("ar1x", None), ("ar2y", None), ("ar3z", None)):
        a = case.view(st.field(n))[2:-2, 2:-2, 2:-2]
        assert np.all(a > 0), n
    st0 = oracle_mod.State.from_case(case, geometry_orient=0)
    # init.f90's verbatim cross products: north/top areas point backwards
    assert np.all(case.view(st0.field("ar2y"))[2:-2, 2:-2, 2:-2] < 0)
    assert np.all(case.view(st0.field("ar3z"))[2:-2, 2:-2, 2:-2] < 0)
    assert np.all(case.view(st0.field("ar1x"))[2:-2, 2:-2, 2:-2] > 0)


def test_intfac_uniform_is_half(oracle_mod):
    case = cappgpu.cases.cavity(N=(5, 6, 7))
    st = oracle_mod.State.from_case(case)
    for n in ("fx", "fy", "fz"):
        f = case.view(st.field(n))[2:-2, 2:-2, 2:-2]
        np.testing.assert_allclose(f, 0.5, atol=1e-12)


def test_gradient_of_linear_field_is_exact(oracle_mod):
    """GRAD_GAUSS on a uniform grid reproduces the gradient of a linear field
    in every interior cell."""
    case = cappgpu.cases.cavity(N=(7, 6, 5))
    st = oracle_mod.State.from_case(case)
    a, b, c = 0.3, -1.7, 2.5
    st.set_field("u", a * st.field("xc") + b * st.field("yc") + c * st.field("zc") + 0.25)
    st.grad_gauss("u", "gradu_x", "gradu_y", "gradu_z")
    for n, g in (("gradu_x", a), ("gradu_y", b), ("gradu_z", c)):
        v = case.view(st.field(n))[2:-2, 2:-2, 2:-2]
        np.testing.assert_allclose(v, g, rtol=0, atol=1e-10)


def _poisson_state(oracle_mod, N=(10, 9, 8)):
    case = cappgpu.cases.poisson(N=N)
    st = oracle_mod.State.from_case(case)
    nj, nij = case.nj, case.ni * case.nj
    for idew, idns, idtb, ar, fif, ae, aw, f, bp in (
            (nj, 1, nij, "ar1", "fx", "ae", "aw", "f1", "be"),
            (1, nij, nj, "ar2", "fy", "an", "as", "f2", "bn"),
            (nij, nj, 1, "ar3", "fz", "at", "ab", "f3", "bt")):
        st.piso_assemble_pressure_eq(idew, idns, idtb, ar + "x", ar + "y", ar + "z", fif, ae, aw, f, 0, bp)
    return case, st


def test_pressure_operator_symmetric(oracle_mod):
    case, st = _poisson_state(oracle_mod)
    v = case.view
    ae, aw = v(st.field("ae")), v(st.field("aw"))
    an, as_ = v(st.field("an")), v(st.field("as"))
    at, ab = v(st.field("at")), v(st.field("ab"))
    np.testing.assert_array_equal(ae[:, 1:-1, :], aw[:, 2:, :])   # acfw(ine) = acfe(inp)
    np.testing.assert_array_equal(an[:, :, 1:-1], as_[:, :, 2:])
    np.testing.assert_array_equal(at[1:-1], ab[2:])
    assert np.all(ae[2:-2, 2:-2, 2:-2] > 0)


def _make_system(oracle_mod, rng, shape=(10, 9, 8), symmetric=True):
    st = oracle_mod.State(*[n + 4 for n in shape])
    diag_dominant_matrix(st, rng, symmetric=symmetric)
    st.params.update(dict(alfa=0.92, sor=[1e-10] * 10, nsw=[500] * 10))
    return st


@pytest.mark.parametrize("solver", ["sipsol", "pcgsip", "iccg", "cgstab", "cgstab_sip", "dpcg"])
def test_solver_reduces_residual(oracle_mod, solver):
    rng = np.random.default_rng(3)
    st = _make_system(oracle_mod, rng)
    rep = st.solve(solver, "p", cappgpu.params.IP)
    assert rep.iters >= 1
    assert rep.resl < 1e-6 * rep.res0, (solver, rep)


def test_solvers_agree(oracle_mod):
    """CG-type solvers reach the same interior solution of a symmetric
    system (pcgsip, iccg, dpcg solve k=3..nkmm; ghost rows fixed)."""
    rng = np.random.default_rng(11)
    sols = {}
    for solver in ("pcgsip", "dpcg", "sipsol"):
        st = _make_system(oracle_mod, np.random.default_rng(11))
        # symmetric: aw(i+1) = ae(i) etc.
        ni, nj, nk = st.dims
        v = lambda a: a.reshape(nk, ni, nj)
        ae, an, at = v(st.field("ae")), v(st.field("an")), v(st.field("at"))
        v(st.field("aw"))[:, 1:, :] = ae[:, :-1, :]
        v(st.field("as"))[:, :, 1:] = an[:, :, :-1]
        v(st.field("ab"))[1:] = at[:-1]
        st.set_field("ap", (st.field("ae") + st.field("aw") + st.field("an") + st.field("as")
                            + st.field("at") + st.field("ab")) * 1.5)
        st.params.update(dict(sor=[1e-12] * 10, nsw=[3000] * 10))
        st.solve(solver, "p", cappgpu.params.IP)
        sols[solver] = v(st.field("p"))[2:-2, 2:-2, 2:-2].copy()
    for s in ("dpcg", "sipsol"):
        np.testing.assert_allclose(sols[s], sols["pcgsip"], rtol=0, atol=1e-8 * np.abs(sols["pcgsip"]).max())


def test_spmv_row_sums(oracle_mod):
    """A p with p = 1 in the interior and 0 outside gives ap - (interior
    neighbour coefficients): checks the 7-point stencil addressing."""
    rng = np.random.default_rng(5)
    st = _make_system(oracle_mod, rng, (6, 5, 4))
    ni, nj, nk = st.dims
    p = np.zeros((nk, ni, nj))
    p[2:-2, 2:-2, 2:-2] = 1.0
    st.set_field("pp", p.reshape(-1))
    st.spmv("pp", "res")
    v = lambda n: st.field(n).reshape(nk, ni, nj)
    expect = v("ap").copy()
    inner = np.zeros_like(p, bool)
    inner[2:-2, 2:-2, 2:-2] = True
    for n, sh in (("ae", (0, 1, 0)), ("aw", (0, -1, 0)), ("an", (0, 0, 1)), ("as", (0, 0, -1)),
                  ("at", (1, 0, 0)), ("ab", (-1, 0, 0))):
        nb = np.roll(p, tuple(-s for s in sh), axis=(0, 1, 2))
        expect = expect - v(n) * nb
    np.testing.assert_allclose(v("res")[inner], expect[inner], rtol=1e-13, atol=1e-13)


def test_piso_steps_run_and_conserve(oracle_mod):
    """PISO steps of a small channel: p solves converge, the fixed-CFL time
    step holds the Courant number, fields stay finite and the continuity
    error decays."""
    case = cappgpu.cases.channel(N=(8, 6, 8))
    st = oracle_mod.State.from_case(case)
    with_fluxes(case, st)
    errs = []
    for _ in range(3):
        rep = st.piso_steps(1)
        errs.append(st.params.sumlocalconterr)
        assert rep.resl < 1e-6 * rep.res0, rep                 # p converged to sor(ip)
        assert abs(st.params.conum - 0.5) < 1e-12              # CourantNo.h fixed-CFL step
    for n in ("u", "v", "w", "p"):
        assert np.all(np.isfinite(st.field(n))), n
    # The explicit non-orthogonal source of PISO_assemble_pressure_eq.f90:186-194
    # is not balanced within a step, so the continuity error only decays.
    assert errs[2] < errs[1] < errs[0]


def test_simple_iterations_run(oracle_mod):
    case = cappgpu.cases.cavity(N=(6, 6, 6))
    st = oracle_mod.State.from_case(case)
    st.simple_iters(3)
    for n in ("u", "v", "w", "p"):
        assert np.all(np.isfinite(st.field(n))), n
    # the lid drives a flow
    assert np.abs(st.field("u")).max() > 1e-3


def test_outbc_restores_the_inflow(oracle_mod):
    """outbc.f90: after the rescale the flux through the outlet faces sums
    to flowin, and an outlet ghost holds the interior velocity times
    fac = flowin/flow, with te copied from the interior."""
    case = cappgpu.cases.cavity(N=(6, 5, 7))
    st = oracle_mod.State.from_case(case, geometry_orient=1)
    with_fluxes(case, st)
    rng = np.random.default_rng(8)
    for n in ("u", "v", "w", "te", "ed", "vis", "t", "den"):
        st.set_field(n, rng.uniform(0.5, 1.5, st.nijk))
    ni, nj, nk = st.dims
    st.bc("lbe")[:] = 2
    st.bc("lbt")[:] = 2
    st.params.update(dict(lout=1, loe=1, lot=1, flowin=0.7))
    v = lambda n: case.view(st.field(n)).copy()
    u0, te0 = v("u"), v("te")
    st.outbc()
    f1, f3, u, te = v("f1"), v("f3"), v("u"), v("te")
    # east fluxes sit at i = nim-1, top fluxes at k = nkm-1 (0-based ni-3, nk-3)
    flow = f1[1:nk - 1, ni - 3, 1:nj - 1].sum() + f3[nk - 3, 1:ni - 1, 1:nj - 1].sum()
    assert flow == pytest.approx(0.7, rel=1e-12)
    # an east ghost away from the top set: u(nim) = u(nim-1) * fac
    k, j = 2, 2
    fac = u[k, ni - 2, j] / u0[k, ni - 3, j]
    assert u[k + 1, ni - 2, j] == pytest.approx(u0[k + 1, ni - 3, j] * fac, rel=1e-14)
    assert te[k, ni - 2, j] == te0[k, ni - 3, j]


def test_outbc_without_outlet_is_a_no_op(oracle_mod):
    case = cappgpu.cases.cavity(N=(5, 4, 6))
    st = oracle_mod.State.from_case(case)
    with_fluxes(case, st)
    st.bc("lbe")[:] = 2
    st.params.update(dict(lout=0, loe=1, flowin=0.7))
    before = {n: st.field(n).copy() for n in ("u", "f1")}
    st.outbc()
    for n, a in before.items():
        np.testing.assert_array_equal(st.field(n), a)
