"""GPU-vs-oracle parity of every hot-path routine, through the C ABI.

Each test fills a full state (ghost and padding cells included, so the
reference's reads of stale ghost values are exercised), copies it to the
GPU context, runs the routine on both sides and compares every module
array.  Routines without reductions must agree bit for bit; where a
deterministic device reduction replaces the reference's serial sum (solver
norms and dot products) fields agree to 1e-10 relative L2, the plain-form
tolerance, and iteration counts must be equal."""
import ctypes

import numpy as np
import pytest

import cappgpu
from cappgpu import FIELD_NAMES
from helpers import compare, diag_dominant_matrix, push, randomize, with_fluxes

pytestmark = pytest.mark.gpu

RTOL = 1e-10   # plain FP64 form vs the FP64 oracle, relative L2
IU, IV, IW, IP = 1, 2, 3, 4


def cases_small():
    return {
        "cavity": lambda: cappgpu.cases.cavity(N=(8, 7, 9)),
        "skewed": lambda: cappgpu.cases.poisson(N=(10, 9, 8)),
        "channel": lambda: cappgpu.cases.channel(N=(8, 6, 8)),
    }


def state(oracle_mod, kind, orient=1):
    case = cases_small()[kind]()
    st = oracle_mod.State.from_case(case, geometry_orient=orient)
    with_fluxes(case, st)
    return case, st


def run_both(gpu_lib, st, fn):
    push(gpu_lib, st)
    r_gpu = fn(gpu_lib)
    r_ora = fn(st)
    return r_gpu, r_ora


# ------------------------------------------------------------------ geometry

@pytest.mark.parametrize("kind", ["cavity", "skewed", "channel"])
@pytest.mark.parametrize("orient", [0, 1])
def test_geometry_bit_exact(gpu_lib, oracle_mod, kind, orient):
    case = cases_small()[kind]()
    st = oracle_mod.State.from_case(case, geometry_orient=orient)
    gpu_lib.load_case(case, geometry_orient=orient)
    compare(gpu_lib, st, exact=["ar1x", "ar1y", "ar1z", "ar2x", "ar2y", "ar2z", "ar3x", "ar3y", "ar3z",
                                "fx", "fy", "fz"],
            names=["ar1x", "ar1y", "ar1z", "ar2x", "ar2y", "ar2z", "ar3x", "ar3y", "ar3z", "fx", "fy", "fz"])


def test_intersection_kat_on_gpu(gpu_lib):
    from test_oracle_kat import KAT
    gpu_lib.init(8, 8, 8)
    for pts, expected in KAT:
        np.testing.assert_array_equal(gpu_lib.find_intersection_point(pts), expected)


def test_index_maps(gpu_lib):
    ni, nj, nk = 13, 9, 7
    gpu_lib.init(ni, nj, nk)
    li, lk = gpu_lib.index_maps()
    np.testing.assert_array_equal(li, (np.arange(1, ni + 1) - 1) * nj)
    np.testing.assert_array_equal(lk, (np.arange(1, nk + 1) - 1) * ni * nj)
    p = gpu_lib.get_params()
    p.ipr, p.jpr, p.kpr = 4, 5, 3
    gpu_lib.set_params(p)
    assert gpu_lib.lib.cappgpu_ijkpr() == (3 - 1) * ni * nj + (4 - 1) * nj + 5   # setind.f90:56


def test_get_field_into_pinned_buffer(gpu_lib):
    """get_field(out=...) copies straight into a caller's array (the
    end-to-end bench reads its fields into page-locked buffers)."""
    gpu_lib.init(9, 8, 7)
    x = np.random.default_rng(1).standard_normal(9 * 8 * 7)
    gpu_lib.set_field("u", x)
    buf = gpu_lib.pinned(x.size)
    try:
        assert gpu_lib.get_field("u", out=buf) is buf
        np.testing.assert_array_equal(buf, x)
        with pytest.raises(ValueError):
            gpu_lib.get_field("u", out=np.empty(3))
    finally:
        gpu_lib.free_pinned()


# --------------------------------------------------------------- ghost cells

@pytest.mark.parametrize("periodic", [0, 1])
def test_ghost_update_bit_exact(gpu_lib, oracle_mod, periodic):
    case, st = state(oracle_mod, "skewed")
    rng = np.random.default_rng(10 + periodic)
    randomize(st, rng, ["u", "v", "w", "te", "ed", "t", "vis"], 0.1, 1.0)
    for face in cappgpu.params.BC_NAMES:
        st.bc(face)[:] = rng.integers(1, 5, st.bc(face).size)   # inlet/outlet/symmetry/wall mixed
    st.params.periodic = periodic
    st.params.update(dict(uin=0.3, vin=-0.2, win=0.1, tein=0.05, edin=0.7, tin=1.5))
    run_both(gpu_lib, st, lambda s: s.update_values_at_ghostcells())
    compare(gpu_lib, st, exact=FIELD_NAMES)


def test_exchange_and_global_reductions_are_identity(gpu_lib, oracle_mod):
    case, st = state(oracle_mod, "cavity")
    push(gpu_lib, st)
    before = gpu_lib.get_field("p")
    assert gpu_lib.lib.cappgpu_exchange(cappgpu.FIELD["p"]) == 0
    np.testing.assert_array_equal(gpu_lib.get_field("p"), before)
    x = ctypes.c_double(3.25)
    assert gpu_lib.lib.cappgpu_global_sum(ctypes.byref(x)) == 0 and x.value == 3.25
    assert gpu_lib.lib.cappgpu_global_max(ctypes.byref(x)) == 0 and x.value == 3.25


# ------------------------------------------------------------------ gradient

@pytest.mark.parametrize("kind", ["cavity", "skewed", "channel"])
def test_grad_gauss_bit_exact(gpu_lib, oracle_mod, kind):
    case, st = state(oracle_mod, kind)
    randomize(st, np.random.default_rng(2), ["u", "gradu_x", "gradu_y", "gradu_z"])
    run_both(gpu_lib, st, lambda s: s.grad_gauss("u", "gradu_x", "gradu_y", "gradu_z"))
    compare(gpu_lib, st, exact=FIELD_NAMES)


def test_grad_gauss_host_pointer(gpu_lib, oracle_mod):
    case, st = state(oracle_mod, "skewed")
    rng = np.random.default_rng(4)
    u = rng.uniform(-1, 1, st.nijk)
    st.set_field("u", u)
    push(gpu_lib, st)
    st.grad_gauss("u", "gradu_x", "gradu_y", "gradu_z")
    out = [np.empty(st.nijk) for _ in range(3)]
    dp = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    assert gpu_lib.lib.cappgpu_grad_gauss_h(dp(u), *map(dp, out)) == 0
    for a, n in zip(out, ("gradu_x", "gradu_y", "gradu_z")):
        np.testing.assert_array_equal(a, st.field(n))


def test_bpres_bit_exact(gpu_lib, oracle_mod):
    case, st = state(oracle_mod, "skewed")
    randomize(st, np.random.default_rng(6), ["p"])
    run_both(gpu_lib, st, lambda s: s.bpres("p"))
    compare(gpu_lib, st, exact=FIELD_NAMES)


def test_correct_boundary_conditions_bit_exact(gpu_lib, oracle_mod):
    case, st = state(oracle_mod, "cavity")
    randomize(st, np.random.default_rng(8), ["u", "v", "w", "f1", "f2"])
    run_both(gpu_lib, st, lambda s: s.correct_boundary_conditions())
    compare(gpu_lib, st, exact=FIELD_NAMES)


# -------------------------------------------------------------------- solvers

def solver_state(oracle_mod, seed, symmetric):
    st = oracle_mod.State(14, 13, 12)
    rng = np.random.default_rng(seed)
    diag_dominant_matrix(st, rng, symmetric=symmetric)
    # stale SIP factors in every cell: the factorisation reads ghost-layer
    # values of bn, be, bt (sipsol.f90:34-46)
    randomize(st, rng, ["bb", "bs", "bw", "bp", "bn", "be", "bt"], -0.3, 0.3)
    randomize(st, rng, ["p", "res", "u"])
    st.params.update(dict(alfa=0.92, sor=[1e-8] * 10, nsw=[300] * 10, ipr=3, jpr=3, kpr=3))
    return st


def test_spmv_bit_exact(gpu_lib, oracle_mod):
    st = solver_state(oracle_mod, 1, False)
    push(gpu_lib, st)
    dg = gpu_lib.spmv("u", "pp")
    do = st.spmv("u", "pp")
    compare(gpu_lib, st, exact=FIELD_NAMES)
    assert abs(dg - do) <= 1e-13 * abs(do)


@pytest.mark.parametrize("solver,symmetric", [("sipsol", False), ("pcgsip", True), ("iccg", True),
                                              ("cgstab", False), ("cgstab_sip", False), ("dpcg", True)])
def test_solver_parity(gpu_lib, oracle_mod, solver, symmetric):
    st = solver_state(oracle_mod, 20, symmetric)
    push(gpu_lib, st)
    rg = gpu_lib.solve(solver, "p", IP)
    ro = st.solve(solver, "p", IP)
    assert rg.iters == ro.iters, (rg, ro)
    assert rg.status == ro.status
    assert abs(rg.res0 - ro.res0) <= 1e-12 * ro.res0
    assert abs(rg.resl - ro.resl) <= 1e-6 * ro.resl + 1e-300
    params = gpu_lib.get_params()
    assert abs(params.resor[IP - 1] - st.params.resor[IP - 1]) <= 1e-12 * abs(st.params.resor[IP - 1])
    sip = ["bb", "bs", "bw", "bp", "bn", "be", "bt"]
    exact = sip if solver in ("sipsol", "pcgsip", "cgstab_sip") else []
    if solver == "sipsol":
        exact = exact + ["p"]   # no reduction reaches fi: bit-exact at equal sweep count
    compare(gpu_lib, st, exact=exact, rtol=RTOL, names=["p"] + sip)
    r = compare(gpu_lib, st, names=["res"])
    assert r["res"][0] <= 1e-8 * np.abs(st.field("res")).max() + 1e-12


def test_solver_nonfinite_is_reported(gpu_lib, oracle_mod):
    st = solver_state(oracle_mod, 3, True)
    su = st.field("su")
    ni, nj, nk = st.dims
    su[(nk // 2 - 1) * ni * nj + (ni // 2 - 1) * nj + nj // 2 - 1] = np.nan   # an interior cell
    push(gpu_lib, st)
    with pytest.raises(cappgpu.CappError, match="-4"):
        gpu_lib.solve("pcgsip", "p", IP)


def test_solver_host_pointer_dropin(gpu_lib, oracle_mod):
    st = solver_state(oracle_mod, 5, True)
    push(gpu_lib, st)
    host = {n: st.field(n).copy() for n in FIELD_NAMES}
    for n in ("ae", "aw", "an", "as", "at", "ab", "ap", "su", "p", "res",
              "bb", "bs", "bw", "bp", "bn", "be", "bt"):
        assert gpu_lib.lib.cappgpu_register(cappgpu.FIELD[n], host[n].ctypes.data_as(
            ctypes.POINTER(ctypes.c_double))) == 0
    rc = gpu_lib.lib.cappgpu_pcgsip_h(host["p"].ctypes.data_as(ctypes.POINTER(ctypes.c_double)), IP)
    assert rc >= 0
    st.solve("pcgsip", "p", IP)
    np.testing.assert_allclose(host["p"], st.field("p"), rtol=0, atol=1e-10 * np.abs(st.field("p")).max())
    np.testing.assert_array_equal(host["bp"], st.field("bp"))
    gpu_lib.lib.cappgpu_unregister_all()
    with pytest.raises(AssertionError):
        assert gpu_lib.lib.cappgpu_pcgsip_h(host["p"].ctypes.data_as(ctypes.POINTER(ctypes.c_double)), IP) == 0


@pytest.mark.parametrize("solver,code,symmetric", [("sipsol", 1, False), ("cgstab", 2, False), ("iccg", 3, True),
                                                   ("pcgsip", 4, True), ("cgstab_sip", 5, False),
                                                   ("dpcg", 6, True)])
def test_every_solver_host_pointer_dropin_reports(gpu_lib, oracle_mod, solver, code, symmetric):
    """The host-pointer form of each solver (what the Fortran drop-ins
    pcgsip, sipsol, iccg, cgstab, cgstab_sip and
    Diagonally_Preconditioned_CG call) solves the registered host array
    as the oracle does and leaves the numbers of the solve's unit-66 line
    (pcg-sip.f90:195-197, pcg-jacobi.f90:150-152) for cappgpu_last_report."""
    st = solver_state(oracle_mod, 20, symmetric)
    push(gpu_lib, st)
    host = {n: st.field(n).copy() for n in FIELD_NAMES}
    dp = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))  # noqa: E731
    for n in ("ae", "aw", "an", "as", "at", "ab", "ap", "su", "p", "res",
              "bb", "bs", "bw", "bp", "bn", "be", "bt"):
        assert gpu_lib.lib.cappgpu_register(cappgpu.FIELD[n], dp(host[n])) == 0
    try:
        rc = getattr(gpu_lib.lib, f"cappgpu_{solver}_h")(dp(host["p"]), IP)
        ro = st.solve(solver, "p", IP)
        assert rc == ro.status
        ref = st.field("p")
        assert np.linalg.norm(host["p"] - ref) <= RTOL * np.linalg.norm(ref)
        assert np.abs(host["res"] - st.field("res")).max() <= 1e-8 * np.abs(st.field("res")).max() + 1e-12
        s, i, rep = ctypes.c_int(), ctypes.c_int(), cappgpu.SolveReport()
        assert gpu_lib.lib.cappgpu_last_report(ctypes.byref(s), ctypes.byref(i), ctypes.byref(rep)) == 0
        assert (s.value, i.value) == (code, IP)
        assert (rep.iters, rep.status) == (ro.iters, ro.status)
        assert abs(rep.res0 - ro.res0) <= 1e-12 * ro.res0
    finally:
        gpu_lib.lib.cappgpu_unregister_all()


# ------------------------------------------------------------------- assembly

def assembly_state(oracle_mod, kind, seed):
    case, st = state(oracle_mod, kind)
    rng = np.random.default_rng(seed)
    randomize(st, rng, ["u", "v", "w", "p", "pp"])
    randomize(st, rng, ["gradu_x", "gradu_y", "gradu_z", "gradv_x", "gradv_y", "gradv_z",
                        "gradw_x", "gradw_y", "gradw_z", "gradp_x", "gradp_y", "gradp_z"])
    randomize(st, rng, ["f1", "f2", "f3"], -0.5, 0.5)
    randomize(st, rng, ["vis", "den", "apu", "apv", "apw"], 0.5, 1.5)
    randomize(st, rng, ["su", "sv", "sw", "ae", "aw", "an", "as", "at", "ab", "ap", "sp", "spv"])
    randomize(st, rng, ["bb", "bs", "bw", "bp", "bn", "be", "bt", "he", "hw", "hn", "hs", "ht", "hb"])
    randomize(st, rng, ["uo", "vo", "wo", "uoo", "voo", "woo", "t"])
    return case, st


SCHEMES = {
    "uds": {}, "cds": {"lcds": 1}, "cds4": {"lcds4": 1}, "luds": {"lluds": 1}, "quick": {"lquds": 1},
    "smart": {"flux_limiter": 1, "lsmart": 1}, "avl": {"flux_limiter": 1, "lavl": 1},
    "muscl": {"flux_limiter": 1, "lmuscl": 1}, "umist": {"flux_limiter": 1, "lumist": 1},
    "gamma": {"flux_limiter": 1, "lgamma": 1},
}


def dir_args(case, d):
    nj, nij = case.nj, case.ni * case.nj
    return [(nj, 1, nij, "ar1x", "ar1y", "ar1z", "fx", "ae", "aw", "f1"),
            (1, nij, nj, "ar2x", "ar2y", "ar2z", "fy", "an", "as", "f2"),
            (nij, nj, 1, "ar3x", "ar3y", "ar3z", "fz", "at", "ab", "f3")][d]


@pytest.mark.parametrize("scheme", list(SCHEMES))
@pytest.mark.parametrize("d", [0, 1, 2])
def test_fluxuvw_bit_exact(gpu_lib, oracle_mod, scheme, d):
    case, st = assembly_state(oracle_mod, "skewed", 30 + d)
    flags = dict(lcds=0, lcds4=0, lluds=0, lquds=0, flux_limiter=0, lsmart=0, lavl=0, lmuscl=0, lumist=0, lgamma=0)
    flags.update(SCHEMES[scheme])
    st.params.update(flags)
    st.params.gds[0] = 0.9
    a = dir_args(case, d)
    run_both(gpu_lib, st, lambda s: s.fluxuvw(*a))
    compare(gpu_lib, st, exact=FIELD_NAMES)


@pytest.mark.parametrize("ipc", [0, 1])
@pytest.mark.parametrize("d", [0, 1, 2])
def test_piso_assemble_bit_exact(gpu_lib, oracle_mod, ipc, d):
    case, st = assembly_state(oracle_mod, "skewed", 40 + d)
    a = dir_args(case, d)
    bp = ["be", "bn", "bt"][d]
    run_both(gpu_lib, st, lambda s: s.piso_assemble_pressure_eq(*a, ipc, bp))
    compare(gpu_lib, st, exact=FIELD_NAMES)


@pytest.mark.parametrize("d", [0, 1, 2])
def test_face_kernels_without_geometry_cache_bit_exact(gpu_lib, oracle_mod, d):
    """Option face_geo 0: the FP64 face kernels evaluate the geometric part
    of each face, and the gradient 1/vol, on every call instead of reading
    the caches (the tests above run the cached form); both match the
    oracle bit for bit."""
    case, st = assembly_state(oracle_mod, "skewed", 45 + d)
    st.params.gds[0] = 0.9
    a = dir_args(case, d)
    bp = ["be", "bn", "bt"][d]
    push(gpu_lib, st)
    gpu_lib.set_option("face_geo", 0)
    for s in (gpu_lib, st):
        s.fluxuvw(*a)
        s.piso_assemble_pressure_eq(*a, 1, bp)
        s.grad_gauss("v", "gradv_x", "gradv_y", "gradv_z")
    compare(gpu_lib, st, exact=FIELD_NAMES)


def test_face_geometry_cache_follows_grid_writes(gpu_lib, oracle_mod):
    """Writing a geometry field after the caches were built (cell centres,
    face areas and volumes moved by set_field) rebuilds them: the next
    assembly and gradient match the oracle on the new grid bit for bit."""
    case, st = assembly_state(oracle_mod, "skewed", 48)
    a = dir_args(case, 0)
    grad = ("u", "gradu_x", "gradu_y", "gradu_z")
    run_both(gpu_lib, st, lambda s: (s.piso_assemble_pressure_eq(*a, 1, "be"), s.grad_gauss(*grad)))
    compare(gpu_lib, st, exact=FIELD_NAMES)
    rng = np.random.default_rng(3)
    for n in ("xc", "yc", "ar1x", "vol"):
        v = st.field(n) * (1.0 + 1e-3 * rng.standard_normal(st.nijk))
        st.set_field(n, v)
        gpu_lib.set_field(n, v)
    for s in (gpu_lib, st):
        s.piso_assemble_pressure_eq(*a, 1, "be")
        s.fluxuvw(*a)
        s.grad_gauss(*grad)
    compare(gpu_lib, st, exact=FIELD_NAMES)


@pytest.mark.parametrize("d", [0, 1, 2])
def test_assemble_pressure_eq_bit_exact(gpu_lib, oracle_mod, d):
    case, st = assembly_state(oracle_mod, "skewed", 50 + d)
    a = dir_args(case, d)
    run_both(gpu_lib, st, lambda s: s.assemble_pressure_eq(*a))
    compare(gpu_lib, st, exact=FIELD_NAMES)


@pytest.mark.parametrize("d", [0, 1, 2])
def test_fluxmass_bit_exact(gpu_lib, oracle_mod, d):
    case, st = assembly_state(oracle_mod, "skewed", 60 + d)
    a = dir_args(case, d)
    run_both(gpu_lib, st, lambda s: s.fluxmass(*a))
    compare(gpu_lib, st, exact=FIELD_NAMES)


@pytest.mark.parametrize("cn", [0, 1])
def test_gethbya_bit_exact(gpu_lib, oracle_mod, cn):
    case, st = assembly_state(oracle_mod, "skewed", 70)
    st.params.update(dict(bdf=1, btime=1.0, cn=cn, timestep=0.01))
    run_both(gpu_lib, st, lambda s: s.piso_gethbya())
    compare(gpu_lib, st, exact=FIELD_NAMES)


# ---------------------------------------------------------- composite routines

@pytest.mark.parametrize("kind", ["cavity", "channel"])
def test_calcuvw_parity(gpu_lib, oracle_mod, kind):
    case, st = state(oracle_mod, kind)
    st.update_values_at_ghostcells()
    if kind == "channel":
        st.params.update(dict(timestep=0.05))
    rg, ro = run_both(gpu_lib, st, lambda s: s.calcuvw())
    for a, b in zip(rg, ro):
        assert a.iters == b.iters, (rg, ro)
    compare(gpu_lib, st, rtol=RTOL)


def test_piso_multiple_correction_parity(gpu_lib, oracle_mod):
    case, st = state(oracle_mod, "channel")
    st.params.update(dict(timestep=0.05))
    st.update_values_at_ghostcells()
    st.calcuvw()
    rg, ro = run_both(gpu_lib, st, lambda s: s.piso_multiple_correction())
    for a, b in zip(rg[:2], ro[:2]):
        assert a.iters == b.iters, (a, b)
    compare(gpu_lib, st, rtol=RTOL, names=["u", "v", "w", "p", "pp", "f1", "f2", "f3", "su", "ap",
                                           "gradp_x", "gradp_y", "gradp_z", "be", "bn", "bt"])
    P = gpu_lib.get_params()
    assert abs(P.sumlocalconterr - st.params.sumlocalconterr) <= 1e-9 * abs(st.params.sumlocalconterr)


@pytest.mark.parametrize("npcor", [1, 2])
def test_calcp_parity(gpu_lib, oracle_mod, npcor):
    case, st = state(oracle_mod, "cavity")
    st.params.update(dict(npcor=npcor))
    st.update_values_at_ghostcells()
    st.calcuvw()
    run_both(gpu_lib, st, lambda s: s.calcp())
    compare(gpu_lib, st, rtol=RTOL, names=["u", "v", "w", "p", "pp", "f1", "f2", "f3", "gradp_x",
                                           "gradp_y", "gradp_z"])


def test_courant_and_continuity(gpu_lib, oracle_mod):
    case, st = assembly_state(oracle_mod, "channel", 80)
    st.params.update(dict(ltransient=1, conumfix=1, conumfixvalue=0.5, timestep=0.01))
    run_both(gpu_lib, st, lambda s: (s.courant(), s.continuity_errors()))
    P = gpu_lib.get_params()
    for n in ("timestep", "conum", "meanconum", "time", "globalconterr", "sumlocalconterr"):
        a, b = getattr(P, n), getattr(st.params, n)
        assert abs(a - b) <= 1e-12 * max(abs(b), 1e-300), (n, a, b)
    assert P.localconterr == st.params.localconterr
    compare(gpu_lib, st, exact=["su"], names=["su"])


# -------------------------------------------------------------- step drivers

def test_piso_steps_parity(gpu_lib, oracle_mod):
    case, st = state(oracle_mod, "channel")
    rg, ro = run_both(gpu_lib, st, lambda s: s.piso_steps(3))
    assert rg.iters == ro.iters
    compare(gpu_lib, st, rtol=RTOL, names=["u", "v", "w", "p", "f1", "f2", "f3", "uo", "vo", "wo"])
    P = gpu_lib.get_params()
    assert abs(P.timestep - st.params.timestep) <= 1e-12 * st.params.timestep


def test_simple_iters_parity(gpu_lib, oracle_mod):
    case, st = state(oracle_mod, "cavity")
    rg, ro = run_both(gpu_lib, st, lambda s: s.simple_iters(3))
    compare(gpu_lib, st, rtol=RTOL, names=["u", "v", "w", "p", "f1", "f2", "f3"])


@pytest.mark.parametrize("dims,flags", [((9, 8, 7), "all"), ((9, 8, 7), "some"), ((5, 6, 5), "all")])
def test_outbc_bit_exact(gpu_lib, oracle_mod, dims, flags):
    """outbc.f90: outlet faces (code 2) mixed with other codes on all six
    face sets; the flow is summed in the routine's order, so every array
    agrees bit for bit.  The corner ghosts shared by two face sets take the
    later set's values, as in the reference."""
    st = oracle_mod.State(*dims)
    rng = np.random.default_rng(31)
    randomize(st, rng, ["u", "v", "w", "te", "ed", "vis", "t", "f1", "f2", "f3"])
    randomize(st, rng, ["den", "ar1x", "ar1y", "ar1z"], 0.5, 1.5)
    for face in cappgpu.params.BC_NAMES:
        b = st.bc(face)
        b[:] = rng.choice([1, 2, 2, 4], size=b.size)
    on = dict(low=1, loe=1, los=1, lon=1, lob=1, lot=1)
    if flags == "some":
        on.update(los=0, lot=0)
    st.params.update(dict(lout=1, flowin=0.9, **on))
    run_both(gpu_lib, st, lambda s: s.outbc())
    compare(gpu_lib, st, exact=FIELD_NAMES)


def test_simple_iters_with_outlet_parity(gpu_lib, oracle_mod):
    """The SIMPLE loop of an inflow/outflow cavity: inlet (code 1) on the
    west face, outlet (code 2) on the east face, outbc rescaling the outlet
    to flowin in every iteration (main.f90:190, calcp...f90:62)."""
    case, st = state(oracle_mod, "cavity")
    st.bc("lbw")[:] = 1
    st.bc("lbe")[:] = 2
    st.params.update(dict(uin=0.5, lout=1, loe=1, flowin=0.02, const_mflux=0))
    rg, ro = run_both(gpu_lib, st, lambda s: s.simple_iters(3))
    compare(gpu_lib, st, rtol=RTOL, names=["u", "v", "w", "p", "f1", "f2", "f3"])


def test_les_viscosity_parity(gpu_lib, oracle_mod):
    """find_strain_rate + calc_vis_les (LES path, main.f90:205): gradients and
    strain bit-exact; the viscosity (pow, exp, log of CUDA against the
    oracle's libm) and the wall-function ghost values to 1e-13."""
    case, st = state(oracle_mod, "channel")
    p = st.params
    p.lles = 1
    p.lcal[cappgpu.params.IVIS - 1] = 1
    p.urf[cappgpu.params.IVIS - 1] = 0.7   # the under-relaxation of :69 takes part
    # a viscosity field to relax from, and strain-bearing velocities
    rng = np.random.default_rng(21)
    v0 = st.field("vis") * (1 + 0.1 * rng.random(st.field("vis").size))
    st.set_field("vis", v0)
    run_both(gpu_lib, st, lambda s: (s.find_strain_rate(), s.calc_vis_les()))
    grads = [f"grad{c}_{x}" for c in "uvw" for x in "xyz"]
    compare(gpu_lib, st, exact=grads + ["strain"], names=grads + ["strain"])
    compare(gpu_lib, st, rtol=1e-13, names=["vis"])
    g = case.view(gpu_lib.get_field("vis"))
    assert np.all(g[2:-2, 2:-2, 2:-2] >= p.viscos * (1 - 1e-12))


def test_les_piso_steps_parity(gpu_lib, oracle_mod):
    case, st = state(oracle_mod, "channel")
    st.params.lles = 1
    st.params.lcal[cappgpu.params.IVIS - 1] = 1
    rg, ro = run_both(gpu_lib, st, lambda s: s.piso_steps(3))
    assert rg.iters == ro.iters
    compare(gpu_lib, st, rtol=RTOL, names=["u", "v", "w", "p", "f1", "f2", "f3", "vis", "strain"])


def test_const_massflux_correction_parity(gpu_lib, oracle_mod):
    case, st = state(oracle_mod, "channel")
    rng = np.random.default_rng(5)
    st.set_field("apu", 0.01 + 0.01 * rng.random(st.field("apu").size))
    st.params.uin = 1.3
    st.params.gradpcmf = 0.2
    run_both(gpu_lib, st, lambda s: s.const_massflux_correction())
    compare(gpu_lib, st, rtol=1e-13, names=["u"])
    g = gpu_lib.get_params().gradpcmf
    assert abs(g - st.params.gradpcmf) <= 1e-12 * abs(st.params.gradpcmf)
    # the bulk velocity is restored (to the rounding of the sums)
    v = case.view
    vol = v(st.field("vol"))[1:-1, 2:-2, 2:-2]
    u = v(gpu_lib.get_field("u"))[1:-1, 2:-2, 2:-2]
    a = v(st.field("apu"))[1:-1, 2:-2, 2:-2]
    ubar = (vol * u).sum() / vol.sum()
    assert abs(ubar - 1.3) < 1e-12


def test_top_wall_index_guard(gpu_lib, oracle_mod):
    """calcuvw.f90:254 addresses the top wall with lk(nimm); a grid with
    ni > nk would put it outside the array: refused, not run."""
    gpu_lib.init(14, 8, 8)
    with pytest.raises(cappgpu.CappError):
        gpu_lib.piso_steps(1)


# ------------------------------------------------ persistent wavefront path

@pytest.mark.parametrize("shape", [(40, 12, 30), (37, 21, 19), (5, 3, 70)])
@pytest.mark.parametrize("wave", [1, 0])
@pytest.mark.parametrize("solver", ["pcgsip", "sipsol", "cgstab_sip", "iccg"])
def test_sip_wavefront_multiblock(gpu_lib, oracle_mod, shape, wave, solver):
    """pcgsip, sipsol, cgstab_sip and iccg with the persistent wavefront over
    many line blocks (and with one launch per hyperplane) against the
    oracle: SIP factors bit-exact (sipsol: the solution too), same iteration
    count.  The loops of cgstab_sip and iccg take the k ghost layers in
    (k = 2..nkm): their wavefronts run on that box."""
    st = oracle_mod.State(*[n + 4 for n in shape])
    rng = np.random.default_rng(sum(shape))
    diag_dominant_matrix(st, rng, symmetric=solver in ("pcgsip", "iccg"))
    randomize(st, rng, ["bb", "bs", "bw", "bp", "bn", "be", "bt"], -0.3, 0.3)
    randomize(st, rng, ["p", "res"])
    st.params.update(dict(alfa=0.92, sor=[1e-9] * 10, nsw=[400] * 10, ipr=3, jpr=3, kpr=3))
    push(gpu_lib, st)
    gpu_lib.set_option("wave", wave)
    try:
        rg = gpu_lib.solve(solver, "p", IP)
    finally:
        gpu_lib.set_option("wave", 1)
    ro = st.solve(solver, "p", IP)
    assert rg.iters == ro.iters, (rg, ro)
    exact = ["bb", "bs", "bw", "bp", "bn", "be", "bt"] + (["p"] if solver == "sipsol" else [])
    compare(gpu_lib, st, exact=exact, rtol=RTOL, names=["p", "bb", "bs", "bw", "bp", "bn", "be", "bt"])
    r = compare(gpu_lib, st, names=["res"])
    assert r["res"][0] <= 1e-8 * np.abs(st.field("res")).max() + 1e-12


def test_pcgsip_wavefront_repeated_calls_are_deterministic(gpu_lib, oracle_mod):
    st = oracle_mod.State(44, 16, 36)
    rng = np.random.default_rng(9)
    diag_dominant_matrix(st, rng, symmetric=True)
    st.params.update(dict(alfa=0.92, sor=[1e-9] * 10, nsw=[400] * 10, ipr=3, jpr=3, kpr=3))
    push(gpu_lib, st)
    outs = []
    for _ in range(3):
        gpu_lib.set_field("p", st.field("p"))
        gpu_lib.solve("pcgsip", "p", IP)
        outs.append(gpu_lib.get_field("p"))
    np.testing.assert_array_equal(outs[0], outs[1])
    np.testing.assert_array_equal(outs[0], outs[2])
