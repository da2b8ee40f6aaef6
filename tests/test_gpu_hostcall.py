"""The host-pointer drop-ins, called through ctypes exactly as the Fortran
shim calls them: the module arrays live in host memory (numpy arrays
standing for the reference's module arrays, the gradients interleaved as
gradu(3,nxyza)), are registered once by address, and every routine gets
its array arguments as host pointers.  After each call the host arrays
must equal the oracle's arrays bit for bit (1e-10 for the routines with
solver reductions), and arguments that are not registered (gfortran
temporaries of array sections) must take the staging path with the same
result."""
import ctypes

import numpy as np
import pytest

import cappgpu
from cappgpu import FIELD, FIELD_NAMES, SolveReport
from helpers import GEOMETRY, push, randomize, with_fluxes

pytestmark = pytest.mark.gpu
DP = ctypes.POINTER(ctypes.c_double)
GRADS = ("gradu", "gradv", "gradw", "gradp")


def dp(a):
    return a.ctypes.data_as(DP)


class HostModules:
    """The reference's module arrays in host memory, registered with the
    library as the shim's cappgpu_attach does."""

    def __init__(self, lib, st):
        self.lib, self.st = lib, st
        n = st.nijk
        self.a = {name: st.field(name).copy() for name in FIELD_NAMES
                  if not any(name.startswith(g + "_") for g in GRADS)}
        self.g3 = {g: np.stack([st.field(f"{g}_{c}") for c in "xyz"], axis=1).reshape(3 * n).copy()
                   for g in GRADS}
        L = lib.lib
        assert L.cappgpu_unregister_all() == 0
        for name, arr in self.a.items():
            assert L.cappgpu_register(FIELD[name], dp(arr)) == 0
        for g, arr in self.g3.items():
            assert L.cappgpu_register_vec3(FIELD[g + "_x"], dp(arr)) == 0

    def field(self, name):
        for g in GRADS:
            if name.startswith(g + "_"):
                return self.g3[g].reshape(-1, 3)[:, "xyz".index(name[-1])]
        return self.a[name]

    def check(self, names=None, rtol=None):
        for name in names or FIELD_NAMES:
            h, o = self.field(name), self.st.field(name)
            if rtol is None:
                bad = np.flatnonzero(h != o)
                assert bad.size == 0, f"{name}: {bad.size} elements differ, first at {bad[:5]}"
            else:
                nrm = np.linalg.norm(o)
                rel = np.linalg.norm(h - o) / (nrm if nrm else 1.0)
                assert rel <= rtol, f"{name}: relative L2 {rel:.2e}"


def small_state(oracle_mod, kind, seed):
    mk = {"skewed": lambda: cappgpu.cases.poisson(N=(10, 9, 8)),
          "channel": lambda: cappgpu.cases.channel(N=(8, 6, 8))}[kind]
    case = mk()
    st = oracle_mod.State.from_case(case)
    with_fluxes(case, st)
    rng = np.random.default_rng(seed)
    randomize(st, rng, ["u", "v", "w", "p", "pp"])
    randomize(st, rng, [f"{g}_{c}" for g in GRADS for c in "xyz"])
    randomize(st, rng, ["f1", "f2", "f3"], -0.5, 0.5)
    randomize(st, rng, ["vis", "den", "apu", "apv", "apw"], 0.5, 1.5)
    randomize(st, rng, ["su", "sv", "sw", "ae", "aw", "an", "as", "at", "ab", "ap", "sp", "spv"])
    randomize(st, rng, ["bb", "bs", "bw", "bp", "bn", "be", "bt", "he", "hw", "hn", "hs", "ht", "hb"])
    randomize(st, rng, ["uo", "vo", "wo", "uoo", "voo", "woo", "t"])
    return case, st


def dir_args(case, d):
    nj, nij = case.nj, case.ni * case.nj
    return [(nj, 1, nij, "ar1x", "ar1y", "ar1z", "fx", "ae", "aw", "f1"),
            (1, nij, nj, "ar2x", "ar2y", "ar2z", "fy", "an", "as", "f2"),
            (nij, nj, 1, "ar3x", "ar3y", "ar3z", "fz", "at", "ab", "f3")][d]


@pytest.mark.parametrize("d", [0, 1, 2])
def test_fluxuvw_h(gpu_lib, oracle_mod, d):
    case, st = small_state(oracle_mod, "skewed", 100 + d)
    st.params.gds[0] = 0.9
    push(gpu_lib, st)
    H = HostModules(gpu_lib, st)
    a = dir_args(case, d)
    rc = gpu_lib.lib.cappgpu_fluxuvw_h(*a[:3], *(dp(H.field(n)) for n in a[3:]))
    assert rc == 0, gpu_lib.lib.cappgpu_last_error()
    st.fluxuvw(*a)
    H.check()


def test_fluxuvw_h_staged_arguments(gpu_lib, oracle_mod):
    """acfe, acfw and fcf passed as unregistered copies (array-section
    temporaries): the copies receive the result, the registered arrays of
    those names are left alone."""
    case, st = small_state(oracle_mod, "skewed", 110)
    push(gpu_lib, st)
    H = HostModules(gpu_lib, st)
    a = dir_args(case, 0)
    acfe, acfw, fcf = (H.field(n).copy() for n in ("ae", "aw", "f1"))
    ae0, aw0 = H.field("ae").copy(), H.field("aw").copy()
    geo = [dp(H.field(n)) for n in a[3:7]]
    assert gpu_lib.lib.cappgpu_fluxuvw_h(*a[:3], *geo, dp(acfe), dp(acfw), dp(fcf)) == 0
    st.fluxuvw(*a)
    np.testing.assert_array_equal(acfe, st.field("ae"))
    np.testing.assert_array_equal(acfw, st.field("aw"))
    np.testing.assert_array_equal(H.field("ae"), ae0)
    np.testing.assert_array_equal(H.field("aw"), aw0)
    H.check(["su", "sv", "sw", "bp", "bt", "bb"])


@pytest.mark.parametrize("ipc", [0, 1])
@pytest.mark.parametrize("d", [0, 2])
def test_piso_assemble_pressure_eq_h(gpu_lib, oracle_mod, ipc, d):
    case, st = small_state(oracle_mod, "skewed", 120 + d + 3 * ipc)
    push(gpu_lib, st)
    H = HostModules(gpu_lib, st)
    a = dir_args(case, d)
    bp = ["be", "bn", "bt"][d]
    rc = gpu_lib.lib.cappgpu_piso_assemble_pressure_eq_h(*a[:3], *(dp(H.field(n)) for n in a[3:]), ipc,
                                                          dp(H.field(bp)))
    assert rc == 0, gpu_lib.lib.cappgpu_last_error()
    st.piso_assemble_pressure_eq(*a, ipc, bp)
    H.check()


@pytest.mark.parametrize("d", [0, 1])
def test_assemble_pressure_eq_h(gpu_lib, oracle_mod, d):
    case, st = small_state(oracle_mod, "skewed", 130 + d)
    push(gpu_lib, st)
    H = HostModules(gpu_lib, st)
    a = dir_args(case, d)
    assert gpu_lib.lib.cappgpu_assemble_pressure_eq_h(*a[:3], *(dp(H.field(n)) for n in a[3:])) == 0
    st.assemble_pressure_eq(*a)
    H.check()


def test_ghost_cells_bpres_exchange_h(gpu_lib, oracle_mod):
    case, st = small_state(oracle_mod, "skewed", 140)
    rng = np.random.default_rng(141)
    for face in cappgpu.params.BC_NAMES:
        st.bc(face)[:] = rng.integers(1, 5, st.bc(face).size)
    st.params.update(dict(uin=0.3, vin=-0.2, win=0.1, tein=0.05, edin=0.7, tin=1.5))
    push(gpu_lib, st)
    H = HostModules(gpu_lib, st)
    L = gpu_lib.lib
    assert L.cappgpu_update_values_at_ghostcells_h() == 0
    st.update_values_at_ghostcells()
    H.check()
    assert L.cappgpu_bpres_h(dp(H.field("p"))) == 0
    st.bpres("p")
    H.check()
    before = H.field("p").copy()
    assert L.cappgpu_exchange_h(dp(H.field("p"))) == 0
    np.testing.assert_array_equal(H.field("p"), before)
    # an unregistered copy of p takes the staging path
    pcopy = H.field("pp").copy()
    st2 = st.field("pp").copy()
    assert L.cappgpu_bpres_h(dp(pcopy)) == 0
    st.bpres("pp")
    np.testing.assert_array_equal(pcopy, st.field("pp"))
    assert not np.array_equal(st2, st.field("pp"))


def test_composite_routines_h(gpu_lib, oracle_mod):
    """calcuvw, PISO_getHbyA and PISO_multiple_correction on the channel,
    host arrays through the frames, against the oracle; the solver reports
    come back and format as the reference's unit-66 lines."""
    case = cappgpu.cases.channel(N=(8, 6, 8))
    st = oracle_mod.State.from_case(case)
    with_fluxes(case, st)
    st.params.update(dict(timestep=0.05))
    st.update_values_at_ghostcells()
    push(gpu_lib, st)
    H = HostModules(gpu_lib, st)
    L = gpu_lib.lib
    reps = (SolveReport * 3)()
    assert L.cappgpu_calcuvw_h(reps) == 0
    ro = st.calcuvw()
    assert [r.iters for r in reps] == [r.iters for r in ro]
    H.check(rtol=1e-10)
    assert L.cappgpu_piso_gethbya_h() == 0
    st.piso_gethbya()
    H.check(rtol=1e-10)
    # PISO_multiple_correction from the state after calcuvw
    st2 = oracle_mod.State.from_case(case)
    with_fluxes(case, st2)
    st2.params.update(dict(timestep=0.05))
    st2.update_values_at_ghostcells()
    st2.calcuvw()
    push(gpu_lib, st2)
    H2 = HostModules(gpu_lib, st2)
    preps = (SolveReport * 8)()
    assert L.cappgpu_piso_multiple_correction_h(preps) == 0
    ro2 = st2.piso_multiple_correction()
    assert [preps[q].iters for q in range(2)] == [ro2[q].iters for q in range(2)]
    H2.check(["u", "v", "w", "p", "pp", "f1", "f2", "f3", "su", "ap"], rtol=1e-10)
    solver, ifi, rep = ctypes.c_int(), ctypes.c_int(), SolveReport()
    assert L.cappgpu_last_report(ctypes.byref(solver), ctypes.byref(ifi), ctypes.byref(rep)) == 0
    assert (solver.value, ifi.value) == (cappgpu.SOLVER["pcgsip"], 4)
    assert rep.iters == preps[1].iters and rep.res0 == preps[1].res0
    buf = ctypes.create_string_buffer(256)
    assert L.cappgpu_solver_report_line(solver, ifi, ctypes.byref(rep), 0, 0, buf, 256) == 0
    line = buf.value.decode()
    assert line.startswith("PCG(SIP):  Solving for p, Initial residual = ") and line.endswith(
        f", No Iterations {rep.iters}"), line
