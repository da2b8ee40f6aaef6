"""The CUDA library against the reference's own routines, directly.

tests/golden/reference_outputs.json records what the reference's Fortran
source computes on each case of tests/golden/golden_cases.py (run by
tests/golden/make_golden.py).  Here the library runs every case whose
device routine is free of reductions and of transcendental functions --
ghost cells, gradient, bpres, boundary correction, fluxuvw (10 schemes x 3
directions), both pressure assemblies, fluxmass, PISO_getHbyA, outbc and
the grid geometry -- on the same inputs, and every module array must have
the reference's digest: the GPU matches the reference bit for bit.  The
solvers, whose sums run in another order, leave the reference's own
unit-66 report line.  The other cases (CUDA's pow/exp/log/tanh, composite
routines) are held to the oracle at 1e-10 by the other GPU tests, and the
oracle to the reference bit for bit by tests/test_golden_reference.py."""
import ctypes
import json
import pathlib
import sys

import pytest

HERE = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(HERE / "golden"))

from cappgpu import FIELD_NAMES, SOLVER, SolveReport  # noqa: E402
import f90exec as F  # noqa: E402
import golden_cases as G  # noqa: E402
from helpers import push  # noqa: E402

pytestmark = pytest.mark.gpu

GOLDEN = json.loads((HERE / "golden" / "reference_outputs.json").read_text())
CASES = {c.name: c for c in G.all_cases()}
BIT_EXACT_PREFIXES = ("ghost_cells_", "grad_gauss_", "bpres_", "correct_boundary_conditions_", "fluxuvw_",
                      "piso_assemble_pressure_eq_", "assemble_pressure_eq_", "fluxmass_", "piso_gethbya_",
                      "outbc_", "geometry_")
NAMES = sorted(n for n in GOLDEN if n.startswith(BIT_EXACT_PREFIXES))


def test_the_bit_exact_set_is_complete():
    assert len(NAMES) >= 50


@pytest.mark.parametrize("name", NAMES)
def test_gpu_matches_the_reference(gpu_lib, oracle_mod, name):
    rec, c = GOLDEN[name], CASES[name]
    grid_case, st = c.build(oracle_mod)
    assert G.state_digest(st) == rec["inputs"], "the seeded inputs are not the ones the reference ran on"
    push(gpu_lib, st)
    if name.startswith("geometry_"):
        gpu_lib.build_geometry(0)        # init.f90's cross products as written
    else:
        G.run_oracle(c, grid_case, gpu_lib)
    got = {n: G.field_digest(gpu_lib.get_field(n)) for n in FIELD_NAMES}
    differing = [n for n, d in rec["fields"].items() if got[n] != d]
    assert not differing, f"{name}: arrays differing from the reference's: {differing}"
    assert G.all_fields_digest(got) == rec["all_fields"], f"{name}: an array the reference left alone changed"


SOLVER_CASES = sorted(n for n in GOLDEN if n.startswith("solve_"))


@pytest.mark.parametrize("name", SOLVER_CASES)
def test_gpu_solver_report_is_the_reference_line(gpu_lib, oracle_mod, name):
    """The solvers sum in another order than the reference (block
    reductions), so their fields agree to 1e-10, not bit for bit.  The
    report a solve leaves is the reference's: the unit-66 line that the
    reference's own routine wrote (residuals to its four digits, the
    iteration index exactly, nsw + 1 when the sweep limit stopped it), and
    resor(ifi) to 1e-12."""
    rec, c = GOLDEN[name], CASES[name]
    solver = max((o for o, *_ in G.SOLVERS if name.startswith(f"solve_{o}_")), key=len)
    grid_case, st = c.build(oracle_mod)
    assert G.state_digest(st) == rec["inputs"]
    push(gpu_lib, st)
    rep = gpu_lib.solve(solver, "p", G.IP)
    buf = ctypes.create_string_buffer(256)
    assert gpu_lib.lib.cappgpu_solver_report_line(SOLVER[solver], G.IP, ctypes.byref(rep), 0, 0, buf, 256) == 0
    assert buf.value.decode() == rec["unit66"][-1]
    ref_resor = float.fromhex(rec["params"]["resor"][G.IP - 1]) if "resor" in rec["params"] else None
    if ref_resor is not None:
        assert abs(gpu_lib.get_params().resor[G.IP - 1] - ref_resor) <= 1e-12 * abs(ref_resor)


COMPOSITE_CASES = sorted(n for n in GOLDEN if n.startswith(("calcuvw_", "piso_multiple_correction_")))


def report_line(gpu_lib, solver, ifi, rep):
    buf = ctypes.create_string_buffer(256)
    r = SolveReport(res0=rep.res0, resl=rep.resl, iters=rep.iters, status=rep.status)
    assert gpu_lib.lib.cappgpu_solver_report_line(SOLVER[solver], ifi, ctypes.byref(r), 0, 0, buf, 256) == 0
    return buf.value.decode()


@pytest.mark.parametrize("name", COMPOSITE_CASES)
def test_gpu_composite_reports_are_the_reference_lines(gpu_lib, oracle_mod, name):
    """calcuvw and PISO_multiple_correction on the GPU leave the unit-66
    lines the reference's routines wrote: the three momentum SIP lines
    (calcuvw.f90:388-460 through sipsol.f90:101-103), and the PCG(SIP) line
    of every pressure solve with the last continuity-error line
    (continuityErrors.h), formatted from the GPU's scalars."""
    rec, c = GOLDEN[name], CASES[name]
    grid_case, st = c.build(oracle_mod)
    assert G.state_digest(st) == rec["inputs"]
    push(gpu_lib, st)
    reps = G.run_oracle(c, grid_case, gpu_lib)
    if name.startswith("calcuvw_"):
        got = [report_line(gpu_lib, "sipsol", ifi, reps[ifi - 1]) for ifi in (1, 2, 3)]
        assert got == [x for x in rec["unit66"] if x.startswith("SIP:")]
        return
    P = gpu_lib.get_params()
    got = [report_line(gpu_lib, "pcgsip", G.IP, r) for r in reps[:P.ncorr * P.npcor]]
    assert got == [x for x in rec["unit66"] if x.startswith("PCG(SIP)")]
    cont = F.fortran_format("(3(a,es10.3))", ["time step continuity errors : sum local = ", P.sumlocalconterr,
                                               ", global = ", P.globalconterr, ", cumulative = ",
                                               P.cumulativeconterr])
    assert cont == [x for x in rec["unit66"] if x.startswith("time step continuity")][-1]
