"""The oracle against the reference's own routines (no GPU).

tests/golden/reference_outputs.json holds what the reference's Fortran
source produced on each case of tests/golden/golden_cases.py: digests of
the module arrays the routine changed and one over all arrays, the module
scalars it changed (as exact hex floats) and a digest over all of them,
the index maps of setind.f90 and the unit-66 report lines.
make_golden.py made it by running the reference's subroutines through a
Fortran-subset executor (tests/golden/f90exec.py), as no Fortran compiler
exists here.  Every case must agree bit for bit: the oracle, and with it
the CUDA path that the GPU tests hold to the oracle, computes what the
reference computes, not only what its restatement says.
"""
import ctypes
import json
import pathlib
import sys

import pytest

HERE = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(HERE / "golden"))

import cappgpu  # noqa: E402
from cappgpu import FIELD_NAMES, SOLVER, SolveReport  # noqa: E402
import golden_cases as G  # noqa: E402

GOLDEN = json.loads((HERE / "golden" / "reference_outputs.json").read_text())
CASES = {c.name: c for c in G.all_cases()}


def test_every_case_has_a_reference_record():
    assert set(GOLDEN) == set(CASES), set(GOLDEN) ^ set(CASES)
    assert len(GOLDEN) >= 60


@pytest.mark.parametrize("name", sorted(GOLDEN))
def test_oracle_matches_the_reference(oracle_mod, name):
    rec, c = GOLDEN[name], CASES[name]
    grid_case, st = c.build(oracle_mod)
    assert G.state_digest(st) == rec["inputs"], "the seeded inputs are not the ones the reference ran on"
    assert [int(x) for x in st.li()] == rec["li"] and [int(x) for x in st.lk()] == rec["lk"]
    out = G.run_oracle(c, grid_case, st)
    got = {n: G.field_digest(st.field(n)) for n in FIELD_NAMES}
    differing = [n for n, d in rec["fields"].items() if got[n] != d]
    assert not differing, f"{name}: arrays differing from the reference's: {differing}"
    assert G.all_fields_digest(got) == rec["all_fields"], f"{name}: an array the reference left alone changed"
    params = G.oracle_params(st)
    pdiff = {k: (params[k], v) for k, v in rec["params"].items() if params[k] != v}
    assert not pdiff, f"{name}: module scalars differing from the reference's: {pdiff}"
    assert G.params_digest(params) == rec["all_params"], f"{name}: a module scalar the reference left alone changed"
    if name.startswith("solve_"):
        check_report_line(name, out, rec["unit66"])


def check_report_line(name, rep, lines):
    """The library's unit-66 line for the oracle's report is the line the
    reference wrote (same numbers, same format)."""
    solver = max((o for o, *_ in G.SOLVERS if name.startswith(f"solve_{o}_")), key=len)
    L = cappgpu.load_library()
    buf = ctypes.create_string_buffer(256)
    r = SolveReport(res0=rep.res0, resl=rep.resl, iters=rep.iters, status=rep.status)
    assert L.cappgpu_solver_report_line(SOLVER[solver], G.IP, ctypes.byref(r), 0, 0, buf, 256) == 0
    assert lines and buf.value.decode() == lines[-1], (buf.value.decode(), lines)

