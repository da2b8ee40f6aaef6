"""The C ABI: the library builds for sm_103a, loads, and exports every
entry point that include/cappgpu.h declares (no GPU work here)."""
import re

import pytest

import cappgpu
from conftest import ROOT

HEADER = ROOT / "include" / "cappgpu.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(cappgpu_\w+)\s*\(", text)))


def test_header_declares_the_routine_set():
    names = declared_functions()
    # the reference routines of the hot path each have an entry point
    for ref in ("sipsol", "pcgsip", "iccg", "cgstab", "cgstab_sip", "dpcg", "grad_gauss", "fluxuvw",
                "calcuvw", "piso_assemble_pressure_eq", "assemble_pressure_eq",
                "update_values_at_ghostcells", "exchange", "global_sum", "global_max", "bpres",
                "piso_gethbya", "piso_multiple_correction", "fluxmass", "calcp", "courant",
                "continuity_errors", "outbc", "correct_boundary_conditions"):
        assert "cappgpu_" + ref in names, ref


def test_library_exports_every_declared_symbol():
    lib_path = cappgpu.build()
    import ctypes
    lib = ctypes.CDLL(str(lib_path))
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_every_symbol():
    assert set(declared_functions()) == set(cappgpu.SIGNATURES), (
        set(declared_functions()) ^ set(cappgpu.SIGNATURES))


def test_calls_without_init_fail_cleanly():
    lib = cappgpu.Library()
    lib.lib.cappgpu_finalize()
    with pytest.raises(cappgpu.CappError):
        lib.dims = (8, 8, 8)
        lib.get_field("u")
    assert lib.lib.cappgpu_ijkpr() < 0


def test_every_run_time_option_is_documented():
    """Every key cappgpu_set_option accepts (csrc/context.cu) is described
    in the header, and the header names no key the library refuses."""
    src = (ROOT / "cappuccino-ghostcells-mpi_gb300" / "csrc" / "context.cu").read_text()
    accepted = set(re.findall(r'strcmp\(key, "(\w+)"\)', src))
    assert {"sip_slabs", "fused_dot", "sweep_timing", "learn_loss"} <= accepted
    doc = HEADER.read_text()
    i = doc.index("cappgpu_set_option")
    documented = set(re.findall(r'"(\w+)":', doc[doc.rfind("/*", 0, i):i]))
    assert accepted - documented == set(), accepted - documented
    assert documented - accepted == set(), documented - accepted
