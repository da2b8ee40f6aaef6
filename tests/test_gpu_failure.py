"""Failure detection of the wavefront engines, without a GPU fault.

Every wait of a wavefront block on a predecessor is bounded by the
"spin_limit" option.  With a limit of one poll the blocks of a many-block
grid give up on their predecessors, the kernel raises its device-wide abort
flag and returns, and the solve reports CAPPGPU_E_SPIN.  The library then
resets the block tickets and edge mailboxes, so the next solve on the same
context, at the default limit, must equal the oracle again."""
import numpy as np
import pytest

import cappgpu
from cappgpu import CappError
from helpers import compare, ctypes_copy, diag_dominant_matrix, push, randomize

pytestmark = pytest.mark.gpu

IP = 4
DEFAULT_SPIN = 1 << 21
SHAPE = (64, 24, 64)   # 4 x 8 wavefront blocks of 16 x 8 lines


def reload(lib, st):
    """The oracle state's arrays and parameters into the existing context
    (no re-initialisation: the wavefront's tickets and mailboxes stay the
    ones the failed solve left behind)."""
    for n in cappgpu.FIELD_NAMES:
        lib.set_field(n, st.field(n))
    p = cappgpu.Params()
    ctypes_copy(p, st.params)
    lib.set_params(p)


def system(oracle_mod, solver, seed=5):
    st = oracle_mod.State(*[n + 4 for n in SHAPE])
    rng = np.random.default_rng(seed)
    diag_dominant_matrix(st, rng, symmetric=solver == "pcgsip")
    randomize(st, rng, ["bb", "bs", "bw", "bp", "bn", "be", "bt"], -0.3, 0.3)
    randomize(st, rng, ["p", "res"])
    st.params.update(dict(alfa=0.92, sor=[1e-9] * 10, nsw=[400] * 10, ipr=3, jpr=3, kpr=3))
    return st


@pytest.mark.parametrize("solver", ["pcgsip", "sipsol"])
def test_spin_limit_reports_and_next_solve_recovers(gpu_lib, oracle_mod, solver):
    st = system(oracle_mod, solver)
    push(gpu_lib, st)
    gpu_lib.set_option("spin_limit", 1)
    try:
        with pytest.raises(CappError) as ei:
            gpu_lib.solve(solver, "p", IP)
    finally:
        gpu_lib.set_option("spin_limit", DEFAULT_SPIN)
    msg = str(ei.value)
    assert "(-5)" in msg and "spin limit" in msg, msg
    # same context, default limit: tickets and mailboxes were reset
    reload(gpu_lib, st)
    rg = gpu_lib.solve(solver, "p", IP)
    ro = st.solve(solver, "p", IP)
    assert rg.iters == ro.iters, (rg, ro)
    exact = ["bb", "bs", "bw", "bp", "bn", "be", "bt"] + (["p"] if solver == "sipsol" else [])
    compare(gpu_lib, st, exact=exact, rtol=1e-10, names=["p", "bb", "bs", "bw", "bp", "bn", "be", "bt"])


@pytest.mark.parametrize("engine", [0, 2])
def test_spin_limit_in_the_refinement_form(gpu_lib, oracle_mod, engine):
    """The FP32 wavefronts of precision mode 1 (one line per thread, or the
    multi-line engine) report the same way, and the next mode-1 solve
    reaches the same result as one on a fresh start."""
    st = system(oracle_mod, "pcgsip", seed=6)
    push(gpu_lib, st)
    gpu_lib.precision(1)
    gpu_lib.set_option("lane_wave", engine)
    try:
        good = gpu_lib.solve("pcgsip", "p", IP)
        p_good = gpu_lib.get_field("p")
        reload(gpu_lib, st)
        gpu_lib.set_option("spin_limit", 1)
        try:
            with pytest.raises(CappError) as ei:
                gpu_lib.solve("pcgsip", "p", IP)
        finally:
            gpu_lib.set_option("spin_limit", DEFAULT_SPIN)
        assert "(-5)" in str(ei.value)
        reload(gpu_lib, st)
        again = gpu_lib.solve("pcgsip", "p", IP)
        np.testing.assert_array_equal(gpu_lib.get_field("p"), p_good)
        assert again.iters == good.iters
    finally:
        gpu_lib.precision(0)
        gpu_lib.set_option("lane_wave", 0)
