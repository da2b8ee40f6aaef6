"""The FP32 + FP64-refinement form of the pressure solve (cappgpu_precision(1)).

Not bit-compatible with the reference by design: the checks are the
reference's own exit test on the FP64 residual and closeness to the FP64
plain solution."""
import numpy as np
import pytest

import cappgpu
from helpers import diag_dominant_matrix, push, randomize

pytestmark = pytest.mark.gpu
IP = 4


def _state(oracle_mod, dims, seed, sor):
    st = oracle_mod.State(*dims)
    rng = np.random.default_rng(seed)
    diag_dominant_matrix(st, rng, symmetric=True)
    randomize(st, rng, ["bb", "bs", "bw", "bp", "bn", "be", "bt"], -0.3, 0.3)
    randomize(st, rng, ["p", "res"])
    st.params.update(dict(alfa=0.92, sor=[sor] * 10, nsw=[2000] * 10, ipr=3, jpr=3, kpr=3))
    return st


@pytest.mark.parametrize("dims,sor", [((14, 13, 12), 1e-8), ((40, 37, 35), 1e-6), ((21, 36, 19), 1e-10)])
def test_mixed_pcgsip_meets_fp64_exit_test(gpu_lib, oracle_mod, dims, sor):
    st = _state(oracle_mod, dims, 3, sor)
    push(gpu_lib, st)
    gpu_lib.precision(0)
    r64 = gpu_lib.pcgsip("p", IP)
    p64 = gpu_lib.get_field("p")
    push(gpu_lib, st)
    gpu_lib.precision(1)
    try:
        r32 = gpu_lib.pcgsip("p", IP)
    finally:
        gpu_lib.precision(0)
    p32 = gpu_lib.get_field("p")
    assert r32.status == 0 and r64.status == 0
    assert r32.res0 == pytest.approx(r64.res0, rel=1e-12)
    assert r32.resl / r32.res0 < sor                  # FP64 residual, the reference's test
    # the module residual array holds the true FP64 residual of the result
    ni, nj, nk = dims
    res = gpu_lib.get_field("res").reshape(nk, ni, nj)[2:-2, 2:-2, 2:-2]
    assert abs(np.abs(res).sum() - r32.resl) <= 1e-9 * r32.res0
    # both solves stop within the tolerance of the exact solution
    assert np.linalg.norm(p32 - p64) <= 1e3 * sor * np.linalg.norm(p64)


def test_mixed_piso_step_channel(gpu_lib):
    case = cappgpu.cases.channel(N=(10, 8, 12))
    gpu_lib.load_case(case)
    gpu_lib.precision(1)
    try:
        rep = gpu_lib.piso_steps(2)
    finally:
        gpu_lib.precision(0)
    assert rep.status == 0
    assert rep.resl / rep.res0 < case.params["sor"][IP - 1]


def test_precision_rejects_unknown_mode(gpu_lib):
    gpu_lib.init(8, 8, 8)
    with pytest.raises(cappgpu.CappError):
        gpu_lib.precision(3)


def _channel_run(gpu_lib, case, mode, tight, steps=3):
    gpu_lib.load_case(case)
    if tight:   # the momentum solves to 1e-9 too (sor 1e-3 and 20 sweeps otherwise)
        pr = gpu_lib.get_params()
        for q in range(3):
            pr.sor[q] = 1e-9
            pr.nsw[q] = 400
        gpu_lib.set_params(pr)
    gpu_lib.set_option("tight_correctors", tight)
    gpu_lib.precision(mode)
    try:
        rep = gpu_lib.piso_steps(steps)
    finally:
        gpu_lib.precision(0)
        gpu_lib.set_option("tight_correctors", 0)
    assert rep.status == 0
    return {k: gpu_lib.get_field(k) for k in ("u", "v", "w", "p")}


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_mixed_piso_agrees_with_fp64_when_every_corrector_is_converged(gpu_lib):
    # The reference stops the first corrector's p solve at sor = 0.1 and the
    # momentum solves at 1e-3, and where they stop moves the step's result
    # far above FP32 rounding.  With every corrector solved to the last one's
    # tolerance (1e-6) and the momentum solves to 1e-9, the FP32 form (FP32
    # SIP factors and sweeps, FP32 velocity gradients) must land on the FP64
    # result within that tolerance's reach.
    case = cappgpu.cases.channel(N=(24, 20, 28))
    ref = _channel_run(gpu_lib, case, 0, 0)
    t64 = _channel_run(gpu_lib, case, 0, 1)
    t32 = _channel_run(gpu_lib, case, 1, 1)
    spread = {k: _rel(t64[k], ref[k]) for k in ref}
    err = {k: _rel(t32[k], t64[k]) for k in ref}
    print("first-corrector spread", spread, "FP32 form vs FP64", err)
    for k in ("u", "v", "w"):
        assert err[k] < 1e-5, (k, err[k])
    assert err["p"] < 1e-4


def _rel_all(x, ref):
    return {k: _rel(x[k], ref[k]) for k in ("u", "v", "w", "p")}


def test_mixed_channel128_twenty_steps_per_field_errors(gpu_lib):
    """The bench's workload: 5 warm-up steps of the 128^3 channel in the
    reference's form, then 20 steps with every p corrector solved to the
    same tolerance and the momentum solves to 1e-9, in FP64 and in
    precision mode 1 with its default FP32 parts.
    At the reference's p tolerance 1e-6: each velocity component within
    1e-5 (relative L2) of the FP64 result; p within twice the distance the
    1e-6 tolerance itself lets an FP64 solution lie from the converged one
    (FP64 against FP64 with the p solves 100x tighter) -- two solutions that
    each satisfy the exit test differ by up to the sum of their distances to
    the converged solution (PISO_multiple_correction.f90:131-141).
    At an equal tighter tolerance (1e-8) every field, p included, within
    1e-5 of the FP64 result."""
    case = cappgpu.cases.channel(N=(128, 128, 128))
    gpu_lib.load_case(case)
    gpu_lib.piso_steps(5)
    snap = {n: gpu_lib.get_field(n) for n in cappgpu.FIELD_NAMES}
    params = gpu_lib.get_params()

    def run(mode, p_factor=1.0):
        for n, a in snap.items():
            gpu_lib.set_field(n, a)
        pr = cappgpu.Params()
        import ctypes
        ctypes.memmove(ctypes.addressof(pr), ctypes.addressof(params), ctypes.sizeof(pr))
        for q in range(3):
            pr.sor[q] = 1e-9
            pr.nsw[q] = 400
        pr.sor[3] = pr.sor[3] * p_factor
        pr.nsw[3] = max(pr.nsw[3], 4000)
        gpu_lib.set_params(pr)
        gpu_lib.set_option("tight_correctors", 1)
        gpu_lib.precision(mode)
        try:
            rep = gpu_lib.piso_steps(20)
        finally:
            gpu_lib.precision(0)
            gpu_lib.set_option("tight_correctors", 0)
        assert rep.status == 0
        return {k: gpu_lib.get_field(k) for k in ("u", "v", "w", "p")}

    t64 = run(0)
    fine = run(0, 1e-2)
    t32 = run(1)
    t32_fine = run(1, 1e-2)
    spread = _rel_all(t64, fine)
    err = _rel_all(t32, t64)
    err_fine = _rel_all(t32_fine, fine)
    fmt = lambda d: {k: f"{v:.2e}" for k, v in d.items()}
    print("20 steps, 128^3: FP64 vs FP64 solved 100x tighter", fmt(spread), "| mode 1 vs FP64", fmt(err),
          "| mode 1 vs FP64, both with p to 1e-8", fmt(err_fine))
    for k in ("u", "v", "w"):
        assert err[k] <= 1e-5, (k, err[k])
    assert err["p"] <= max(1e-5, 2.0 * spread["p"]), (err["p"], spread["p"])
    for k in ("u", "v", "w", "p"):
        assert err_fine[k] <= 1e-5, (k, err_fine[k])


@pytest.mark.parametrize("axis,slabs", [(0, 2), (0, 4), (1, 2)])
@pytest.mark.parametrize("solver", ["pcgsip", "sipsol"])
@pytest.mark.parametrize("dims", [(36, 37, 68), (34, 37, 68)])
def test_block_local_sip_per_slab(gpu_lib, oracle_mod, axis, slabs, solver, dims):
    """The FP32 SIP of the refinement form restarted at every i-slab (axis 0)
    or k-slab (axis 1) (options sip_slabs, sip_slab_axis; interior 32 or 30
    x 33 x 64: 4 FP32 block columns of 8 lines, the last one partial in the
    second case, whose mirrored backward blocks then start 2 lines outside
    the box; 2 block rows of 32): both solvers still meet the reference's
    exit test on the FP64 residual, within the tolerance's reach of the FP64
    solution, with the SIP over the whole box and with the slabs."""
    sor = 1e-6
    st = _state(oracle_mod, dims, 11, sor)
    st.set_field("res", np.zeros_like(st.field("res")))
    push(gpu_lib, st)
    gpu_lib.precision(0)
    r64 = getattr(gpu_lib, solver)("p", IP)
    p64 = gpu_lib.get_field("p")
    out, sol = {}, {}
    for n in (1, slabs):
        push(gpu_lib, st)
        gpu_lib.set_option("sip_slabs", n)
        gpu_lib.set_option("sip_slab_axis", axis)
        gpu_lib.precision(1)
        try:
            out[n] = getattr(gpu_lib, solver)("p", IP)
        finally:
            gpu_lib.precision(0)
            gpu_lib.set_option("sip_slabs", 4096)
            gpu_lib.set_option("sip_slab_axis", 0)
        sol[n] = gpu_lib.get_field("p")
        r = out[n]
        assert r.status == 0 and r64.status == 0
        assert r.res0 == pytest.approx(r64.res0, rel=1e-12)
        assert r.resl / r.res0 < sor
        assert np.linalg.norm(sol[n] - p64) <= 1e3 * sor * np.linalg.norm(p64)
    # the slabs change the preconditioner: a different iteration path
    assert out[slabs].iters != out[1].iters or not np.array_equal(sol[slabs], sol[1])
    print(f"{solver}: whole box {out[1].iters} it, {slabs} {'ik'[axis]}-slabs {out[slabs].iters} it, "
          f"FP64 {r64.iters} it")


@pytest.mark.parametrize("dims,sor", [((14, 13, 12), 1e-6), ((40, 37, 35), 1e-4)])
def test_mixed_sipsol_meets_fp64_exit_test(gpu_lib, oracle_mod, dims, sor):
    """sipsol in precision mode 1: FP64 residual and exit test, FP32 SIP
    factorisation and substitutions."""
    st = _state(oracle_mod, dims, 4, sor)
    # the reference's forward recurrence reads the ghost layers of res; start
    # both forms from a clean res so that the FP64 form converges too
    st.set_field("res", np.zeros_like(st.field("res")))
    push(gpu_lib, st)
    gpu_lib.precision(0)
    r64 = gpu_lib.sipsol("p", IP)
    p64 = gpu_lib.get_field("p")
    push(gpu_lib, st)
    gpu_lib.precision(1)
    try:
        r32 = gpu_lib.sipsol("p", IP)
    finally:
        gpu_lib.precision(0)
    p32 = gpu_lib.get_field("p")
    assert r32.status == 0 and r64.status == 0
    assert r32.res0 == pytest.approx(r64.res0, rel=1e-12)   # the first sweep's FP64 residual
    assert r32.resl / r32.res0 < sor
    assert abs(r32.iters - r64.iters) <= max(2, r64.iters // 10)
    assert np.linalg.norm(p32 - p64) <= 1e3 * sor * np.linalg.norm(p64)


@pytest.mark.parametrize("solver", ["pcgsip", "sipsol"])
@pytest.mark.parametrize("dims", [(14, 13, 12), (40, 37, 35), (70, 9, 45), (104, 23, 71)])
def test_fp32_substitution_engines_agree_bit_for_bit(gpu_lib, oracle_mod, solver, dims):
    """The FP32 substitutions of the refinement form run on the wavefront of
    wave.cuh (option lane_wave 0), on the warp-tile engine (lane_wave 1) or
    on the multi-line wavefront (lane_wave 2).  All evaluate each cell's
    expression on the same operands in the same order, so the whole solve
    -- iterations, residuals, solution -- is the same to the bit.  The
    shapes cover one tile or block, several along a and c, and extents that
    are not multiples of either."""
    st = _state(oracle_mod, dims, 5, 1e-6)
    st.set_field("res", np.zeros_like(st.field("res")))
    out = {}
    for lw in (0, 1, 2):
        push(gpu_lib, st)
        gpu_lib.set_option("lane_wave", lw)
        gpu_lib.set_option("sip_slabs", 1)   # the other engines run the SIP over the whole box
        gpu_lib.set_option("fused_dot", 0)   # and form r.z in a vector pass
        gpu_lib.precision(1)
        try:
            r = getattr(gpu_lib, solver)("p", IP)
        finally:
            gpu_lib.precision(0)
            gpu_lib.set_option("lane_wave", 0)
            gpu_lib.set_option("sip_slabs", 4096)
            gpu_lib.set_option("fused_dot", 1)
        out[lw] = (r, gpu_lib.get_field("p"), gpu_lib.get_field("res"))
    r0, p0, q0 = out[0]
    assert r0.status == 0
    for lw in (1, 2):
        r1, p1, q1 = out[lw]
        assert r1.status == 0
        assert r1.iters == r0.iters, lw
        assert r1.resl == r0.resl and r1.res0 == r0.res0, lw
        np.testing.assert_array_equal(p1, p0)
        np.testing.assert_array_equal(q1, q0)


@pytest.mark.parametrize("make", ["channel", "poisson"])
def test_fp32_gradient_from_cached_fp32_geometry(gpu_lib, make):
    """The FP32 velocity gradient of precision modes 1-2 from the FP32 copy of
    the geometry (option face_geo 1, the default) gives the bits of the
    per-call conversion (face_geo 0), ghost and padding cells included, and
    lies within FP32 rounding of the FP64 gradient; a geometry write
    rebuilds the copy."""
    case = getattr(cappgpu.cases, make)(N=(20, 12, 16))
    gpu_lib.load_case(case)
    names = ("gradu_x", "gradu_y", "gradu_z")
    u = gpu_lib.get_field("u")
    rng = np.random.default_rng(3)
    gpu_lib.set_field("u", u + 0.1 * rng.standard_normal(u.shape))

    def grad(mode, face_geo):
        gpu_lib.set_option("face_geo", face_geo)
        gpu_lib.precision(mode)
        try:
            gpu_lib.grad_gauss("u", *names)
        finally:
            gpu_lib.precision(0)
            gpu_lib.set_option("face_geo", 1)
        return [gpu_lib.get_field(n) for n in names]

    g64 = grad(0, 1)
    g32c = grad(1, 1)
    g32 = grad(1, 0)
    for a, b, c in zip(g32c, g32, g64):
        np.testing.assert_array_equal(a, b)
        assert np.linalg.norm(a - c) <= 1e-5 * np.linalg.norm(c)
    # a geometry write (vol) invalidates the FP32 copy
    vol = gpu_lib.get_field("vol")
    gpu_lib.set_field("vol", 2.0 * vol)
    h32c, h32 = grad(1, 1), grad(1, 0)
    for a, b, c in zip(h32c, h32, g32):
        np.testing.assert_array_equal(a, b)
        assert not np.array_equal(a, c)
    gpu_lib.set_field("vol", vol)


@pytest.mark.parametrize("batch", [1, 4, 7])
def test_sweep_timing_counts_the_forward_substitutions(gpu_lib, oracle_mod, batch):
    """Option sweep_timing: CUDA events around every FP64 pcgsip forward
    substitution; one per iteration that ran (the launches after the exit
    test, which return at once, are not counted), whatever the batch, and
    the same solution as without the events."""
    st = _state(oracle_mod, (40, 37, 35), 9, 1e-6)
    st.set_field("res", np.zeros_like(st.field("res")))
    push(gpu_lib, st)
    r0 = gpu_lib.pcgsip("p", IP)
    p0 = gpu_lib.get_field("p")
    push(gpu_lib, st)
    gpu_lib.set_option("cg_batch", batch)
    gpu_lib.set_option("sweep_timing", 1)
    try:
        gpu_lib.sweep_stats(reset=True)
        r1 = gpu_lib.pcgsip("p", IP)
        ms, n = gpu_lib.sweep_stats(reset=True)
    finally:
        gpu_lib.set_option("sweep_timing", 0)
        gpu_lib.set_option("cg_batch", 4)
    assert r1.iters == r0.iters and r1.resl == r0.resl
    np.testing.assert_array_equal(gpu_lib.get_field("p"), p0)
    assert n == r1.iters and ms > 0.0
    assert gpu_lib.sweep_stats() == (0.0, 0)


@pytest.mark.parametrize("dims", [(14, 13, 12), (40, 37, 68), (104, 23, 71)])
def test_fused_dot_in_the_backward_substitution(gpu_lib, oracle_mod, dims):
    """sk = r.z formed in the FP32 backward substitution (option fused_dot,
    the default) or in a vector pass after it: the same sum in another
    order, so both solves meet the FP64 exit test within an iteration or two
    of each other and agree to the tolerance's reach; the fused form gives
    the same bits when repeated."""
    sor = 1e-6
    st = _state(oracle_mod, dims, 7, sor)
    st.set_field("res", np.zeros_like(st.field("res")))
    out = {}
    for fused in (1, 0, 1):
        push(gpu_lib, st)
        gpu_lib.set_option("fused_dot", fused)
        gpu_lib.precision(1)
        try:
            r = gpu_lib.pcgsip("p", IP)
        finally:
            gpu_lib.precision(0)
            gpu_lib.set_option("fused_dot", 1)
        assert r.status == 0 and r.resl / r.res0 < sor
        p = gpu_lib.get_field("p")
        if fused in out:
            assert r.iters == out[fused][0].iters and r.resl == out[fused][0].resl
            np.testing.assert_array_equal(p, out[fused][1])
        out[fused] = (r, p)
    (r1, p1), (r0, p0) = out[1], out[0]
    assert abs(r1.iters - r0.iters) <= 2
    assert np.linalg.norm(p1 - p0) <= 1e3 * sor * np.linalg.norm(p0)


@pytest.mark.parametrize("engine", [1, 2])
def test_fp32_substitution_engine_repeated_calls(gpu_lib, oracle_mod, engine):
    """Mailboxes and the block ticket are left clean by every launch: the
    same solve repeated on the warp-tile or multi-line engine gives the
    same bits."""
    st = _state(oracle_mod, (70, 37, 45), 6, 1e-6)
    res = []
    for _ in range(3):
        push(gpu_lib, st)
        gpu_lib.set_option("lane_wave", engine)
        gpu_lib.precision(1)
        try:
            r = gpu_lib.pcgsip("p", IP)
        finally:
            gpu_lib.precision(0)
            gpu_lib.set_option("lane_wave", 0)
        res.append((r.iters, r.resl, gpu_lib.get_field("p")))
    for it, rl, p in res[1:]:
        assert it == res[0][0] and rl == res[0][1]
        np.testing.assert_array_equal(p, res[0][2])
