"""Standalone pressure-correction solve on the skewed 256^3 grid: PCG-SIP in
FP64, in the FP32 refinement form (precision 1) and from the learned initial
guess (precision 2), each to a 1e-6 relative L1 residual.

The system: piso_assemble_pressure_eq in the three directions with
vol*apu*den = 1 (PISO_assemble_pressure_eq.f90:48-237), boundary links
removed (pure Neumann, boundary face fluxes zero), ap = the sum of the
links, su = -div F of a seeded Gaussian face-velocity field with its mean
removed, and the reference cell pinned as in PISO_multiple_correction.f90:
117-129.  The net of the learned guess is trained on six such systems with
other seeds and judged on a seventh."""
import numpy as np
import pytest

import cappgpu

pytestmark = pytest.mark.gpu
IP = 4
N = 256


@pytest.fixture(scope="module")
def poisson_case():
    return cappgpu.cases.poisson(N=(N, N, N))


def assemble(lib, case, seed):
    ni, nj, nk = case.ni, case.nj, case.nk
    nij = ni * nj
    rng = np.random.default_rng(seed)
    for c in "uvw":
        lib.set_field(c, rng.standard_normal(ni * nj * nk))
    for n in ("p", "su", "gradp_x", "gradp_y", "gradp_z"):
        lib.set_field(n, np.zeros(ni * nj * nk))
    for idew, idns, idtb, ar, fif, ae, aw, f, bp in (
            (nj, 1, nij, "ar1", "fx", "ae", "aw", "f1", "be"),
            (1, nij, nj, "ar2", "fy", "an", "as", "f2", "bn"),
            (nij, nj, 1, "ar3", "fz", "at", "ab", "f3", "bt")):
        # ipc = 1: the face flux is formed in the corrector branch
        # (PISO_assemble_pressure_eq.f90:204-229); with p = 0 its explicit
        # non-orthogonal source is zero
        lib.piso_assemble_pressure_eq(idew, idns, idtb, ar + "x", ar + "y", ar + "z", fif, ae, aw, f, 1, bp)
    v = lambda n: lib.get_field(n).reshape(nk, ni, nj)
    I = (slice(2, nk - 2), slice(2, ni - 2), slice(2, nj - 2))        # interior (k, i, j)
    a = {n: v(n) for n in ("ae", "aw", "an", "as", "at", "ab")}
    # no links to ghost cells: i (E/W), j (N/S), k (T/B)
    a["aw"][:, 2, :] = 0.0
    a["ae"][:, ni - 3, :] = 0.0
    a["as"][:, :, 2] = 0.0
    a["an"][:, :, nj - 3] = 0.0
    a["ab"][2, :, :] = 0.0
    a["at"][nk - 3, :, :] = 0.0
    f1, f2, f3 = v("f1").copy(), v("f2").copy(), v("f3").copy()
    # closed boundary: the boundary faces carry no flux
    f1[:, 1, :] = 0.0
    f1[:, ni - 3, :] = 0.0
    f2[:, :, 1] = 0.0
    f2[:, :, nj - 3] = 0.0
    f3[1, :, :] = 0.0
    f3[nk - 3, :, :] = 0.0
    div = (f1[I] - f1[2:nk - 2, 1:ni - 3, 2:nj - 2] + f2[I] - f2[2:nk - 2, 2:ni - 2, 1:nj - 3]
           + f3[I] - f3[1:nk - 3, 2:ni - 2, 2:nj - 2])
    su = np.zeros((nk, ni, nj))
    su[I] = -(div - div.mean())
    ap = np.zeros((nk, ni, nj))
    ap[I] = sum(a[n][I] for n in a)
    # reference cell (ipr, jpr, kpr), 1-based, as in
    # PISO_multiple_correction.f90:117-129: ap = 1, no links, su = p = 0
    pr = lib.get_params()
    kp, ip, jp = pr.kpr - 1, pr.ipr - 1, pr.jpr - 1
    for n in a:
        a[n][kp, ip, jp] = 0.0
    ap[kp, ip, jp] = 1.0
    su[kp, ip, jp] = 0.0
    for n, arr in a.items():
        lib.set_field(n, arr.reshape(-1))
    lib.set_field("ap", ap.reshape(-1))
    lib.set_field("su", su.reshape(-1))
    lib.set_field("p", np.zeros(ni * nj * nk))


def _level_free_diff(case, p, ref):
    """Relative L2 difference of the interior fields with their means removed.
    One pinned cell hardly constrains the near-constant mode of a Neumann
    problem, so two solutions within the same residual tolerance may differ
    in level; only pressure differences enter the flow."""
    I = (slice(2, case.nk - 2), slice(2, case.ni - 2), slice(2, case.nj - 2))
    a = case.view(p)[I]
    b = case.view(ref)[I]
    a = a - a.mean()
    b = b - b.mean()
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def solve(lib, mode):
    lib.set_field("p", np.zeros(lib.nijk))
    lib.precision(mode)
    try:
        lib.timer_start()
        rep = lib.pcgsip("p", IP)
        ms = lib.timer_stop()
    finally:
        lib.precision(0)
    return rep, ms, lib.get_field("p")


def test_poisson_256_fp64_fp32_and_learned(gpu_lib, poisson_case):
    case = poisson_case
    gpu_lib.load_case(case)
    tol = case.params["sor"][IP - 1]
    assert tol == 1e-6
    # FP64 plain against the FP32 refinement form on one system
    assemble(gpu_lib, case, seed=7)
    r64, ms64, p64 = solve(gpu_lib, 0)
    r32, ms32, p32 = solve(gpu_lib, 1)
    assert r64.status == 0 and r32.status == 0
    assert r64.resl / r64.res0 < tol and r32.resl / r32.res0 < tol
    assert r32.res0 == pytest.approx(r64.res0, rel=1e-12)
    d32 = _level_free_diff(case, p32, p64)
    # the learned guess: trained on six other systems, judged on this one
    gpu_lib.learn_reset(6, seed=11)
    gpu_lib.learn_collect(True)
    for seed in range(1, 7):
        assemble(gpu_lib, case, seed=seed)
        solve(gpu_lib, 1)
    gpu_lib.learn_collect(False)
    assert gpu_lib.learn_stats()["samples"] == 6
    loss = gpu_lib.learn_train(10, block=64, lr=1e-3)
    assemble(gpu_lib, case, seed=7)
    s0 = gpu_lib.learn_stats()
    rl, msl, pl = solve(gpu_lib, 2)
    s1 = gpu_lib.learn_stats()
    dl = _level_free_diff(case, pl, p64)
    kept = s1["guesses"] - s0["guesses"]
    print(f"poisson {N}^3: FP64 {r64.iters} it {ms64:.1f} ms; FP32+IR {r32.iters} it {ms32:.1f} ms "
          f"(diff {d32:.2e}); learned (loss {loss:.3f}, guess {'kept' if kept else 'discarded'}, "
          f"ratio {s1['last_ratio']:.3f}) {rl.iters} it {msl:.1f} ms (diff {dl:.2e})")
    assert rl.status == 0 and rl.resl / rl.res0 < tol
    assert rl.res0 == pytest.approx(r64.res0, rel=1e-12)   # res0 of the solve's own start
    assert s1["guesses"] + s1["fallbacks"] == s0["guesses"] + s0["fallbacks"] + 1
    assert d32 < 1e3 * tol and dl < 1e3 * tol
