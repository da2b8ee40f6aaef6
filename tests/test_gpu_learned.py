"""The learned initial guess (precision mode 2): the library's U-Net forward
and backward kernels against the CPU oracle, and what a trained net gains."""
import numpy as np
import pytest

import cappgpu

pytestmark = pytest.mark.gpu
IP = 4


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


def _window_operator(rng, dims):
    """A diagonally dominant 7-point operator like a normalised p-equation."""
    off = rng.uniform(0.3, 1.2, (6,) + dims).astype(np.float32)
    diag = off.sum(0, keepdims=True) * np.float32(1.01)
    return np.concatenate([off, diag], 0)


def _check(gpu_lib, impl, rhs, coef):
    gpu_lib.set_option("learn_conv", impl)
    try:
        return gpu_lib.learn_check(rhs, coef)
    finally:
        gpu_lib.set_option("learn_conv", 0)


@pytest.mark.parametrize("impl", [1, 2])
@pytest.mark.parametrize("dims", [(8, 12, 16), (16, 16, 20), (4, 12, 20), (8, 36, 20)])
def test_tensor_core_convolutions_match_mma_sync(gpu_lib, dims, impl):
    """tcgen05 implicit GEMMs (forward and input gradient; impl 1 halo tiles
    where the weights fit, impl 2 per-tap gathers) against the mma.sync
    kernels on the same weights and data; the extents include voxel counts
    that are not multiples of the 128-voxel tile and x/y extents that are
    not multiples of the 8 x 16 halo tile."""
    import learned_oracle as lo
    gpu_lib.init(12, 12, 12)
    gpu_lib.learn_reset(0, seed=7)
    rng = np.random.default_rng(9)
    rhs = rng.standard_normal(dims).astype(np.float32)
    coef = _window_operator(rng, dims)
    out0, grad0, loss0 = _check(gpu_lib, 0, rhs, coef)
    out1, grad1, loss1 = _check(gpu_lib, impl, rhs, coef)
    assert np.all(np.isfinite(out1)) and np.all(np.isfinite(grad1))
    assert _rel(out1, out0) < 1e-2
    assert abs(loss1 - loss0) <= 1e-2 * loss0
    for name, sl in lo.param_slices():
        assert _rel(grad1[sl], grad0[sl]) < 5e-2, name


@pytest.mark.parametrize("impl", [0, 1, 2])
@pytest.mark.parametrize("dims", [(8, 12, 16), (16, 16, 20)])
def test_forward_and_gradients_match_cpu_oracle(gpu_lib, dims, impl):
    pytest.importorskip("torch")
    import learned_oracle as lo
    gpu_lib.init(12, 12, 12)
    gpu_lib.learn_reset(0, seed=11)
    p = gpu_lib.learn_params()            # the library's He-uniform start
    assert p.size == lo.NPARAMS
    rng = np.random.default_rng(5)
    rhs = rng.standard_normal(dims).astype(np.float32)
    coef = _window_operator(rng, dims)
    out, grad, loss = _check(gpu_lib, impl, rhs, coef)
    loss_o, out_o, grad_o = lo.loss_and_grad(p, rhs, coef)
    assert _rel(out, out_o) < 2e-2
    assert abs(loss - loss_o) <= 2e-2 * loss_o
    assert _rel(grad, grad_o) < 5e-2
    # every layer's weight and bias gradient, not only the total
    for name, sl in lo.param_slices():
        assert _rel(grad[sl], grad_o[sl]) < 1e-1, name


@pytest.mark.parametrize("kind", [1, 2])
@pytest.mark.parametrize("dims", [(8, 12, 16), (16, 16, 20)])
def test_target_losses_match_cpu_oracle(gpu_lib, dims, kind):
    """The supervised (1) and energy-norm (2) losses against a converged
    correction: loss, output and every layer's gradients against the CPU
    oracle (halo-tile tensor-core convolutions)."""
    pytest.importorskip("torch")
    import learned_oracle as lo
    gpu_lib.init(12, 12, 12)
    gpu_lib.learn_reset(0, seed=13)
    p = gpu_lib.learn_params()
    rng = np.random.default_rng(6)
    rhs = rng.standard_normal(dims).astype(np.float32)
    coef = _window_operator(rng, dims)
    target = rng.standard_normal(dims).astype(np.float32)
    gpu_lib.set_option("learn_conv", 1)
    out, grad, loss = gpu_lib.learn_check(rhs, coef, target=target, kind=kind)
    loss_o, out_o, grad_o = lo.loss_and_grad(p, rhs, coef, target=target, kind=kind)
    assert _rel(out, out_o) < 2e-2
    assert abs(loss - loss_o) <= 2e-2 * loss_o
    assert _rel(grad, grad_o) < 5e-2
    for name, sl in lo.param_slices():
        assert _rel(grad[sl], grad_o[sl]) < 1e-1, name
    with pytest.raises(cappgpu.CappError):   # a target loss without a target
        gpu_lib.learn_check(rhs, coef, kind=kind)


def test_recorded_target_is_the_converged_correction(gpu_lib):
    """Each recorded pair carries the solve's converged correction on the
    pair's scale: A^ t^ - r^ is the solve's final residual over its initial
    one (relative L1), and training on the supervised and energy-norm losses
    against it lowers them."""
    torch = pytest.importorskip("torch")
    import learned_oracle as lo
    case = cappgpu.cases.channel(N=(16, 16, 24))
    gpu_lib.load_case(case)
    ni, nj, nk = case.interior
    gpu_lib.precision(1)
    try:
        gpu_lib.learn_reset(8, seed=5)
        gpu_lib.learn_collect(True)
        rep = gpu_lib.piso_steps(2)                 # 4 pressure solves recorded
        gpu_lib.learn_collect(False)
        assert gpu_lib.learn_stats()["samples"] == 4
        smp = gpu_lib.learn_sample(3, (nk, ni, nj))   # the last solve
        r, coef, t = smp[0], smp[1:8], smp[8]
        p0 = gpu_lib.learn_params()
        losses = {}
        for kind in (1, 2):
            # from the same start each time; the loss on the whole last pair
            # before and after training
            gpu_lib.learn_params(p0)
            gpu_lib.set_option("learn_loss", kind)
            l0 = gpu_lib.learn_check(r, coef, target=t, kind=kind)[2]
            gpu_lib.learn_train(30, block=16, lr=1e-3)
            l1 = gpu_lib.learn_check(r, coef, target=t, kind=kind)[2]
            losses[kind] = (l0, l1)
    finally:
        gpu_lib.precision(0)
        gpu_lib.set_option("learn_loss", 0)
    at = lo.apply_a(coef, torch.as_tensor(t)).numpy()
    ratio = float(np.abs(at - r).sum() / np.abs(r).sum())
    assert rep.status == 0 and np.abs(t).max() > 0
    assert abs(ratio - rep.resl / rep.res0) <= 1e-3 + 0.05 * rep.resl / rep.res0, (ratio, rep.resl / rep.res0)
    for kind, (l0, l1) in losses.items():
        assert np.isfinite(l1) and l1 < l0, (kind, l0, l1)
    print(f"recorded target: |A^t^ - r^|/|r^| {ratio:.2e} (solve {rep.resl / rep.res0:.2e}); "
          f"supervised loss {losses[1][0]:.3f} -> {losses[1][1]:.3f}, energy {losses[2][0]:.3f} -> {losses[2][1]:.3f}")


def test_learn_check_rejects_extents_not_multiple_of_4(gpu_lib):
    gpu_lib.init(12, 12, 12)
    gpu_lib.learn_reset(0, seed=1)
    with pytest.raises(cappgpu.CappError):
        gpu_lib.learn_check(np.zeros((8, 9, 8), np.float32), np.zeros((7, 8, 9, 8), np.float32))


def test_trained_guess_lowers_the_initial_residual(gpu_lib):
    case = cappgpu.cases.channel(N=(16, 16, 24))
    gpu_lib.load_case(case)
    gpu_lib.precision(1)
    try:
        gpu_lib.learn_reset(64, seed=3)
        gpu_lib.learn_collect(True)
        gpu_lib.piso_steps(12)                      # 24 pressure solves recorded
        gpu_lib.learn_collect(False)
        st = gpu_lib.learn_stats()
        assert st["samples"] == 24
        loss0 = gpu_lib.learn_train(1, block=16, lr=1e-3)
        loss = gpu_lib.learn_train(40, block=16, lr=1e-3)
        assert loss < loss0
        # the same step from the same state without and with the guess
        snap = {n: gpu_lib.get_field(n) for n in cappgpu.FIELD_NAMES}
        par = gpu_lib.get_params()
        r1 = gpu_lib.piso_steps(1)
        for n, a in snap.items():
            gpu_lib.set_field(n, a)
        gpu_lib.set_params(par)
        gpu_lib.precision(2)
        r2 = gpu_lib.piso_steps(1)
        st = gpu_lib.learn_stats()
    finally:
        gpu_lib.precision(0)
    assert r1.status == 0 and r2.status == 0
    # both of the step's pressure solves start from a guess with a lower FP64
    # residual; a guess that raises it would be discarded
    assert st["guesses"] == 2 and st["fallbacks"] == 0
    assert 0.0 < st["last_ratio"] < 1.0
    assert r2.resl / r2.res0 < case.params["sor"][IP - 1]
    print(f"learned guess: loss {loss0:.3f} -> {loss:.3f}, last residual ratio {st['last_ratio']:.3f}, "
          f"last solve {r2.iters} iterations vs {r1.iters} without")


def test_window_recording_and_training(gpu_lib):
    """The training set as the learned-guess configuration builds it: random
    block^3 windows of each recorded solve (per_solve of them), the store
    cycling at its room; training on the windows lowers the loss; window
    sizes that are not a multiple of 4 or exceed the interior are refused."""
    case = cappgpu.cases.channel(N=(16, 16, 24))
    gpu_lib.load_case(case)
    gpu_lib.precision(1)
    try:
        gpu_lib.learn_reset(20, seed=4)
        gpu_lib.learn_windows(8, 3)
        gpu_lib.learn_collect(True)
        gpu_lib.piso_steps(2)                      # 4 solves x 3 windows
        assert gpu_lib.learn_stats()["samples"] == 12
        gpu_lib.piso_steps(2)
        assert gpu_lib.learn_stats()["samples"] == 20
        gpu_lib.learn_collect(False)
        loss0 = gpu_lib.learn_train(1, block=8, lr=1e-3)
        loss = gpu_lib.learn_train(30, block=8, lr=1e-3)
        assert np.isfinite(loss) and loss < loss0
        for bad in (6, 20):
            with pytest.raises(cappgpu.CappError):
                gpu_lib.learn_windows(bad, 1)
    finally:
        gpu_lib.precision(0)


def test_guess_that_raises_the_residual_is_discarded(gpu_lib, oracle_mod):
    """A net whose output is the constant 1 (all weights zero, the last
    bias 1): the fitted guess is a level shift fi + alpha, and with the
    right-hand side a single spike the shift spreads residual over every
    cell, so the guess's FP64 L1 residual is about twice res0.  The guess
    must be discarded (one more fallback, no guess kept) and the solve must
    then be the precision-1 solve from the original start, bit for bit."""
    from helpers import diag_dominant_matrix, push
    st = oracle_mod.State(24, 20, 28)
    rng = np.random.default_rng(17)
    diag_dominant_matrix(st, rng, symmetric=True)
    ni, nj, nk = st.dims
    su = np.zeros(st.nijk)
    su[(12 - 1) * ni * nj + (9 - 1) * nj + (11 - 1)] = 1.0   # cell (i, j, k) = (9, 11, 12)
    st.set_field("su", su)
    st.set_field("p", np.zeros(st.nijk))
    st.params.update(dict(alfa=0.92, sor=[1e-8] * 10, nsw=[2000] * 10, ipr=3, jpr=3, kpr=3))
    push(gpu_lib, st)
    gpu_lib.learn_reset(1, seed=3)
    n = gpu_lib.learn_params().size
    w = np.zeros(n, np.float32)
    w[-1] = 1.0
    gpu_lib.learn_params(w)
    try:
        gpu_lib.precision(1)
        r1 = gpu_lib.pcgsip("p", IP)
        p1 = gpu_lib.get_field("p")
        gpu_lib.set_field("p", np.zeros(st.nijk))
        s0 = gpu_lib.learn_stats()
        gpu_lib.precision(2)
        r2 = gpu_lib.pcgsip("p", IP)
        p2 = gpu_lib.get_field("p")
        s1 = gpu_lib.learn_stats()
    finally:
        gpu_lib.precision(0)
    assert s1["fallbacks"] == s0["fallbacks"] + 1 and s1["guesses"] == s0["guesses"]
    assert s1["last_ratio"] > 1.5, s1
    assert r1.status == 0 and r2.status == 0
    assert r2.res0 == r1.res0 and r2.iters == r1.iters and r2.resl == r1.resl
    np.testing.assert_array_equal(p2, p1)
