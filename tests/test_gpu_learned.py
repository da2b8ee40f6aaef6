"""The learned initial guess (precision mode 2): the library's forward and
backward kernels against the CPU oracle, and what a trained net gains."""
import numpy as np
import pytest

import cappgpu

pytestmark = pytest.mark.gpu
IP = 4


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


@pytest.mark.parametrize("dims", [(8, 9, 10), (20, 17, 18)])
def test_forward_and_gradients_match_cpu_oracle(gpu_lib, dims):
    torch = pytest.importorskip("torch")
    import learned_oracle as lo
    gpu_lib.init(12, 12, 12)
    gpu_lib.learn_reset(0, seed=11)
    rng = np.random.default_rng(5)
    p = (rng.standard_normal(lo.NPARAMS) * 0.15).astype(np.float32)
    gpu_lib.learn_params(p)
    x = rng.standard_normal(dims).astype(np.float32)
    t = rng.standard_normal(dims).astype(np.float32)
    out, grad, loss = gpu_lib.learn_check(x, t)
    loss_o, out_o, grad_o = lo.loss_and_grad(p, x, t)
    assert _rel(out, out_o) < 2e-2
    assert abs(loss - loss_o) <= 2e-2 * loss_o
    assert _rel(grad, grad_o) < 5e-2
    # every layer's weight gradient, not only the total
    o = 0
    for l in range(lo.LAYERS):
        sl = slice(o, o + lo.WCONV)
        assert _rel(grad[sl], grad_o[sl]) < 8e-2, l
        o += lo.WCONV + lo.C


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
    # at least one of the step's two pressure solves started from a guess
    # with a lower FP64 residual; a guess that raises it is discarded
    assert st["guesses"] >= 1 and st["guesses"] + st["fallbacks"] == 2
    assert r2.resl / r2.res0 < case.params["sor"][IP - 1]
    print(f"learned guess: kept {st['guesses']} of 2, last ratio {st['last_ratio']:.3f}, "
          f"last solve {r2.iters} iterations vs {r1.iters} without")
