"""The learned block correction of the device solve, on the GPU through the
C ABI: the FP32 training gradient and the BF16 tensor-core forward against
the CPU restatement (oracle/nn_oracle.py, pinned by finite differences),
training on the plain solver's own pairs, the gain of the trained network on a
held-out problem, the correction inside the solve, and the fallback to plain MG when the correction
stalls the solve."""
import numpy as np
import pytest

import sayakaamr_gb300 as sg
from oracle import nn_oracle as nn

pytestmark = pytest.mark.gpu

GRAD_RTOL = 2e-3   # FP32 accumulation over 64..256 cells x 288 taps vs float64
BF16_RTOL = 2e-2   # BF16 hidden layer (8-bit mantissa) vs the oracle's BF16 emulation


def small_solver(nb):
    t = sg.AmrTree(2, nb, 2, 2, 64)
    t.init_uniform_root((1, 1, 1), (0, 0, 0), (1, 1, 0), (-20,) * 6, (0,) * 6)
    t.init_refine_to_min_level()
    return sg.MacSolver(t.tables())


@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("nb", [8, 16])
def test_training_gradient_matches_oracle(nb, mode):
    S = small_solver(nb)
    S.set_params(learned_loss=mode)
    rng = np.random.default_rng(nb)
    w = nn.init(nb)
    S.set_learned_weights(w)
    n = 3
    feat = rng.standard_normal((n, 3, nb * nb)).astype(np.float32)
    aux = nn.random_aux(rng, n, nb)
    loss, g = S.learned_loss_grad(feat, aux)
    lref, gref = nn.loss_grad(w, feat, aux, nb, mode)
    assert abs(loss - lref) <= GRAD_RTOL * abs(lref)
    scale = np.abs(gref).max()
    assert np.max(np.abs(g - gref)) <= GRAD_RTOL * scale, np.max(np.abs(g - gref)) / scale


@pytest.mark.parametrize("nb", [8, 16])
def test_tensor_core_forward_matches_oracle(nb):
    S = small_solver(nb)
    rng = np.random.default_rng(100 + nb)
    w = nn.init(7 + nb)
    S.set_learned_weights(w)
    feat = rng.standard_normal((5, 3, nb * nb)).astype(np.float32)
    y = S.learned_forward(feat)
    ref = nn.forward(w, feat, nb, bf16=True, project=False)
    scale = np.abs(ref).max()
    assert np.max(np.abs(y - ref)) <= BF16_RTOL * scale


def test_tcgen05_forward_matches_warp_mma():
    """16x16 blocks: the hidden layer as a tcgen05 implicit GEMM (tensor
    memory accumulator) and as mma.sync warp MMAs give the same network
    output up to the order of the FP32 sums"""
    S = small_solver(16)
    rng = np.random.default_rng(7)
    S.set_learned_weights(nn.init(31))
    feat = rng.standard_normal((6, 3, 256)).astype(np.float32)
    out = {}
    for tc in (1, 0):
        S.set_params(learned_tc05=tc)
        out[tc] = S.learned_forward(feat)
    scale = np.abs(out[0]).max()
    assert scale > 0
    assert np.max(np.abs(out[1] - out[0])) <= 1e-4 * scale, np.max(np.abs(out[1] - out[0])) / scale


@pytest.fixture(scope="module")
def trained_config2():
    from sayakaamr_gb300 import workloads
    prob = workloads.config2()
    S = workloads.make_solver(prob)
    S.set_params(tol_rel=1e-8, tol_abs=0.0, use_mg_precond=1, max_iter=500, precision=1, bottom=1)
    S.prepare()
    iters = S.learned_collect(200)
    first = S.learned_train(epochs=1, lr=1e-3, batch=256, seed=3)
    last = S.learned_train(epochs=9, lr=1e-3, batch=256, seed=4)
    return prob, S, iters, first, last


def test_training_lowers_the_loss_on_solver_pairs(trained_config2):
    """the block-local residual left after the correction falls with training"""
    prob, S, iters, first, last = trained_config2
    assert iters > 5
    assert last < 0.9 * first, (first, last)


def test_trained_network_gains_on_a_held_out_problem(trained_config2):
    """what the trained network gains over the method without it: on the
    V-cycle residuals of another problem of the same family (different
    seed: geometry, density ellipse and right-hand side), the block-local
    residual left by the trained correction against the one left with no
    correction (the network's output layer zeroed, u = 0)"""
    from sayakaamr_gb300 import workloads
    prob, S, iters, first, last = trained_config2
    p2 = workloads.config2(seed=12)
    S2 = workloads.make_solver(p2)
    S2.set_params(tol_rel=1e-8, tol_abs=0.0, use_mg_precond=1, max_iter=500, precision=1, bottom=1)
    S2.prepare()
    assert S2.learned_collect(200) > 5
    w = S.learned_weights()
    S2.set_learned_weights(w)
    trained = S2.learned_eval()
    w0 = w.copy()
    w0[nn.OW3:nn.OB3 + 1] = 0.0
    S2.set_learned_weights(w0)
    none = S2.learned_eval()
    print("held-out block-local residual: no correction %.4g, trained correction %.4g" % (none, trained))
    assert trained < 0.8 * none, (trained, none)


def test_learned_correction_in_the_solve(trained_config2):
    """the trained correction inside the FP32 V-cycle solve converges to
    1e-8, but does not save iterations: the block-local gain measured above
    does not carry over to BiCGSTAB, whose recurrences the changing
    correction perturbs.  When the residual does not halve within two
    iterations the device switches the correction off (status
    STALL_FALLBACK) and goes on with plain MG from a restarted search
    direction, which bounds the cost (measured on config2: 9 iterations
    plain, 16 with the correction)"""
    prob, S, iters, first, last = trained_config2
    res, st = {}, {}
    for on in (0, 1):
        S.set_rhs_compact(prob.rhs)
        S.set_zero_sol()
        S.set_params(learned=on)
        info = S.cg_solve()
        assert info["status"] in (sg.OK, sg.STALL_FALLBACK), info
        assert info["rnorm"] < 1e-8 * info["rnorm0"]
        res[on], st[on] = info["iterations"], info["status"]
    S.set_params(learned=0)
    print("iterations plain FP32 V-cycle %d, with the learned correction %d (status %d)" % (res[0], res[1], st[1]))
    assert st[0] == sg.OK
    assert res[1] <= 2 * res[0] + 2, res


def test_stalled_correction_falls_back_to_plain_mg(trained_config2):
    """a correction that stalls the solve (weights scaled up 50x) is switched
    off on the device; the solve still converges with plain MG and reports
    the fallback"""
    prob, S, iters, first, last = trained_config2
    good = S.learned_weights()
    bad = good.copy()
    bad[nn.OW3:nn.OB3 + 1] *= 50.0
    S.set_learned_weights(bad)
    try:
        S.set_rhs_compact(prob.rhs)
        S.set_zero_sol()
        S.set_params(learned=1)
        info = S.cg_solve()
        assert info["status"] in (sg.STALL_FALLBACK, sg.OK), info
        assert info["rnorm"] < 1e-8 * info["rnorm0"]
    finally:
        S.set_learned_weights(good)
