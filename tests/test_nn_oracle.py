"""The CPU restatement of the learned correction's network (oracle/nn_oracle)
against central finite differences of its own loss, so that the GPU
gradient test compares against a pinned oracle."""
import numpy as np
import pytest

from oracle import nn_oracle as nn


@pytest.mark.parametrize("mode", [0, 1])
def test_oracle_gradient_matches_finite_differences(mode):
    nb = 8
    rng = np.random.default_rng(5)
    w = nn.init(3).astype(np.float64)
    feat = rng.standard_normal((2, 3, nb * nb))
    aux = nn.random_aux(rng, 2, nb).astype(np.float64)
    _, g = nn.loss_grad(w, feat, aux, nb, mode)
    idx = np.concatenate([rng.choice(np.arange(lo, hi), 6, replace=False) for lo, hi in
                          ((nn.OW1, nn.OB1), (nn.OB1, nn.OW2), (nn.OW2, nn.OB2), (nn.OB2, nn.OW3),
                           (nn.OW3, nn.OB3))] + [np.array([nn.OB3])])
    h = 1e-6
    for k in idx:
        wp, wm = w.copy(), w.copy()
        wp[k] += h
        wm[k] -= h
        fd = (nn.loss_grad(wp, feat, aux, nb, mode)[0] - nn.loss_grad(wm, feat, aux, nb, mode)[0]) / (2 * h)
        assert abs(fd - g[k]) <= 1e-6 * max(1.0, abs(g[k])), (k, fd, g[k])


def test_bf16_rounding_is_round_to_nearest_even():
    x = np.array([1.0, 1.00390625, 1.005859375, -3.0e-3, 65504.0], dtype=np.float32)
    r = nn.to_bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0078125
    assert abs(r[3] - (-3.0e-3)) <= 2 ** -8 * 3e-3 and r[4] == 65536.0
