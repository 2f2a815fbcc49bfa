"""The learned-guess network's CPU oracle: its hand-derived backward pass
against central finite differences (FP64, no rounding), its BF16 rounding,
and its parameter count against the library's."""
import numpy as np
import pytest

import guess_oracle as G


def test_bf16_round_to_nearest_even():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -9, -2.5, 3.0e-3, 0.0])
    r = G.bf16_round(x)
    assert r[0] == 1.0 and r[1] == 1.0          # tie -> even (1.0)
    assert r[2] == 1.0 + 2 ** -7                 # above the tie -> up
    assert r[3] == -2.5 and r[5] == 0.0
    assert abs(r[4] - 3.0e-3) / 3.0e-3 < 2 ** -8


def test_param_count_matches_library(lib):
    from baorec import _lib
    assert lib.baorec_guess_num_params() == G.num_params() == 431969


@pytest.mark.parametrize("seed,loss", [(0, "mse"), (1, "laplacian")])
def test_backward_matches_finite_differences(seed, loss):
    n = 8
    rng = np.random.default_rng(seed)
    p = G.init_params(seed, head_scale=0.3)
    feats = rng.normal(size=(n, n, n, 8))
    target = rng.normal(size=(n, n, n))
    _, _, grad = G.loss_and_grads(p, feats, target, n, bf16=False, loss=loss)
    lay, total = G.layout()
    # a few weights and the bias of every layer, and the head
    idx = []
    for (wo, shape, bo, nb) in lay:
        idx += list(rng.integers(wo, wo + int(np.prod(shape)), 3)) + [bo]
    eps = 1e-6
    for i in idx:
        pp, pm = p.copy(), p.copy()
        pp[i] += eps
        pm[i] -= eps
        lp = G.loss_and_grads(pp, feats, target, n, bf16=False, loss=loss)[0]
        lm = G.loss_and_grads(pm, feats, target, n, bf16=False, loss=loss)[0]
        fd = (lp - lm) / (2 * eps)
        assert abs(fd - grad[i]) <= 1e-5 * max(1e-3, abs(fd)) + 1e-9, (i, fd, grad[i])
