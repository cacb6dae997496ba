"""CPU pin of the U-Net oracle (oracle/unet_ref.py): its analytic gradient
against central finite differences, and its parameter count against the
library's."""
import numpy as np

from oracle import unet_ref as U


def random_params(rng):
    p = np.zeros(U.num_params())
    off = U.offsets()
    p[:off[0]] = rng.normal(0, np.sqrt(2 / 9), off[0])
    for k, (a, b, c) in enumerate(U.LAYERS):
        p[off[k]:off[k + 1]] = rng.normal(0, np.sqrt(2 / (9 * (a + b))), off[k + 1] - off[k])
    p[off[-1]:] = rng.normal(0, np.sqrt(1 / 32), 32)
    return p


def test_parameter_count_matches_library():
    from carpio_gb300 import unet
    assert unet.num_params() == U.num_params() == 1944896


import pytest


@pytest.mark.parametrize("loss", ["mse", "energy"])
def test_oracle_gradient_matches_finite_differences(loss):
    rng = np.random.default_rng(0)
    p = random_params(rng)
    x = rng.normal(size=(2, 16, 16))
    t = rng.normal(size=(2, 16, 16))
    value, g = U.loss_and_grad(p, x, t, loss=loss)
    off = U.offsets()
    # a few parameters of every layer with a non-negligible gradient
    picks = []
    bounds = [0] + off + [U.num_params()]
    for a, b in zip(bounds[:-1], bounds[1:]):
        seg = np.arange(a, b)
        big = seg[np.abs(g[seg]) > 1e-4 * np.abs(g).max()]
        if big.size:
            picks += list(rng.choice(big, size=min(3, big.size), replace=False))
    assert len(picks) >= 30
    eps = 1e-6
    for i in picks:
        pp, pm = p.copy(), p.copy()
        pp[i] += eps
        pm[i] -= eps
        fd = (U.loss_and_grad(pp, x, t, loss=loss)[0]
              - U.loss_and_grad(pm, x, t, loss=loss)[0]) / (2 * eps)
        assert abs(fd - g[i]) <= 1e-5 * abs(g[i]) + 1e-9, (i, fd, g[i])


def test_bf16_rounding_is_round_to_nearest_even():
    v = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 2 ** -7 + 2 ** -8, -3.14159, 0.0])
    r = U.bf16_round(v)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0 + 2 ** -6
    assert abs(r[3] - -3.140625) < 1e-12 and r[4] == 0.0
