"""CPU checks of the learned-network oracle: its backward pass against
central differences of its own float64 forward."""

from __future__ import annotations

import numpy as np

from oracle import cnn_oracle as cnn


def test_backward_matches_central_differences():
    rng = np.random.default_rng(0)
    weights, biases, w6, b6 = cnn.init(1)
    x0 = rng.normal(0, 1, (2, 64, 64, 2))
    target = rng.normal(0, 1, (2, 6))
    acts, out = cnn.forward(x0, weights, biases, w6, b6, rounded=False)
    dws, dbs, dw6, db6 = cnn.backward(acts, out, target, weights, w6, rounded=False)

    def objective():
        return cnn.loss(cnn.forward(x0, weights, biases, w6, b6, rounded=False)[1], target)

    eps = 1e-6
    checks = [(weights[0], dws[0], (3, 5)), (weights[2], dws[2], (17, 100)), (weights[4], dws[4], (60, 1000)),
              (biases[1], dbs[1], (7,)), (w6, dw6, (2, 33)), (b6, db6, (4,))]
    for param, grad, index in checks:
        saved = param[index]
        param[index] = saved + eps
        up = objective()
        param[index] = saved - eps
        down = objective()
        param[index] = saved
        numeric = (up - down) / (2 * eps)
        assert abs(numeric - grad[index]) <= 1e-5 * max(1.0, abs(numeric)), (index, numeric, grad[index])


def test_bf16_rounding_is_nearest_even():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 2 ** -9, 1.0 + 3 * 2 ** -9, -3.14159], np.float32)
    r = cnn.bf16(x)
    assert r[0] == 1.0
    assert r[1] == 1.0  # exactly halfway between 1 and 1 + 2^-7: ties to the even mantissa
    assert r[2] == 1.0  # below halfway rounds down
    assert r[3] == 1.0 + 2 ** -7  # above halfway rounds up
    assert abs(r[4] + 3.140625) < 1e-9
