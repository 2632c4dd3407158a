"""The surrogate's CPU restatement (oracle/mlp_oracle.py): its analytic
gradients agree with central finite differences (without BF16 rounding, where
the function is smooth), and its BF16 rounding is round-to-nearest-even."""
import numpy as np

from oracle import mlp_oracle as M


def _params(rng, scale=0.3):
    return (rng.normal(0, scale, M.N_PARAMS)).astype(np.float32)


def test_bf16_rounding():
    a = np.array([1.0, 1.00390625, 1.005859375, 3.0e-40, -2.5, 65504.0], np.float32)
    b = M.bf16(a)
    assert b[0] == 1.0 and b[1] == 1.0          # halfway -> even
    assert b[2] == np.float32(1.0078125)        # above halfway -> up
    assert b[4] == -2.5
    assert np.all(M.bf16_bits(a) == (M.bf16(a).view(np.uint32) >> 16))


def test_gradients_match_finite_differences():
    rng = np.random.default_rng(0)
    p = _params(rng).astype(np.float64)
    x = rng.normal(0, 0.5, (24, M.IN))
    t = rng.normal(0, 0.3, (24, 2))
    g, l0 = M.gradients(p, x, t, round_bf16=False)
    assert abs(l0 - M.loss(p, x, t, round_bf16=False)) < 1e-12
    idx = rng.choice(M.N_PARAMS, 40, replace=False)
    # the padded outputs 2..7 of the last layer have zero gradient
    for i in idx:
        e = np.zeros(M.N_PARAMS)
        e[i] = 1e-6
        fd = (M.loss(p + e, x, t, False) - M.loss(p - e, x, t, False)) / 2e-6
        assert abs(fd - g[i]) <= 1e-6 + 1e-5 * abs(fd), (i, fd, g[i])


def test_padding_outputs_get_no_gradient():
    rng = np.random.default_rng(1)
    p = _params(rng)
    g, _ = M.gradients(p, rng.normal(0, 0.5, (8, M.IN)), rng.normal(0, 0.3, (8, 2)))
    w1, b1, w2, b2, w3, b3 = M.unpack(g)
    assert np.all(w3[:, 2:] == 0) and np.all(b3[2:] == 0)
