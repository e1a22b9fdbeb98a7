"""CPU pins of the surrogate oracle (oracle/mlp_oracle.py).

The oracle's analytic gradient is checked against central finite differences, its BF16
rounding against torch's float32 -> bfloat16 conversion (round to nearest even), and its
scale-free flow-rule target against the Drucker-Prager plastic source in physical units.
"""
import numpy as np
import pytest

import mlp_oracle as mo


def random_tuples(rng, n):
    x = rng.uniform(-1.0, 1.0, (n, mo.NIN))
    t = rng.uniform(-1.0, 1.0, (n, mo.NOUT))
    return np.concatenate([x, t], axis=1)


def random_params(rng, scale=0.3):
    p = rng.uniform(-scale, scale, mo.NPARAM)
    # padding rows / columns are zero in the product
    off, k, n = mo.LAYERS[0]
    p[off + 14 * n:off + 16 * n] = 0.0
    off, k, n = mo.LAYERS[3]
    W = p[off:off + k * n].reshape(k, n)
    W[:, 4:] = 0.0
    p[off + k * n + 4:off + k * n + n] = 0.0
    return p


def test_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    p = random_params(rng)
    t = random_tuples(rng, 8)
    _, g = mo.loss_grad(p, t)
    idx = np.concatenate([rng.choice(mo.NPARAM, 60, replace=False),
                          [mo.B1, mo.B2 + 5, mo.B3 + 7, mo.B4, mo.B4 + 3]])
    h = 1e-6
    for i in idx:
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        fd = (mo.loss_grad(pp, t)[0] - mo.loss_grad(pm, t)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-7 + 1e-5 * abs(g[i]), (i, fd, g[i])


def test_bf16_rounding_matches_torch():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(1)
    v = np.concatenate([rng.normal(0, 3, 10000).astype(np.float32),
                        np.float32([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -9, -2.5, 0.0, 1e-30])])
    ref = torch.from_numpy(v).to(torch.bfloat16).to(torch.float32).numpy()
    np.testing.assert_array_equal(mo.bf16(v).astype(np.float32), ref)


def test_flow_rule_target_is_scale_free():
    rng = np.random.default_rng(2)
    for _ in range(200):
        s = rng.uniform(-2e5, 1e4, 4)
        gu = rng.normal(0, 1e-2, 4)
        tanfi = np.tan(np.radians(rng.uniform(20, 40)))
        young, poiss = rng.uniform(5e6, 5e7), rng.uniform(0.2, 0.35)
        x, scale = mo.features(s, gu, tanfi, 1e3, young, poiss, 1900.0)
        np.testing.assert_allclose(mo.dp_target(x)[0] * scale,
                                   mo.dp_source(s, gu, tanfi, young, poiss),
                                   rtol=1e-10, atol=1e-12 * scale)
