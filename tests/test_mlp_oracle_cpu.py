"""CPU checks of the warm-start MLP oracle: its back-propagation against
central finite differences (float64 mode), the parameter count of the C ABI,
and BF16 rounding."""
import numpy as np

import mlp_oracle as mo


def test_parameter_count():
    assert mo.N_PARAMS == 34434
    from pd_gpu1_gb300._lib import lib

    assert lib().pd_mlp_num_params() == 34434


def test_bf16_rounding():
    v = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -9, -2.5, 3.0e-3], dtype=np.float32)
    r = mo.bf16(v)
    assert r[0] == 1.0 and r[1] == 1.0 + 2 ** -7 - 2 ** -7  # tie to even: 1 + 2^-8 -> 1
    assert r[2] == 1.0 + 2 ** -7  # 1 + 1.5 * 2^-8 -> up
    assert r[3] == -2.5
    assert abs(r[4] - 3.0e-3) <= 3.0e-3 * 2 ** -8


def test_oracle_gradient_finite_differences():
    rng = np.random.default_rng(3)
    p = mo.init_params(1).astype(np.float64)
    x = rng.standard_normal((9, 8))
    t = rng.standard_normal((9, 2))
    g, _ = mo.grad(p, x, t, bf=False)
    idx = np.concatenate([rng.choice(range(0, 1024), 6, replace=False),      # W1
                          rng.choice(range(1024, 1152), 3, replace=False),   # b1
                          rng.choice(range(1152, 17536), 6, replace=False),  # W2, b2
                          rng.choice(range(17536, 34176), 6, replace=False),  # W3, b3
                          rng.choice(range(34176, 34434), 5, replace=False)])  # W4, b4
    h = 1e-6
    for i in idx:
        q = p.copy()
        q[i] += h
        lp = mo.grad(q, x, t, bf=False)[1]
        q[i] -= 2 * h
        lm = mo.grad(q, x, t, bf=False)[1]
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(g[i])), (i, fd, g[i])
