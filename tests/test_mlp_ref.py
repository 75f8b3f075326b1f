"""The FP64 CPU reference of the step-size MLP checked by finite differences
(CPU only); the GPU training kernel is checked against this reference in
tests/test_gpu_learned.py."""
import numpy as np

from oracle import mlp_ref


def test_reference_backprop_matches_finite_differences():
    rng = np.random.default_rng(0)
    p = rng.standard_normal(mlp_ref.NPARAM) * 0.2
    f = rng.standard_normal((40, 8))
    t = rng.standard_normal(40)
    mu, isg = np.zeros(8), np.ones(8)
    mlp_ref.EXACT = True
    try:
        g, _ = mlp_ref.loss_grad(p, f, t, mu, isg, 0.0, 1.0)
        eps = 1e-6
        idx = np.concatenate([rng.choice(range(0, 512), 6), rng.choice(range(512, 576), 4),
                              rng.choice(range(576, 4672), 8), rng.choice(range(4672, 4736), 4),
                              rng.choice(range(4736, 4800), 4), [4800]])
        for k in idx:
            pp, pm = p.copy(), p.copy()
            pp[k] += eps
            pm[k] -= eps
            lp = mlp_ref.loss_grad(pp, f, t, mu, isg, 0.0, 1.0)[1]
            lm = mlp_ref.loss_grad(pm, f, t, mu, isg, 0.0, 1.0)[1]
            fd = (lp - lm) / (2 * eps) / len(t)
            assert abs(fd - g[k]) <= 1e-6 * max(1.0, abs(fd)), (k, fd, g[k])
    finally:
        mlp_ref.EXACT = False


def test_bf16_rounding():
    x = np.array([1.0, 1.00390625, 1.001953125, -3.14159265, 65504.0], np.float32)
    r = mlp_ref.bf16(x)
    assert r[0] == 1.0
    assert r[1] == 1.0  # 1 + 2^-8 is a tie between 1 and 1 + 2^-7: rounds to even
    assert r[2] == 1.0
    assert r[3] == -3.140625
    # every result is exactly representable with an 8-bit significand
    m, _ = np.frexp(r)
    assert np.all(np.abs(m * 256 - np.round(m * 256)) < 1e-9)
