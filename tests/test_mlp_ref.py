"""The NumPy MLP restatement (the checker of the BF16 kernels) against
finite differences, in float64."""
import numpy as np

from oracle import mlp_ref


def test_mlp_ref_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    lay, npar = mlp_ref.layout(3, 16, 2, 2)
    p = rng.normal(0, 0.5, npar)
    x = rng.normal(size=(40, 3))
    t = rng.normal(size=(40, 2))
    loss, g = mlp_ref.loss_grad(p, lay, x, t, 2, bf16_ops=False)
    for k in rng.choice(npar, 60, replace=False):
        e = np.zeros(npar)
        e[k] = 1e-6
        lp, _ = mlp_ref.loss_grad(p + e, lay, x, t, 2, bf16_ops=False)
        lm, _ = mlp_ref.loss_grad(p - e, lay, x, t, 2, bf16_ops=False)
        fd = (lp - lm) / 2e-6
        assert abs(fd - g[k]) <= 1e-6 * max(1.0, abs(fd)), (k, fd, g[k])


def test_bf16_rounding():
    a = np.array([1.0, 1.00390625, 1.005859375, -3.0e-3, 65504.0], dtype=np.float32)
    r = mlp_ref.bf16(a)
    # 1 + 2^-8 is a tie between 1 and 1 + 2^-7: rounds to even (1.0)
    assert r[0] == 1.0 and r[1] == 1.0
    assert r[2] == np.float32(1.0078125)
    assert abs(r[3] - a[3]) <= abs(a[3]) * 2 ** -8
    assert r[4] == 65536.0
