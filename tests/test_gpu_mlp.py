"""BF16 tensor-core MLP kernels (nlm_mlp_*) against the NumPy restatement
with the same bf16 operand rounding (oracle/mlp_ref.py).

Tolerances: the kernels accumulate in FP32 where the restatement uses
float64, so a hidden activation can land on the other side of a bf16
rounding boundary (one bf16 ulp, 2^-8 relative); outputs are compared to
1e-2 of their scale and gradients to 2e-2 relative L2 per layer.
"""
import numpy as np
import pytest

from oracle import mlp_ref

pytestmark = pytest.mark.gpu


def _net(gpu, shape, seed=1):
    m = gpu.MLP(*shape, seed=seed)
    lay, npar = mlp_ref.layout(*shape)
    assert npar == m.nparams
    return m, lay


def test_mlp_padding_is_zero(gpu):
    m, lay = _net(gpu, (10, 128, 3, 2))
    p = m.params()
    di, do, wo, bo = lay[0]
    W0 = p[wo:wo + di * do].reshape(di, do)
    assert np.all(W0[10:] == 0)
    di, do, wo, bo = lay[-1]
    WL = p[wo:wo + di * do].reshape(di, do)
    assert np.all(WL[:, 2:] == 0)
    assert np.all(p[bo:bo + do] == 0)


@pytest.mark.parametrize("rows", [1, 37, 4096, 20000])
def test_mlp_forward_matches_restatement(gpu, rows):
    m, lay = _net(gpu, (10, 128, 3, 2))
    rng = np.random.default_rng(rows)
    p = m.params()
    p = p + (p != 0) * rng.normal(0, 0.02, p.size).astype(np.float32)
    di, do, wo, bo = lay[1]
    p[bo:bo + do] = rng.normal(0, 0.1, do)  # non-zero hidden biases
    m.set_params(p)
    x = rng.normal(size=(rows, 10)).astype(np.float32)
    y = m.forward(x)
    yr, _ = mlp_ref.forward(p, lay, x, 2)
    scale = max(np.abs(yr).max(), 1e-3)
    assert np.abs(y - yr).max() <= 1e-2 * scale


@pytest.mark.parametrize("shape", [(10, 128, 3, 2), (5, 48, 2, 3)])
def test_mlp_gradient_matches_restatement(gpu, shape):
    m, lay = _net(gpu, shape, seed=3)
    rng = np.random.default_rng(7)
    rows = 3000
    x = rng.normal(size=(rows, shape[0])).astype(np.float32)
    t = rng.normal(size=(rows, shape[3])).astype(np.float32)
    loss, g = m.grad(x, t)
    p = m.params()
    lr, gr = mlp_ref.loss_grad(p, lay, x, t, shape[3])
    assert abs(loss - lr) <= 1e-3 * abs(lr)
    for di, do, wo, bo in lay:
        for a, b in ((wo, wo + di * do), (bo, bo + do)):
            ref = gr[a:b]
            err = np.linalg.norm(g[a:b] - ref)
            assert err <= 2e-2 * max(np.linalg.norm(ref), 1e-6), (a, b, err, np.linalg.norm(ref))


def test_mlp_training_reduces_loss(gpu):
    m, lay = _net(gpu, (10, 128, 3, 2), seed=5)
    rng = np.random.default_rng(11)
    x = rng.uniform(-1, 1, size=(60000, 10)).astype(np.float32)
    t = np.stack([np.sin(2 * x[:, 0]) + x[:, 1] * x[:, 2], np.abs(x[:, 3]) - x[:, 4] ** 2],
                 axis=1).astype(np.float32)
    m.set_data(x, t)
    l0 = m.grad(x[:8192], t[:8192])[0]
    losses = m.train(20, batch=1024, lr=2e-3, seed=1)
    l1 = m.grad(x[:8192], t[:8192])[0]
    assert np.all(np.isfinite(losses))
    assert l1 < 0.05 * l0, (l0, l1, losses)
    # padding stays zero under training
    p = m.params()
    di, do, wo, bo = lay[0]
    assert np.all(p[wo:wo + di * do].reshape(di, do)[10:] == 0)
