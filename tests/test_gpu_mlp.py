"""Rank model kernels (ttg_mlp_*): gradients against the CPU reference,
training reduces the loss."""
import numpy as np
import pytest

from oracle import mlp_ref

pytestmark = pytest.mark.gpu


def test_mlp_forward_and_gradients_match_cpu(ttg):
    from tensor_train_gb300.mlp import RankModel
    F, H = 8, 128
    m = RankModel(F, H, seed=3)
    rng = np.random.default_rng(0)
    x = rng.standard_normal((1000, F)).astype(np.float32)
    t = rng.standard_normal(1000).astype(np.float32)
    p = m.params()
    y = m.forward(x)  # normaliser is identity before training
    yr = mlp_ref.forward(p, x, F, H)
    assert np.max(np.abs(y - yr)) <= 1e-4 * (1 + np.max(np.abs(yr)))
    g, loss = m.gradients(x, t)
    lr, gr = mlp_ref.loss_and_grad(p, x, t, F, H)
    assert abs(loss - lr) <= 1e-4 * (1 + lr)
    # FP32 GPU vs FP64 CPU: relative error of the whole gradient vector
    assert np.linalg.norm(g - gr) <= 1e-4 * np.linalg.norm(gr)


def test_mlp_training_reduces_loss(ttg):
    from tensor_train_gb300.mlp import RankModel
    F = 8
    rng = np.random.default_rng(1)
    x = rng.standard_normal((8192, F)).astype(np.float32)
    t = (np.sin(x[:, 0]) + 0.5 * x[:, 1] * x[:, 2]).astype(np.float32)
    m = RankModel(F, 128, seed=1)
    hist = m.train(x, t, epochs=40, lr=3e-3, batch=2048)
    assert hist[-1] < 0.1 * hist[0]
    assert m.kernel_launches() > 0
