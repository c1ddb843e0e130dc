"""The calibration-step network on the tensor cores (csrc/wg_mlp.cu) against its
CPU restatement (oracle/mlp_oracle.py): forward outputs, the gradient of every
parameter, and a training run that fits a known function."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _net(seed=3):
    from watergap2_gb300.mlp import Mlp
    return Mlp(seed=seed)


def test_forward_matches_cpu_restatement():
    from oracle import mlp_oracle as mo
    net = _net()
    rng = np.random.default_rng(1)
    x = rng.normal(size=(300, 128)).astype(np.float32)   # 3 tiles, the last one partial
    y = net.forward(x)
    y_ref, _ = mo.forward(net.params(), x)
    scale = np.abs(y_ref).max()
    print(f"forward: max {np.abs(y - y_ref).max() / scale:.2e}, median {np.median(np.abs(y - y_ref)) / scale:.2e} "
          "of the output scale")
    # FP32 accumulation order differs, so a BF16 rounding of a hidden activation
    # can land one unit apart (measured on GB300: max 3.5e-5, median 3e-9 of the
    # output scale)
    assert np.abs(y - y_ref).max() <= 1e-3 * scale, (np.abs(y - y_ref).max(), scale)
    assert np.median(np.abs(y - y_ref)) <= 1e-6 * scale


def test_gradient_matches_cpu_restatement():
    from oracle import mlp_oracle as mo
    net = _net(seed=4)
    rng = np.random.default_rng(2)
    x = rng.normal(size=(256, 128)).astype(np.float32)
    t = rng.normal(size=(256, 2)).astype(np.float32)
    g, loss = net.gradient(x, t)
    g_ref, loss_ref = mo.gradient(net.params(), x, t)
    assert abs(loss - loss_ref) <= 1e-6 * loss_ref
    rel = np.linalg.norm(g - g_ref) / np.linalg.norm(g_ref)
    print(f"gradient: relative norm error {rel:.2e}, loss {abs(loss - loss_ref) / loss_ref:.2e}")
    assert rel <= 1e-4, rel   # measured on GB300: 3.4e-6
    # every layer's block agrees, biases included
    o = 0
    for n_out in (128, 128, 128, 16):
        for size in (n_out * 128, n_out):
            a, b = g[o:o + size], g_ref[o:o + size]
            assert np.linalg.norm(a - b) <= 1e-3 * np.linalg.norm(b) + 1e-9, o
            o += size


def test_training_fits_a_smooth_function():
    net = _net(seed=5)
    rng = np.random.default_rng(3)
    n = 8192
    x = rng.uniform(-1, 1, size=(n, 8)).astype(np.float32)
    t = np.stack([np.sin(2 * x[:, 0]) + x[:, 1] * x[:, 2], np.cos(x[:, 3]) - 0.5 * x[:, 4] ** 2], 1).astype(np.float32)
    y0 = net.forward(x)[:, :2]
    mse0 = float(((y0 - t) ** 2).mean())
    final = net.train(x, t, epochs=30, batch=512, lr=2e-3, seed=1)
    y1 = net.forward(x)[:, :2]
    mse1 = float(((y1 - t) ** 2).mean())
    assert mse1 < 0.05 * mse0, (mse0, mse1, final)
