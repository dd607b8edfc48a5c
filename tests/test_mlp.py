"""The warm-start surrogate's network: the GPU kernels (forward, backward, Adam) against the
CPU restatement (tests/mlp_np.py), whose own gradients are checked by finite differences."""
import numpy as np
import pytest

from mlp_np import loss_and_grads, predict, round_bf16

WIDTHS = [12, 32, 32, 16]


def small_problem(seed=0, n=24):
    rng = np.random.default_rng(seed)
    x = rng.normal(size=(n, WIDTHS[0])).astype(np.float32)
    y = rng.normal(size=(n, WIDTHS[-1])).astype(np.float32)
    sizes = [a * b + b for a, b in zip(WIDTHS[:-1], WIDTHS[1:])]
    p = np.concatenate([np.concatenate([rng.normal(0, 1 / np.sqrt(a), a * b), rng.normal(0, 0.1, b)])
                        for a, b in zip(WIDTHS[:-1], WIDTHS[1:])]).astype(np.float32)
    assert len(p) == sum(sizes)
    return x, y, p


def test_restatement_gradients_match_finite_differences():
    x, y, p = small_problem()
    p = p.astype(np.float64)
    loss, g = loss_and_grads(p, WIDTHS, x.astype(np.float64), y.astype(np.float64), bf16=False)
    rng = np.random.default_rng(1)
    for i in rng.choice(len(p), size=40, replace=False):
        e = np.zeros_like(p)
        e[i] = 1e-6
        lp, _ = loss_and_grads(p + e, WIDTHS, x, y, bf16=False)
        lm, _ = loss_and_grads(p - e, WIDTHS, x, y, bf16=False)
        fd = (lp - lm) / 2e-6
        assert abs(fd - g[i]) <= 1e-6 + 1e-5 * abs(g[i]), (i, fd, g[i])


def test_bf16_rounding_is_round_to_nearest_even():
    v = np.array([1.0, 1.00390625, 1.005859375, -3.0e-3, 65504.0], dtype=np.float32)
    r = round_bf16(v)
    assert r[0] == 1.0 and r[1] == 1.0          # halfway between 1 and 1.0078125: the even one
    assert r[2] == 1.0078125                     # above halfway: up
    assert abs(r[3] + 3.0e-3) < 3.0e-3 * 2 ** -8
    assert r[4] == 65536.0


@pytest.mark.gpu
def test_gpu_gradients_match_restatement(gpu):
    from psim_gb300 import api
    x, y, p = small_problem(2, n=40)
    net = api.Mlp(WIDTHS, seed=3)
    net.params = p
    loss, g = net.gradients(x, y)
    want_loss, want = loss_and_grads(p.astype(np.float64), WIDTHS, x, y, bf16=True)
    assert abs(loss - want_loss) <= 1e-4 * want_loss
    err = np.linalg.norm(g - want) / np.linalg.norm(want)
    cos = float(g @ want / (np.linalg.norm(g) * np.linalg.norm(want)))
    assert err < 1e-2 and cos > 0.9999, (err, cos)
    # and the forward pass
    out = net.predict(x)
    ref = predict(p.astype(np.float64), WIDTHS, x, bf16=True)
    assert np.allclose(out, ref, rtol=1e-3, atol=1e-4)


@pytest.mark.gpu
def test_gpu_training_fits_a_smooth_map(gpu):
    """Adam on a smooth 12 -> 64 map: the loss falls by more than an order of magnitude and the
    fit generalises to new inputs."""
    from psim_gb300 import api
    rng = np.random.default_rng(4)
    A = rng.normal(size=(12, 64)) / np.sqrt(12)

    def target(x):
        return np.tanh(x @ A) + 0.1 * (x[:, :1] ** 2)

    x = rng.uniform(-1, 1, size=(1024, 12)).astype(np.float32)
    y = target(x).astype(np.float32)
    net = api.Mlp([12, 128, 128, 64], seed=5)
    loss0, _ = net.gradients(x, y)
    loss = net.train(x, y, batch=128, epochs=60, lr=1e-3, seed=6)
    assert loss < loss0 / 10, (loss0, loss)
    xt = rng.uniform(-1, 1, size=(256, 12)).astype(np.float32)
    test_mse = float(np.mean((net.predict(xt) - target(xt)) ** 2))
    assert test_mse < 3 * loss + 1e-3, (test_mse, loss)
