"""GPU parity of the keypoint-credibility MLP against the FP64 oracle
(oracle/mlp.py): scores, loss and gradient (relative tolerance 1e-4 on the
gradient norm, FP32 accumulation vs FP64), one Adam step, and training
progress on a separable problem."""
import numpy as np
import pytest

from oracle import mlp as OM

pytestmark = pytest.mark.gpu


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda()


def _data(seed, n):
    rng = np.random.default_rng(seed)
    X = np.abs(rng.standard_normal((n, 352))).astype(np.float32)
    X /= np.linalg.norm(X, axis=1, keepdims=True)  # SHOT-like: non-negative, unit norm
    w = rng.standard_normal(352)
    y = ((X @ w) > np.median(X @ w)).astype(np.float32)
    return X, y


def test_mlp_scores_match_oracle(ctx, rtr):
    theta = OM.init_params(1)
    X, _ = _data(2, 3000)
    m = rtr.Mlp(ctx, theta)
    got = m.score(_dev(X)).cpu().numpy()
    ref = OM.score(theta, X)
    np.testing.assert_allclose(got, ref, rtol=1e-5, atol=1e-6)
    assert np.array_equal(m.params(), theta)


@pytest.mark.parametrize("n", [1, 257, 4096])
def test_mlp_gradient_matches_oracle(ctx, rtr, n):
    theta = OM.init_params(3)
    X, y = _data(4, n)
    m = rtr.Mlp(ctx, theta)
    loss, g = m.loss_grad(_dev(X), _dev(y))
    rl, rg = OM.loss_and_grad(theta, X, y)
    g = g.cpu().numpy().astype(np.float64)
    assert abs(float(loss.item()) - rl) <= 1e-5 * max(1.0, abs(rl))
    rel = np.linalg.norm(g - rg) / max(np.linalg.norm(rg), 1e-30)
    assert rel < 1e-4, rel
    # every block of the parameter vector, not only the large W1
    o = 0
    for name, shape in OM.SIZES:
        k = int(np.prod(shape))
        a, b = g[o:o + k], rg[o:o + k]
        assert np.linalg.norm(a - b) <= 1e-4 * np.linalg.norm(rg) + 1e-9, name
        o += k


def test_mlp_adam_step_matches_oracle(ctx, rtr):
    theta = OM.init_params(5)
    X, y = _data(6, 512)
    m = rtr.Mlp(ctx, theta)
    m.train_step(_dev(X), _dev(y), lr=1e-3)
    got = m.params().astype(np.float64)
    _, rg = OM.loss_and_grad(theta, X, y)
    ref, _, _ = OM.adam_step(theta, rg, np.zeros_like(rg), np.zeros_like(rg), 1, lr=1e-3)
    # the first Adam step moves each weight by ~lr * sign(g): compare the moves
    dg, dr = got - theta, ref - theta
    big = np.abs(rg) > 1e-4 * np.abs(rg).max()  # sign-stable coordinates
    np.testing.assert_allclose(dg[big], dr[big], rtol=1e-3, atol=1e-7)


def test_mlp_training_learns_a_separable_rule(ctx, rtr):
    X, y = _data(7, 8192)
    m = rtr.Mlp(ctx, seed=11)
    losses = m.train(_dev(X), _dev(y), batch=1024, epochs=8, lr=3e-3, seed=1)
    assert losses[-1] < 0.5 * losses[0], losses
    acc = ((m.score(_dev(X)).cpu().numpy() > 0.5) == (y > 0.5)).mean()
    assert acc > 0.9, acc
