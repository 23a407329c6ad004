"""CPU checks of the screening oracle: the MLP restatement's gradient and the block filter rule."""
import numpy as np

from oracle import mlp
from oracle.rpa_oracle import screen_blocks, _filter_g


def _problem(seed=3, n=40):
    rng = np.random.default_rng(seed)
    params = rng.normal(0.0, 0.3, mlp.NPARAM)
    # feature means, feature scales, target mean and scale, margin
    norm = np.concatenate([[3.0, 0.0, -2.0, -3.0, -3.0, 3.2, 2.2, 0.5, 0.5], [2.0, 1.0, 1.0, 2.0, 2.0, 0.4, 0.3, 0.5, 0.5],
                           [-5.0, 2.0, 0.5]])
    assert norm.size == mlp.NNORM
    x = rng.normal(0.0, 1.0, (n, mlp.IN)) * norm[mlp.IN:2 * mlp.IN] + norm[:mlp.IN]
    y = rng.normal(-5.0, 2.0, n)
    return params, norm, x, y


def test_mlp_oracle_gradient_matches_finite_differences():
    params, norm, x, y = _problem()
    loss, grad = mlp.loss_grad(params, norm, x, y, round16=False)
    rng = np.random.default_rng(7)
    idx = np.concatenate([rng.choice(mlp.NPARAM - 1, 24, replace=False), [mlp.NPARAM - 1]])
    h = 1e-6
    for i in idx:
        pp, pm = params.copy(), params.copy()
        pp[i] += h
        pm[i] -= h
        fd = (mlp.loss_grad(pp, norm, x, y, round16=False)[0] - mlp.loss_grad(pm, norm, x, y, round16=False)[0]) / (2 * h)
        assert abs(fd - grad[i]) <= 1e-6 + 1e-5 * abs(fd), (i, fd, grad[i])
    assert loss > 0


def test_mlp_oracle_forward_consistent_with_loss():
    params, norm, x, y = _problem(5)
    pred = mlp.forward(params, norm, x)
    loss, _ = mlp.loss_grad(params, norm, x, y)
    tn = (y - norm[2 * mlp.IN]) / norm[2 * mlp.IN + 1]
    pn = (pred - norm[2 * mlp.IN]) / norm[2 * mlp.IN + 1]
    assert np.isclose(loss, np.mean((pn - tn) ** 2), rtol=1e-12)


def test_block_filter_keeps_max_norm_above_threshold():
    """LibRI's filter keeps a block whose max-norm exceeds the threshold (LRI.hpp:20-25)."""
    blocks = {(0, 0, (0, 0, 0)): np.array([[1e-3, -2e-3]]), (0, 1, (0, 0, 0)): np.array([[1e-4, -1e-4]]),
              (1, 1, (0, 0, 0)): np.array([[0.0]])}
    kept = screen_blocks(blocks, 1e-4)
    assert set(kept) == {(0, 0, (0, 0, 0))}
    assert set(_filter_g(blocks, 1e-4)) == {(0, 0, (0, 0, 0))}
    assert set(screen_blocks(blocks, 0.0)) == {(0, 0, (0, 0, 0)), (0, 1, (0, 0, 0))}
