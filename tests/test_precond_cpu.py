"""The FP64 oracle of the learned preconditioner's network: its analytic
weight gradients agree with central finite differences of its loss, so the
GPU training kernels can be checked against it."""
import numpy as np

from oracle import precond_oracle as PO


def test_oracle_gradients_match_finite_differences():
    rng = np.random.default_rng(0)
    x = rng.standard_normal((1, 1000, 3))
    e = rng.standard_normal((1, 512, 3))
    w = [0.1 * rng.standard_normal(s) for s in ((27, 3, 32), (27, 32, 32), (27, 32, 3))]
    _, g = PO.loss_grad(x, e, *w)
    h = 1e-6
    for layer in range(3):
        for _ in range(2):
            idx = tuple(int(rng.integers(0, n)) for n in w[layer].shape)
            wp = [a.copy() for a in w]
            wm = [a.copy() for a in w]
            wp[layer][idx] += h
            wm[layer][idx] -= h
            fd = (PO.loss_grad(x, e, *wp)[0] - PO.loss_grad(x, e, *wm)[0]) / (2 * h)
            assert abs(fd - g[layer][idx]) <= 1e-6 * max(1.0, abs(fd)), (layer, idx)


def test_oracle_identity_network_is_jacobi():
    # zero output layer: z = x, loss = mean (x - e)^2 over the owned corners
    rng = np.random.default_rng(1)
    x = rng.standard_normal((2, 1000, 3))
    e = rng.standard_normal((2, 512, 3))
    w = [rng.standard_normal((27, 3, 32)), rng.standard_normal((27, 32, 32)), np.zeros((27, 32, 3))]
    loss, _ = PO.loss_grad(x, e, *w)
    xo = PO.owned(x.reshape(2, 10, 10, 10, 3))
    assert np.isclose(loss, np.mean((xo - e) ** 2))
