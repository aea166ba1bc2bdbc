"""The float64 network oracle's backward against finite differences (no GPU)."""
import numpy as np

from oracle import kpcn


def test_oracle_gradients_match_finite_differences():
    rng = np.random.default_rng(0)
    n = sum(co * 9 * ci + co for _, ci, co in kpcn.LAYERS)
    params = np.zeros(n)
    off = 0
    for _, ci, co in kpcn.LAYERS:
        params[off:off + co * 9 * ci] = rng.normal(0, np.sqrt(2.0 / (9 * ci)), co * 9 * ci)
        off += co * 9 * ci
        params[off:off + co] = rng.normal(0, 0.05, co)
        off += co
    B, H, W = 1, 8, 8
    feat = rng.normal(0, 1, (B, H, W, 16))
    noisy = rng.uniform(0, 2, (B, H, W, 3))
    prev = rng.uniform(0, 2, (B, H, W, 3))
    target = rng.uniform(0, 2, (B, H, W, 3))
    loss, g, _ = kpcn.loss_and_grads(params, feat, noisy, prev, target)
    assert np.isfinite(loss) and g.shape == params.shape
    # central differences on parameters spread over every layer
    idx = rng.choice(n, 40, replace=False)
    eps = 1e-6
    worst = 0.0
    for i in idx:
        p1, p2 = params.copy(), params.copy()
        p1[i] += eps
        p2[i] -= eps
        fd = (kpcn.loss_and_grads(p1, feat, noisy, prev, target)[0] -
              kpcn.loss_and_grads(p2, feat, noisy, prev, target)[0]) / (2 * eps)
        worst = max(worst, abs(fd - g[i]) / (abs(g[i]) + 1e-7))
        assert abs(fd - g[i]) <= 1e-4 * abs(g[i]) + 1e-8, (i, fd, g[i])
