"""The U-Net oracle's backward pass against finite differences (CPU)."""
import numpy as np
import pytest

from oracle import unet as U


@pytest.mark.parametrize("chans", [(4, 8, 8, 16), (8, 8, 16, 16)])
def test_unet_oracle_gradients_match_finite_differences(chans):
    rng = np.random.default_rng(1)
    shapes = U.layer_shapes(3, chans, 2)
    params = {n: (rng.standard_normal((co, t, ci)) * np.sqrt(2 / (t * ci)), rng.standard_normal(co) * 0.1)
              for n, ci, co, t in shapes}
    x = rng.standard_normal((2, 16, 16, 3))
    tgt = rng.standard_normal((2, 16, 16, 2))
    loss, g, _ = U.loss_and_grads(params, x, tgt, chans)
    eps = 1e-6
    for name, ci, co, t in shapes:
        W, b = params[name]
        for _ in range(2):
            idx = tuple(int(rng.integers(0, s)) for s in W.shape)
            W2 = W.copy()
            W2[idx] += eps
            l2 = U.loss_and_grads({**params, name: (W2, b)}, x, tgt, chans)[0]
            assert (l2 - loss) / eps == pytest.approx(g[name][0][idx], rel=1e-3, abs=1e-7), name
        b2 = b.copy()
        b2[0] += eps
        l3 = U.loss_and_grads({**params, name: (W, b2)}, x, tgt, chans)[0]
        assert (l3 - loss) / eps == pytest.approx(g[name][1][0], rel=1e-3, abs=1e-7), name


def test_conv_adjoints():
    """<conv(x), y> = <x, dgrad(y)> and <conv(x), y> = <W, wgrad(x, y)>."""
    rng = np.random.default_rng(2)
    x = rng.standard_normal((2, 9, 7, 5))
    w = rng.standard_normal((6, 9, 5))
    y = rng.standard_normal((2, 9, 7, 6))
    lhs = np.sum(U.conv(x, w) * y)
    assert np.sum(x * U.conv_dgrad(y, w)) == pytest.approx(lhs, rel=1e-12)
    assert np.sum(w * U.conv_wgrad(x, y)) == pytest.approx(lhs, rel=1e-12)
