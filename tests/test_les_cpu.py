"""CPU checks of the closure oracle itself (finite differences, filter identities)."""
import numpy as np

from oracle import les_ref


def test_conv_gradients_by_finite_differences():
    rng = np.random.default_rng(0)
    n = (4, 4, 4)
    x = rng.standard_normal(n + (3,))
    W = rng.standard_normal((27, 2, 3))
    g = rng.standard_normal(n + (2,))

    def L(x, W):
        return np.sum(les_ref.conv3d(x, W) * g)
    gx = les_ref.conv3d_bwd_data(g, W)
    dW, db = les_ref.conv3d_bwd_weight(x, g)
    e = 1e-6
    for i in [(1, 2, 3, 1), (0, 0, 0, 2), (3, 3, 1, 0)]:
        xp = x.copy()
        xp[i] += e
        assert abs((L(xp, W) - L(x, W)) / e - gx[i]) < 1e-4
    for j in [(5, 1, 2), (0, 0, 0), (26, 1, 1)]:
        Wp = W.copy()
        Wp[j] += e
        assert abs((L(x, Wp) - L(x, W)) / e - dW[j]) < 1e-4
    assert np.allclose(db, g.reshape(-1, 2).sum(0))


def test_box_filter_identities():
    rng = np.random.default_rng(1)
    u = rng.standard_normal((3, 16, 16, 16))
    ub, tau = les_ref.box_filter(u, 4)
    assert np.allclose(ub.mean(axis=(1, 2, 3)), u.mean(axis=(1, 2, 3)))
    assert tau[..., :3].min() >= -1e-12  # diagonal of tau is a variance
    ub1, tau1 = les_ref.box_filter(np.ones_like(u), 4)
    assert np.allclose(tau1, 0)
