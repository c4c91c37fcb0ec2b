"""Self-consistency of the surrogate's float64 oracle (oracle/nn_oracle.py),
which the GPU gradient checks trust: the data gradient is the adjoint of the
convolution, the weight gradient and the loss gradient match finite
differences, and so do the whole network's parameter gradients."""
import numpy as np

import nn_oracle as NO


def test_dgrad_is_adjoint_of_forward():
    rng = np.random.default_rng(0)
    for dil in (1, 2, 3):
        x = rng.standard_normal((2, 5, 6, 7, 4))
        w = rng.standard_normal((27, 3, 4))
        dy = rng.standard_normal((2, 5, 6, 7, 3))
        lhs = np.sum(dy * NO.conv_fwd(x, w, None, dil))
        rhs = np.sum(NO.conv_dgrad(dy, w, dil) * x)
        assert abs(lhs - rhs) <= 1e-9 * max(1.0, abs(lhs))


def test_wgrad_matches_finite_differences():
    rng = np.random.default_rng(1)
    x = rng.standard_normal((1, 4, 5, 6, 2))
    w = rng.standard_normal((27, 2, 2))
    dy = rng.standard_normal((1, 4, 5, 6, 2))
    g = NO.conv_wgrad(x, dy, 2)
    eps = 1e-6
    for t, co, ci in ((0, 0, 0), (13, 1, 0), (26, 1, 1), (7, 0, 1)):
        wp, wm = w.copy(), w.copy()
        wp[t, co, ci] += eps
        wm[t, co, ci] -= eps
        num = (np.sum(dy * NO.conv_fwd(x, wp, None, 2)) - np.sum(dy * NO.conv_fwd(x, wm, None, 2))) / (2 * eps)
        assert abs(num - g[t, co, ci]) <= 1e-6 * max(1.0, abs(num))


def test_xent_gradient_matches_finite_differences():
    rng = np.random.default_rng(2)
    z = rng.standard_normal((3, 4, 5, 16))
    p = rng.dirichlet(np.ones(4), size=(3, 4, 5))
    wgt = (rng.random((3, 4, 5)) < 0.8).astype(np.float64)
    _, g = NO.xent(z, p, wgt, 4)
    eps = 1e-6
    for idx in ((0, 0, 0, 0), (1, 2, 3, 2), (2, 3, 1, 3)):
        zp, zm = z.copy(), z.copy()
        zp[idx] += eps
        zm[idx] -= eps
        num = (NO.xent(zp, p, wgt, 4)[0] - NO.xent(zm, p, wgt, 4)[0]) / (2 * eps)
        assert abs(num - g[idx]) <= 1e-6
    assert np.all(g[..., 4:] == 0)


def test_network_gradients_match_finite_differences():
    """Without the bf16 rounding (float64 weights/activations, rounding off)
    the network's parameter gradients are the loss derivatives."""
    rng = np.random.default_rng(3)
    shape = (1, 4, 5, 4)
    x = rng.uniform(0, 1, shape + (16,))
    dils = [1, 2]
    ws = [rng.standard_normal((27, 16, 16)) * 0.05 for _ in range(2 + 2 * len(dils))]
    bs = [rng.standard_normal(16) * 0.05 for _ in ws]
    p = rng.dirichlet(np.ones(3), size=shape)
    wgt = np.ones(shape)
    grads = lambda w_, b_: NO.network_grads(x, w_, b_, dils, p, wgt, 3, rounding=False)
    loss, _, dws, dbs = grads(ws, bs)
    eps = 1e-6
    for k, (t, co, ci) in ((0, (13, 2, 3)), (2, (4, 7, 1)), (len(ws) - 1, (26, 0, 5))):
        wp = [w.copy() for w in ws]
        wm = [w.copy() for w in ws]
        wp[k][t, co, ci] += eps
        wm[k][t, co, ci] -= eps
        num = (grads(wp, bs)[0] - grads(wm, bs)[0]) / (2 * eps)
        assert abs(num - dws[k][t, co, ci]) <= 1e-5 * max(1e-3, abs(num)), (k, num, dws[k][t, co, ci])
    bp = [b.copy() for b in bs]
    bm = [b.copy() for b in bs]
    bp[1][4] += eps
    bm[1][4] -= eps
    num = (grads(ws, bp)[0] - grads(ws, bm)[0]) / (2 * eps)
    assert abs(num - dbs[1][4]) <= 1e-5 * max(1e-3, abs(num))
