"""CPU checks of the learned preconditioner's oracle (oracle/convnet.py):
the backward formulas against central finite differences of the FP64 loss,
and the BF16 rounding helper.  The device network is compared with this
oracle in tests/test_gpu_learned.py."""
import numpy as np

import convnet as cn


def make_case(seed=0, b=2, P=7):
    rng = np.random.default_rng(seed)
    p = np.zeros(3 * cn.PL)
    for l in range(3):
        W = np.zeros((cn.TAPS, cn.CH, cn.CH))
        W[:, :cn.CIN[l], :cn.COUT[l]] = rng.standard_normal((cn.TAPS, cn.CIN[l], cn.COUT[l])) * 0.2
        p[l * cn.PL:l * cn.PL + cn.WL] = W.reshape(-1)
        p[l * cn.PL + cn.WL:l * cn.PL + cn.WL + cn.COUT[l]] = rng.standard_normal(cn.COUT[l]) * 0.1
    x = np.zeros((b, P, P, P, cn.CH))
    x[..., :3] = rng.standard_normal((b, P, P, P, 3))
    tgt = rng.standard_normal((b, P, P, P, 2))
    return p, x, tgt


def test_backward_matches_finite_differences():
    p, x, tgt = make_case()
    margin = 1
    loss, g = cn.loss_grad(p, x, tgt, margin, bf16_round=False)
    rng = np.random.default_rng(1)
    live = np.flatnonzero(g)
    for k in rng.choice(live, 24, replace=False):
        h = 1e-5
        pp, pm = p.copy(), p.copy()
        pp[k] += h
        pm[k] -= h
        fd = (cn.loss_grad(pp, x, tgt, margin, False)[0] - cn.loss_grad(pm, x, tgt, margin, False)[0]) / (2 * h)
        assert abs(fd - g[k]) <= 1e-6 * max(1.0, abs(g[k])) + 1e-9, (k, fd, g[k])


def test_padded_channels_have_no_gradient():
    p, x, tgt = make_case(2)
    _, g = cn.loss_grad(p, x, tgt, 1, bf16_round=False)
    for l in range(3):
        W = g[l * cn.PL:l * cn.PL + cn.WL].reshape(cn.TAPS, cn.CH, cn.CH)
        assert np.all(W[:, cn.CIN[l]:, :] == 0) and np.all(W[:, :, cn.COUT[l]:] == 0)


def test_bf16_rounding():
    v = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -9, -2.5, 3.14159], np.float32)
    r = cn.bf16(v)
    assert r[0] == 1.0 and r[1] == 1.0  # tie to even
    assert r[2] == 1.0 + 2 ** -7       # tie to even (odd neighbour)
    assert r[3] == -2.5
    assert abs(r[4] - 3.14159) < 2 ** -7 * 4
    assert np.array_equal(cn.from_bits(cn.bf16_bits(v)), r)
