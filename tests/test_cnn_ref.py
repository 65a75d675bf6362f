"""The CPU reference of the learned stage's CNN checked against finite differences (exact
mode, float64), so the GPU's gradient checks rest on a verified reference."""
import numpy as np

from climage_gb300 import gls
from tests import cnn_ref


def test_backward_matches_finite_differences():
    rng = np.random.default_rng(1)
    params = gls.cnn_init(3).astype(np.float64)
    params += rng.normal(0, 0.02, params.size)  # non-zero biases and head
    inp = np.concatenate([rng.uniform(0, 1, (1, 6, 7, 3)), rng.uniform(0.02, 0.05, (1, 6, 7, 1))], axis=-1)
    gt = rng.uniform(0, 1, (1, 6, 7, 3))
    acts, head = cnn_ref.forward(params, inp, exact=True)
    tgt = cnn_ref.strength_target(inp, head, gt)
    _, _, dhead = cnn_ref.loss_grad(inp, head, gt, exact=True, tgt=tgt)
    g = cnn_ref.backward(params, acts, dhead, exact=True)

    def loss(p):
        _, hd = cnn_ref.forward(p, inp, exact=True)
        l0, l1, _ = cnn_ref.loss_grad(inp, hd, gt, exact=True, tgt=tgt)
        return l0 + cnn_ref.STRENGTH_WEIGHT * l1

    idx = np.concatenate([rng.choice(np.arange(a, c), 12, replace=False) for a, _, c in cnn_ref.layer_slices()])
    eps = 1e-6
    for i in idx:
        p1, p2 = params.copy(), params.copy()
        p1[i] += eps
        p2[i] -= eps
        fd = (loss(p1) - loss(p2)) / (2 * eps)
        assert abs(fd - g[i]) <= 1e-6 + 1e-4 * abs(fd), (i, fd, g[i])


def test_bf16_rounding():
    x = np.array([1.0, 1.00390625, 1.005859375, -3.14159, 0.0], np.float32)
    r = cnn_ref.bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0  # tie to even
    assert r[2] == 1.0078125
    assert abs(r[3] + 3.140625) < 1e-12
    assert r[4] == 0.0
