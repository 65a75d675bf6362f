"""The learned stage's CNN on the GPU (tensor-core implicit-GEMM kernels, through the C ABI)
against the CPU reference (tests/cnn_ref.py, itself checked by finite differences):
forward output, the gradients of every layer, and training that lowers the loss.

Tolerances: the GPU accumulates in FP32 in its own order and rounds hidden activations
and gradients to bfloat16 where the reference does, so a value next to a bfloat16
rounding boundary can land one bfloat16 step away; the head output must agree within 1 %
of its range and every layer's gradient within 3 % (relative L2)."""
import numpy as np
import pytest

from climage_gb300 import gls
from tests import cnn_ref

pytestmark = pytest.mark.gpu


def batch(rng, n, h, w, sigma=0.03):
    """Smooth random images in [0.05, 0.95] (the clean target) and noisy inputs with their
    sigma map: (inp (n, h, w, 4), gt (n, h, w, 3))."""
    yy, xx = np.meshgrid(np.linspace(0, 1, h), np.linspace(0, 1, w), indexing="ij")
    gt = np.empty((n, h, w, 3), np.float32)
    for i in range(n):
        for c in range(3):
            a, b, d, f = rng.uniform(-1, 1, 4)
            gt[i, :, :, c] = 0.5 + 0.3 * np.sin(3 * a * xx + 3 * b * yy + f) * np.cos(4 * d * (xx - yy))
        k = rng.integers(1, 4)
        for _ in range(k):  # a sharp-edged block
            y0, x0 = rng.integers(0, h // 2), rng.integers(0, w // 2)
            gt[i, y0:y0 + h // 3, x0:x0 + w // 3, :] = rng.uniform(0.1, 0.9, 3)
    noisy = gt + rng.normal(0, sigma, gt.shape).astype(np.float32)
    inp = np.concatenate([noisy, np.full((n, h, w, 1), sigma, np.float32)], axis=-1)
    return inp.astype(np.float32), gt


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


@pytest.fixture
def cnn(ctx):
    c = gls.Cnn(ctx)
    yield c
    c.close()


@pytest.mark.parametrize("backend", [0, 1, 2], ids=["mma_sync", "tcgen05", "fused"])
def test_forward_matches_reference(cnn, backend):
    import torch
    cnn.set_backend(backend)
    rng = np.random.default_rng(5)
    params = gls.cnn_init(7) + rng.normal(0, 0.01, gls.lib().gls_cnn_param_count()).astype(np.float32)
    cnn.set_params(params)
    inp, _ = batch(rng, 2, 21, 37)
    out = torch.empty((2, 21, 37, 4), dtype=torch.float32, device="cuda")
    cnn.forward(torch.from_numpy(inp).cuda(), out)
    torch.cuda.synchronize()
    got = out.cpu().numpy()
    cnn.status()
    _, ref = cnn_ref.forward(params, inp)
    span = float(ref.max() - ref.min())
    assert np.max(np.abs(got - ref)) <= 0.01 * span, (np.max(np.abs(got - ref)), span)
    assert rel_l2(got, ref) < 3e-3


def test_backends_agree(cnn):
    """tcgen05 (per layer or all five layers fused in one kernel) and mma.sync accumulate the
    same products in FP32 in different orders: the hidden activations can differ by one
    bfloat16 step where a value sits on a rounding boundary, nothing more."""
    import torch
    rng = np.random.default_rng(11)
    cnn.set_params(gls.cnn_init(3, head_std=0.05))
    inp, _ = batch(rng, 3, 50, 70)
    x = torch.from_numpy(inp).cuda()
    outs = []
    for backend in (0, 1, 2):
        cnn.set_backend(backend)
        o = torch.empty_like(x)
        cnn.forward(x, o)
        torch.cuda.synchronize()
        outs.append(o.cpu().numpy())
    cnn.status()
    assert rel_l2(outs[1], outs[0]) < 2e-3, rel_l2(outs[1], outs[0])
    assert rel_l2(outs[2], outs[0]) < 2e-3, rel_l2(outs[2], outs[0])


@pytest.mark.parametrize("w,h,n", [(24, 24, 1), (1, 1, 1), (25, 47, 2), (200, 9, 1), (300, 230, 1)])
def test_fused_forward_sizes(cnn, w, h, n):
    """Tile edges, images smaller than a tile, several images: the fused kernel against the
    per-layer tcgen05 path."""
    import torch
    cnn.set_params(gls.cnn_init(4, head_std=0.05))
    rng = np.random.default_rng(w * 1000 + h)
    x = torch.from_numpy(rng.uniform(0, 1, (n, h, w, 4)).astype(np.float32)).cuda()
    outs = []
    for backend in (1, 2):
        cnn.set_backend(backend)
        o = torch.full_like(x, 123.0)
        cnn.forward(x, o)
        torch.cuda.synchronize()
        outs.append(o.cpu().numpy())
    cnn.status()
    assert np.all(np.isfinite(outs[1]))
    assert rel_l2(outs[1], outs[0]) < 2e-3, rel_l2(outs[1], outs[0])


def test_gradients_match_reference(cnn):
    import torch
    rng = np.random.default_rng(6)
    params = gls.cnn_init(8) + rng.normal(0, 0.01, gls.lib().gls_cnn_param_count()).astype(np.float32)
    cnn.set_params(params)
    inp, gt = batch(rng, 2, 24, 40)
    loss = cnn.train_step(torch.from_numpy(inp).cuda(), torch.from_numpy(gt).cuda(), 0.0)
    g = cnn.grads()
    assert np.array_equal(cnn.params(), params)  # lr = 0 leaves the parameters
    acts, head = cnn_ref.forward(params, inp)
    l0, l1, dhead = cnn_ref.loss_grad(inp, head, gt)
    ref = cnn_ref.backward(params, acts, dhead)
    assert abs(loss[0] - l0) <= 1e-3 * l0 and abs(loss[1] - l1) <= 1e-2 * max(l1, 1e-6)
    for l, (a, b, c) in enumerate(cnn_ref.layer_slices()):
        assert rel_l2(g[a:b], ref[a:b]) < 3e-2, ("weights", l, rel_l2(g[a:b], ref[a:b]))
        assert rel_l2(g[b:c], ref[b:c]) < 3e-2, ("biases", l, rel_l2(g[b:c], ref[b:c]))


def test_training_lowers_the_loss(cnn):
    import torch
    rng = np.random.default_rng(9)
    cnn.set_params(gls.cnn_init(1))
    vin, vgt = batch(rng, 4, 48, 48)
    vin_d, vgt_d = torch.from_numpy(vin).cuda(), torch.from_numpy(vgt).cuda()
    before = cnn.train_step(vin_d, vgt_d, 0.0)[0]
    for step in range(400):  # past the plateau of the zero-initialised head
        inp, gt = batch(rng, 8, 48, 48)
        cnn.train_step(torch.from_numpy(inp).cuda(), torch.from_numpy(gt).cuda(), 1e-3)
    after = cnn.train_step(vin_d, vgt_d, 0.0)[0]
    assert after < 0.7 * before, (before, after)


def test_bounded_wait_runs_out_and_reports(cnn):
    """A tensor-core wait that never completes: the kernels' bounded mbarrier wait, run on a
    barrier that nothing arrives at (no MMA committed, nothing in flight), gives up after
    its polls and flags the error; status() raises GLS_ERR_TIMEOUT once, and the network
    then runs and reports normally (the context stays usable)."""
    import torch
    cnn.wait_probe(1 << 10)
    with pytest.raises(gls.GlsError) as err:
        cnn.status()
    assert err.value.status == gls.GLS_ERR_TIMEOUT
    cnn.status()  # reported once
    rng = np.random.default_rng(13)
    inp, _ = batch(rng, 1, 40, 56)
    x = torch.from_numpy(inp).cuda()
    cnn.set_params(gls.cnn_init(3))
    first = cnn.forward(x, torch.empty_like(x)).cpu().numpy()
    cnn.status()
    again = cnn.forward(x, torch.empty_like(x)).cpu().numpy()
    cnn.status()
    np.testing.assert_array_equal(first, again)
    with pytest.raises(gls.GlsError) as bad:
        cnn.wait_probe(0)
    assert bad.value.status == gls.GLS_ERR_INVALID_ARGUMENT
