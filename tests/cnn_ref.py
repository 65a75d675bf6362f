"""CPU reference of the learned stage's CNN (test infrastructure): forward, loss and
backward in float64, rounding to bfloat16 where the GPU kernels store bfloat16 (network
input, weights, hidden activations, head and hidden gradients).  exact=True skips every
rounding, for finite-difference checks of the reference itself."""
import numpy as np

from climage_gb300.gls import CNN_LAYERS

STRENGTH_WEIGHT = 0.1
SIGMA_SCALE = 64.0  # the network sees the sigma channel scaled by this


def cnn_split(params):
    """Flat parameters -> [(W (cout, 3, 3, cin), b)], float64 (no rounding of the values)."""
    out, o = [], 0
    p = np.asarray(params, np.float64)
    for cin, cout in CNN_LAYERS:
        W = p[o:o + cout * 9 * cin].reshape(cout, 3, 3, cin)
        o += cout * 9 * cin
        out.append((W, p[o:o + cout]))
        o += cout
    return out


def bf16(x):
    """Round to bfloat16 (nearest, ties to even), returned as float64."""
    f = np.ascontiguousarray(x, np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def conv3x3(x, W, b=None):
    """'same' 3x3 convolution with zero padding; x (n, h, w, cin), W (cout, 3, 3, cin)."""
    n, h, w, _ = x.shape
    xp = np.pad(x, ((0, 0), (1, 1), (1, 1), (0, 0)))
    out = np.zeros((n, h, w, W.shape[0]))
    for dy in range(3):
        for dx in range(3):
            out += xp[:, dy:dy + h, dx:dx + w, :] @ W[:, dy, dx, :].T
    if b is not None:
        out += b
    return out


def forward(params, inp, exact=False):
    """Returns (activations [input, a0..a3], head (n, h, w, 4))."""
    r = (lambda v: np.asarray(v, np.float64)) if exact else bf16
    layers = cnn_split(params)
    x = np.array(inp, np.float64)
    x[..., 3] = (np.asarray(inp, np.float32)[..., 3] * np.float32(SIGMA_SCALE)).astype(np.float64)
    acts = [r(x)]
    a = acts[0]
    for l, (W, b) in enumerate(layers):
        z = conv3x3(a, r(W), np.asarray(b, np.float64))
        if l == len(layers) - 1:
            return acts, z
        a = r(np.maximum(z, 0.0))
        acts.append(a)


def corrected(inp, head):
    """The network's RGB output applied: input RGB + sigma * residual."""
    x = np.asarray(inp, np.float64)
    return x[..., :3] + x[..., 3:4] * head[..., 1:4]


def strength_target(inp, head, gt):
    x = np.asarray(inp, np.float64)
    e = corrected(inp, head) - np.asarray(gt, np.float64)
    return 0.5 * np.minimum(1.0, np.mean(e * e, axis=-1) / np.maximum(x[..., 3] ** 2, 1e-8))


def loss_grad(inp, head, gt, exact=False, tgt=None):
    """Residual and strength losses (means) and the gradient at the head of
    l0 + STRENGTH_WEIGHT * l1, the strength target held fixed (given, or from this head)."""
    r = (lambda v: np.asarray(v, np.float64)) if exact else bf16
    x = np.asarray(inp, np.float64)
    e = corrected(inp, head) - np.asarray(gt, np.float64)
    npx = e.shape[0] * e.shape[1] * e.shape[2]
    if tgt is None:
        tgt = strength_target(inp, head, gt)
    s = 1.0 / (1.0 + np.exp(-head[..., 0]))
    l0 = float(np.sum(e * e) / (3 * npx))
    l1 = float(np.sum((s - tgt) ** 2) / npx)
    d = np.zeros(head.shape)
    d[..., 1:4] = 2.0 * e * x[..., 3:4] / (3 * npx)
    d[..., 0] = STRENGTH_WEIGHT * 2.0 * (s - tgt) * s * (1 - s) / npx
    return l0, l1, r(d)


def backward(params, acts, dhead, exact=False):
    """Flat gradient of the parameters (same layout as the parameters)."""
    r = (lambda v: np.asarray(v, np.float64)) if exact else bf16
    layers = cnn_split(params)
    grads = [None] * len(layers)
    dz = dhead
    for l in range(len(layers) - 1, -1, -1):
        W = r(layers[l][0])
        a = acts[l]
        n, h, w, _ = a.shape
        ap = np.pad(a, ((0, 0), (1, 1), (1, 1), (0, 0)))
        dW = np.zeros(W.shape)
        for dy in range(3):
            for dx in range(3):
                dW[:, dy, dx, :] = np.einsum("nhwo,nhwi->oi", dz, ap[:, dy:dy + h, dx:dx + w, :])
        grads[l] = (dW, dz.sum(axis=(0, 1, 2)))
        if l > 0:
            Wt = W[:, ::-1, ::-1, :].transpose(3, 1, 2, 0)  # [cin][dy][dx][cout], taps flipped
            da = conv3x3(dz, Wt)
            dz = r(da * (acts[l] > 0))
    return np.concatenate([np.concatenate([g[0].ravel(), g[1].ravel()]) for g in grads])


def layer_slices():
    out, o = [], 0
    for cin, cout in CNN_LAYERS:
        out.append((o, o + cout * 9 * cin, o + cout * 9 * cin + cout))
        o += cout * 9 * cin + cout
    return out
