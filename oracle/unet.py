"""CPU restatement of the learned denoiser (test infrastructure only: the
checker for libvpt's tcgen05 U-Net kernels, never part of the product path).

The reference (swr06/VoxelPathTracer) has no learned denoiser; the network is
this build's (a 3-level U-Net, 32/64/96 channels, 3x3 convolutions, ReLU,
nearest upsampling with skip concatenation, 2x2 average pooling) and this file
restates exactly what libvpt computes, in numpy:

  * `forward` / `backward` in float64 with optional BF16 rounding at the same
    points as the GPU (every stored activation and gradient, the weights),
    so GPU results can be compared within BF16 tolerance;
  * `numeric_grad` central finite differences of the float64 loss, which
    pins `backward` itself (parity of the gradient formulas, not of rounding).

Tensors are NHWC. Parameters are one flat vector laid out as libvpt's
vpt_unet_layer_info describes: per layer weights [Np][9][Cin] (tap =
(dy+1)*3 + (dx+1)) then bias [Np].
"""
from __future__ import annotations

import numpy as np

# (cin, cout, cin_real, cout_real, relu), the order of vpt_unet_layer_info
LAYERS = [(16, 32, 11, 32, 1), (32, 32, 32, 32, 1), (32, 64, 32, 64, 1), (64, 64, 64, 64, 1),
          (64, 96, 64, 96, 1), (96, 96, 96, 96, 1), (160, 64, 160, 64, 1), (64, 64, 64, 64, 1),
          (96, 32, 96, 32, 1), (32, 32, 32, 32, 1), (32, 16, 32, 3, 0)]


def offsets():
    off, o = [], 0
    for cin, cout, *_ in LAYERS:
        off.append(o)
        o += cout * 9 * cin + cout
    return off, o


def unpack(params):
    off, _ = offsets()
    out = []
    for (cin, cout, *_), o in zip(LAYERS, off):
        w = params[o:o + cout * 9 * cin].reshape(cout, 9, cin)
        b = params[o + cout * 9 * cin:o + cout * 9 * cin + cout]
        out.append((w, b))
    return out


def init_params(seed=0):
    """He-normal weights over the real fan-in, zero bias; padded channels zero."""
    rng = np.random.default_rng(seed)
    _, n = offsets()
    p = np.zeros(n, np.float32)
    for (w, _), (cin, cout, cin_r, cout_r, _relu) in zip(unpack(p), LAYERS):
        std = np.sqrt(2.0 / (9 * cin_r)) if _relu else np.sqrt(1.0 / (9 * cin_r))
        w[:cout_r, :, :cin_r] = rng.normal(0.0, std, (cout_r, 9, cin_r)).astype(np.float32)
    return p


def bf16(x, on=True):
    """Round to BF16 (nearest even), returned as float64; identity when off."""
    if not on:
        return np.asarray(x, np.float64)
    f = np.ascontiguousarray(x, np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def _shift(x, dy, dx):
    """x[n, y+dy, x+dx, c], zero outside."""
    N, H, W, C = x.shape
    out = np.zeros_like(x)
    ys, yd = (slice(dy, H), slice(0, H - dy)) if dy >= 0 else (slice(0, H + dy), slice(-dy, H))
    xs, xd = (slice(dx, W), slice(0, W - dx)) if dx >= 0 else (slice(0, W + dx), slice(-dx, W))
    out[:, yd, xd, :] = x[:, ys, xs, :]
    return out


def conv(x, w, b=None):
    """3x3 'same' convolution: y[p, co] = sum_tap,ci x[p+tap, ci] w[co, tap, ci] (+ b)."""
    N, H, W, _ = x.shape
    y = np.zeros((N, H, W, w.shape[0]))
    for tap in range(9):
        dy, dx = tap // 3 - 1, tap % 3 - 1
        y += np.einsum("nhwc,oc->nhwo", _shift(x, dy, dx), w[:, tap, :], optimize=True)
    if b is not None:
        y += b
    return y


def conv_bwd_data(g, w):
    """Gradient of conv's input: dx[p, ci] = sum_tap,co g[p-tap, co] w[co, tap, ci]."""
    N, H, W, _ = g.shape
    dx = np.zeros((N, H, W, w.shape[2]))
    for tap in range(9):
        dy_, dx_ = tap // 3 - 1, tap % 3 - 1
        dx += np.einsum("nhwo,oc->nhwc", _shift(g, -dy_, -dx_), w[:, tap, :], optimize=True)
    return dx


def conv_bwd_weight(x, g):
    """dW[co, tap, ci] = sum_p g[p, co] x[p+tap, ci]; db[co] = sum_p g[p, co]."""
    co, ci = g.shape[3], x.shape[3]
    dw = np.zeros((co, 9, ci))
    for tap in range(9):
        dy, dx = tap // 3 - 1, tap % 3 - 1
        dw[:, tap, :] = np.einsum("nhwo,nhwc->oc", g, _shift(x, dy, dx), optimize=True)
    return dw, g.sum(axis=(0, 1, 2))


def pool(x):
    return 0.25 * (x[:, 0::2, 0::2] + x[:, 0::2, 1::2] + x[:, 1::2, 0::2] + x[:, 1::2, 1::2])


def up(x):
    return x.repeat(2, axis=1).repeat(2, axis=2)


def upsum(g):
    return g[:, 0::2, 0::2] + g[:, 0::2, 1::2] + g[:, 1::2, 0::2] + g[:, 1::2, 1::2]


def forward(params, x, rounding=True):
    """Returns (out [N,H,W,16] float64, activations dict)."""
    r = lambda t: bf16(t, rounding)  # noqa: E731
    P = np.asarray(params, np.float32 if rounding else np.float64)
    L = [(r(w), np.asarray(b, np.float64)) for w, b in unpack(P)]
    relu = lambda t: np.maximum(t, 0.0)  # noqa: E731
    a = {"x": r(x)}
    a["e1a"] = r(relu(conv(a["x"], *L[0])))
    a["e1"] = r(relu(conv(a["e1a"], *L[1])))
    a["p1"] = r(pool(a["e1"]))
    a["e2a"] = r(relu(conv(a["p1"], *L[2])))
    a["e2"] = r(relu(conv(a["e2a"], *L[3])))
    a["p2"] = r(pool(a["e2"]))
    a["e3a"] = r(relu(conv(a["p2"], *L[4])))
    a["e3"] = r(relu(conv(a["e3a"], *L[5])))
    a["c2"] = np.concatenate([up(a["e3"]), a["e2"]], axis=3)
    a["d2a"] = r(relu(conv(a["c2"], *L[6])))
    a["d2"] = r(relu(conv(a["d2a"], *L[7])))
    a["c1"] = np.concatenate([up(a["d2"]), a["e1"]], axis=3)
    a["d1a"] = r(relu(conv(a["c1"], *L[8])))
    a["d1"] = r(relu(conv(a["d1a"], *L[9])))
    out = conv(a["d1"], *L[10])
    if rounding:
        out = out.astype(np.float32).astype(np.float64)
    return out, a


def loss(out, target):
    d = out[..., :3] - target
    return float(np.mean(d * d))


def backward(params, x, target, rounding=True):
    """Loss and the flat parameter gradient, in the GPU's order and rounding."""
    r = lambda t: bf16(t, rounding)  # noqa: E731
    L = [(r(w), b) for w, b in unpack(np.asarray(params, np.float32 if rounding else np.float64))]
    out, a = forward(params, x, rounding)
    N, H, W, _ = out.shape
    P = N * H * W
    g_out = np.zeros_like(out)
    g_out[..., :3] = 2.0 * (out[..., :3] - target) / (3 * P)
    g_out = r(g_out)
    grads = [None] * len(LAYERS)
    mask = lambda t, act: np.where(act > 0, t, 0.0)  # noqa: E731

    grads[10] = conv_bwd_weight(a["d1"], g_out)
    g = r(mask(conv_bwd_data(g_out, L[10][0]), a["d1"]))
    grads[9] = conv_bwd_weight(a["d1a"], g)
    g = r(mask(conv_bwd_data(g, L[9][0]), a["d1a"]))
    grads[8] = conv_bwd_weight(a["c1"], g)
    g_cat1 = r(conv_bwd_data(g, L[8][0]))
    g = r(mask(upsum(g_cat1[..., :64]), a["d2"]))
    grads[7] = conv_bwd_weight(a["d2a"], g)
    g = r(mask(conv_bwd_data(g, L[7][0]), a["d2a"]))
    grads[6] = conv_bwd_weight(a["c2"], g)
    g_cat2 = r(conv_bwd_data(g, L[6][0]))
    g = r(mask(upsum(g_cat2[..., :96]), a["e3"]))
    grads[5] = conv_bwd_weight(a["e3a"], g)
    g = r(mask(conv_bwd_data(g, L[5][0]), a["e3a"]))
    grads[4] = conv_bwd_weight(a["p2"], g)
    g_p2 = r(conv_bwd_data(g, L[4][0]))
    g = r(mask(g_cat2[..., 96:] + 0.25 * up(g_p2), a["e2"]))
    grads[3] = conv_bwd_weight(a["e2a"], g)
    g = r(mask(conv_bwd_data(g, L[3][0]), a["e2a"]))
    grads[2] = conv_bwd_weight(a["p1"], g)
    g_p1 = r(conv_bwd_data(g, L[2][0]))
    g = r(mask(g_cat1[..., 64:] + 0.25 * up(g_p1), a["e1"]))
    grads[1] = conv_bwd_weight(a["e1a"], g)
    g = r(mask(conv_bwd_data(g, L[1][0]), a["e1a"]))
    grads[0] = conv_bwd_weight(a["x"], g)

    flat = np.concatenate([np.concatenate([dw.ravel(), db.ravel()]) for dw, db in grads])
    return loss(out, target), flat


def numeric_grad(params, x, target, index, h=1e-4):
    """Central difference of the float64 (unrounded) loss in parameter `index`."""
    p = np.asarray(params, np.float64).copy()
    p[index] += h
    lp = loss(forward(p, x, rounding=False)[0], target)
    p[index] -= 2 * h
    lm = loss(forward(p, x, rounding=False)[0], target)
    return (lp - lm) / (2 * h)
