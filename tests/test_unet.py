"""The learned denoiser's tcgen05 kernels against the numpy restatement
(oracle/unet.py), and that restatement against finite differences.

Tolerances: the GPU multiplies BF16 operands exactly and accumulates in FP32
(the oracle in float64) and rounds stored activations and gradients to BF16,
so single values may differ by one BF16 step (2^-8 relative) where the two
roundings fall on opposite sides; the checks bound relative L2 errors."""
import numpy as np
import pytest

from oracle import unet as U


def rel_l2(a, b):
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


def rand_input(rng, n, h, w):
    x = np.zeros((n, h, w, 16), np.float32)
    x[..., :11] = rng.normal(size=(n, h, w, 11))
    return x


# --------------------------------------------------------------- oracle --
def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(3)
    p = U.init_params(1).astype(np.float64)
    p[::7] += 0.01          # non-zero biases too
    x = rand_input(rng, 2, 8, 8)
    t = rng.normal(size=(2, 8, 8, 3))
    _, g = U.backward(p, x, t, rounding=False)
    off, n = U.offsets()
    picks = [off[k] + int(rng.integers(0, 9 * U.LAYERS[k][0] * U.LAYERS[k][3])) for k in range(len(off))]
    picks += [off[k] + U.LAYERS[k][1] * 9 * U.LAYERS[k][0] for k in (0, 5, 9)]   # a bias of three layers
    for i in picks:
        ng = U.numeric_grad(p, x, t, i, 1e-5)
        assert abs(g[i] - ng) <= 1e-6 * max(1.0, abs(ng)) + 1e-7 * abs(ng), (i, g[i], ng)


def test_oracle_bf16_rounding():
    v = np.array([1.0, 1.00390625, 1.005859375, -3.1415927, 65504.0], np.float32)
    r = U.bf16(v)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0078125   # ties to even, then up
    assert abs(r[3] + 3.140625) < 1e-9


# ------------------------------------------------------------------ GPU --
def bf16_tensor(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda().to(torch.bfloat16)


@pytest.mark.gpu
@pytest.mark.parametrize("cin,cout,h,w,relu", [(16, 32, 6, 40, 1), (32, 64, 5, 130, 1), (96, 32, 4, 257, 0),
                                               (64, 96, 3, 128, 1), (32, 16, 4, 20, 0)])
def test_conv_forward(vpt, gpu, cin, cout, h, w, relu):
    import torch
    rng = np.random.default_rng(cin + cout + w)
    n = 2
    x = U.bf16(rng.normal(size=(n, h, w, cin)))
    wt = U.bf16(rng.normal(size=(cout, 9, cin)) / np.sqrt(9 * cin))
    b = rng.normal(size=cout).astype(np.float32)
    ref = U.conv(x, wt, b)
    if relu:
        ref = np.maximum(ref, 0)
    xt, wtt, bt = bf16_tensor(torch, x), bf16_tensor(torch, wt), torch.from_numpy(b).cuda()
    out = torch.empty((n, h, w, cout), dtype=torch.bfloat16, device="cuda")
    o32 = torch.empty((n, h, w, cout), dtype=torch.float32, device="cuda")
    vpt.nn_conv3x3(xt, cin, None, 0, n, h, w, wtt, bt, cout, relu=relu, out=out, out_f32=o32)
    vpt.nn_status()
    got32 = o32.cpu().numpy()
    assert rel_l2(got32, ref) < 1e-5, rel_l2(got32, ref)
    assert np.array_equal(out.float().cpu().numpy(), U.bf16(got32))


@pytest.mark.gpu
@pytest.mark.parametrize("c0,c1,cout,h,w", [(64, 32, 32, 8, 136), (96, 64, 64, 6, 200), (96, 64, 64, 4, 48),
                                            (64, 64, 96, 4, 256)],
                         ids=["rows", "staged-split", "staged-assembled", "staged-split-wide"])
def test_conv_upsample_concat_and_mask(vpt, gpu, c0, c1, cout, h, w):
    """Channels [0, c0) nearest-upsampled from half size, [c0, c0 + c1) full
    size, masked output: through the row-resident kernel's two-source loads,
    the staged kernel's even / odd half boxes (rows of at least 128 pixels,
    one ragged tile) and its assembled fallback (narrower rows)."""
    import torch
    rng = np.random.default_rng(5 + c0 + w)
    n = 2
    cin = c0 + c1
    low = U.bf16(rng.normal(size=(n, h // 2, w // 2, c0)))
    skip = U.bf16(rng.normal(size=(n, h, w, c1)))
    wt = U.bf16(rng.normal(size=(cout, 9, cin)) / np.sqrt(9 * cin))
    mask = U.bf16(rng.normal(size=(n, h, w, cout)))
    ref = U.conv(np.concatenate([U.up(low), skip], axis=3), wt)
    ref = np.where(mask > 0, ref, 0.0)
    o32 = torch.empty((n, h, w, cout), dtype=torch.float32, device="cuda")
    vpt.nn_conv3x3(bf16_tensor(torch, low), c0, bf16_tensor(torch, skip), c1, n, h, w, bf16_tensor(torch, wt), None,
                   cout, mask=bf16_tensor(torch, mask), out_f32=o32, up0=True)
    vpt.nn_status()
    assert rel_l2(o32.cpu().numpy(), ref) < 1e-5


@pytest.mark.gpu
@pytest.mark.parametrize("cin,cout,up0", [(16, 32, False), (160, 64, True), (32, 16, False), (96, 96, False)])
def test_conv_weight_gradient(vpt, gpu, cin, cout, up0):
    import torch
    rng = np.random.default_rng(cin * 3 + cout)
    n, h, w = 2, 12, 72
    if up0:
        c0 = 96
        low = U.bf16(rng.normal(size=(n, h // 2, w // 2, c0)))
        skip = U.bf16(rng.normal(size=(n, h, w, cin - c0)))
        x = np.concatenate([U.up(low), skip], axis=3)
        srcs = (bf16_tensor(torch, low), c0, bf16_tensor(torch, skip), cin - c0)
    else:
        x = U.bf16(rng.normal(size=(n, h, w, cin)))
        srcs = (bf16_tensor(torch, x), cin, None, 0)
    g = U.bf16(rng.normal(size=(n, h, w, cout)))
    ref, _ = U.conv_bwd_weight(x, g)
    dw = torch.zeros((cout, 9, cin), dtype=torch.float32, device="cuda")
    vpt.nn_conv3x3_dw(srcs[0], srcs[1], srcs[2], srcs[3], n, h, w, bf16_tensor(torch, g), cout, dw, up0=up0)
    vpt.nn_status()
    assert rel_l2(dw.cpu().numpy(), ref) < 1e-5, rel_l2(dw.cpu().numpy(), ref)


@pytest.mark.gpu
def test_unet_forward_and_gradient_match_oracle(vpt, gpu):
    """The whole network: output and every layer's gradient against the oracle
    with the same BF16 rounding points."""
    import torch
    rng = np.random.default_rng(11)
    n, h, w = 2, 16, 24
    p = U.init_params(2)
    p += (rng.normal(size=p.size) * 1e-3 * (p != 0)).astype(np.float32)
    off, total = U.offsets()
    for k, (cin, cout, cin_r, cout_r, _r) in enumerate(U.LAYERS):   # small non-zero biases
        bias = p[off[k] + cout * 9 * cin: off[k] + cout * 9 * cin + cout]
        bias[:cout_r] = rng.normal(size=cout_r) * 0.02
    x = rand_input(rng, n, h, w)
    t = rng.normal(size=(n, h, w, 3)).astype(np.float32)
    ref_out, _ = U.forward(p, x)
    ref_loss, ref_g = U.backward(p, x, t)
    with vpt.UNet(n, h, w) as net:
        net.set_params(p)
        xt = bf16_tensor(torch, x)
        out = torch.empty((n, h, w, 16), dtype=torch.float32, device="cuda")
        net.forward(xt, out)
        net.synchronize()
        got = out.cpu().numpy()
        assert rel_l2(got[..., :3], ref_out[..., :3]) < 1e-2
        loss = net.backward(xt, torch.from_numpy(t).cuda())
        g = net.grads()
    assert abs(loss - ref_loss) <= 1e-2 * ref_loss
    for k, (cin, cout, cin_r, cout_r, _r) in enumerate(U.LAYERS):
        end = off[k + 1] if k + 1 < len(off) else total
        err = rel_l2(g[off[k]:end], ref_g[off[k]:end])
        assert err < 5e-2, f"layer {k}: relative gradient error {err}"


@pytest.mark.gpu
def test_unet_training_reduces_loss(vpt, gpu):
    """A few Adam steps on a fixed smoothing task lower the loss."""
    import torch
    rng = np.random.default_rng(4)
    n, h, w = 4, 32, 32
    clean = rng.random((n, h // 8, w // 8, 3)).repeat(8, 1).repeat(8, 2)
    noisy = clean + 0.3 * rng.normal(size=clean.shape)
    x = np.zeros((n, h, w, 16), np.float32)
    x[..., :3] = noisy
    with vpt.UNet(n, h, w) as net:
        net.set_params(U.init_params(0))
        xt = bf16_tensor(torch, x)
        tt = torch.from_numpy(clean.astype(np.float32)).cuda()
        losses = []
        for _ in range(60):
            losses.append(net.backward(xt, tt))
            net.adam(lr=2e-3)
        net.synchronize()
    assert losses[-1] < 0.5 * losses[0], losses[::10]
