"""Training data, training and evaluation of the learned denoiser.

The network (vpt_unet, tcgen05 BF16 kernels) replaces the SVGF a-trous
iterations as the spatial denoiser: its input is the frame shaded from the
temporally accumulated 1-spp GI plus albedo, normal, depth and the SVGF
variance (vpt_learned_features), its target the same frame shaded from the
FP64 ground-truth GI (vpt_ground_truth, `spp` samples per pixel), both in
log(1 + RGB); the network predicts the correction target - input (a residual,
so an untrained network passes the noisy frame through). Pairs come from seeded worlds and random cameras rendered by
this tracer; every step of data generation, training and inference runs on
the GPU through libvpt. SVGF is the fallback (vpt_render_frame_learned
without a network) and the yardstick: `evaluate` reports the error of the
noisy input, of SVGF and of the network against the same ground truth.

    python -m voxelpathtracer_gb300.learned train --pairs 2000 --out weights.npz
    python -m voxelpathtracer_gb300.learned evaluate --weights weights.npz
"""
from __future__ import annotations

import argparse
import json
import pathlib
import time

import numpy as np

from . import (Context, UNet, camera_from_pose, default_frame, generate_block_table, generate_world, quality)

WEIGHTS = pathlib.Path(__file__).resolve().parent / "weights" / "unet_denoiser.npz"
# trained for the large combined configuration (512^3, 3840x2160, 2 bounces, FP16 planes, orbit camera)
WEIGHTS_LARGE = pathlib.Path(__file__).resolve().parent / "weights" / "unet_denoiser_large.npz"


def he_init(seed: int = 0) -> np.ndarray:
    """He-normal weights over each layer's real fan-in, zero biases and padding."""
    from . import unet_layers
    rng = np.random.default_rng(seed)
    layers = unet_layers()
    last = layers[-1]
    n = last[4] + last[1] * 9 * last[0] + last[1]
    p = np.zeros(n, np.float32)
    for k, (cin, cout, cin_r, cout_r, off) in enumerate(layers):
        w = p[off:off + cout * 9 * cin].reshape(cout, 9, cin)
        # the last layer starts small: the residual output begins near zero
        std = np.sqrt(2.0 / (9 * cin_r)) if k < len(layers) - 1 else 0.1 * np.sqrt(1.0 / (9 * cin_r))
        w[:cout_r, :, :cin_r] = rng.normal(0.0, std, (cout_r, 9, cin_r))
    return p


def random_pose(rng, dims):
    X, Y, Z = dims
    pos = (float(rng.uniform(0.25 * X, 0.75 * X)), float(min(Y - 3.0, 90.0)), float(rng.uniform(0.25 * Z, 0.75 * Z)))
    return pos, float(rng.uniform(0.0, 360.0)), float(rng.uniform(-40.0, -10.0))


def drift_camera(pos, yaw, pitch, k, aspect):
    """The camera k frames before the sampled one (a slow pan, as the bench moves)."""
    return camera_from_pose((pos[0] - 0.05 * k, pos[1], pos[2]), yaw - 0.25 * k, pitch, 90.0, aspect)


def orbit_camera(dims, theta_deg, aspect, radius=200.0, height=150.0, ground=40.0):
    """On a circle of `radius` at `height` around the world's centre column,
    looking at the terrain (near y = `ground`) below the centre."""
    X, Y, Z = dims
    th = np.radians(theta_deg)
    pos = (X / 2 + radius * np.cos(th), height, Z / 2 + radius * np.sin(th))
    yaw = float(np.degrees(np.arctan2(Z / 2 - pos[2], X / 2 - pos[0])))
    pitch = float(-np.degrees(np.arctan2(height - ground, radius)))
    return camera_from_pose(pos, yaw, pitch, 90.0, aspect)


def pan_sequence(rng, dims, W, H, history):
    """A random pan: (length, camera of frame k), ending at a random pose."""
    pos, yaw, pitch = random_pose(rng, dims)
    length = int(rng.integers(*history))
    return length, (lambda k: drift_camera(pos, yaw, pitch, length - 1 - k, W / H))


def orbit_sequence(rng, dims, W, H, history, deg_per_frame=1.0):
    """A stretch of the orbit at a random start angle: (length, camera of frame k)."""
    theta0 = float(rng.uniform(0.0, 360.0))
    length = int(rng.integers(*history))
    return length, (lambda k: orbit_camera(dims, theta0 + deg_per_frame * k, W / H))


def generate_pairs(n_pairs: int, crop=(256, 256), spp: int = 1024, n_worlds: int = 8, dims=(256, 256, 256),
                   frame_size=(1920, 1080), history=(1, 65), per_sequence: int = 4, seed: int = 0, device: int = 0,
                   log=None, bounces: int = 1, storage: int = 0, camera: str = "pan"):
    """(X [n, h, w, 16] bfloat16, T [n, h, w, 3] float32) on the GPU.

    Each camera sequence (a pan, or a stretch of the orbit) has a random
    length in `history` (frames of temporal accumulation); at up to
    `per_sequence` random frames of it a random crop is sampled: its features
    (vpt_learned_features) from a context with `storage` planes, and
    log(1 + colour) of the same frame shaded from the FP64 ground-truth GI."""
    import torch
    cw, ch = crop
    W, H = frame_size
    dev = f"cuda:{device}"
    X = torch.zeros((n_pairs, ch, cw, 16), dtype=torch.bfloat16, device=dev)
    T = torch.zeros((n_pairs, ch, cw, 3), dtype=torch.float32, device=dev)
    rng = np.random.default_rng(seed)
    per_world = -(-n_pairs // n_worlds)
    make_seq = orbit_sequence if camera == "orbit" else pan_sequence
    i = 0
    t0 = time.perf_counter()
    for wi in range(n_worlds):
        if i >= n_pairs:
            break
        wseed = 10_000 * (seed + 1) + wi
        vox = generate_world(*dims, seed=wseed)
        blocks = generate_block_table(100, seed=wseed)
        stop = min(n_pairs, i + per_world)
        ctx = Context(width=W, height=H, device=device, storage=storage, bounces=bounces)
        ctx.upload_world(vox)
        ctx.set_block_table(blocks)
        ctx.build_df()
        # the ground truth needs FP32 planes: a second context when the input is FP16
        gt = ctx if storage == 0 else quality.make_gt_context(W, H, vox, blocks, device=device, bounces=bounces)
        try:
            while i < stop:
                length, cam_at = make_seq(rng, dims, W, H, history)
                picks = set(int(v) for v in rng.choice(length, size=min(per_sequence, length), replace=False))
                fseed = int(rng.integers(0, 2**31))
                ctx.reset_history()
                for f in range(length):
                    cam = cam_at(f)
                    fr = default_frame(seed=fseed, frame_index=f, time=1.0 + f / 60.0)
                    if f in picks and i < stop:
                        ctx.learned_input(cam, fr)
                        x0 = int(rng.integers(0, W - cw + 1))
                        y0 = int(rng.integers(0, H - ch + 1))
                        ctx.learned_features((x0, y0, cw, ch), X[i])
                        if gt is not ctx:
                            ctx.end_frame()
                        rgb, _ = quality.ground_truth_color(gt, cam, fr, (x0, y0, cw, ch), spp=spp)   # ends gt's frame
                        T[i] = torch.from_numpy(np.log1p(np.maximum(rgb, 0.0)).astype(np.float32)).to(dev)
                        i += 1
                        if log and i % 100 == 0:
                            log(f"pairs {i}/{n_pairs} ({time.perf_counter() - t0:.1f} s)")
                    else:
                        ctx.render_frame(cam, fr, readback=False)
        finally:
            if gt is not ctx:
                gt.close()
            ctx.close()
    torch.cuda.synchronize()
    return X, T


def train(net: UNet, X, T, steps: int, batch: int = 8, lr: float = 1e-3, seed: int = 0, log=None,
          log_every: int = 100):
    """Adam on random mini-batches with random flips; returns the loss curve."""
    import torch
    g = torch.Generator(device="cpu").manual_seed(seed)
    n = X.shape[0]
    losses = []
    t0 = time.perf_counter()
    for s in range(steps):
        idx = torch.randint(0, n, (batch,), generator=g)
        xb, tb = X[idx], T[idx]
        if s % 2:   # horizontal flip; it mirrors the x component of the normal feature
            xb, tb = xb.flip(2).clone(), tb.flip(2)
            xb[..., 6] = -xb[..., 6]
        tb = (tb - xb[..., :3].float()).contiguous()    # the residual target
        xb = xb.contiguous()
        lr_s = lr * (0.5 * (1.0 + np.cos(np.pi * s / steps)) * 0.9 + 0.1)
        loss = net.backward(xb, tb)
        net.adam(lr=float(lr_s))
        losses.append(loss)
        if log and (s + 1) % log_every == 0:
            log(f"step {s + 1}/{steps}: loss {np.mean(losses[-log_every:]):.5f} ({time.perf_counter() - t0:.1f} s)")
    net.synchronize()
    return losses


def predict_crops(net: UNet, X, batch: int = 8):
    """Denoised log(1 + RGB) for every crop of X: the noisy input plus the network's correction."""
    import torch
    n, h, w, _ = X.shape
    out = torch.empty((n, h, w, 16), dtype=torch.float32, device=X.device)
    for s in range(0, n, batch):
        e = min(n, s + batch)
        net.forward(X[s:e].contiguous(), out[s:e])
    net.synchronize()
    return out[..., :3] + X[..., :3].float()


def crop_rmse(a_log, b_log) -> float:
    """RMSE in linear RGB between two log(1 + RGB) tensors."""
    import torch
    d = torch.expm1(a_log.double()) - torch.expm1(b_log.double())
    return float(torch.sqrt(torch.mean(d * d)))


def save(path, params: np.ndarray, meta: dict):
    path = pathlib.Path(path)
    path.parent.mkdir(parents=True, exist_ok=True)
    np.savez_compressed(path, params=params.astype(np.float32), meta=json.dumps(meta))


def load(path=WEIGHTS):
    d = np.load(path)
    return d["params"], json.loads(str(d["meta"]))


def evaluate_frame(net: UNet | None, vox, blocks, pos, yaw, pitch, frames: int, size=(1920, 1080),
                   crop=quality.DEFAULT_CROP_1080P, gt_spp: int = 4096, device: int = 0, storage: int = 0):
    """Render `frames` frames of a pan twice (SVGF path and learned path, two
    contexts with the same inputs) and score the last frame against the FP64
    ground truth on `crop`: RMSE of the noisy network input, of SVGF and of
    the network. Returns a dict of the three errors and whether the network ran."""
    W, H = size
    x0, y0, cw, ch = crop
    with Context(width=W, height=H, device=device, storage=storage) as a, \
            Context(width=W, height=H, device=device, storage=storage) as b:
        for c in (a, b):
            c.upload_world(vox)
            c.set_block_table(blocks)
            c.build_df()
        for k in range(frames - 1, 0, -1):
            fr = default_frame(seed=7, frame_index=frames - 1 - k, time=1.0 + (frames - 1 - k) / 60.0)
            cam = drift_camera(pos, yaw, pitch, k, W / H)
            a.render_frame(cam, fr, readback=False)
            b.render_frame_learned(cam, fr, net, readback=False)
        fr = default_frame(seed=7, frame_index=frames - 1, time=1.0 + (frames - 1) / 60.0)
        cam = drift_camera(pos, yaw, pitch, 0, W / H)
        learned, used = b.render_frame_learned(cam, fr, net)
        a.learned_input(cam, fr)
        noisy = a.read_plane("COLOR").astype(np.float64)
        a.svgf(None, fr)
        a.shade(fr)
        svgf = a.read_plane("COLOR").astype(np.float64)
        if storage == 0:
            gt, _ = quality.ground_truth_color(a, cam, fr, crop, spp=gt_spp)
        else:
            with quality.make_gt_context(W, H, vox, blocks, device=device) as g:
                gt, _ = quality.ground_truth_color(g, cam, fr, crop, spp=gt_spp)
    sl = (slice(y0, y0 + ch), slice(x0, x0 + cw))
    return {"rmse_noisy": quality.rmse(noisy[sl], gt), "rmse_svgf": quality.rmse(svgf[sl], gt),
            "rmse_learned": quality.rmse(learned.astype(np.float64)[sl], gt), "used_net": used}


def main():
    ap = argparse.ArgumentParser()
    sub = ap.add_subparsers(dest="cmd", required=True)
    t = sub.add_parser("train")
    t.add_argument("--pairs", type=int, default=2000)
    t.add_argument("--crop", type=int, default=256)
    t.add_argument("--spp", type=int, default=1024)
    t.add_argument("--worlds", type=int, default=10)
    t.add_argument("--steps", type=int, default=3000)
    t.add_argument("--batch", type=int, default=8)
    t.add_argument("--lr", type=float, default=1e-3)
    t.add_argument("--holdout", type=int, default=100)
    t.add_argument("--seed", type=int, default=0)
    t.add_argument("--out", default=None)
    t.add_argument("--profile", choices=["frame", "large"], default="frame",
                   help="frame: 256^3 worlds, 1920x1080 pans, 1 bounce, FP32 planes; large: 512^3 worlds, "
                        "3840x2160 orbits, 2 bounces, FP16 planes")
    e = sub.add_parser("evaluate")
    e.add_argument("--weights", default=str(WEIGHTS))
    e.add_argument("--world-seed", type=int, default=0)
    e.add_argument("--frames", type=int, default=16)
    e.add_argument("--gt-spp", type=int, default=4096)
    a = ap.parse_args()
    if a.cmd == "evaluate":
        params, meta = load(a.weights)
        vox = generate_world(256, 256, 256, seed=a.world_seed)
        blocks = generate_block_table(100, seed=a.world_seed)
        with UNet(1, 1080, 1920) as net:
            net.set_params(params)
            r = evaluate_frame(net, vox, blocks, (128.0, 90.0, 128.0), 229.3, -31.9, a.frames, gt_spp=a.gt_spp)
        print(json.dumps(r), flush=True)
        return
    import torch
    log = lambda m: print(m, flush=True)  # noqa: E731
    t0 = time.perf_counter()
    if a.profile == "large":
        gen = dict(dims=(512, 512, 512), frame_size=(3840, 2160), bounces=2, storage=1, camera="orbit")
        out = a.out or str(WEIGHTS_LARGE)
    else:
        gen = {}
        out = a.out or str(WEIGHTS)
    X, T = generate_pairs(a.pairs + a.holdout, crop=(a.crop, a.crop), spp=a.spp, n_worlds=a.worlds, seed=a.seed,
                          log=log, **gen)
    gen_s = time.perf_counter() - t0
    Xtr, Ttr, Xva, Tva = X[:a.pairs], T[:a.pairs], X[a.pairs:], T[a.pairs:]
    with UNet(a.batch, a.crop, a.crop) as net:
        net.set_params(he_init(a.seed))
        t1 = time.perf_counter()
        losses = train(net, Xtr, Ttr, a.steps, batch=a.batch, lr=a.lr, seed=a.seed, log=log)
        train_s = time.perf_counter() - t1
        pred = predict_crops(net, Xva, batch=a.batch)
        noisy = Xva[..., :3].float()
        res = {"profile": a.profile, "pairs": a.pairs, "holdout": a.holdout, "crop": a.crop, "spp": a.spp, "worlds": a.worlds,
               "steps": a.steps, "batch": a.batch, "lr": a.lr, "generate_seconds": gen_s, "train_seconds": train_s,
               "final_loss": float(np.mean(losses[-100:])), "first_loss": float(np.mean(losses[:20])),
               "holdout_rmse_noisy": crop_rmse(noisy, Tva), "holdout_rmse_net": crop_rmse(pred, Tva),
               "loss_curve": [float(np.mean(losses[k:k + 50])) for k in range(0, len(losses), 50)]}
        save(out, net.params(), res)
    log(json.dumps({k: v for k, v in res.items() if k != "loss_curve"}))
    del torch


if __name__ == "__main__":
    main()
