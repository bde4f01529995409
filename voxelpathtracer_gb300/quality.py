"""Image error against the FP64 ground truth.

The ground truth of a frame is the converged output of this renderer: the
primary and sun-shadow rays are deterministic, and the diffuse GI (SH, CoCg,
AO) is replaced by its FP64 Welford mean over many samples
(vpt_ground_truth); that mean goes through the same colour pass as a
denoised frame. The error of a pipeline variant (plain fp32 SVGF, fp16
storage, learned denoiser, ...) is the RMSE of its colour against that image
on a crop, evaluated in float64.
"""
from __future__ import annotations

import numpy as np

from . import Context, Camera, Frame, default_config

DEFAULT_CROP_1080P = (800, 450, 320, 180)   # centre 320x180 of a 1920x1080 frame


def ground_truth_color(ctx: Context, cam: Camera, frame: Frame, crop, spp: int = 4096, chunk: int = 256,
                       seed: int = 0x5eed):
    """Colour of the converged frame on `crop`, with the per-pixel standard
    error of the GI luminance channel. `ctx` must be an fp32 context with at
    least one a-trous iteration and the world loaded."""
    x0, y0, w, h = crop
    ctx.trace_primary(cam)
    if getattr(ctx, "_textures", None) is not None:   # block textures: the textured G-buffer
        ctx.generate_gbuffer()
    ctx.trace_shadow(frame)
    mean, m2 = ctx.ground_truth(frame, crop, spp=spp, chunk=chunk, seed=seed)
    H, W = ctx.height, ctx.width
    sh = np.zeros((H, W, 4), np.float32)
    cocg = np.zeros((H, W, 2), np.float32)
    ao = np.zeros((H, W, 2), np.float32)
    sh[y0:y0 + h, x0:x0 + w] = mean[..., 0:4]
    cocg[y0:y0 + h, x0:x0 + w] = mean[..., 4:6]
    ao[y0:y0 + h, x0:x0 + w, 0] = mean[..., 6]
    ctx.write_plane("DEN_SH", sh)
    ctx.write_plane("DEN_COCG", cocg)
    ctx.write_plane("DEN_AOSKY", ao)
    ctx.shade(frame)
    rgb = ctx.read_plane("COLOR")[y0:y0 + h, x0:x0 + w].astype(np.float64)
    stderr = np.sqrt(m2[..., 3] / max(spp - 1, 1) / spp)
    ctx.end_frame()
    return rgb, stderr


def rmse(a: np.ndarray, b: np.ndarray) -> float:
    d = np.asarray(a, np.float64) - np.asarray(b, np.float64)
    return float(np.sqrt(np.mean(d * d)))


def make_gt_context(width: int, height: int, vox, blocks, textures=None, **cfg) -> Context:
    c = default_config(width=width, height=height, **cfg)
    c.storage = 0
    ctx = Context(c)
    ctx.upload_world(vox)
    ctx.set_block_table(blocks)
    ctx.build_df()
    if textures is not None:
        ctx.set_block_textures(textures)
    return ctx


def error_by_history(ctx: Context, gt_ctx: Context, cameras, frames, crop, sample_at, spp: int = 1024) -> dict:
    """RMSE against the FP64 ground truth as the temporal history grows.

    Renders frame k = 0, 1, ... with cameras[k] / frames[k] through ctx (its
    history carried) and, at every k in sample_at, compares on `crop` the
    denoised colour (SVGF or the plain a-trous path), the colour shaded from the
    temporally accumulated GI before any spatial filter, and the colour shaded
    from this frame's raw 1-spp GI with the ground-truth colour of that frame
    (gt_ctx, an fp32 context of the same world). Returns {k: {denoised,
    temporal, raw}}."""
    x0, y0, w, h = crop
    out = {}
    for k in range(max(sample_at) + 1):
        cam, frame = cameras[k], frames[k]
        ctx.trace_primary(cam)
        ctx.trace_shadow(frame)
        ctx.trace_diffuse(frame)
        ctx.svgf(cameras[k - 1] if k > 0 else cam, frame)
        if k in sample_at:
            row = {}
            for name, source in (("temporal", 1), ("raw", 2), ("denoised", 0)):
                ctx.shade_from(frame, source)
                row[name] = ctx.read_plane("COLOR")[y0:y0 + h, x0:x0 + w].astype(np.float64)
            gt, _ = ground_truth_color(gt_ctx, cam, frame, crop, spp=spp)
            out[k] = {name: rmse(img, gt) for name, img in row.items()}
        else:
            ctx.shade(frame)
        ctx.end_frame()
    return out
