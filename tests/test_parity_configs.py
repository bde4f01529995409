"""Bit-exact parity of whole frames at the benchmark's own sizes.

The other parity tests run small images; these render the two measured
configurations at full size, pass by pass in the order vpt_render_frame runs
them (primary, shadow and diffuse traces, SVGF, colour pass, end of frame),
and compare every plane each frame writes against the oracle's restatement
of the same frame (Core/Pipeline.cpp:1959-3821):

* the full-frame workload: the 256^3 world of seed 0, 1920x1080, 1 spp,
  sun shadow, one diffuse bounce with its shadow ray, SVGF (pre-temporal 3x3,
  temporal, variance, 5 a-trous iterations) and the colour pass, FP32 and
  FP16 storage, over two frames of the benchmark's camera pan so the temporal
  pass reprojects;
* the large combined workload: the 512^3 world of seed 0, 3840x2160, two
  diffuse bounces, FP16 storage, two frames of the seeded orbit (the SVGF
  path, which is also the learned denoiser's fallback).

Sizes that only these frames reach (index products above 2^24, history planes
of 8.3 M pixels, the last partial tile rows of 1080 = 33.75 x 32) are covered
here. Every plane must match bit for bit (+0 and -0 treated as equal).
"""
import numpy as np
import pytest

from test_gpu_parity import assert_same

pytestmark = pytest.mark.gpu


def compare_frame(ctx, ref, what):
    """Every plane of a rendered frame (before its end_frame swap) against the
    oracle's frame dict."""
    g = ref["g"]
    for name, plane in (("t", "T"), ("face", "FACE"), ("block", "BLOCK"), ("hit", "HIT"), ("steps", "STEPS")):
        assert_same(ctx.read_plane(plane), g[name], f"{what}: G-buffer {name}")
    assert_same(ctx.read_plane("SHADOW"), ref["shadow"], f"{what}: sun shadow")
    for k in ("sh", "cocg", "luma", "aosky"):
        assert_same(ctx.read_plane("GI_" + k.upper()), ref["gi"][k], f"{what}: diffuse GI {k}")
    sv = ref["svgf"]
    for k in ("sh", "cocg", "luma", "aosky"):
        assert_same(ctx.read_plane("PRE_" + k.upper()), sv["pre"][k], f"{what}: pre-temporal {k}")
    for k in ("sh", "cocg", "util", "aosky"):
        assert_same(ctx.read_plane("TEMP_" + k.upper()), sv["temporal"][k], f"{what}: temporal {k}")
    for k in ("sh", "cocg", "variance"):
        assert_same(ctx.read_plane("VAR_" + k.upper()), sv["variance"][k], f"{what}: variance {k}")
    last = sv["atrous"][-1]
    for k in ("sh", "cocg", "variance", "aosky"):
        assert_same(ctx.read_plane("DEN_" + k.upper()), last[k], f"{what}: a-trous {k}")
    assert_same(ctx.read_plane("COLOR"), ref["rgb"], f"{what}: colour")


def render_and_compare(vpt, oracle, vox, blocks, cams, frames, what, **cfg):
    df = oracle.build_df(vox)
    world = oracle.World(vox, df, blocks)
    with vpt.Context(**cfg) as ctx:
        ctx.upload_world(vox)
        ctx.set_block_table(blocks)
        ctx.build_df()
        assert_same(ctx.read_df(), df, f"{what}: distance field")
        c = ctx.config
        prev_g, hist = oracle.empty_history(c.height, c.width)
        prev_cam = cams[0]
        hits = []
        for fi, (cam, frame) in enumerate(zip(cams, frames)):
            ctx.trace_primary(cam)
            ctx.trace_shadow(frame)
            ctx.trace_diffuse(frame)
            ctx.svgf(prev_cam, frame)
            ctx.shade(frame)
            ref = oracle.render_frame(world, cam, prev_cam, c, frame, prev_g, hist)
            compare_frame(ctx, ref, f"{what} frame {fi}")
            ctx.end_frame()
            hits.append(float((ref["g"]["t"] > 0).mean()))
            prev_g = {k: ref["g"][k] for k in ("t", "face", "block")}
            hist = ref["svgf"]["temporal"]
            prev_cam = cam
            del ref
    # the views mix terrain and sky, so every branch of the filters runs
    assert all(0.2 < h < 0.98 for h in hits), hits


@pytest.mark.parametrize("storage", [0, 1], ids=["f32", "f16"])
def test_full_frame_1080p_two_frames(vpt, oracle, storage, gpu):
    """256^3 seed 0, 1920x1080, 1 spp + shadow + 1 bounce, SVGF, colour:
    the benchmark's first two frames (its 0.25 degree / 0.05 voxel pan)."""
    W, H = 1920, 1080
    vox = vpt.generate_world(256, 256, 256, seed=0)
    blocks = vpt.generate_block_table(100, seed=0)
    yaw, pitch = vpt.seeded_pose(0)
    cams = [vpt.camera_from_pose((128.0 + 0.05 * s, 90.0, 128.0), yaw + 0.25 * s, pitch, 90.0, W / H)
            for s in range(2)]
    frames = [vpt.default_frame(frame_index=s, seed=0, time=1.0 + s / 60.0) for s in range(2)]
    render_and_compare(vpt, oracle, vox, blocks, cams, frames, f"1080p storage {storage}", width=W, height=H,
                       storage=storage)


def test_large_combined_4k_two_bounces_fp16(vpt, oracle, gpu):
    """512^3 seed 0, 3840x2160, 1 spp with 2 diffuse bounces, FP16 storage,
    SVGF: the first two frames of the seeded orbit (radius 200, height 150,
    1 degree per frame)."""
    from voxelpathtracer_gb300 import learned
    W, H = 3840, 2160
    dims = (512, 512, 512)
    vox = vpt.generate_world(*dims, seed=0)
    blocks = vpt.generate_block_table(100, seed=0)
    theta0 = float(np.random.default_rng(0).uniform(0.0, 360.0))
    cams = [learned.orbit_camera(dims, theta0 + k, W / H) for k in range(2)]
    frames = [vpt.default_frame(frame_index=k, seed=0, time=1.0 + k / 60.0) for k in range(2)]
    render_and_compare(vpt, oracle, vox, blocks, cams, frames, "4K 2-bounce fp16", width=W, height=H, storage=1,
                       bounces=2)
