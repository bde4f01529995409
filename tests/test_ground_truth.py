"""FP64 Welford ground truth: the oracle's accumulation is chunk-invariant
and statistically sound (CPU), and libvpt's GPU accumulation reproduces it bit
for bit (GPU)."""
import numpy as np
import pytest

W, H = 48, 32


@pytest.fixture(scope="module")
def small(vpt, oracle):
    vox = vpt.generate_world(40, 48, 40, seed=9)
    blocks = vpt.generate_block_table(100, seed=9)
    df = oracle.build_df(vox)
    world = oracle.World(vox, df, blocks)
    cam = vpt.camera_from_pose((20.0, 46.0, 20.0), 60.0, -30.0, 90.0, W / H)
    cfg = vpt.default_config(width=W, height=H, primary_max_steps=256)
    g = oracle.trace_primary(world, cam, cfg)
    frame = vpt.default_frame(seed=1)
    return {"vox": vox, "blocks": blocks, "world": world, "cam": cam, "cfg": cfg, "g": g, "frame": frame}


def test_oracle_welford_is_chunk_invariant(oracle, small):
    s = small
    crop = (10, 8, 14, 9)
    a_mean, a_m2 = oracle.ground_truth(s["world"], s["cam"], s["cfg"], s["frame"], s["g"]["t"], s["g"]["face"],
                                       crop, spp=64, chunk=64)
    b_mean, b_m2 = oracle.ground_truth(s["world"], s["cam"], s["cfg"], s["frame"], s["g"]["t"], s["g"]["face"],
                                       crop, spp=64, chunk=5)
    assert np.allclose(a_mean, b_mean, rtol=1e-12, atol=1e-12)
    assert np.allclose(a_m2, b_m2, rtol=1e-9, atol=1e-9)
    assert (a_m2 >= -1e-12).all()
    hit = s["g"]["t"][8:17, 10:24] > 0
    assert hit.any() and (a_m2[..., 3][hit] > 0).any()      # the diffuse signal is noisy on hit pixels
    assert np.allclose(a_m2[..., :6][~hit], 0.0)             # sky pixels are deterministic


def test_oracle_ground_truth_converges(oracle, small):
    """The mean of the first 256 samples and of samples 256..511 agree within
    a few standard errors (independent streams per sample index)."""
    s = small
    crop = (12, 10, 8, 6)
    m_all, m2_all = oracle.ground_truth(s["world"], s["cam"], s["cfg"], s["frame"], s["g"]["t"], s["g"]["face"],
                                        crop, spp=512, chunk=256)
    m_lo, _ = oracle.ground_truth(s["world"], s["cam"], s["cfg"], s["frame"], s["g"]["t"], s["g"]["face"], crop,
                                  spp=256, chunk=256)
    m_hi = 2.0 * m_all - m_lo                     # mean of samples 256..511
    se = np.sqrt(np.maximum(m2_all, 0) / 511.0 / 256.0) + 1e-9
    z = np.abs(m_lo - m_hi) / (np.sqrt(2.0) * se)
    assert np.mean(z < 4.0) > 0.97


@pytest.mark.gpu
@pytest.mark.parametrize("textured", [False, True], ids=["flat", "block-textures"])
def test_gpu_ground_truth_bit_exact(vpt, oracle, small, textured, gpu):
    """FP64 means and M2 equal the oracle's to the bit, with flat materials
    and with the bounce hits sampling block textures."""
    s = small
    crop = (6, 4, 30, 20)
    tex = vpt.generate_block_textures(16, 6, seed=3) if textured else None
    with vpt.Context(s["cfg"]) as ctx:
        ctx.upload_world(s["vox"])
        ctx.set_block_table(s["blocks"])
        ctx.build_df()
        if tex is not None:
            ctx.set_block_textures(tex)
        ctx.trace_primary(s["cam"])
        mean, m2 = ctx.ground_truth(s["frame"], crop, spp=40, chunk=16, seed=77)
    r_mean, r_m2 = oracle.ground_truth(s["world"], s["cam"], s["cfg"], s["frame"], s["g"]["t"], s["g"]["face"],
                                       crop, spp=40, chunk=16, seed=77, textures=tex)
    assert np.array_equal(mean.view(np.uint64), r_mean.view(np.uint64))
    assert np.array_equal(m2.view(np.uint64), r_m2.view(np.uint64))
    if textured:   # the textures change the converged GI
        f_mean, _ = oracle.ground_truth(s["world"], s["cam"], s["cfg"], s["frame"], s["g"]["t"], s["g"]["face"],
                                        crop, spp=40, chunk=16, seed=77)
        assert not np.array_equal(f_mean, r_mean)


@pytest.mark.gpu
def test_gpu_ground_truth_color_and_error(vpt, small, gpu):
    """A denoised frame is closer to the converged image than the raw 1-spp
    GI, and the ground-truth image is stable against a second seed."""
    from voxelpathtracer_gb300 import quality
    s = small
    crop = (8, 6, 32, 20)
    gt_ctx = quality.make_gt_context(W, H, s["vox"], s["blocks"], primary_max_steps=256)
    gt, se = quality.ground_truth_color(gt_ctx, s["cam"], s["frame"], crop, spp=1024, chunk=128, seed=1)
    gt2, _ = quality.ground_truth_color(gt_ctx, s["cam"], s["frame"], crop, spp=1024, chunk=128, seed=2)
    gt_ctx.close()
    assert quality.rmse(gt, gt2) < 0.05 * float(np.sqrt(np.mean(gt * gt)))
    with vpt.Context(s["cfg"]) as ctx:
        ctx.upload_world(s["vox"])
        ctx.set_block_table(s["blocks"])
        ctx.build_df()
        for k in range(12):                       # static camera: the history accumulates
            rgb = ctx.render_frame(s["cam"], vpt.default_frame(seed=1, frame_index=k))
        x0, y0, w, h = crop
        denoised = rgb[y0:y0 + h, x0:x0 + w]
        # raw 1-spp GI straight into the colour pass
        ctx.trace_primary(s["cam"])
        ctx.trace_shadow(s["frame"])
        ctx.trace_diffuse(s["frame"])
        for src, dst in (("GI_SH", "DEN_SH"), ("GI_COCG", "DEN_COCG"), ("GI_AOSKY", "DEN_AOSKY")):
            ctx.write_plane(dst, ctx.read_plane(src))
        ctx.shade(s["frame"])
        raw = ctx.read_plane("COLOR")[y0:y0 + h, x0:x0 + w]
    assert quality.rmse(denoised, gt) < quality.rmse(raw, gt)
