"""The reflection pass (ReflectionTraceFrag.glsl, the two bilateral passes
over its hit distance, SpecularTemporalFilter.glsl with TEMPORAL_SPEC on or
off, the two separable passes of ReflectionDenoiserNew.glsl with
DenoiseReflections on or off) and the specular indirect it feeds into the
colour pass (ColorPassFrag.glsl :595-603, :901-909). Every plane is
bit-identical to the oracle.
"""
import numpy as np
import pytest

from test_gpu_parity import assert_same

W, H = 96, 64
DIMS = (64, 64, 64)


def scene_inputs(vpt, oracle, seed=1):
    X, Y, Z = DIMS
    vox = vpt.generate_world(X, Y, Z, seed=seed)
    blocks = vpt.generate_block_table(100, seed=seed)
    df = oracle.build_df(vox)
    yaw, pitch = vpt.seeded_pose(seed)
    cam0 = vpt.camera_from_pose((X / 2, 58.0, Z / 2), yaw, pitch, 90.0, W / H)
    cam1 = vpt.camera_from_pose((X / 2 + 0.7, 58.2, Z / 2 - 0.4), yaw + 2.0, pitch + 1.0, 90.0, W / H)
    return {"vox": vox, "blocks": blocks, "world": oracle.World(vox, df, blocks), "cams": [cam0, cam1]}


# ------------------------------------------------------------------ CPU --
def test_oracle_reflection_properties(vpt, oracle):
    """Sky texels reflect nothing, every other texel is finite and positive,
    hit distances lie in the shader's clamp, masks are 0/1, the resolved plane
    differs from the raw one only where an emissive block was hit, and the
    colour pass with reflections adds light on average."""
    sc = scene_inputs(vpt, oracle)
    cfg = vpt.default_config(width=W, height=H, primary_max_steps=256, reflection_spp=2, reflection_temporal=0)
    cam = sc["cams"][0]
    frame = vpt.default_frame(frame_index=0, seed=9)
    prev_g, hist = oracle.empty_history(H, W)
    ref = oracle.render_frame(sc["world"], cam, cam, cfg, frame, prev_g, hist)
    r, g = ref["refl"], ref["g"]
    sky = g["t"] < 0
    assert (r["spec"][sky] == 0).all() and (r["hit"][sky] == -1).all()
    assert np.isfinite(r["spec"]).all() and (r["spec"][~sky] > 0).all()
    assert ((r["hit"] >= -10) & (r["hit"] <= 200)).all() and (r["hit"][~sky] > 0).any()
    assert set(np.unique(r["mask"])) <= {0.0, 1.0}
    assert (r["acc"] == -1).all()
    changed = (r["out"] != r["spec"]).any(axis=-1)
    assert not (changed & (r["mask"] <= 0.05)).any()
    cfg0 = vpt.default_config(width=W, height=H, primary_max_steps=256)
    base = oracle.render_frame(sc["world"], cam, cam, cfg0, frame, prev_g, hist)
    hit = ~sky
    assert (ref["rgb"][sky] == base["rgb"][sky]).all()
    assert ref["rgb"][hit].mean() > base["rgb"][hit].mean() and (ref["rgb"][hit] != base["rgb"][hit]).any()


def test_oracle_reflection_temporal_accumulates(vpt, oracle):
    """With TEMPORAL_SPEC the second frame of a still camera reprojects onto
    itself: accumulation factors in (0, 0.95] where history was valid, and
    the output moves towards last frame's."""
    sc = scene_inputs(vpt, oracle)
    cfg = vpt.default_config(width=W, height=H, primary_max_steps=256, reflection_spp=2)
    cam = sc["cams"][0]
    prev_g, hist = oracle.empty_history(H, W)
    f0 = oracle.render_frame(sc["world"], cam, cam, cfg, vpt.default_frame(frame_index=0, seed=9), prev_g, hist)
    assert (f0["refl"]["acc"] == 0).all()          # nothing to reproject from
    g0 = {k: f0["g"][k] for k in ("t", "face", "block")}
    f1 = oracle.render_frame(sc["world"], cam, cam, cfg, vpt.default_frame(frame_index=1, seed=9), g0,
                             f0["svgf"]["temporal"], f0["refl"])
    acc = f1["refl"]["acc"]
    hits = f1["g"]["t"] > 0
    assert ((acc == 0) | ((acc >= 0.001) & (acc <= 0.95))).all() and (acc[hits] > 0.5).mean() > 0.5
    hist_ok = acc > 0
    d_new = np.abs(f1["refl"]["out"] - f1["refl"]["spec"])[hist_ok].mean()
    d_old = np.abs(f1["refl"]["out"] - f0["refl"]["out"])[hist_ok].mean()
    assert d_old < d_new


def test_oracle_reflection_denoiser_smooths(vpt, oracle):
    """The separable denoiser keeps sky texels and the mean of the hit
    texels' radiance (within 10%) and lowers its local variation."""
    sc = scene_inputs(vpt, oracle)
    cfg = vpt.default_config(width=W, height=H, primary_max_steps=256, reflection_spp=1, reflection_temporal=0)
    cam = sc["cams"][0]
    prev_g, hist = oracle.empty_history(H, W)
    ref = oracle.render_frame(sc["world"], cam, cam, cfg, vpt.default_frame(frame_index=0, seed=3), prev_g, hist)
    r, hit = ref["refl"], ref["g"]["t"] > 0
    assert (r["den"][~hit] == r["out"][~hit]).all()
    a, b = r["out"][..., :3], r["den"][..., :3]
    assert abs(b[hit].mean() - a[hit].mean()) < 0.1 * a[hit].mean()
    both = hit[:, 1:] & hit[:, :-1]
    assert np.abs(np.diff(b, axis=1))[both].mean() < np.abs(np.diff(a, axis=1))[both].mean()


def test_oracle_reflection_counts_rays(vpt, oracle):
    sc = scene_inputs(vpt, oracle)
    cfg = vpt.default_config(width=W, height=H, primary_max_steps=256, reflection_spp=3)
    cam = sc["cams"][0]
    frame = vpt.default_frame(frame_index=1, seed=9)
    prev_g, hist = oracle.empty_history(H, W)
    with oracle.Counting() as cnt:
        ref = oracle.render_frame(sc["world"], cam, cam, cfg, frame, prev_g, hist)
    hits = int((ref["g"]["t"] > 0).sum())
    assert cnt.rays["reflection"] == 3 * hits
    assert 0 < cnt.rays["reflection_shadow"] <= hits


# ------------------------------------------------------------------ GPU --
@pytest.mark.gpu
@pytest.mark.parametrize("d,storage,denoiser,temporal,rden", [
    (1, 0, 0, 1, 1), (2, 0, 0, 1, 1), (1, 1, 0, 1, 1), (4, 1, 0, 1, 1), (1, 0, 1, 1, 1), (1, 0, 0, 0, 1),
    (2, 0, 0, 1, 0)], ids=["d1-f32", "d2-f32", "d1-f16", "d4-f16", "d1-plain", "d1-no-temporal", "d2-no-denoise"])
def test_reflection_planes_bit_exact(vpt, oracle, d, storage, denoiser, temporal, rden, gpu):
    sc = scene_inputs(vpt, oracle)
    world = sc["world"]
    X, Z = DIMS[0], DIMS[2]
    yaw, pitch = vpt.seeded_pose(1)
    cams = sc["cams"] + [vpt.camera_from_pose((X / 2 + 1.1, 58.1, Z / 2 - 0.9), yaw + 3.5, pitch + 1.5, 90.0, W / H)]
    ctx = vpt.Context(width=W, height=H, primary_max_steps=256, storage=storage, gi_divisor=d, reflection_spp=2,
                      denoiser=denoiser, reflection_temporal=temporal, reflection_denoise=rden)
    ctx.upload_world(sc["vox"])
    ctx.set_block_table(sc["blocks"])
    ctx.build_df()
    cfg = ctx.config
    prev_g, hist = oracle.empty_history(H, W, d)
    prev_refl = None
    prev_cam = cams[0]
    for fi, cam in enumerate(cams):
        frame = vpt.default_frame(frame_index=fi, seed=13, time=0.7 + 0.2 * fi)
        ctx.set_stats(True)
        ctx.trace_primary(cam)
        ctx.trace_shadow(frame)
        ctx.trace_diffuse(frame)
        ctx.svgf(prev_cam, frame)
        ctx.trace_reflections(frame)
        ctx.shade(frame)
        rgb = ctx.read_plane("COLOR")
        stats = ctx.read_stats()
        with oracle.Counting() as cnt:
            ref = oracle.render_frame(world, cam, prev_cam, cfg, frame, prev_g, hist, prev_refl)
        r = ref["refl"]
        assert_same(ctx.read_plane("SPEC"), r["spec"], f"{d} frame {fi} spec")
        assert_same(ctx.read_plane("SPEC_MASK")[..., 0], r["mask"], f"{d} frame {fi} mask")
        assert_same(ctx.read_plane("SPEC_HIT")[..., 0], r["hit"], f"{d} frame {fi} blurred hit")
        assert_same(ctx.read_plane("SPEC_OUT"), r["out"], f"{d} frame {fi} temporal colour")
        assert_same(ctx.read_plane("SPEC_ACC")[..., 0], r["acc"], f"{d} frame {fi} accumulation")
        assert_same(ctx.read_plane("SPEC_STABLE_HIT")[..., 0], r["stable"], f"{d} frame {fi} stable hit")
        if rden:
            assert_same(ctx.read_plane("SPEC_DEN"), r["den"], f"{d} frame {fi} denoised")
        assert_same(rgb, ref["rgb"], f"{d} frame {fi} colour")
        assert stats["rays"] == cnt.rays and stats["steps"] == cnt.steps
        if temporal and fi > 0:
            assert (r["acc"] > 0).any()
        ctx.end_frame()
        prev_g = {k: ref["g"][k] for k in ("t", "face", "block")}
        hist = ref["svgf"]["temporal"]
        prev_refl = r
        prev_cam = cam
    ctx.close()


@pytest.mark.gpu
def test_reflection_pass_order_and_guards(vpt, oracle, gpu):
    """The pass API in the reference's order gives the render_frame result;
    without reflections the planes are absent and the pass is refused."""
    sc = scene_inputs(vpt, oracle, seed=2)
    cam = sc["cams"][0]
    frame = vpt.default_frame(frame_index=0, seed=4)
    with vpt.Context(width=W, height=H, primary_max_steps=256, reflection_spp=1) as a, \
            vpt.Context(width=W, height=H, primary_max_steps=256, reflection_spp=1) as b:
        for c in (a, b):
            c.upload_world(sc["vox"])
            c.set_block_table(sc["blocks"])
            c.build_df()
        rgb = a.render_frame(cam, frame)
        b.trace_primary(cam)
        b.trace_shadow(frame)
        b.trace_diffuse(frame)
        b.svgf(None, frame)
        b.trace_reflections(frame)
        b.shade(frame)
        assert_same(b.read_plane("COLOR"), rgb, "pass-by-pass colour")
    with vpt.Context(width=W, height=H) as c:
        c.upload_world(sc["vox"])
        c.set_block_table(sc["blocks"])
        c.build_df()
        c.trace_primary(cam)
        with pytest.raises(vpt.VPTError):
            c.trace_reflections(frame)
        with pytest.raises(vpt.VPTError):
            c.read_plane("SPEC")
