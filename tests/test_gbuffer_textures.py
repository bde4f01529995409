"""The textured G-buffer pass (GenerateGBuffer.glsl main with parallax off):
block texture arrays sampled with textureGrad at the face UV. The CPU half
checks the oracle's restatement against properties the shader fixes (sky
texels, constant textures, the tangent basis, the grass override, the light
leak fix, mip-level selection); the GPU half holds the CUDA pass to the
oracle's bits through the C ABI."""
import numpy as np
import pytest

from test_gpu_parity import assert_same

W, H = 96, 64
DIMS = (64, 64, 64)


def scene(vpt, oracle, seed=1):
    X, Y, Z = DIMS
    vox = vpt.generate_world(X, Y, Z, seed=seed)
    blocks = vpt.generate_block_table(100, seed=seed)
    world = oracle.World(vox, oracle.build_df(vox), blocks)
    yaw, pitch = vpt.seeded_pose(seed)
    cams = [vpt.camera_from_pose((X / 2, 58.0, Z / 2), yaw, pitch, 90.0, W / H),
            vpt.camera_from_pose((8.5, 42.0, 8.5), 30.0, -20.0, 90.0, W / H)]
    return vox, blocks, world, cams


def constant_textures(vpt, layers=4, size=8):
    """Every layer one constant value per channel: layer l albedo (40 l + 20, 100, 200 - 30 l)."""
    t = vpt.generate_block_textures(size, layers, seed=3)
    for l in range(layers):
        t["albedo"][l, ..., :3] = (40 * l + 20, 100, 200 - 30 * l)
        t["normal"][l, ..., :3] = (128, 128, 255)
        t["pbr"][l] = (30 + 40 * l, 0, 128, 200)
        t["emissive"][l] = 255
    return t


def srgb(b):
    x = np.float32(b) / np.float32(255.0)
    return x / np.float32(12.92) if x <= 0.04045 else ((x + 0.055) / 1.055) ** 2.4


# ------------------------------------------------------------------ CPU --
def test_oracle_gbuffer_sky_and_constant_textures(vpt, oracle):
    vox, blocks, world, cams = scene(vpt, oracle)
    cfg = vpt.default_config(width=W, height=H, primary_max_steps=256)
    tex = constant_textures(vpt)
    g = oracle.trace_primary(world, cams[0], cfg)
    gb = oracle.generate_gbuffer(cams[0], cfg, tex, g["t"], g["face"], g["block"])
    sky, hit = g["t"] < 0, g["t"] > 0
    assert sky.any() and hit.any()
    assert (gb["albedo"][sky] == 0).all() and (gb["normal"][sky] == 1).all()
    assert (gb["pbr"][sky] == 0).all() and (gb["ao"][sky] == 0).all()
    # constant layers: every level and every filter weight gives the layer's value
    ids = tex["albedo_id"][g["block"][hit]]
    grass = g["block"][hit] == tex["grass"][0]
    face = g["face"][hit]
    layer = np.where(grass, np.where(face == 2, tex["grass"][1], np.where(face == 3, tex["grass"][7],
                                                                           tex["grass"][4])), ids)
    want = np.array([[srgb(40 * l + 20), srgb(100), srgb(200 - 30 * l)] for l in range(4)], np.float32)
    np.testing.assert_allclose(gb["albedo"][hit], want[np.clip(layer, 0, 3)], rtol=2e-6)
    # the flat normal map gives the face normal plus the (1/255) tangent and bitangent tilt
    n_face = np.array([[0, 0, 1], [0, 0, -1], [0, 1, 0], [0, -1, 0], [-1, 0, 0], [1, 0, 0]], np.float32)
    tang = np.array([[1, 0, 0]] * 4 + [[0, 0, -1]] * 2, np.float32)
    bitang = np.array([[0, 1, 0]] * 2 + [[0, 0, 1]] * 2 + [[0, -1, 0]] * 2, np.float32)
    e = np.float32(128) / np.float32(255) * 2 - 1
    np.testing.assert_allclose(gb["normal"][hit], n_face[face] + e * (tang[face] + bitang[face]), atol=1e-6)
    pl = np.where(grass, np.where(face == 2, tex["grass"][3], np.where(face == 3, tex["grass"][9],
                                                                        tex["grass"][6])), tex["pbr_id"][g["block"][hit]])
    np.testing.assert_allclose(gb["pbr"][hit][:, 0], (30 + 40 * np.clip(pl, 0, 3)) / 255.0, rtol=2e-6)
    np.testing.assert_allclose(gb["ao"][hit], 200 / 255.0, rtol=2e-6)
    # emissive texture of 1: 1 inside the face, 0 in its 2% border band (BloomLightLeakFix)
    em = gb["pbr"][hit][:, 3]
    has = tex["emissive_id"][g["block"][hit]] > -1
    assert set(np.unique(em[has])) <= {0.0, 1.0} and (em[has] == 1).mean() > 0.8
    assert (em[~has] == 0).all()


def test_oracle_gbuffer_grass_override(vpt, oracle):
    """A grass block's top, side and bottom faces read their own layers."""
    vox, blocks, world, cams = scene(vpt, oracle)
    cfg = vpt.default_config(width=W, height=H, primary_max_steps=256)
    tex = constant_textures(vpt)
    g = oracle.trace_primary(world, cams[0], cfg)
    common = np.bincount(g["block"][g["t"] > 0]).argmax()
    tex["grass"][:] = (common, 0, 0, 0, 1, 1, 1, 2, 2, 2)
    tex["albedo_id"][:] = 3
    gb = oracle.generate_gbuffer(cams[0], cfg, tex, g["t"], g["face"], g["block"])
    sel = (g["block"] == common) & (g["t"] > 0)
    want = {2: 0, 3: 2, 0: 1, 1: 1, 4: 1, 5: 1}
    for f, l in want.items():
        m = sel & (g["face"] == f)
        if m.any():
            np.testing.assert_allclose(gb["albedo"][m][:, 0], srgb(40 * l + 20), rtol=2e-6)
    other = (g["block"] != common) & (g["t"] > 0)
    np.testing.assert_allclose(gb["albedo"][other][:, 0], srgb(40 * 3 + 20), rtol=2e-6)


def test_oracle_gbuffer_filters_towards_the_mean_with_distance(vpt, oracle):
    """A texel checkerboard: near faces resolve it, far faces read the coarse
    mip levels, whose texels are all the mean."""
    vox, blocks, world, cams = scene(vpt, oracle)
    cfg = vpt.default_config(width=W, height=H, primary_max_steps=256)
    tex = constant_textures(vpt, size=32)
    yy, xx = np.meshgrid(np.arange(32), np.arange(32), indexing="ij")
    tex["pbr"][..., 0] = np.where((xx + yy) % 2 == 0, 0, 254).astype(np.uint8)[None]
    g = oracle.trace_primary(world, cams[1], cfg)
    gb = oracle.generate_gbuffer(cams[1], cfg, tex, g["t"], g["face"], g["block"])
    hit = g["t"] > 0
    r = gb["pbr"][..., 0]
    near, far = hit & (g["t"] < 6), hit & (g["t"] > 30)
    assert near.sum() > 20 and far.sum() > 20
    assert np.abs(r[far] - 127 / 255.0).mean() < np.abs(r[near] - 127 / 255.0).mean()


# ------------------------------------------------------------------ GPU --
@pytest.mark.gpu
@pytest.mark.parametrize("storage,size,emissive", [(0, 16, True), (1, 16, True), (0, 64, False), (1, 8, True)],
                         ids=["f32-16", "f16-16", "f32-64-no-emissive", "f16-8"])
def test_gbuffer_planes_bit_exact(vpt, oracle, storage, size, emissive, gpu):
    vox, blocks, world, cams = scene(vpt, oracle, seed=2)
    solid = vox[vox > 0]
    tex = vpt.generate_block_textures(size, 7, seed=size, emissive=emissive,
                                      grass_block=int(np.bincount(solid).argmax()))   # the most common block
    with vpt.Context(width=W, height=H, primary_max_steps=256, storage=storage) as ctx:
        ctx.upload_world(vox)
        ctx.set_block_table(blocks)
        ctx.build_df()
        ctx.set_block_textures(tex)
        cfg = ctx.config
        for k, cam in enumerate(cams):
            ctx.trace_primary(cam)
            ctx.generate_gbuffer()
            g = oracle.trace_primary(world, cam, cfg)
            ref = oracle.generate_gbuffer(cam, cfg, tex, g["t"], g["face"], g["block"])
            assert_same(ctx.read_plane("GB_ALBEDO"), ref["albedo"], f"cam {k} albedo")
            assert_same(ctx.read_plane("GB_NORMAL"), ref["normal"], f"cam {k} normal")
            assert_same(ctx.read_plane("GB_PBR"), ref["pbr"], f"cam {k} pbr")
            assert_same(ctx.read_plane("GB_AO")[..., 0], ref["ao"], f"cam {k} ao")
            ctx.end_frame()


@pytest.mark.gpu
def test_gbuffer_needs_textures_and_a_gbuffer(vpt, oracle, gpu):
    vox, blocks, world, cams = scene(vpt, oracle)
    with vpt.Context(width=W, height=H) as ctx:
        ctx.upload_world(vox)
        ctx.set_block_table(blocks)
        ctx.build_df()
        with pytest.raises(vpt.VPTError):
            ctx.read_plane("GB_ALBEDO")
        ctx.trace_primary(cams[0])
        with pytest.raises(vpt.VPTError):
            ctx.generate_gbuffer()
        bad = vpt.generate_block_textures(8, 2)
        bad["size"] = 12
        with pytest.raises(vpt.VPTError):
            ctx.set_block_textures(bad)
        ctx.set_block_textures(vpt.generate_block_textures(8, 2))
        ctx.generate_gbuffer()
        assert ctx.read_plane("GB_PBR").shape == (H, W, 4)
        ctx.set_block_textures(None)
        with pytest.raises(vpt.VPTError):
            ctx.generate_gbuffer()


# ------------------------------------------------ colour pass with textures --
def test_oracle_textured_colour_pass(vpt, oracle):
    """The colour pass reads the textured G-buffer: sky unchanged, a brighter
    albedo texture brightens the lit pixels, and an emissive texel over 0.05
    switches the direct light off."""
    vox, blocks, world, cams = scene(vpt, oracle)
    cfg = vpt.default_config(width=W, height=H, primary_max_steps=256)
    frame = vpt.default_frame(frame_index=0, seed=9)
    prev_g, hist = oracle.empty_history(H, W)
    flat = oracle.render_frame(world, cams[0], cams[0], cfg, frame, prev_g, hist)
    dark, bright = constant_textures(vpt), constant_textures(vpt)
    dark["emissive_id"][:] = -1
    bright["emissive_id"][:] = -1
    dark["albedo"][..., :3] = 60
    bright["albedo"][..., :3] = 200
    fd = oracle.render_frame(world, cams[0], cams[0], cfg, frame, prev_g, hist, textures=dark)
    fb = oracle.render_frame(world, cams[0], cams[0], cfg, frame, prev_g, hist, textures=bright)
    sky, hit = flat["g"]["t"] < 0, flat["g"]["t"] > 0
    assert (fd["rgb"][sky] == flat["rgb"][sky]).all() and (fb["rgb"][sky] == flat["rgb"][sky]).all()
    assert fb["rgb"][hit].mean() > 1.5 * fd["rgb"][hit].mean()
    # the bounce hits read the textures too: brighter texels, more bounced light
    assert fb["gi"]["luma"][hit].mean() > fd["gi"]["luma"][hit].mean()
    assert not np.array_equal(fd["gi"]["sh"], flat["gi"]["sh"])
    # the same colour pass inputs but an emissive G-buffer texel: no direct light there
    g, sv = fd["g"], fd["svgf"]["atrous"][-1]
    glow = {k: v.copy() for k, v in fd["gbt"].items()}
    glow["pbr"][..., 3] = np.where(hit, 1.0, 0.0)
    args = (world, cams[0], cfg, frame, g["t"], g["face"], g["block"], fd["shadow"], sv["sh"], sv["cocg"], sv["aosky"])
    lit = oracle.shade(*args, gbt=fd["gbt"])
    dark = oracle.shade(*args, gbt=glow)
    assert (lit == fd["rgb"]).all()
    assert (dark[hit] <= lit[hit]).all() and dark[hit].mean() < lit[hit].mean() and (dark[sky] == lit[sky]).all()


@pytest.mark.gpu
@pytest.mark.parametrize("storage,d,rspp", [(0, 1, 0), (1, 1, 0), (0, 2, 2), (1, 1, 2)],
                         ids=["f32", "f16", "f32-d2-reflections", "f16-reflections"])
def test_textured_frames_bit_exact(vpt, oracle, storage, d, rspp, gpu):
    """Whole frames through vpt_render_frame with block textures: the
    textured G-buffer, the colour pass over it (with the GI upscale and the
    reflection gather) and the history across frames equal the oracle's."""
    vox, blocks, world, cams = scene(vpt, oracle, seed=3)
    tex = vpt.generate_block_textures(16, 9, seed=7, grass_block=int(np.bincount(vox[vox > 0]).argmax()))
    X, Z = DIMS[0], DIMS[2]
    yaw, pitch = vpt.seeded_pose(3)
    poses = [cams[0], vpt.camera_from_pose((X / 2 + 0.6, 58.1, Z / 2 - 0.3), yaw + 2.0, pitch + 1.0, 90.0, W / H)]
    with vpt.Context(width=W, height=H, primary_max_steps=256, storage=storage, gi_divisor=d,
                     reflection_spp=rspp) as ctx:
        ctx.upload_world(vox)
        ctx.set_block_table(blocks)
        ctx.build_df()
        ctx.set_block_textures(tex)
        cfg = ctx.config
        prev_g, hist = oracle.empty_history(H, W, d)
        prev_refl, prev_cam = None, poses[0]
        for k, cam in enumerate(poses):
            frame = vpt.default_frame(frame_index=k, seed=5, time=0.3 + 0.2 * k)
            rgb = ctx.render_frame(cam, frame)
            ref = oracle.render_frame(world, cam, prev_cam, cfg, frame, prev_g, hist, prev_refl, textures=tex)
            for name, key in (("GI_SH", "sh"), ("GI_COCG", "cocg"), ("GI_LUMA", "luma"), ("GI_AOSKY", "aosky")):
                got = ctx.read_plane(name)
                assert_same(got[..., 0] if key == "luma" else got, ref["gi"][key], f"frame {k} {name}")
            assert_same(rgb, ref["rgb"], f"frame {k} colour")
            prev_g = {n: ref["g"][n] for n in ("t", "face", "block")}
            hist = ref["svgf"]["temporal"]
            prev_refl = ref["refl"]
            prev_cam = cam


@pytest.mark.gpu
def test_textured_shade_needs_this_frames_gbuffer(vpt, oracle, gpu):
    vox, blocks, world, cams = scene(vpt, oracle)
    frame = vpt.default_frame(frame_index=0, seed=1)
    with vpt.Context(width=W, height=H) as ctx:
        ctx.upload_world(vox)
        ctx.set_block_table(blocks)
        ctx.build_df()
        ctx.set_block_textures(vpt.generate_block_textures(8, 3))
        ctx.trace_primary(cams[0])
        ctx.trace_shadow(frame)
        ctx.trace_diffuse(frame)
        ctx.svgf(None, frame)
        with pytest.raises(vpt.VPTError):
            ctx.shade(frame)
        ctx.generate_gbuffer()
        ctx.shade(frame)


def test_oracle_textured_reflections_read_the_textures(vpt, oracle):
    """With block textures the reflection pass reads the textured G-buffer
    and samples the textures at its hits: brighter albedo texels, brighter
    reflections; sky texels reflect nothing either way."""
    vox, blocks, world, cams = scene(vpt, oracle)
    cfg = vpt.default_config(width=W, height=H, primary_max_steps=256, reflection_spp=2, reflection_temporal=0)
    frame = vpt.default_frame(frame_index=0, seed=9)
    prev_g, hist = oracle.empty_history(H, W)
    dark, bright = constant_textures(vpt), constant_textures(vpt)
    for t in (dark, bright):
        t["emissive_id"][:] = -1
        t["pbr"][..., 0] = 40          # smooth enough to reflect
    dark["albedo"][..., :3] = 60
    bright["albedo"][..., :3] = 200
    fd = oracle.render_frame(world, cams[0], cams[0], cfg, frame, prev_g, hist, textures=dark)
    fb = oracle.render_frame(world, cams[0], cams[0], cfg, frame, prev_g, hist, textures=bright)
    sky = fd["g"]["t"] < 0
    hits = (fd["refl"]["hit"] > 0) & ~sky
    assert hits.any() and (fd["refl"]["spec"][sky] == 0).all()
    assert fb["refl"]["spec"][hits][:, :3].mean() > 1.2 * fd["refl"]["spec"][hits][:, :3].mean()


# ------------------------------------------------ alpha-tested traversal --
def test_oracle_alpha_test(vpt, oracle):
    """u_ShouldAlphaTest: with every block transparent to it, rays pass the
    cut-out texels and end farther; with none transparent, or without the
    flag, the G-buffer is the plain traversal's."""
    vox, blocks, world, cams = scene(vpt, oracle)
    tex = vpt.generate_block_textures(16, 6, seed=1)
    plain = oracle.trace_primary(world, cams[0], vpt.default_config(width=W, height=H, primary_max_steps=256))
    cfg = vpt.default_config(width=W, height=H, primary_max_steps=256, alpha_test=1)
    tex["transparent"][:] = 0
    opaque = oracle.trace_primary(world, cams[0], cfg, textures=tex)
    for k in ("t", "face", "block", "hit", "steps"):
        assert np.array_equal(opaque[k], plain[k]), k
    tex["transparent"][:] = 1
    cut = oracle.trace_primary(world, cams[0], cfg, textures=tex)
    hit = plain["t"] > 0
    assert (cut["t"][hit] > plain["t"][hit] + 0.5).mean() > 0.2
    assert (cut["t"][~hit] == plain["t"][~hit]).all()


@pytest.mark.gpu
@pytest.mark.parametrize("storage,frac", [(0, 1.0), (1, 0.5), (0, 0.0)], ids=["f32-all", "f16-half", "f32-none"])
def test_alpha_tested_gbuffer_bit_exact(vpt, oracle, storage, frac, gpu):
    vox, blocks, world, cams = scene(vpt, oracle, seed=2)
    tex = vpt.generate_block_textures(32, 5, seed=4)
    tex["transparent"][:] = (np.random.default_rng(1).random(128) < frac).astype(np.int32)
    with vpt.Context(width=W, height=H, primary_max_steps=256, storage=storage, alpha_test=1) as ctx:
        ctx.upload_world(vox)
        ctx.set_block_table(blocks)
        ctx.build_df()
        ctx.set_block_textures(tex)
        cfg = ctx.config
        for k, cam in enumerate(cams):
            ctx.set_stats(True)
            ctx.trace_primary(cam)
            stats = ctx.read_stats()
            with oracle.Counting() as cnt:
                ref = oracle.trace_primary(world, cam, cfg, textures=tex)
            for name, key in (("T", "t"), ("FACE", "face"), ("BLOCK", "block"), ("HIT", "hit"), ("STEPS", "steps")):
                got = ctx.read_plane(name)
                assert_same(got[..., 0] if got.ndim == 3 and key != "hit" else got, ref[key], f"cam {k} {name}")
            assert stats["steps"]["primary"] == cnt.steps["primary"]
            ctx.end_frame()


def test_oracle_alpha_tested_shadows(vpt, oracle):
    """ShouldAlphaTestShadows: sun rays pass the cut-out texels of transparent
    blocks, so fewer texels are shadowed; with no transparent block the
    shadow plane is the plain one."""
    vox, blocks, world, cams = scene(vpt, oracle)
    tex = vpt.generate_block_textures(16, 6, seed=1)
    frame = vpt.default_frame(frame_index=0, seed=3)
    base = vpt.default_config(width=W, height=H, primary_max_steps=256)
    g = oracle.trace_primary(world, cams[1], base)
    plain = oracle.trace_shadow(world, cams[1], base, frame, g["t"], g["face"])
    cfg = vpt.default_config(width=W, height=H, primary_max_steps=256, alpha_test_shadows=1)
    tex["transparent"][:] = 0
    assert np.array_equal(oracle.trace_shadow(world, cams[1], cfg, frame, g["t"], g["face"], textures=tex), plain)
    tex["transparent"][:] = 1
    cut = oracle.trace_shadow(world, cams[1], cfg, frame, g["t"], g["face"], textures=tex)
    assert cut.sum() < plain.sum() and (cut <= plain).mean() > 0.9


@pytest.mark.gpu
@pytest.mark.parametrize("storage", [0, 1], ids=["f32", "f16"])
def test_alpha_tested_shadows_bit_exact(vpt, oracle, storage, gpu):
    vox, blocks, world, cams = scene(vpt, oracle, seed=2)
    tex = vpt.generate_block_textures(32, 5, seed=4)
    tex["transparent"][:] = (np.random.default_rng(2).random(128) < 0.6).astype(np.int32)
    frame = vpt.default_frame(frame_index=0, seed=3)
    with vpt.Context(width=W, height=H, primary_max_steps=256, storage=storage, alpha_test=1,
                     alpha_test_shadows=1) as ctx:
        ctx.upload_world(vox)
        ctx.set_block_table(blocks)
        ctx.build_df()
        ctx.set_block_textures(tex)
        cfg = ctx.config
        for k, cam in enumerate(cams):
            ctx.trace_primary(cam)
            ctx.trace_shadow(frame)
            g = oracle.trace_primary(world, cam, cfg, textures=tex)
            ref = oracle.trace_shadow(world, cam, cfg, frame, g["t"], g["face"], textures=tex)
            assert_same(ctx.read_plane("SHADOW")[..., 0] if ctx.read_plane("SHADOW").ndim == 3
                        else ctx.read_plane("SHADOW"), ref, f"cam {k} shadow")
            ctx.end_frame()
