"""The diffuse GI on a grid coarser than the G-buffer.

The reference traces and denoises the GI at DiffuseTraceResolution =
DiffuseIndirectSuperSampleRes = 1/d of the G-buffer (d = 4 by default, 2 in
its higher presets, Core/Pipeline.cpp:72, :79, :1256-1282) and brings it back
to full resolution with the colour pass's joint-bilateral upscale
(ColorPassFrag.glsl:535-653). Covered here: the GI-grid reading of the
G-buffer, every GI pass, the upscale, the plane sizes and the guards of the
paths that need the two grids to coincide. Every plane is bit-identical to
the oracle.
"""
import ctypes as C

import numpy as np
import pytest

from test_gpu_parity import assert_same

W, H = 96, 64
DIMS = (64, 64, 64)


# ------------------------------------------------------------------ CPU --
def test_oracle_view_is_the_gbuffer_on_the_same_grid(oracle):
    rng = np.random.default_rng(0)
    t = rng.uniform(-1, 90, (16, 24)).astype(np.float32)
    face = rng.integers(0, 11, (16, 24)).astype(np.uint8)
    block = rng.integers(0, 100, (16, 24)).astype(np.uint8)
    cfg = oracle.OParams(width=24, height=16, gi_divisor=1)
    v = oracle.gi_view(cfg, t, face, block)
    assert np.array_equal(v["t"].view(np.uint32), t.view(np.uint32))
    assert np.array_equal(v["face"], face) and np.array_equal(v["block"], block)


@pytest.mark.parametrize("d", [2, 4])
def test_oracle_view_samples_texel_centres(oracle, d):
    """Bilinear depth at each GI texel centre (the 2x2 G-buffer texels around
    it, equal weights when d is even) and a nearest face / block from the
    texels under it."""
    rng = np.random.default_rng(d)
    Hf, Wf = 8 * d, 12 * d
    t = rng.uniform(0, 90, (Hf, Wf)).astype(np.float32)
    face = rng.integers(0, 6, (Hf, Wf)).astype(np.uint8)
    block = rng.integers(0, 100, (Hf, Wf)).astype(np.uint8)
    cfg = oracle.OParams(width=Wf, height=Hf, gi_divisor=d)
    v = oracle.gi_view(cfg, t, face, block)
    assert v["t"].shape == (8, 12)
    h = d // 2
    quad = (t[h - 1::d, h - 1::d].astype(np.float64) + t[h - 1::d, h::d] + t[h::d, h - 1::d] + t[h::d, h::d]) / 4
    assert np.allclose(v["t"], quad, rtol=1e-5, atol=1e-5)
    for name, plane in (("face", face), ("block", block)):
        cands = np.stack([plane[h - 1::d, h - 1::d], plane[h - 1::d, h::d], plane[h::d, h - 1::d], plane[h::d, h::d]])
        assert (cands == v[name][None]).any(axis=0).all(), name


def test_create_rejects_bad_gi_divisor(vpt):
    for w, h, d in ((97, 64, 2), (96, 66, 4), (96, 64, -1), (96, 64, 32)):
        cfg = vpt.default_config(width=w, height=h, gi_divisor=d)
        ctx = C.c_void_p()
        assert vpt.lib.vpt_create(C.byref(ctx), C.byref(cfg)) == vpt.ERR_INVALID_ARG, (w, h, d)


# ------------------------------------------------------------------ GPU --
@pytest.fixture(scope="module")
def scene(vpt, oracle):
    X, Y, Z = DIMS
    vox = vpt.generate_world(X, Y, Z, seed=1)
    blocks = vpt.generate_block_table(100, seed=1)
    df = oracle.build_df(vox)
    yaw, pitch = vpt.seeded_pose(1)
    cam0 = vpt.camera_from_pose((X / 2, 58.0, Z / 2), yaw, pitch, 90.0, W / H)
    cam1 = vpt.camera_from_pose((X / 2 + 0.7, 58.2, Z / 2 - 0.4), yaw + 2.0, pitch + 1.0, 90.0, W / H)
    return {"vox": vox, "blocks": blocks, "world": oracle.World(vox, df, blocks), "cams": [cam0, cam1]}


def make_ctx(vpt, scene, **kw):
    ctx = vpt.Context(width=W, height=H, primary_max_steps=256, **kw)
    ctx.upload_world(scene["vox"])
    ctx.set_block_table(scene["blocks"])
    ctx.build_df()
    return ctx


@pytest.mark.gpu
@pytest.mark.parametrize("d,storage", [(2, 0), (4, 0), (2, 1), (4, 1)], ids=["d2-f32", "d4-f32", "d2-f16", "d4-f16"])
def test_gi_grid_passes_bit_exact(vpt, oracle, scene, d, storage, gpu):
    world = scene["world"]
    ctx = make_ctx(vpt, scene, storage=storage, gi_divisor=d)
    cfg = ctx.config
    assert ctx.plane_dims("GI_SH") == (H // d, W // d) and ctx.plane_dims("T") == (H, W)
    assert ctx.plane_dims("COLOR") == (H, W) and ctx.plane_dims("DEN_AOSKY") == (H // d, W // d)
    prev_g, hist = oracle.empty_history(H, W, d)
    prev_cam = scene["cams"][0]
    for fi, cam in enumerate(scene["cams"]):
        frame = vpt.default_frame(frame_index=fi, seed=11, time=1.3 + 0.37 * fi)
        ctx.trace_primary(cam)
        g = oracle.trace_primary(world, cam, cfg)
        assert_same(ctx.read_plane("T"), g["t"], f"d={d} frame {fi} primary t")
        ctx.trace_shadow(frame)
        shadow = oracle.trace_shadow(world, cam, cfg, frame, g["t"], g["face"])
        assert_same(ctx.read_plane("SHADOW"), shadow, f"d={d} frame {fi} shadow")
        ctx.trace_diffuse(frame)
        view = oracle.gi_view(cfg, g["t"], g["face"], g["block"])
        gi = oracle.trace_diffuse(world, cam, cfg, frame, view["t"], view["face"])
        for k in ("sh", "cocg", "luma", "aosky"):
            assert_same(ctx.read_plane("GI_" + k.upper()), gi[k], f"d={d} frame {fi} diffuse {k}")
        ctx.svgf(prev_cam, frame)
        sv = oracle.svgf(cam, prev_cam, cfg, frame, g, prev_g, gi, hist)
        for k in ("sh", "cocg", "luma", "aosky"):
            assert_same(ctx.read_plane("PRE_" + k.upper()), sv["pre"][k], f"d={d} frame {fi} pre-temporal {k}")
        for k in ("sh", "cocg", "util", "aosky"):
            assert_same(ctx.read_plane("TEMP_" + k.upper()), sv["temporal"][k], f"d={d} frame {fi} temporal {k}")
        for k in ("sh", "cocg", "variance"):
            assert_same(ctx.read_plane("VAR_" + k.upper()), sv["variance"][k], f"d={d} frame {fi} variance {k}")
        last = sv["atrous"][-1]
        for k in ("sh", "cocg", "variance", "aosky"):
            assert_same(ctx.read_plane("DEN_" + k.upper()), last[k], f"d={d} frame {fi} a-trous {k}")
        ctx.shade(frame)
        rgb = oracle.shade(world, cam, cfg, frame, g["t"], g["face"], g["block"], shadow, last["sh"], last["cocg"],
                           last["aosky"])
        assert_same(ctx.read_plane("COLOR"), rgb, f"d={d} frame {fi} colour")
        ctx.end_frame()
        prev_g = {"t": g["t"], "face": g["face"], "block": g["block"]}
        hist = sv["temporal"]
        prev_cam = cam
    ctx.close()


@pytest.mark.gpu
@pytest.mark.parametrize("denoiser", [0, 1], ids=["svgf", "plain"])
def test_gi_grid_render_frame(vpt, oracle, scene, denoiser, gpu):
    """Whole frames at the reference's default quarter-resolution GI, with the
    fused-trace tuning asked for (it needs one grid, so the passes run)."""
    world = scene["world"]
    ctx = make_ctx(vpt, scene, gi_divisor=4, denoiser=denoiser)
    ctx.set_tuning(fused_trace=True)
    prev_g, hist = oracle.empty_history(H, W, 4)
    prev_cam = scene["cams"][0]
    for fi, cam in enumerate(scene["cams"]):
        frame = vpt.default_frame(frame_index=fi, seed=3, time=0.5 * fi)
        rgb = ctx.render_frame(cam, frame)
        ref = oracle.render_frame(world, cam, prev_cam, ctx.config, frame, prev_g, hist)
        assert np.isfinite(rgb).all()
        assert_same(rgb, ref["rgb"], f"render_frame {fi}")
        prev_g = {k: ref["g"][k] for k in ("t", "face", "block")}
        hist = ref["svgf"]["temporal"]
        prev_cam = cam
    with pytest.raises(vpt.VPTError):
        ctx.trace_frame(scene["cams"][0], vpt.default_frame())
    with pytest.raises(vpt.VPTError):
        ctx.learned_input(scene["cams"][0], vpt.default_frame())
    ctx.close()


@pytest.mark.gpu
def test_gi_grid_learned_falls_back_to_svgf(vpt, scene, gpu):
    """The learned denoiser works on the G-buffer's grid only; with a coarser
    GI grid vpt_render_frame_learned renders the SVGF frame."""
    net = vpt.UNet(1, H, W)
    a = make_ctx(vpt, scene, gi_divisor=2)
    b = make_ctx(vpt, scene, gi_divisor=2)
    for fi, cam in enumerate(scene["cams"]):
        frame = vpt.default_frame(frame_index=fi, seed=7)
        got, used = a.render_frame_learned(cam, frame, net)
        ref = b.render_frame(cam, frame)
        assert not used
        assert_same(got, ref, f"fallback frame {fi}")
    a.close()
    b.close()
    net.close()
