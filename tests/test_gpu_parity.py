"""Parity of every libvpt pass with the CPU oracle, through the C ABI.

Traversal outputs (distance field, hit distance, face, block, hit voxel, step
count, shadow) must be bit-identical. The radiance and filter planes are also
held to bit-identity: libvpt and the oracle evaluate the same IEEE fp32
operations in the same order (no fused multiply-add, IEEE division and square
root, the same polynomial exp/log/sin/cos), so any difference is a bug. The
FP16-storage variant is compared against the oracle emulating half stores.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

W, H = 96, 64
DIMS = (64, 64, 64)   # X, Y, Z


def same_bits(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    if a.dtype == np.float16:
        a = a.astype(np.float32)
    if b.dtype == np.float16:
        b = b.astype(np.float32)
    if a.dtype.kind == "f":
        a32, b32 = a.astype(np.float32), b.astype(np.float32)
        eq = (a32.view(np.uint32) == b32.view(np.uint32)) | (np.isnan(a32) & np.isnan(b32))
        # +0 and -0 compare equal as values; only their sign bit differs
        eq |= (a32 == 0) & (b32 == 0)
        return eq
    return a == b


def assert_same(gpu, ref, what):
    gpu = np.asarray(gpu).reshape(np.asarray(ref).shape)
    eq = same_bits(gpu, ref)
    if not eq.all():
        bad = np.argwhere(~eq)
        g = gpu.astype(np.float64)
        r = np.asarray(ref).astype(np.float64)
        diff = np.nanmax(np.abs(g - r)[~eq]) if g.dtype.kind == "f" else None
        first = [tuple(int(v) for v in i) for i in bad[:5]]
        vals = [(float(g[tuple(i)]), float(r[tuple(i)])) for i in bad[:5]]
        pytest.fail(f"{what}: {len(bad)} of {eq.size} values differ; max |diff| {diff}; first {first} {vals}")


@pytest.fixture(scope="module")
def scene(vpt, oracle):
    X, Y, Z = DIMS
    vox = vpt.generate_world(X, Y, Z, seed=1)
    blocks = vpt.generate_block_table(100, seed=1)
    df = oracle.build_df(vox)
    yaw, pitch = vpt.seeded_pose(1)
    cam0 = vpt.camera_from_pose((X / 2, 58.0, Z / 2), yaw, pitch, 90.0, W / H)
    cam1 = vpt.camera_from_pose((X / 2 + 0.7, 58.2, Z / 2 - 0.4), yaw + 2.0, pitch + 1.0, 90.0, W / H)
    return {"vox": vox, "blocks": blocks, "df": df, "world": oracle.World(vox, df, blocks), "cams": [cam0, cam1]}


def make_ctx(vpt, scene, storage):
    ctx = vpt.Context(width=W, height=H, primary_max_steps=256, storage=storage)
    ctx.upload_world(scene["vox"])
    ctx.set_block_table(scene["blocks"])
    ctx.build_df()
    return ctx


def test_distance_field_bit_exact(vpt, oracle, scene, gpu):
    with make_ctx(vpt, scene, vpt.STORAGE_F32) as ctx:
        assert_same(ctx.read_df(), scene["df"], "distance field")


# shapes for both paths of the build: the 128-bit one (X % 16 == 0, X <= 1024:
# one to 32 rows per warp, lanes without a segment, two segments per lane,
# lines along y / z from 1 to 1536 voxels, tiles narrower than 64 bytes) and
# the generic one (other X, lines over 1536)
@pytest.mark.parametrize("dims", [(16, 16, 16), (37, 21, 50), (200, 40, 9), (1, 1, 1), (64, 1, 3), (48, 20, 30),
                                  (1024, 8, 6), (528, 5, 7), (80, 33, 17), (16, 1536, 2), (32, 3, 800),
                                  (2048, 2, 2), (96, 1537, 1), (272, 12, 12)])
def test_distance_field_shapes(vpt, oracle, dims, gpu):
    X, Y, Z = dims
    rng = np.random.default_rng(sum(dims))
    vox = (rng.random((Z, Y, X)) < 0.02).astype(np.uint8) * rng.integers(1, 200, (Z, Y, X)).astype(np.uint8)
    with vpt.Context(width=8, height=8) as ctx:
        ctx.upload_world(vox)
        ctx.set_block_table(vpt.generate_block_table(100, 0))
        ctx.build_df()
        assert_same(ctx.read_df(), oracle.build_df(vox), f"distance field {dims}")


def test_distance_field_empty_and_full(vpt, oracle, gpu):
    for fill in (0, 7):
        vox = np.full((20, 30, 40), fill, np.uint8)
        with vpt.Context(width=8, height=8) as ctx:
            ctx.upload_world(vox)
            ctx.set_block_table(vpt.generate_block_table(100, 0))
            ctx.build_df()
            got = ctx.read_df()
        assert_same(got, oracle.build_df(vox), f"distance field fill={fill}")
        assert (got == (0 if fill else min(254, 90))).all()


def check_passes_two_frames(vpt, oracle, scene, storage, fused, w=W, h=H, cams=None):
    """Every plane of every pass over two frames (the second reprojects the
    first), pass by pass against the oracle, at a w x h image."""
    world = scene["world"]
    cams = cams or scene["cams"]
    ctx = vpt.Context(width=w, height=h, primary_max_steps=256, storage=storage)
    ctx.upload_world(scene["vox"])
    ctx.set_block_table(scene["blocks"])
    ctx.build_df()
    ctx.set_tuning(fused_prefilter=fused)
    cfg = ctx.config
    prev_g, hist = oracle.empty_history(h, w)
    prev_cam = cams[0]
    for fi, cam in enumerate(cams):
        frame = vpt.default_frame(frame_index=fi, seed=11, time=1.3 + 0.37 * fi)
        ctx.trace_primary(cam)
        g = oracle.trace_primary(world, cam, cfg)
        for name, plane in (("t", "T"), ("face", "FACE"), ("block", "BLOCK"), ("hit", "HIT"), ("steps", "STEPS")):
            assert_same(ctx.read_plane(plane), g[name], f"frame {fi} primary {name}")
        ctx.trace_shadow(frame)
        shadow = oracle.trace_shadow(world, cam, cfg, frame, g["t"], g["face"])
        assert_same(ctx.read_plane("SHADOW"), shadow, f"frame {fi} shadow")
        ctx.trace_diffuse(frame)
        gi = oracle.trace_diffuse(world, cam, cfg, frame, g["t"], g["face"])
        for k in ("sh", "cocg", "luma", "aosky"):
            assert_same(ctx.read_plane("GI_" + k.upper()), gi[k], f"frame {fi} diffuse {k}")
        ctx.svgf(prev_cam, frame)
        sv = oracle.svgf(cam, prev_cam, cfg, frame, g, prev_g, gi, hist)
        for k in ("sh", "cocg", "luma", "aosky"):
            assert_same(ctx.read_plane("PRE_" + k.upper()), sv["pre"][k], f"frame {fi} pre-temporal {k}")
        for k in ("sh", "cocg", "util", "aosky"):
            assert_same(ctx.read_plane("TEMP_" + k.upper()), sv["temporal"][k], f"frame {fi} temporal {k}")
        for k in ("sh", "cocg", "variance"):
            assert_same(ctx.read_plane("VAR_" + k.upper()), sv["variance"][k], f"frame {fi} variance {k}")
        last = sv["atrous"][-1]
        for k in ("sh", "cocg", "variance", "aosky"):
            assert_same(ctx.read_plane("DEN_" + k.upper()), last[k], f"frame {fi} a-trous {k}")
        ctx.shade(frame)
        rgb = oracle.shade(world, cam, cfg, frame, g["t"], g["face"], g["block"], shadow, last["sh"], last["cocg"],
                           last["aosky"])
        assert_same(ctx.read_plane("COLOR"), rgb, f"frame {fi} colour")
        ctx.end_frame()
        prev_g = {"t": g["t"], "face": g["face"], "block": g["block"]}
        hist = sv["temporal"]
        prev_cam = cam
    ctx.close()


@pytest.mark.parametrize("fused", [False, True], ids=["split_prefilter", "fused_prefilter"])
@pytest.mark.parametrize("storage", [0, 1], ids=["f32", "f16"])
def test_passes_bit_exact_two_frames(vpt, oracle, scene, storage, fused, gpu):
    check_passes_two_frames(vpt, oracle, scene, storage, fused)


@pytest.mark.parametrize("size", [(101, 67), (45, 13), (7, 5), (1, 1)], ids=lambda s: f"{s[0]}x{s[1]}")
@pytest.mark.parametrize("storage", [0, 1], ids=["f32", "f16"])
def test_passes_bit_exact_ragged_sizes(vpt, oracle, scene, storage, size, gpu):
    """Images whose sides are no multiple of any block shape (the 16x16 trace
    tiles, the 16x32 staged diffuse blocks, the 32x8 filter blocks and their
    shared-memory neighbourhoods), down to a single texel: the border blocks'
    fallbacks and every image-edge test, pass by pass."""
    w, h = size
    X, Y, Z = DIMS
    yaw, pitch = vpt.seeded_pose(1)
    cams = [vpt.camera_from_pose((X / 2, 58.0, Z / 2), yaw, pitch, 90.0, w / h),
            vpt.camera_from_pose((X / 2 + 0.7, 58.2, Z / 2 - 0.4), yaw + 2.0, pitch + 1.0, 90.0, w / h)]
    check_passes_two_frames(vpt, oracle, scene, storage, False, w, h, cams)


TRACE_PLANES = [("t", "T"), ("face", "FACE"), ("block", "BLOCK"), ("hit", "HIT"), ("steps", "STEPS")]
GI_PLANES = ["sh", "cocg", "luma", "aosky"]


@pytest.mark.parametrize("storage,threshold,blocks,spp,bounces", [
    (0, 16, 0, 1, 1), (0, 1, 0, 1, 1), (0, 32, 3, 1, 1), (1, 16, 0, 1, 1), (0, 8, 0, 2, 2), (1, 24, 7, 2, 2)])
def test_fused_trace_frame_bit_exact(vpt, oracle, scene, storage, threshold, blocks, spp, bounces, gpu):
    """The persistent fused kernel writes the same G-buffer, shadow and GI
    planes as the oracle's three passes, for any refill threshold and grid size."""
    world = scene["world"]
    with vpt.Context(width=W, height=H, primary_max_steps=256, storage=storage, spp=spp, bounces=bounces) as ctx:
        ctx.upload_world(scene["vox"])
        ctx.set_block_table(scene["blocks"])
        ctx.build_df()
        ctx.set_tuning(refill_threshold=threshold, trace_blocks=blocks)
        for fi, cam in enumerate(scene["cams"]):
            frame = vpt.default_frame(frame_index=fi, seed=21)
            ctx.set_stats(True)
            ctx.trace_frame(cam, frame)
            stats = ctx.read_stats()
            cfg = ctx.config
            with oracle.Counting() as cnt:
                g = oracle.trace_primary(world, cam, cfg)
                shadow = oracle.trace_shadow(world, cam, cfg, frame, g["t"], g["face"])
                gi = oracle.trace_diffuse(world, cam, cfg, frame, g["t"], g["face"])
            for name, plane in TRACE_PLANES:
                assert_same(ctx.read_plane(plane), g[name], f"fused {name} frame {fi}")
            assert_same(ctx.read_plane("SHADOW"), shadow, f"fused shadow frame {fi}")
            for k in GI_PLANES:
                assert_same(ctx.read_plane("GI_" + k.upper()), gi[k], f"fused GI {k} frame {fi}")
            assert stats["rays"] == cnt.rays and stats["steps"] == cnt.steps
            ctx.end_frame()


@pytest.mark.parametrize("storage,bounces", [(0, 1), (0, 2), (1, 2)])
def test_diffuse_pass_bit_exact(vpt, oracle, scene, storage, bounces, gpu):
    """The diffuse pass at one sample (the staged kernel for one bounce, the
    per-texel kernel for two) writes the oracle's GI planes and counts its
    rays and steps."""
    world = scene["world"]
    with vpt.Context(width=W, height=H, primary_max_steps=256, storage=storage, bounces=bounces) as ctx:
        ctx.upload_world(scene["vox"])
        ctx.set_block_table(scene["blocks"])
        ctx.build_df()
        for fi, cam in enumerate(scene["cams"]):
            frame = vpt.default_frame(frame_index=fi, seed=29)
            ctx.trace_primary(cam)
            ctx.set_stats(True)
            ctx.trace_diffuse(frame)
            stats = ctx.read_stats()
            ctx.set_stats(False)
            cfg = ctx.config
            g = oracle.trace_primary(world, cam, cfg)
            with oracle.Counting() as cnt:
                gi = oracle.trace_diffuse(world, cam, cfg, frame, g["t"], g["face"])
            for k in GI_PLANES:
                assert_same(ctx.read_plane("GI_" + k.upper()), gi[k], f"bounces {bounces} GI {k} frame {fi}")
            for kind in ("diffuse", "bounce_shadow"):
                assert stats["rays"][kind] == cnt.rays[kind] and stats["steps"][kind] == cnt.steps[kind], kind
            ctx.end_frame()


@pytest.mark.parametrize("mode", ["passes", "fused", "overlap_shadow", "overlap_unsplit"])
def test_render_frame_matches_oracle(vpt, oracle, scene, mode, gpu):
    """Whole frames through vpt_render_frame: passes in line, the fused
    trace, the sun-shadow trace and the temporal history gather on the second
    stream (split_temporal), and the shadow alone there (the default)."""
    world = scene["world"]
    ctx = make_ctx(vpt, scene, vpt.STORAGE_F32)
    ctx.set_tuning(fused_trace=mode == "fused", overlap_shadow=mode.startswith("overlap"),
                   split_temporal=mode == "overlap_shadow")
    prev_g, hist = oracle.empty_history(H, W)
    prev_cam = scene["cams"][0]
    for fi, cam in enumerate(scene["cams"]):
        frame = vpt.default_frame(frame_index=fi, seed=3, time=0.5 * fi)
        rgb = ctx.render_frame(cam, frame)
        ref = oracle.render_frame(world, cam, prev_cam, ctx.config, frame, prev_g, hist)
        assert_same(rgb, ref["rgb"], f"render_frame {fi}")
        prev_g = {k: ref["g"][k] for k in ("t", "face", "block")}
        hist = ref["svgf"]["temporal"]
        prev_cam = cam
    ctx.close()


@pytest.mark.parametrize("iterations", [0, 1, 2, 3, 5])
def test_atrous_iteration_counts(vpt, oracle, scene, iterations, gpu):
    """Whole frames with 0 to 5 a-trous iterations (each count ends on a
    different step and ping-pong buffer): the final planes and the colour
    equal the oracle's."""
    world = scene["world"]
    with vpt.Context(width=W, height=H, primary_max_steps=256, atrous_iterations=iterations) as ctx:
        ctx.upload_world(scene["vox"])
        ctx.set_block_table(scene["blocks"])
        ctx.build_df()
        prev_g, hist = oracle.empty_history(H, W)
        prev_cam = scene["cams"][0]
        for fi, cam in enumerate(scene["cams"]):
            frame = vpt.default_frame(frame_index=fi, seed=7, time=0.25 * fi)
            rgb = ctx.render_frame(cam, frame)
            ref = oracle.render_frame(world, cam, prev_cam, ctx.config, frame, prev_g, hist)
            if iterations:
                last = ref["svgf"]["atrous"][-1]
                for k in ("sh", "cocg", "variance", "aosky"):
                    assert_same(ctx.read_plane("DEN_" + k.upper()), last[k], f"frame {fi} a-trous {k}")
            assert_same(rgb, ref["rgb"], f"frame {fi} colour")
            prev_g = {k: ref["g"][k] for k in ("t", "face", "block")}
            hist = ref["svgf"]["temporal"]
            prev_cam = cam


def test_render_frame_ragged_size(vpt, oracle, scene, gpu):
    """Whole frames at 101 x 67 with the default tuning (sun shadow on the
    second stream, staged diffuse trace, tiled filter steps)."""
    w, h = 101, 67
    X, Y, Z = DIMS
    yaw, pitch = vpt.seeded_pose(1)
    cams = [vpt.camera_from_pose((X / 2, 58.0, Z / 2), yaw, pitch, 90.0, w / h),
            vpt.camera_from_pose((X / 2 + 0.7, 58.2, Z / 2 - 0.4), yaw + 2.0, pitch + 1.0, 90.0, w / h)]
    world = scene["world"]
    with vpt.Context(width=w, height=h, primary_max_steps=256) as ctx:
        ctx.upload_world(scene["vox"])
        ctx.set_block_table(scene["blocks"])
        ctx.build_df()
        prev_g, hist = oracle.empty_history(h, w)
        prev_cam = cams[0]
        for fi, cam in enumerate(cams):
            frame = vpt.default_frame(frame_index=fi, seed=3, time=0.5 * fi)
            rgb = ctx.render_frame(cam, frame)
            ref = oracle.render_frame(world, cam, prev_cam, ctx.config, frame, prev_g, hist)
            assert_same(rgb, ref["rgb"], f"render_frame {fi}")
            prev_g = {k: ref["g"][k] for k in ("t", "face", "block")}
            hist = ref["svgf"]["temporal"]
            prev_cam = cam


@pytest.mark.parametrize("storage", [0, 1], ids=["f32", "f16"])
def test_plain_atrous_path_bit_exact(vpt, oracle, scene, storage, gpu):
    """The non-SVGF denoiser (temporal + 5x5 a-trous) over two frames."""
    world = scene["world"]
    ctx = vpt.Context(width=W, height=H, primary_max_steps=256, storage=storage, denoiser=vpt.DENOISER_ATROUS)
    ctx.upload_world(scene["vox"])
    ctx.set_block_table(scene["blocks"])
    ctx.build_df()
    cfg = ctx.config
    prev_g, hist = oracle.empty_history(H, W)
    prev_cam = scene["cams"][0]
    for fi, cam in enumerate(scene["cams"]):
        frame = vpt.default_frame(frame_index=fi, seed=5)
        rgb = ctx.render_frame(cam, frame)
        ref = oracle.render_frame(world, cam, prev_cam, cfg, frame, prev_g, hist)
        tmp = ref["svgf"]["temporal"]
        assert_same(ctx.read_plane("HIST_SH"), tmp["sh"], f"frame {fi} plain temporal sh")   # swapped by end_frame
        assert_same(ctx.read_plane("HIST_COCG"), tmp["cocg"], f"frame {fi} plain temporal cocg")
        assert_same(rgb, ref["rgb"], f"frame {fi} plain colour")
        prev_g = {k: ref["g"][k] for k in ("t", "face", "block")}
        hist = tmp
        prev_cam = cam
    ctx.close()


def test_primary_steps_cap_and_inside_solid(vpt, oracle, scene, gpu):
    """A camera buried in stone misses everywhere (InitialRayTraceFrag.glsl:322-335);
    a tiny step cap truncates every ray at the cap."""
    world = scene["world"]
    with make_ctx(vpt, scene, vpt.STORAGE_F32) as ctx:
        cam = vpt.camera_from_pose((10.5, 5.5, 10.5), 30.0, 10.0, 90.0, W / H)
        ctx.trace_primary(cam)
        assert (ctx.read_plane("T") == -1).all()
        assert (ctx.read_plane("STEPS") == 0).all()
    with vpt.Context(width=W, height=H, primary_max_steps=3) as ctx:
        ctx.upload_world(scene["vox"])
        ctx.set_block_table(scene["blocks"])
        ctx.build_df()
        cam = scene["cams"][0]
        ctx.trace_primary(cam)
        g = oracle.trace_primary(world, cam, ctx.config)
        assert_same(ctx.read_plane("STEPS"), g["steps"], "capped steps")
        assert_same(ctx.read_plane("HIT"), g["hit"], "capped hit voxel")
        assert ctx.read_plane("STEPS").max() <= 3


def test_detmath_device_equals_host(vpt, gpu):
    rng = np.random.default_rng(5)
    xs = {
        0: rng.uniform(-110, 90, 20000).astype(np.float32),
        1: rng.uniform(-160, 130, 20000).astype(np.float32),
        2: np.exp(rng.uniform(-100, 80, 20000)).astype(np.float32),
        3: rng.uniform(0, 3, 20000).astype(np.float32),
        4: rng.uniform(-50, 50, 20000).astype(np.float32),
        5: rng.uniform(-50, 50, 20000).astype(np.float32),
    }
    y = rng.uniform(-4, 140, 20000).astype(np.float32)
    for op, x in xs.items():
        host = vpt.detmath(op, x, y, on_device=False)
        dev = vpt.detmath(op, x, y, on_device=True)
        assert_same(dev, host, f"detmath op {op}")


def test_packed_pairs_device_equals_host(vpt, gpu):
    """The filters' packed fp32 pairs (two adds or multiplies per
    instruction) round every lane as the scalar operation does."""
    rng = np.random.default_rng(11)
    n = 50000

    def wide():
        return (rng.uniform(-1, 1, n) * np.exp2(rng.integers(-30, 30, n))).astype(np.float32)

    x, y = wide(), wide()
    for op, want in ((6, x * y), (7, x * y), (8, x + y), (9, x + y)):
        dev = vpt.detmath(op, x, y, on_device=True)
        assert_same(dev, want, f"packed op {op}")
        assert_same(vpt.detmath(op, x, y, on_device=False), want, f"host op {op}")
    e = rng.uniform(-110, 90, n).astype(np.float32)
    f = rng.uniform(-20, 0, n).astype(np.float32)
    f[::7] = e[::7]   # some pairs with a lane outside the polynomial's range
    for op in (10, 11):
        assert_same(vpt.detmath(op, e, f, on_device=True), vpt.detmath(0, e, on_device=False), f"packed exp op {op}")
    # the form for non-positive arguments (the filters' negated distances),
    # down to and beyond the polynomial's range, zeros of both signs and NaN
    en = -np.abs(e) * np.float32(1.2)
    fn = -np.abs(f)
    fn[::7] = en[::7]
    en[:4] = [0.0, -0.0, np.nan, -1e-40]
    fn[:4] = [-0.0, np.nan, -3.0, -104.5]
    for op in (16, 17):
        assert_same(vpt.detmath(op, en, fn, on_device=True), vpt.detmath(0, en, on_device=False),
                    f"packed non-positive exp op {op}")
    w = rng.uniform(0, 8, n).astype(np.float32)
    bad = []
    for op, b in ((12, y), (13, w), (14, w), (15, y)):
        d, h = vpt.detmath(op, x, b, on_device=True), vpt.detmath(op, x, b, on_device=False)
        if not same_bits(d, h).all():
            bad.append((op, int((~same_bits(d, h)).sum())))
    assert not bad, f"packed ops differing from the scalar operations (op, count): {bad}"


def test_stats_count_rays(vpt, oracle, scene, gpu):
    with make_ctx(vpt, scene, vpt.STORAGE_F32) as ctx:
        ctx.set_stats(True)
        cam = scene["cams"][0]
        frame = vpt.default_frame()
        ctx.trace_primary(cam)
        ctx.trace_shadow(frame)
        ctx.trace_diffuse(frame)
        s = ctx.read_stats()
        steps = ctx.read_plane("STEPS")
        assert s["rays"]["primary"] == W * H
        assert s["steps"]["primary"] == int(steps.astype(np.int64).sum())
        hits = int((ctx.read_plane("T") > 0).sum())
        assert s["rays"]["diffuse"] == hits   # 1 spp, 1 bounce: one GI ray per hit pixel
        assert 0 < s["rays"]["shadow"] <= hits
