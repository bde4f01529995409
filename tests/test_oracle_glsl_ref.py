"""The oracle against the reference's own shader code, compiled as C++.

oracle/build_glsl_ref.py takes ManhattanDistance{X,Y,Z}.comp,
InitialRayTraceFrag.glsl, ShadowRayTraceFrag.glsl, Spatial3x3Initial.glsl and
SVGF/{TemporalFilter,VarianceEstimate,SpatialFilter}.glsl, TemporalFilter.glsl
and AtrousSpatialFilter.glsl from the reference tree, rewrites only GLSL syntax
(qualifiers, swizzles, literals, interface variables) and compiles them with
GLSL's types and built-ins from oracle/glsl_compat.h into
oracle/_ref/libglsl_ref.so; oracle/glsl_ref.cpp runs them as the
reference's dispatches and draws do. Where they and the oracle take the same
inputs, every output must be bit-identical: the distance field of every
world, the primary G-buffer (hit distance, face id, block id), the sun
shadow, the pre-temporal 3x3 filter, the temporal pass over a moving camera,
the variance estimate and the five a-trous iterations of every texel, and
the non-SVGF denoiser's temporal pass and five a-trous iterations; and the
SH / YCoCg encoding of a diffuse sample and the bounce rays' Hammon BRDF
(DiffuseRayTraceFrag.glsl) and the decoding in the colour pass
(ColorPassFrag.glsl), function by function. That pins the oracle's restatement of those passes to the reference's
own code; the built-ins (normalize, texel fetch of R8 data, matrix times
vector) are the conventions the oracle fixes for them. Skipped where the
reference tree is absent (the GPU machines).
"""
import ctypes as C

import numpy as np
import pytest

import oracle
from oracle import build_glsl_ref, inputs


@pytest.fixture(scope="module")
def ref():
    if build_glsl_ref.build() is None or not build_glsl_ref.OUT.exists():
        pytest.skip("the reference tree (its shaders) is not present")
    L = C.CDLL(str(build_glsl_ref.OUT))
    P = C.c_void_p
    L.glslref_build_df.argtypes = [P, C.c_int, C.c_int, C.c_int, P]
    L.glslref_trace_primary.argtypes = [P, P, C.c_int, C.c_int, C.c_int, P, P, C.c_int, C.c_int, C.c_int,
                                        C.c_float, P, P, P]
    L.glslref_trace_shadow.argtypes = [P, P, C.c_int, C.c_int, C.c_int, P, P, C.c_int, C.c_int, P, P, P, P]
    L.glslref_spatial_initial.argtypes = [P, P, C.c_int, C.c_int] + [P] * 10
    L.glslref_variance.argtypes = [P, P, C.c_int, C.c_int] + [P] * 8
    L.glslref_atrous.argtypes = [C.c_int, C.c_int, C.c_int, C.c_float, C.c_float, C.c_float] + [P] * 11
    L.glslref_temporal.argtypes = [P] * 4 + [C.c_int] * 3 + [P] * 18
    L.glslref_plain_atrous.argtypes = [P] * 2 + [C.c_int] * 3 + [P] * 8
    L.glslref_plain_temporal.argtypes = [P] * 4 + [C.c_int] * 2 + [P] * 8
    L.glslref_sh_codec.argtypes = [C.c_int, C.c_int, P, P]
    L.glslref_diffuse_brdf.argtypes = [C.c_int, P, P]
    return L


def ref_df(L, vox):
    vox = np.ascontiguousarray(vox, np.uint8)
    Z, Y, X = vox.shape
    out = np.zeros_like(vox)
    L.glslref_build_df(vox.ctypes.data, X, Y, Z, out.ctypes.data)
    return out


def ref_primary(L, vox, df, cam, W, H, steps):
    Z, Y, X = vox.shape
    iv = np.ascontiguousarray(np.asarray(cam.inv_view, np.float32))
    ip = np.ascontiguousarray(np.asarray(cam.inv_proj, np.float32))
    t, n, b = (np.zeros((H, W), np.float32) for _ in range(3))
    L.glslref_trace_primary(vox.ctypes.data, df.ctypes.data, X, Y, Z, iv.ctypes.data, ip.ctypes.data, W, H, steps,
                            90.0, t.ctypes.data, n.ctypes.data, b.ctypes.data)
    return t, n, b


@pytest.mark.parametrize("dims", [(32, 32, 32), (64, 32, 96), (33, 17, 5), (1, 1, 1), (200, 3, 7)])
@pytest.mark.parametrize("fill", [0.0, 0.02, 0.3, 1.0])
def test_distance_field_equals_the_reference_shaders(ref, dims, fill):
    X, Y, Z = dims
    rng = np.random.default_rng(X * 131 + Y * 7 + Z + int(fill * 100))
    vox = ((rng.random((Z, Y, X)) < fill) * rng.integers(1, 128, (Z, Y, X))).astype(np.uint8)
    assert np.array_equal(ref_df(ref, vox), oracle.build_df(vox))


def test_distance_field_of_generated_worlds(ref):
    for seed, dims in ((0, (128, 64, 96)), (3, (64, 64, 64))):
        vox = inputs.generate_world(*dims, seed=seed)
        assert np.array_equal(ref_df(ref, vox), oracle.build_df(vox)), seed


@pytest.mark.parametrize("case", [
    # (world dims, seed, camera position, yaw / pitch offsets, W, H, step cap, rays that hit)
    ((64, 64, 64), 1, (32.0, 58.0, 32.0), (0.0, 0.0), 96, 64, 256, True),
    ((64, 64, 64), 1, (32.7, 58.2, 31.6), (2.0, 1.0), 80, 48, 256, True),
    ((128, 64, 96), 5, (40.5, 60.0, 50.25), (-35.0, -20.0), 72, 40, 350, True),
    ((64, 64, 64), 2, (10.5, 5.5, 10.5), (30.0, 10.0), 48, 32, 256, False),   # camera inside the terrain
    ((64, 64, 64), 1, (32.0, 58.0, 32.0), (0.0, 0.0), 64, 40, 3, False),      # step cap before any hit
])
def test_primary_gbuffer_equals_the_reference_shader(ref, case):
    dims, seed, pos, (dyaw, dpitch), W, H, steps, hits = case
    X, Y, Z = dims
    vox = inputs.generate_world(X, Y, Z, seed=seed)
    blocks = inputs.generate_block_table(100, seed=seed)
    df = oracle.build_df(vox)
    yaw, pitch = inputs.seeded_pose(seed)
    cam = inputs.camera_from_pose(pos, yaw + dyaw, pitch + dpitch, 90.0, W / H)
    cfg = inputs.default_config(width=W, height=H, primary_max_steps=steps)
    g = oracle.trace_primary(oracle.World(vox, df, blocks), cam, cfg)
    t, n, b = ref_primary(ref, vox, df, cam, W, H, steps)
    assert np.array_equal(t.view(np.uint32), g["t"].view(np.uint32)) or np.array_equal(t, g["t"])
    # o_Normal holds the face id / 10 (1.0 for a miss, the oracle's 10), o_BlockID the R8 block id / 255
    assert np.array_equal(np.rint(n * np.float32(10)).astype(np.int32), g["face"].astype(np.int32))
    assert np.array_equal(np.rint(b * np.float32(255)).astype(np.int32), g["block"].astype(np.int32))
    assert (t > 0).any() == hits


@pytest.mark.parametrize("sun", [(0.3, 0.8, 0.5), (0.9, 0.15, 0.3), (-0.5, 0.6, -0.6), (0.05, 0.99, -0.1)])
@pytest.mark.parametrize("seed", [1, 5])
def test_sun_shadow_equals_the_reference_shader(ref, sun, seed):
    """The reference's shadow pass reads the G-buffer its initial trace wrote
    (here the reference's own, equal to the oracle's by the test above)."""
    X, Y, Z = 64, 64, 64
    W, H = 80, 48
    vox = inputs.generate_world(X, Y, Z, seed=seed)
    blocks = inputs.generate_block_table(100, seed=seed)
    df = oracle.build_df(vox)
    yaw, pitch = inputs.seeded_pose(seed)
    cam = inputs.camera_from_pose((X / 2 + 0.3, 58.0, Z / 2 - 0.2), yaw, pitch, 90.0, W / H)
    cfg = inputs.default_config(width=W, height=H, primary_max_steps=256)
    frame = inputs.default_frame(frame_index=0, seed=3)
    s = np.asarray(sun, np.float64)
    frame.sun_dir[:] = [float(v) for v in (s / np.linalg.norm(s)).astype(np.float32)]
    world = oracle.World(vox, df, blocks)
    g = oracle.trace_primary(world, cam, cfg)
    t, n, _ = ref_primary(ref, vox, df, cam, W, H, 256)
    iv = np.ascontiguousarray(np.asarray(cam.inv_view, np.float32))
    ip = np.ascontiguousarray(np.asarray(cam.inv_proj, np.float32))
    light = np.ascontiguousarray(np.asarray(frame.sun_dir, np.float32))
    out = np.zeros((H, W), np.float32)
    ref.glslref_trace_shadow(vox.ctypes.data, df.ctypes.data, X, Y, Z, iv.ctypes.data, ip.ctypes.data, W, H,
                             t.ctypes.data, n.ctypes.data, light.ctypes.data, out.ctypes.data)
    want = oracle.trace_shadow(world, cam, cfg, frame, g["t"], g["face"])
    assert set(np.unique(out).tolist()) <= {0.0, 1.0}
    assert np.array_equal(out.astype(np.uint8), want)
    assert (want[g["t"] > 0] == 1).any()


def f32(a):
    return np.ascontiguousarray(a, np.float32)


def same(a, b):
    a, b = f32(a), f32(b)
    eq = (a.view(np.uint32) == b.view(np.uint32)) | ((a == 0) & (b == 0)) | (np.isnan(a) & np.isnan(b))
    return bool(eq.all())


@pytest.fixture(scope="module", params=[1, 5])
def gi_frame(request):
    """A traced frame (G-buffer and diffuse GI) and its SVGF intermediates."""
    seed = request.param
    X, Y, Z = 64, 64, 64
    W, H = 96, 64
    vox = inputs.generate_world(X, Y, Z, seed=seed)
    blocks = inputs.generate_block_table(100, seed=seed)
    df = oracle.build_df(vox)
    world = oracle.World(vox, df, blocks)
    yaw, pitch = inputs.seeded_pose(seed)
    cam = inputs.camera_from_pose((X / 2, 58.0, Z / 2), yaw, pitch, 90.0, W / H)
    cfg = inputs.default_config(width=W, height=H, primary_max_steps=256)
    frame = inputs.default_frame(frame_index=0, seed=11, time=1.3)
    g = oracle.trace_primary(world, cam, cfg)
    gi = oracle.trace_diffuse(world, cam, cfg, frame, g["t"], g["face"])
    prev_g, hist = oracle.empty_history(H, W)
    sv = oracle.svgf(cam, cam, cfg, frame, g, prev_g, gi, hist)
    # the face plane as the initial trace writes it (GetNormalID: k / 10, 1.0 for a miss)
    normal = np.array([np.float32(k) / np.float32(10) for k in range(11)], np.float32)[g["face"]]
    return dict(W=W, H=H, cam=cam, cfg=cfg, frame=frame, g=g, gi=gi, sv=sv, normal=normal,
                iv=f32(cam.inv_view), ip=f32(cam.inv_proj))


def test_pre_temporal_filter_equals_the_reference_shader(ref, gi_frame):
    F = gi_frame
    W, H, gi = F["W"], F["H"], F["gi"]
    want = oracle.spatial_initial(F["cam"], F["cfg"], F["g"]["t"], F["g"]["face"], gi)
    o = {"sh": np.zeros((H, W, 4), np.float32), "cocg": np.zeros((H, W, 2), np.float32),
         "aosky": np.zeros((H, W, 2), np.float32), "luma": np.zeros((H, W), np.float32)}
    ins = [f32(F["g"]["t"]), F["normal"], f32(gi["sh"]), f32(gi["cocg"]), f32(gi["aosky"]), f32(gi["luma"])]
    ref.glslref_spatial_initial(F["iv"].ctypes.data, F["ip"].ctypes.data, W, H, *[a.ctypes.data for a in ins],
                                *[o[k].ctypes.data for k in ("sh", "cocg", "aosky", "luma")])
    for k in o:
        assert same(o[k], want[k]), k


def test_variance_estimate_equals_the_reference_shader(ref, gi_frame):
    """Both branches: the accumulated-frame count of every texel drawn from
    young (< 12, the 81-tap estimate) and old histories."""
    F = gi_frame
    W, H = F["W"], F["H"]
    tmp = F["sv"]["temporal"]
    util = f32(tmp["util"]).copy()
    rng = np.random.default_rng(W + H)
    util[..., 0] = rng.choice(np.array([1, 2, 5, 11, 11.5, 12, 13, 30], np.float32), size=(H, W))
    want = oracle.variance(F["cam"], F["cfg"], F["g"]["t"], F["g"]["face"], dict(tmp, util=util))
    o = {"sh": np.zeros((H, W, 4), np.float32), "cocg": np.zeros((H, W, 2), np.float32),
         "variance": np.zeros((H, W), np.float32)}
    ins = [f32(F["g"]["t"]), F["normal"], f32(tmp["sh"]), f32(tmp["cocg"]), util]
    ref.glslref_variance(F["iv"].ctypes.data, F["ip"].ctypes.data, W, H, *[a.ctypes.data for a in ins],
                         *[o[k].ctypes.data for k in ("sh", "cocg", "variance")])
    for k in o:
        assert same(o[k], want[k]), k


@pytest.mark.parametrize("history", ["young", "old"])
def test_atrous_iterations_equal_the_reference_shader(ref, gi_frame, history):
    """The five iterations (steps 16, 8, 4, 2, 1: gathered taps at fractional
    offsets, jittered, with and without the AO / sky filter), each from the
    oracle's previous output; young histories take the strong spatial branch
    at steps <= 8, old ones the luminance weight at every step."""
    F = gi_frame
    W, H, sv = F["W"], F["H"], F["sv"]
    p = oracle.params(F["cfg"])
    util = f32(sv["temporal"]["util"]).copy()
    if history == "old":
        util[..., 0] = 30.0
    cur, ao = sv["variance"], sv["temporal"]["aosky"]
    for it in range(p.atrous_iterations):
        step = max(16 >> it, 1)
        want = oracle.atrous(F["cam"], F["cfg"], F["frame"], step, F["g"]["t"], F["g"]["face"], util, cur, ao)
        o = {"sh": np.zeros((H, W, 4), np.float32), "cocg": np.zeros((H, W, 2), np.float32),
             "variance": np.zeros((H, W), np.float32), "aosky": np.zeros((H, W, 2), np.float32)}
        ins = [f32(F["g"]["t"]), F["normal"], util, f32(cur["sh"]), f32(cur["cocg"]), f32(cur["variance"]), f32(ao)]
        ref.glslref_atrous(W, H, step, p.resolution_scale, p.color_phi_bias, F["frame"].time,
                           *[a.ctypes.data for a in ins], *[o[k].ctypes.data for k in ("sh", "cocg", "variance", "aosky")])
        for k in o:
            assert same(o[k], want[k]), (step, k)
        cur, ao = want, want["aosky"]


@pytest.mark.parametrize("seed", [1, 5])
def test_temporal_pass_equals_the_reference_shader(ref, seed):
    """Three frames: an empty history, a moved and turned camera (the history
    reprojected through the previous view-projection and sampled between
    texels), then the same camera again (reprojection onto the texel centres)."""
    X, Y, Z = 64, 64, 64
    W, H = 96, 64
    vox = inputs.generate_world(X, Y, Z, seed=seed)
    blocks = inputs.generate_block_table(100, seed=seed)
    world = oracle.World(vox, oracle.build_df(vox), blocks)
    yaw, pitch = inputs.seeded_pose(seed)
    cams = [inputs.camera_from_pose((X / 2, 58.0, Z / 2), yaw, pitch, 90.0, W / H),
            inputs.camera_from_pose((X / 2 + 0.7, 58.2, Z / 2 - 0.4), yaw + 2.0, pitch + 1.0, 90.0, W / H)]
    cfg = inputs.default_config(width=W, height=H, primary_max_steps=256)
    ids = np.array([np.float32(k) / np.float32(10) for k in range(11)], np.float32)
    prev_g, hist = oracle.empty_history(H, W)
    prev_cam = cams[0]
    reprojected = 0
    for fi, cam in enumerate(cams + [cams[1]]):
        frame = inputs.default_frame(frame_index=fi, seed=11, time=1.3 + 0.37 * fi)
        g = oracle.trace_primary(world, cam, cfg)
        gi = oracle.trace_diffuse(world, cam, cfg, frame, g["t"], g["face"])
        sv = oracle.svgf(cam, prev_cam, cfg, frame, g, prev_g, gi, hist)
        pre, want = sv["pre"], sv["temporal"]
        blk, pblk = (f32(b.astype(np.float32) / np.float32(255)) for b in (g["block"], prev_g["block"]))
        ins = [f32(g["t"]), ids[g["face"]], blk, f32(pre["sh"]), f32(pre["cocg"]), f32(pre["luma"]),
               f32(pre["aosky"]), f32(prev_g["t"]), ids[prev_g["face"]], pblk, f32(hist["sh"]), f32(hist["cocg"]),
               f32(hist["util"]), f32(hist["aosky"])]
        o = {"sh": np.zeros((H, W, 4), np.float32), "cocg": np.zeros((H, W, 2), np.float32),
             "util": np.zeros((H, W, 3), np.float32), "aosky": np.zeros((H, W, 2), np.float32)}
        mats = [f32(cam.inv_view), f32(cam.inv_proj), f32(prev_cam.view), f32(prev_cam.proj)]
        ref.glslref_temporal(*[m.ctypes.data for m in mats], W, H, int(frame.temporal), *[a.ctypes.data for a in ins],
                             *[o[k].ctypes.data for k in ("sh", "cocg", "util", "aosky")])
        assert same(o["sh"], want["sh"]) and same(o["cocg"], want["cocg"]), fi
        assert same(o["util"], f32(want["util"])[..., :3]) and same(o["aosky"], want["aosky"]), fi
        reprojected += int((f32(want["util"])[..., 0] > 1).sum())
        prev_g, hist, prev_cam = {k: g[k] for k in ("t", "face", "block")}, want, cam
    assert reprojected > 1000


@pytest.mark.parametrize("seed", [1, 5])
def test_plain_atrous_iterations_equal_the_reference_shader(ref, seed):
    """The non-SVGF denoiser's five a-trous iterations (steps 12, 8, 4, 2, 1,
    5 x 5 taps), each from the oracle's previous output."""
    X, Y, Z = 64, 64, 64
    W, H = 96, 64
    vox = inputs.generate_world(X, Y, Z, seed=seed)
    world = oracle.World(vox, oracle.build_df(vox), inputs.generate_block_table(100, seed=seed))
    yaw, pitch = inputs.seeded_pose(seed)
    cam = inputs.camera_from_pose((X / 2, 58.0, Z / 2), yaw, pitch, 90.0, W / H)
    cfg = inputs.default_config(width=W, height=H, primary_max_steps=256, denoiser=1)
    frame = inputs.default_frame(frame_index=0, seed=5)
    g = oracle.trace_primary(world, cam, cfg)
    gi = oracle.trace_diffuse(world, cam, cfg, frame, g["t"], g["face"])
    prev_g, hist = oracle.empty_history(H, W)
    out = oracle.plain_denoise(cam, cam, cfg, g, prev_g, gi, hist)
    ids = np.array([np.float32(k) / np.float32(10) for k in range(11)], np.float32)
    blk = f32(g["block"].astype(np.float32) / np.float32(255))
    iv, ip = f32(cam.inv_view), f32(cam.inv_proj)   # kept alive across the calls
    sh, cocg = out["temporal"]["sh"], out["temporal"]["cocg"]
    for it, want in enumerate(out["atrous"]):
        o_sh, o_cc = np.zeros((H, W, 4), np.float32), np.zeros((H, W, 2), np.float32)
        ins = [f32(g["t"]), ids[g["face"]], blk, f32(out["variance"]), f32(sh), f32(cocg)]
        ref.glslref_plain_atrous(iv.ctypes.data, ip.ctypes.data, W, H, (12, 8, 4, 2, 1)[it],
                                 *[a.ctypes.data for a in ins], o_sh.ctypes.data, o_cc.ctypes.data)
        assert same(o_sh, want["sh"]) and same(o_cc, want["cocg"]), it
        sh, cocg = want["sh"], want["cocg"]


@pytest.mark.parametrize("seed", [1, 5])
def test_plain_temporal_pass_equals_the_reference_shader(ref, seed):
    """The non-SVGF temporal pass (TemporalFilter.glsl in its diffuse mode)
    over an empty history, a moved camera and a repeated one."""
    X, Y, Z = 64, 64, 64
    W, H = 96, 64
    vox = inputs.generate_world(X, Y, Z, seed=seed)
    world = oracle.World(vox, oracle.build_df(vox), inputs.generate_block_table(100, seed=seed))
    yaw, pitch = inputs.seeded_pose(seed)
    cams = [inputs.camera_from_pose((X / 2, 58.0, Z / 2), yaw, pitch, 90.0, W / H),
            inputs.camera_from_pose((X / 2 + 0.7, 58.2, Z / 2 - 0.4), yaw + 2.0, pitch + 1.0, 90.0, W / H)]
    cfg = inputs.default_config(width=W, height=H, primary_max_steps=256, denoiser=1)
    prev_g, hist = oracle.empty_history(H, W)
    prev_cam = cams[0]
    blended = 0
    for fi, cam in enumerate(cams + [cams[1]]):
        frame = inputs.default_frame(frame_index=fi, seed=5)
        g = oracle.trace_primary(world, cam, cfg)
        gi = oracle.trace_diffuse(world, cam, cfg, frame, g["t"], g["face"])
        want = oracle.plain_denoise(cam, prev_cam, cfg, g, prev_g, gi, hist)["temporal"]
        o_sh, o_cc = np.zeros((H, W, 4), np.float32), np.zeros((H, W, 2), np.float32)
        mats = [f32(cam.inv_view), f32(cam.inv_proj), f32(prev_cam.view), f32(prev_cam.proj)]
        ins = [f32(g["t"]), f32(prev_g["t"]), f32(gi["sh"]), f32(gi["cocg"]), f32(hist["sh"]), f32(hist["cocg"])]
        ref.glslref_plain_temporal(*[m.ctypes.data for m in mats], W, H, *[a.ctypes.data for a in ins],
                                   o_sh.ctypes.data, o_cc.ctypes.data)
        assert same(o_sh, want["sh"]) and same(o_cc, want["cocg"]), fi
        blended += int((np.abs(f32(want["sh"]) - f32(gi["sh"])).sum(-1) > 0).sum())
        prev_g, hist, prev_cam = {k: g[k] for k in ("t", "face", "block")}, want, cam
    assert blended > 1000


def test_sh_encoding_and_decoding_equal_the_reference_shaders(ref):
    """IrridianceToSH and SHToIrridiance on 200,000 random radiances (four
    decades), unit directions and normals, against the oracle's own."""
    lib = oracle.lib()
    lib.vpto_sh_codec.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p]
    rng = np.random.default_rng(4)
    n = 200000
    rad = rng.random((n, 3)) * rng.choice([0.01, 1.0, 8.0, 100.0], (n, 1))
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    enc_in = f32(np.concatenate([rad, d], 1))
    got, want = np.zeros((n, 6), np.float32), np.zeros((n, 6), np.float32)
    ref.glslref_sh_codec(0, n, enc_in.ctypes.data, got.ctypes.data)
    lib.vpto_sh_codec(0, n, enc_in.ctypes.data, want.ctypes.data)
    assert same(got, want)
    dec_in = f32(np.concatenate([want, rng.normal(size=(n, 3))], 1))
    got3, want3 = np.zeros((n, 3), np.float32), np.zeros((n, 3), np.float32)
    ref.glslref_sh_codec(1, n, dec_in.ctypes.data, got3.ctypes.data)
    lib.vpto_sh_codec(1, n, dec_in.ctypes.data, want3.ctypes.data)
    assert same(got3, want3)


def test_bounce_brdf_equals_the_reference_shader(ref):
    """DiffuseRayBRDF / DiffuseHammon on 200,000 random normals, incident and
    new directions and roughnesses (0 and 1 included), against the oracle's."""
    lib = oracle.lib()
    lib.vpto_diffuse_brdf.argtypes = [C.c_int, C.c_void_p, C.c_void_p]
    rng = np.random.default_rng(6)
    n = 200000

    def unit():
        v = rng.normal(size=(n, 3))
        return v / np.linalg.norm(v, axis=1, keepdims=True)

    inp = np.concatenate([unit(), unit(), unit(), rng.random((n, 1))], 1).astype(np.float32)
    inp[::5, 9], inp[1::5, 9] = 0.0, 1.0
    inp = f32(inp)
    got, want = np.zeros(n, np.float32), np.zeros(n, np.float32)
    ref.glslref_diffuse_brdf(n, inp.ctypes.data, got.ctypes.data)
    lib.vpto_diffuse_brdf(n, inp.ctypes.data, want.ctypes.data)
    assert same(got, want)
    assert (want > 0).sum() > n // 4
