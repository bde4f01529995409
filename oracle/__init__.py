"""CPU oracle for the VoxelPathTracer hot path (ctypes binding).

TEST INFRASTRUCTURE ONLY. The oracle is a C++17 restatement of the reference
shaders (see vpt_oracle.h for the file list and vpt_oracle.cpp for the
per-function citations). Only the tests, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py use it, as the checker or as the timed CPU
baseline; the product (voxelpathtracer_gb300) never imports it.

Parity is unpinned by the reference itself (it has no tests, golden vectors
or CPU implementation of this path); the oracle is pinned by analytic
known-answer tests and brute-force cross-checks under tests/.

Struct layouts are byte-compatible with include/vpt.h, so any ctypes
structure of the same size (e.g. voxelpathtracer_gb300.Camera) is accepted.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "_build" / "libvpt_oracle.so"


class OCamera(C.Structure):
    _fields_ = [("view", C.c_float * 16), ("proj", C.c_float * 16), ("inv_view", C.c_float * 16),
                ("inv_proj", C.c_float * 16), ("position", C.c_float * 3), ("pad", C.c_float)]


class OFrame(C.Structure):
    _fields_ = [("sun_dir", C.c_float * 3), ("time", C.c_float), ("sun_radiance", C.c_float * 3),
                ("frame_index", C.c_uint32), ("moon_radiance", C.c_float * 3), ("seed", C.c_uint32),
                ("gi_sun_strength", C.c_float), ("gi_sky_strength", C.c_float),
                ("diffuse_light_intensity", C.c_float), ("temporal", C.c_int32)]


class OParams(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("primary_max_steps", C.c_int32),
                ("shadow_max_steps", C.c_int32), ("diffuse_max_steps", C.c_int32),
                ("bounce_shadow_max_steps", C.c_int32), ("bounces", C.c_int32), ("spp", C.c_int32),
                ("storage", C.c_int32), ("atrous_iterations", C.c_int32), ("resolution_scale", C.c_float),
                ("color_phi_bias", C.c_float), ("device", C.c_int32), ("denoiser", C.c_int32),
                ("gi_divisor", C.c_int32), ("reflection_spp", C.c_int32), ("reflection_max_steps", C.c_int32),
                ("reflection_shadow_max_steps", C.c_int32), ("reflection_temporal", C.c_int32),
                ("reflection_denoise", C.c_int32), ("alpha_test", C.c_int32), ("alpha_test_shadows", C.c_int32),
                ("reserved", C.c_int32 * 1)]


class OWorld(C.Structure):
    _fields_ = [("vox", C.c_void_p), ("df", C.c_void_p), ("X", C.c_int32), ("Y", C.c_int32), ("Z", C.c_int32),
                ("blocks", C.c_void_p), ("n_blocks", C.c_int32)]


class OGBuffer(C.Structure):
    _fields_ = [("t", C.c_void_p), ("face", C.c_void_p), ("block", C.c_void_p), ("hit", C.c_void_p),
                ("steps", C.c_void_p)]


class OPlanes4(C.Structure):   # vpto_gi / vpto_history / vpto_filtered share this shape
    _fields_ = [("a", C.c_void_p), ("b", C.c_void_p), ("c", C.c_void_p), ("d", C.c_void_p)]


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            import importlib.util
            build_py = LIB_PATH.parent.parent.parent / "voxelpathtracer_gb300" / "_build.py"
            spec = importlib.util.spec_from_file_location("vpt_build", build_py)
            mod = importlib.util.module_from_spec(spec)
            spec.loader.exec_module(mod)
            mod.build_oracle()
        L = C.CDLL(str(LIB_PATH))
        P = C.c_void_p
        L.vpto_build_df.argtypes = [P, C.c_int, C.c_int, C.c_int, P]
        L.vpto_trace_primary.argtypes = [P, P, P, C.c_int, C.c_int, P]
        L.vpto_trace_shadow.argtypes = [P, P, P, P, P, P, C.c_int, C.c_int, P]
        L.vpto_trace_diffuse.argtypes = [P, P, P, P, P, P, C.c_int, C.c_int, P]
        L.vpto_spatial_initial.argtypes = [P, P, P, P, P, P]
        L.vpto_temporal.argtypes = [P, P, P, P, P, P, P, P, P, P, P, P, P]
        L.vpto_variance.argtypes = [P, P, P, P, P, P]
        L.vpto_reproject.argtypes = [P, P, C.c_int, C.c_int, P, P, P]
        L.vpto_vecmath.argtypes = [C.c_int, P, P, P, P, C.c_int]
        L.vpto_check_div_const.argtypes = [C.c_float, C.c_uint32, C.c_uint32]
        L.vpto_check_div_const.restype = C.c_uint64
        L.vpto_atrous.argtypes = [P, P, P, C.c_int, P, P, P, P, P, P, P, P]
        L.vpto_gi_view.argtypes = [P, P, P, P, P, P, P]
        L.vpto_shade.argtypes = [P, P, P, P, P, P, P, P, P, P, P, P, C.c_int, C.c_int, P]
        L.vpto_trace_reflection.argtypes = [P] * 13 + [C.c_int, C.c_int, P, P, P]
        L.vpto_spec_hit_blur.argtypes = [P, C.c_int, P, P, P, P]
        L.vpto_spec_temporal.argtypes = [P] * 18
        L.vpto_spec_denoise.argtypes = [P, P, P, C.c_int] + [P] * 10
        for name in ("vpto_exp", "vpto_exp2", "vpto_log2", "vpto_sin", "vpto_cos", "vpto_half_round"):
            getattr(L, name).argtypes = [C.c_float]
            getattr(L, name).restype = C.c_float
        L.vpto_pow.argtypes = [C.c_float, C.c_float]
        L.vpto_pow.restype = C.c_float
        L.vpto_omp_threads.restype = C.c_int
        L.vpto_set_counters.argtypes = [P]
        L.vpto_plain_temporal.argtypes = [P, P, P, P, P, P, P, P]
        L.vpto_plain_variance.argtypes = [P, P, P]
        L.vpto_plain_atrous.argtypes = [P, P, C.c_int, P, P, P, P, P, P, P, P, P]
        L.vpto_ground_truth.argtypes = [P, P, P, P, P, P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                        C.c_uint32, P, P]
        L.vpto_generate_gbuffer.argtypes = [P, P, P, P, P, P, P, P, P, P]
        L.vpto_set_block_textures.argtypes = [P]
        L.vpto_set_textured_gbuffer.argtypes = [P, P, C.c_int, C.c_int]
        L.vpto_shade_textured.argtypes = [P, P, P, P, P, P, P, P, P, P, P, P, C.c_int, C.c_int, P, P, P, P, P]
        _lib = L
    return _lib


def _p(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def _as(cls, obj):
    if isinstance(obj, cls):
        return obj
    if C.sizeof(obj) != C.sizeof(cls):
        raise TypeError(f"{type(obj).__name__} is not layout-compatible with {cls.__name__}")
    return cls.from_buffer_copy(bytes(memoryview(obj)))


def omp_threads() -> int:
    return lib().vpto_omp_threads()


class Counting:
    """Context manager that counts the oracle's rays and DDA steps."""

    KINDS = ("primary", "shadow", "diffuse", "bounce_shadow", "reflection", "reflection_shadow")

    def __enter__(self):
        self.buf = np.zeros(12, dtype=np.uint64)
        lib().vpto_set_counters(_p(self.buf))
        return self

    def __exit__(self, *exc):
        lib().vpto_set_counters(None)

    @property
    def rays(self) -> dict:
        return {k: int(v) for k, v in zip(self.KINDS, self.buf[:6])}

    @property
    def steps(self) -> dict:
        return {k: int(v) for k, v in zip(self.KINDS, self.buf[6:])}


def build_df(vox: np.ndarray) -> np.ndarray:
    v = np.ascontiguousarray(vox, dtype=np.uint8)
    Z, Y, X = v.shape
    df = np.empty_like(v)
    lib().vpto_build_df(_p(v), X, Y, Z, _p(df))
    return df


class World:
    """Voxels + distance field + block table, kept alive for the C calls."""

    def __init__(self, vox: np.ndarray, df: np.ndarray, blocks: np.ndarray):
        self.vox = np.ascontiguousarray(vox, dtype=np.uint8)
        self.df = np.ascontiguousarray(df, dtype=np.uint8)
        self.blocks = np.ascontiguousarray(blocks)
        Z, Y, X = self.vox.shape
        self.s = OWorld(self.vox.ctypes.data, self.df.ctypes.data, X, Y, Z, self.blocks.ctypes.data,
                        int(self.blocks.size))


def params(config) -> OParams:
    return _as(OParams, config)


def gi_dims(config) -> tuple:
    """(height, width) of the GI planes: the G-buffer's over gi_divisor."""
    p = params(config)
    d = max(int(p.gi_divisor), 1)
    return p.height // d, p.width // d


def gi_view(config, t, face, block) -> dict:
    """The G-buffer read at the GI grid's texel centres (vpto_gi_view)."""
    p = params(config)
    Hg, Wg = gi_dims(p)
    out = {"t": np.zeros((Hg, Wg), np.float32), "face": np.zeros((Hg, Wg), np.uint8),
           "block": np.zeros((Hg, Wg), np.uint8)}
    arrs = [np.ascontiguousarray(a, dtype=dt) for a, dt in ((t, np.float32), (face, np.uint8), (block, np.uint8))]
    lib().vpto_gi_view(C.byref(p), *[_p(a) for a in arrs], _p(out["t"]), _p(out["face"]), _p(out["block"]))
    return out


def _planes(H, W, spec):
    return {k: np.zeros((H, W, c) if c > 1 else (H, W), dtype=dt) for k, (c, dt) in spec.items()}


def trace_primary(world: World, cam, config, rows=None, textures=None) -> dict:
    """The primary G-buffer; with config.alpha_test and block textures, the
    alpha-tested traversal."""
    p = params(config)
    H, W = p.height, p.width
    g = _planes(H, W, {"t": (1, np.float32), "face": (1, np.uint8), "block": (1, np.uint8),
                       "hit": (3, np.int32), "steps": (1, np.uint16)})
    r0, r1 = rows if rows else (0, H)
    gb = OGBuffer(_p(g["t"]), _p(g["face"]), _p(g["block"]), _p(g["hit"]), _p(g["steps"]))
    keep = _set_textures(textures)
    try:
        lib().vpto_trace_primary(C.byref(world.s), C.byref(_as(OCamera, cam)), C.byref(p), r0, r1, C.byref(gb))
    finally:
        lib().vpto_set_block_textures(None)
    del keep
    return g


def trace_shadow(world: World, cam, config, frame, t, face, rows=None, textures=None) -> np.ndarray:
    """Sun shadow; with config.alpha_test_shadows and block textures, alpha-tested rays."""
    p = params(config)
    H, W = p.height, p.width
    out = np.zeros((H, W), dtype=np.uint8)
    t = np.ascontiguousarray(t, dtype=np.float32)
    face = np.ascontiguousarray(face, dtype=np.uint8)
    r0, r1 = rows if rows else (0, H)
    keep = _set_textures(textures)
    try:
        lib().vpto_trace_shadow(C.byref(world.s), C.byref(_as(OCamera, cam)), C.byref(p),
                                C.byref(_as(OFrame, frame)), _p(t), _p(face), r0, r1, _p(out))
    finally:
        lib().vpto_set_block_textures(None)
    del keep
    return out


GI_SPEC = {"sh": (4, np.float32), "cocg": (2, np.float32), "luma": (1, np.float32), "aosky": (2, np.float32)}
HIST_SPEC = {"sh": (4, np.float32), "cocg": (2, np.float32), "util": (4, np.float32), "aosky": (2, np.float32)}
FILT_SPEC = {"sh": (4, np.float32), "cocg": (2, np.float32), "variance": (1, np.float32), "aosky": (2, np.float32)}


def _struct4(d, keys):
    return OPlanes4(*[_p(d[k]) if d.get(k) is not None else None for k in keys])


def _f32(d, keys):
    return {k: np.ascontiguousarray(d[k], dtype=np.float32) for k in keys if d.get(k) is not None}


def trace_diffuse(world: World, cam, config, frame, t, face, rows=None, textures=None) -> dict:
    """Diffuse GI on the GI grid; t and face are the G-buffer's GI-grid view;
    textures (a block-texture dict) textures the bounce hits."""
    p = params(config)
    H, W = gi_dims(p)
    out = _planes(H, W, GI_SPEC)
    t = np.ascontiguousarray(t, dtype=np.float32)
    face = np.ascontiguousarray(face, dtype=np.uint8)
    r0, r1 = rows if rows else (0, H)
    s = _struct4(out, ["sh", "cocg", "luma", "aosky"])
    keep = _set_textures(textures)
    try:
        lib().vpto_trace_diffuse(C.byref(world.s), C.byref(_as(OCamera, cam)), C.byref(p),
                                 C.byref(_as(OFrame, frame)), _p(t), _p(face), r0, r1, C.byref(s))
    finally:
        lib().vpto_set_block_textures(None)
    del keep
    return out


def spatial_initial(cam, config, t, face, gi: dict) -> dict:
    p = params(config)
    out = _planes(*gi_dims(p), GI_SPEC)
    gi = _f32(gi, ["sh", "cocg", "luma", "aosky"])
    t = np.ascontiguousarray(t, dtype=np.float32)
    face = np.ascontiguousarray(face, dtype=np.uint8)
    sin, sout = _struct4(gi, ["sh", "cocg", "luma", "aosky"]), _struct4(out, ["sh", "cocg", "luma", "aosky"])
    lib().vpto_spatial_initial(C.byref(_as(OCamera, cam)), C.byref(p), _p(t), _p(face), C.byref(sin), C.byref(sout))
    return out


def temporal(cam, prev_cam, config, frame, t, face, block, prev_t, prev_face, prev_block, cur: dict,
             hist: dict) -> dict:
    p = params(config)
    out = _planes(*gi_dims(p), HIST_SPEC)
    cur = _f32(cur, ["sh", "cocg", "luma", "aosky"])
    hist = _f32(hist, ["sh", "cocg", "util", "aosky"])
    arrs = [np.ascontiguousarray(a, dtype=dt) for a, dt in
            ((t, np.float32), (face, np.uint8), (block, np.uint8), (prev_t, np.float32), (prev_face, np.uint8),
             (prev_block, np.uint8))]
    sc, sh_, so = (_struct4(cur, ["sh", "cocg", "luma", "aosky"]), _struct4(hist, ["sh", "cocg", "util", "aosky"]),
                   _struct4(out, ["sh", "cocg", "util", "aosky"]))
    lib().vpto_temporal(C.byref(_as(OCamera, cam)), C.byref(_as(OCamera, prev_cam)), C.byref(p),
                        C.byref(_as(OFrame, frame)), *[_p(a) for a in arrs], C.byref(sc), C.byref(sh_), C.byref(so))
    return out


def vecmath(op: int, a, b, c) -> np.ndarray:
    """The oracle's dot / cross / length / normalize / mix / mat4*vec4 (op 0..5)
    over arrays of inputs (n x 3, or n x 16 and n x 4 for op 5)."""
    a = np.ascontiguousarray(a, np.float32)
    b = np.ascontiguousarray(b, np.float32)
    c = np.ascontiguousarray(c, np.float32)
    n = a.shape[0]
    out = np.zeros((n, 4 if op == 5 else 3), np.float32)
    lib().vpto_vecmath(op, _p(a), _p(b), _p(c), _p(out), n)
    return out


def reproject(cam, prev_cam, t) -> tuple:
    """(world position (H, W, 3), previous texture coordinate (H, W, 2)) of every
    texel of the hit-distance plane t, as the temporal pass computes them."""
    t = np.ascontiguousarray(t, dtype=np.float32)
    H, W = t.shape
    pos = np.zeros((H, W, 3), np.float32)
    uv = np.zeros((H, W, 2), np.float32)
    lib().vpto_reproject(C.byref(_as(OCamera, cam)), C.byref(_as(OCamera, prev_cam)), W, H, _p(t), _p(pos), _p(uv))
    return pos, uv


def variance(cam, config, t, face, temporal_out: dict) -> dict:
    p = params(config)
    out = _planes(*gi_dims(p), {k: v for k, v in FILT_SPEC.items() if k != "aosky"})
    h = _f32(temporal_out, ["sh", "cocg", "util", "aosky"])
    t = np.ascontiguousarray(t, dtype=np.float32)
    face = np.ascontiguousarray(face, dtype=np.uint8)
    si, so = _struct4(h, ["sh", "cocg", "util", "aosky"]), _struct4(out, ["sh", "cocg", "variance", "aosky"])
    lib().vpto_variance(C.byref(_as(OCamera, cam)), C.byref(p), _p(t), _p(face), C.byref(si), C.byref(so))
    return out


def atrous(cam, config, frame, step, t, face, temporal_util, filt_in: dict, aosky_in, t_view=None,
           face_view=None) -> dict:
    """t / face: the full-resolution G-buffer; t_view / face_view: its GI-grid
    view (the same planes when the grids coincide)."""
    p = params(config)
    out = _planes(*gi_dims(p), FILT_SPEC)
    fi = _f32(filt_in, ["sh", "cocg", "variance"])
    ao = np.ascontiguousarray(aosky_in, dtype=np.float32)
    tu = np.ascontiguousarray(temporal_util, dtype=np.float32)
    t = np.ascontiguousarray(t, dtype=np.float32)
    face = np.ascontiguousarray(face, dtype=np.uint8)
    tv = t if t_view is None else np.ascontiguousarray(t_view, dtype=np.float32)
    fv = face if face_view is None else np.ascontiguousarray(face_view, dtype=np.uint8)
    si, so = _struct4(fi, ["sh", "cocg", "variance", "aosky"]), _struct4(out, ["sh", "cocg", "variance", "aosky"])
    lib().vpto_atrous(C.byref(_as(OCamera, cam)), C.byref(p), C.byref(_as(OFrame, frame)), int(step), _p(t),
                      _p(face), _p(tv), _p(fv), _p(tu), C.byref(si), _p(ao), C.byref(so))
    return out


class OBlockTextures(C.Structure):   # vpto_block_textures
    _fields_ = [("size", C.c_int32), ("albedo", C.c_void_p), ("albedo_layers", C.c_int32),
                ("normal", C.c_void_p), ("normal_layers", C.c_int32), ("pbr", C.c_void_p),
                ("pbr_layers", C.c_int32), ("emissive", C.c_void_p), ("emissive_layers", C.c_int32),
                ("albedo_id", C.c_int32 * 128), ("normal_id", C.c_int32 * 128), ("pbr_id", C.c_int32 * 128),
                ("emissive_id", C.c_int32 * 128), ("grass", C.c_int32 * 10), ("transparent", C.c_int32 * 128)]


def _block_textures(textures: dict):
    """(vpto_block_textures, the arrays it points into) for a texture dict."""
    keep = {k: np.ascontiguousarray(textures[k], np.uint8) for k in ("albedo", "normal", "pbr")}
    if textures.get("emissive") is not None:
        keep["emissive"] = np.ascontiguousarray(textures["emissive"], np.uint8)
    bt = OBlockTextures()
    bt.size = int(textures["size"])
    for k, arr in keep.items():
        setattr(bt, k, arr.ctypes.data)
        setattr(bt, f"{k}_layers", int(arr.shape[0]))
    for k in ("albedo_id", "normal_id", "pbr_id", "emissive_id"):
        getattr(bt, k)[:] = [int(v) for v in np.asarray(textures[k], np.int64)[:128]]
    bt.grass[:] = [int(v) for v in np.asarray(textures["grass"], np.int64)[:10]]
    if textures.get("transparent") is not None:
        bt.transparent[:] = [int(v) for v in np.asarray(textures["transparent"], np.int64)[:128]]
    return bt, keep


def _set_textures(textures):
    """Sets (or clears, for None) the oracle's bounce-hit textures; returns what must stay alive."""
    if textures is None:
        lib().vpto_set_block_textures(None)
        return None
    bt, keep = _block_textures(textures)
    lib().vpto_set_block_textures(C.byref(bt))   # copies the texels
    return keep


def generate_gbuffer(cam, config, textures: dict, t, face, block) -> dict:
    """The textured G-buffer pass (GenerateGBuffer.glsl main) over the
    G-buffer t / face / block with the block textures (a dict as
    generate_block_textures makes): albedo (3), normal (3), pbr (4), ao."""
    p = params(config)
    H, W = p.height, p.width
    bt, keep = _block_textures(textures)
    out = {"albedo": np.zeros((H, W, 3), np.float32), "normal": np.zeros((H, W, 3), np.float32),
           "pbr": np.zeros((H, W, 4), np.float32), "ao": np.zeros((H, W), np.float32)}
    ts, fs, bs = (np.ascontiguousarray(a, dtype=dt) for a, dt in ((t, np.float32), (face, np.uint8),
                                                                  (block, np.uint8)))
    lib().vpto_generate_gbuffer(C.byref(_as(OCamera, cam)), C.byref(p), C.byref(bt), _p(ts), _p(fs), _p(bs),
                                _p(out["albedo"]), _p(out["normal"]), _p(out["pbr"]), _p(out["ao"]))
    return out


def shade(world: World, cam, config, frame, t, face, block, shadow, sh, cocg, aosky, rows=None,
          spec=None, gbt=None) -> np.ndarray:
    """The colour pass; spec is the resolved reflection (GI grid, 4 ch) or None;
    gbt the textured G-buffer (generate_gbuffer's planes) or None for flat materials."""
    p = params(config)
    H, W = p.height, p.width
    out = np.zeros((H, W, 3), dtype=np.float32)
    arrs = [np.ascontiguousarray(a, dtype=dt) for a, dt in
            ((t, np.float32), (face, np.uint8), (block, np.uint8), (shadow, np.uint8), (sh, np.float32),
             (cocg, np.float32), (aosky, np.float32))]
    sp = None if spec is None else np.ascontiguousarray(spec, dtype=np.float32)
    r0, r1 = rows if rows else (0, H)
    if gbt is None:
        lib().vpto_shade(C.byref(world.s), C.byref(_as(OCamera, cam)), C.byref(p), C.byref(_as(OFrame, frame)),
                         *[_p(a) for a in arrs], None if sp is None else _p(sp), r0, r1, _p(out))
    else:
        gb = [np.ascontiguousarray(gbt[k], dtype=np.float32) for k in ("albedo", "normal", "pbr", "ao")]
        lib().vpto_shade_textured(C.byref(world.s), C.byref(_as(OCamera, cam)), C.byref(p),
                                  C.byref(_as(OFrame, frame)), *[_p(a) for a in arrs], None if sp is None else _p(sp),
                                  r0, r1, _p(out), *[_p(a) for a in gb])
    return out


def trace_reflection(world: World, cam, config, frame, g: dict, shadow, den: dict, rows=None) -> dict:
    """The reflection trace on the GI grid from the full G-buffer g, the sun
    shadow and the denoised diffuse GI den (sh, cocg, aosky); returns spec
    (4 ch), hit and mask."""
    p = params(config)
    H, W = gi_dims(p)
    v = gi_view(p, g["t"], g["face"], g["block"])
    out = {"spec": np.zeros((H, W, 4), np.float32), "hit": np.zeros((H, W), np.float32),
           "mask": np.zeros((H, W), np.float32)}
    arrs = [np.ascontiguousarray(a, dtype=dt) for a, dt in
            ((g["t"], np.float32), (g["face"], np.uint8), (shadow, np.uint8), (v["t"], np.float32),
             (v["face"], np.uint8), (v["block"], np.uint8), (den["sh"], np.float32), (den["cocg"], np.float32),
             (den["aosky"], np.float32))]
    r0, r1 = rows if rows else (0, H)
    lib().vpto_trace_reflection(C.byref(world.s), C.byref(_as(OCamera, cam)), C.byref(p),
                                C.byref(_as(OFrame, frame)), *[_p(a) for a in arrs], r0, r1, _p(out["spec"]),
                                _p(out["hit"]), _p(out["mask"]))
    return out


def spec_hit_blur(config, g: dict, hit) -> np.ndarray:
    """The two bilateral passes over the reflection hit distance."""
    p = params(config)
    v = gi_view(p, g["t"], g["face"], g["block"])
    h0 = np.ascontiguousarray(hit, dtype=np.float32)
    h1, h2 = np.zeros_like(h0), np.zeros_like(h0)
    lib().vpto_spec_hit_blur(C.byref(p), 1, _p(v["t"]), _p(v["face"]), _p(h0), _p(h1))
    lib().vpto_spec_hit_blur(C.byref(p), 2, _p(v["t"]), _p(v["face"]), _p(h1), _p(h2))
    return h2


def empty_reflection_history(config) -> dict:
    """The reflection state libvpt starts from: zero planes on the GI grid."""
    H, W = gi_dims(config)
    return {"out": np.zeros((H, W, 4), np.float32), "hit": np.zeros((H, W), np.float32),
            "stable": np.zeros((H, W), np.float32)}


def spec_temporal(world: World, cam, prev_cam, config, g: dict, prev_g: dict, refl: dict, prev_refl: dict) -> dict:
    """SpecularTemporalFilter: refl holds this frame's spec, (blurred) hit and
    mask, prev_refl last frame's out, hit and stable; returns out, acc, stable."""
    p = params(config)
    H, W = gi_dims(p)
    v = gi_view(p, g["t"], g["face"], g["block"])
    out = {"out": np.zeros((H, W, 4), np.float32), "acc": np.zeros((H, W), np.float32),
           "stable": np.zeros((H, W), np.float32)}
    arrs = [np.ascontiguousarray(a, dtype=dt) for a, dt in
            ((v["t"], np.float32), (v["face"], np.uint8), (v["block"], np.uint8), (prev_g["t"], np.float32),
             (prev_g["face"], np.uint8), (refl["spec"], np.float32), (refl["hit"], np.float32),
             (refl["mask"], np.float32), (prev_refl["out"], np.float32), (prev_refl["hit"], np.float32),
             (prev_refl["stable"], np.float32))]
    lib().vpto_spec_temporal(C.byref(world.s), C.byref(_as(OCamera, cam)), C.byref(_as(OCamera, prev_cam)),
                             C.byref(p), *[_p(a) for a in arrs], _p(out["out"]), _p(out["acc"]), _p(out["stable"]))
    return out


def ground_truth(world: World, cam, config, frame, t, face, crop, spp, chunk, seed=0x5eed, textures=None):
    """FP64 Welford mean and M2 (h, w, 7) of the diffuse GI over crop = (x0, y0, w, h);
    textures (a block-texture dict) textures the bounce hits."""
    p = params(config)
    x0, y0, w, h = crop
    mean = np.empty((h, w, 7), np.float64)
    m2 = np.empty((h, w, 7), np.float64)
    t = np.ascontiguousarray(t, dtype=np.float32)
    face = np.ascontiguousarray(face, dtype=np.uint8)
    keep = _set_textures(textures)
    try:
        lib().vpto_ground_truth(C.byref(world.s), C.byref(_as(OCamera, cam)), C.byref(p),
                                C.byref(_as(OFrame, frame)), _p(t), _p(face), x0, y0, w, h, spp, chunk, seed,
                                _p(mean), _p(m2))
    finally:
        lib().vpto_set_block_textures(None)
    del keep
    return mean, m2


def plain_denoise(cam, prev_cam, config, g: dict, prev_g: dict, gi: dict, hist: dict) -> dict:
    """The non-SVGF path (Core/Pipeline.cpp:2618-2786): temporal, variance and
    5 a-trous iterations with steps 12, 8, 4, 2, 1."""
    p = params(config)
    H, W = gi_dims(p)
    f32 = lambda a: np.ascontiguousarray(a, dtype=np.float32)  # noqa: E731
    cur = _f32(gi, ["sh", "cocg", "luma", "aosky"])
    prev = _f32(hist, ["sh", "cocg", "util", "aosky"])
    tmp = _planes(H, W, HIST_SPEC)
    view = gi_view(p, g["t"], g["face"], g["block"])
    t, pt = f32(view["t"]), f32(prev_g["t"])
    lib().vpto_plain_temporal(C.byref(_as(OCamera, cam)), C.byref(_as(OCamera, prev_cam)), C.byref(p), _p(t), _p(pt),
                              C.byref(_struct4(cur, ["sh", "cocg", "luma", "aosky"])),
                              C.byref(_struct4(prev, ["sh", "cocg", "util", "aosky"])),
                              C.byref(_struct4(tmp, ["sh", "cocg", "util", "aosky"])))
    var = np.zeros((H, W), np.float32)
    lib().vpto_plain_variance(C.byref(p), _p(tmp["sh"]), _p(var))
    face, block = view["face"], view["block"]
    sh, cocg, ao = tmp["sh"], tmp["cocg"], tmp["aosky"]
    dens = []
    for it in range(p.atrous_iterations):
        step = (12, 8, 4, 2, 1)[it] if it < 5 else 1
        o = _planes(H, W, {"sh": (4, np.float32), "cocg": (2, np.float32), "aosky": (2, np.float32)})
        lib().vpto_plain_atrous(C.byref(_as(OCamera, cam)), C.byref(p), step, _p(t), _p(face), _p(block), _p(sh),
                                _p(cocg), _p(ao), _p(o["sh"]), _p(o["cocg"]), _p(o["aosky"]))
        dens.append(o)
        sh, cocg, ao = o["sh"], o["cocg"], o["aosky"]
    return {"temporal": tmp, "variance": var, "atrous": dens}


def svgf(cam, prev_cam, config, frame, g: dict, prev_g: dict, gi: dict, hist: dict) -> dict:
    """Spatial3x3Initial, temporal, variance and the a-trous iterations, as
    Core/Pipeline.cpp:2284-2615 sequences them. Returns every intermediate."""
    p = params(config)
    v = gi_view(p, g["t"], g["face"], g["block"])
    pre = spatial_initial(cam, p, v["t"], v["face"], gi)
    tmp = temporal(cam, prev_cam, p, frame, v["t"], v["face"], v["block"], prev_g["t"], prev_g["face"],
                   prev_g["block"], pre, hist)
    var = variance(cam, p, v["t"], v["face"], tmp)
    cur = {"sh": var["sh"], "cocg": var["cocg"], "variance": var["variance"]}
    ao = tmp["aosky"]
    dens = []
    for it in range(p.atrous_iterations):
        step = max(16 >> it, 1)
        den = atrous(cam, p, frame, step, g["t"], g["face"], tmp["util"], cur, ao, v["t"], v["face"])
        dens.append(den)
        cur, ao = den, den["aosky"]
    return {"pre": pre, "temporal": tmp, "variance": var, "atrous": dens}


def spec_denoise(world: World, cam, config, g: dict, spec_in, hit_data, frames, direction: int) -> np.ndarray:
    """One separable pass of the reflection denoiser (direction 1: x, 0: y)."""
    p = params(config)
    v = gi_view(p, g["t"], g["face"], g["block"])
    arrs = [np.ascontiguousarray(a, dtype=dt) for a, dt in
            ((g["t"], np.float32), (g["face"], np.uint8), (g["block"], np.uint8), (v["t"], np.float32),
             (v["face"], np.uint8), (v["block"], np.uint8), (spec_in, np.float32), (hit_data, np.float32),
             (frames, np.float32))]
    out = np.zeros_like(arrs[6])
    lib().vpto_spec_denoise(C.byref(world.s), C.byref(_as(OCamera, cam)), C.byref(p), int(direction),
                            *[_p(a) for a in arrs], _p(out))
    return out


def render_frame(world: World, cam, prev_cam, config, frame, prev_g: dict, hist: dict, prev_refl=None,
                 textures=None) -> dict:
    """One whole frame in the order of vpt_render_frame; prev_refl is last
    frame's "refl" (zero planes when None)."""
    p = params(config)
    g = trace_primary(world, cam, p, textures=textures)
    shadow = trace_shadow(world, cam, p, frame, g["t"], g["face"], textures=textures)
    v = gi_view(p, g["t"], g["face"], g["block"])
    gi = trace_diffuse(world, cam, p, frame, v["t"], v["face"], textures=textures)
    if p.denoiser == 1:
        sv = plain_denoise(cam, prev_cam, p, g, prev_g, gi, hist)
        last = sv["atrous"][-1] if sv["atrous"] else sv["temporal"]
        sh, cocg, ao = last["sh"], last["cocg"], last["aosky"]
    else:
        sv = svgf(cam, prev_cam, p, frame, g, prev_g, gi, hist)
        if sv["atrous"]:
            last = sv["atrous"][-1]
            sh, cocg, ao = last["sh"], last["cocg"], last["aosky"]
        else:
            sh, cocg, ao = sv["variance"]["sh"], sv["variance"]["cocg"], sv["temporal"]["aosky"]
    gbt = None if textures is None else generate_gbuffer(cam, p, textures, g["t"], g["face"], g["block"])
    refl = None
    if p.reflection_spp > 0:
        # with block textures the reflection passes read the textured G-buffer
        # and sample the textures at their hits
        keep = _set_textures(textures)
        if gbt is not None:
            gbn = np.ascontiguousarray(gbt["normal"], np.float32)
            gbp = np.ascontiguousarray(gbt["pbr"], np.float32)
            lib().vpto_set_textured_gbuffer(_p(gbn), _p(gbp), p.width, p.height)
        try:
            refl = trace_reflection(world, cam, p, frame, g, shadow, {"sh": sh, "cocg": cocg, "aosky": ao})
            refl["raw_hit"] = refl["hit"]
            refl["hit"] = spec_hit_blur(p, g, refl["raw_hit"])
            prev_refl = prev_refl if prev_refl is not None else empty_reflection_history(p)
            refl.update(spec_temporal(world, cam, prev_cam, p, g, prev_g, refl, prev_refl))
            if p.reflection_denoise:
                hd = refl["stable"] if p.reflection_temporal else refl["hit"]
                refl["den1"] = spec_denoise(world, cam, p, g, refl["out"], hd, refl["acc"], 1)
                refl["den"] = spec_denoise(world, cam, p, g, refl["den1"], hd, refl["acc"], 0)
        finally:
            lib().vpto_set_textured_gbuffer(None, None, 0, 0)
            lib().vpto_set_block_textures(None)
        del keep
    spec = None if refl is None else (refl["den"] if p.reflection_denoise else refl["out"])
    rgb = shade(world, cam, p, frame, g["t"], g["face"], g["block"], shadow, sh, cocg, ao, spec=spec, gbt=gbt)
    return {"g": g, "shadow": shadow, "gi": gi, "svgf": sv, "refl": refl, "rgb": rgb, "gbt": gbt}


def empty_history(H: int, W: int, gi_divisor: int = 1):
    """The state libvpt starts from: previous G-buffer all misses, zero history
    (on the GI grid)."""
    prev_g = {"t": np.full((H, W), -1.0, np.float32), "face": np.full((H, W), 10, np.uint8),
              "block": np.zeros((H, W), np.uint8)}
    d = max(int(gi_divisor), 1)
    Hg, Wg = H // d, W // d
    hist = {"sh": np.zeros((Hg, Wg, 4), np.float32), "cocg": np.zeros((Hg, Wg, 2), np.float32),
            "util": np.zeros((Hg, Wg, 4), np.float32), "aosky": np.zeros((Hg, Wg, 2), np.float32)}
    return prev_g, hist
