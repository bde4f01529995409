"""GB300-native VoxelPathTracer hot path: Python host over the libvpt C ABI.

The reference (swr06/VoxelPathTracer) drives its hot path from
Core/Pipeline.cpp: World::Buffer uploads the voxel volume, World::
GenerateDistanceField builds the Manhattan distance field, and each frame runs
the initial (G-buffer) trace, the sun-shadow and diffuse-GI traces, the SVGF
denoiser and the colour pass, then swaps its history framebuffers. `Context`
exposes exactly those steps over libvpt (include/vpt.h); every call goes
through the C ABI into hand-written sm_103a kernels. There is no CPU fallback:
importing this package without a built libvpt raises.

Arrays: voxel volumes are numpy uint8 of shape (Z, Y, X) (x fastest, as
Core/World.h:46-49 lays them out); image planes are (H, W, C) with row 0 at
the bottom (OpenGL convention).
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "libvpt.so"

# ------------------------------------------------------------------ enums --
OK, ERR_INVALID_ARG, ERR_OOM, ERR_DEVICE_TIMEOUT, ERR_CUDA, ERR_STATE, ERR_NO_DEVICE = range(7)
STORAGE_F32, STORAGE_F16 = 0, 1
DENOISER_SVGF, DENOISER_ATROUS = 0, 1
DTYPE_F32, DTYPE_F16, DTYPE_U8, DTYPE_U16, DTYPE_I32 = range(5)
_NP_DTYPE = {DTYPE_F32: np.float32, DTYPE_F16: np.float16, DTYPE_U8: np.uint8, DTYPE_U16: np.uint16,
             DTYPE_I32: np.int32}

PLANES = [
    "T", "FACE", "BLOCK", "HIT", "STEPS", "SHADOW",
    "GI_SH", "GI_COCG", "GI_LUMA", "GI_AOSKY",
    "PRE_SH", "PRE_COCG", "PRE_LUMA", "PRE_AOSKY",
    "TEMP_SH", "TEMP_COCG", "TEMP_UTIL", "TEMP_AOSKY",
    "HIST_SH", "HIST_COCG", "HIST_UTIL", "HIST_AOSKY",
    "PREV_T", "PREV_FACE", "PREV_BLOCK",
    "VAR_SH", "VAR_COCG", "VAR_VARIANCE",
    "DEN_SH", "DEN_COCG", "DEN_VARIANCE", "DEN_AOSKY",
    "COLOR", "SPEC", "SPEC_HIT", "SPEC_MASK", "SPEC_OUT", "SPEC_ACC", "SPEC_STABLE_HIT", "SPEC_DEN",
    "GB_ALBEDO", "GB_NORMAL", "GB_PBR", "GB_AO",
]
PLANE = {name: i for i, name in enumerate(PLANES)}
PASSES = ["primary", "shadow", "diffuse", "spatial_initial", "temporal", "variance", "atrous", "shade", "trace_frame",
          "learned", "reflection", "gbuffer"]
RAY_KINDS = ["primary", "shadow", "diffuse", "bounce_shadow", "reflection", "reflection_shadow"]
FACE_MISS = 10


# ---------------------------------------------------------------- structs --
class Config(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("primary_max_steps", C.c_int32),
                ("shadow_max_steps", C.c_int32), ("diffuse_max_steps", C.c_int32),
                ("bounce_shadow_max_steps", C.c_int32), ("bounces", C.c_int32), ("spp", C.c_int32),
                ("storage", C.c_int32), ("atrous_iterations", C.c_int32), ("resolution_scale", C.c_float),
                ("color_phi_bias", C.c_float), ("device", C.c_int32), ("denoiser", C.c_int32),
                ("gi_divisor", C.c_int32), ("reflection_spp", C.c_int32), ("reflection_max_steps", C.c_int32),
                ("reflection_shadow_max_steps", C.c_int32), ("reflection_temporal", C.c_int32),
                ("reflection_denoise", C.c_int32), ("alpha_test", C.c_int32), ("alpha_test_shadows", C.c_int32),
                ("reserved", C.c_int32 * 1)]


class Camera(C.Structure):
    _fields_ = [("view", C.c_float * 16), ("proj", C.c_float * 16), ("inv_view", C.c_float * 16),
                ("inv_proj", C.c_float * 16), ("position", C.c_float * 3), ("pad", C.c_float)]


class BlockTextures(C.Structure):
    """vpt_block_textures: the four block texture arrays and their per-block layer ids."""
    _fields_ = [("size", C.c_int32), ("albedo", C.c_void_p), ("albedo_layers", C.c_int32),
                ("normal", C.c_void_p), ("normal_layers", C.c_int32), ("pbr", C.c_void_p),
                ("pbr_layers", C.c_int32), ("emissive", C.c_void_p), ("emissive_layers", C.c_int32),
                ("albedo_id", C.c_int32 * 128), ("normal_id", C.c_int32 * 128), ("pbr_id", C.c_int32 * 128),
                ("emissive_id", C.c_int32 * 128), ("grass", C.c_int32 * 10), ("transparent", C.c_int32 * 128)]


class Block(C.Structure):
    _fields_ = [("albedo", C.c_uint8 * 3), ("roughness", C.c_uint8), ("metalness", C.c_uint8),
                ("emissive", C.c_uint8)]


class Frame(C.Structure):
    _fields_ = [("sun_dir", C.c_float * 3), ("time", C.c_float), ("sun_radiance", C.c_float * 3),
                ("frame_index", C.c_uint32), ("moon_radiance", C.c_float * 3), ("seed", C.c_uint32),
                ("gi_sun_strength", C.c_float), ("gi_sky_strength", C.c_float),
                ("diffuse_light_intensity", C.c_float), ("temporal", C.c_int32)]


class Stats(C.Structure):
    _fields_ = [("rays", C.c_uint64 * 6), ("steps", C.c_uint64 * 6)]


class TraceBuffers(C.Structure):
    """vpt_trace_buffers: caller-owned device buffers of vpt_trace_frame_noalloc."""
    _fields_ = [("voxels", C.c_void_p), ("df", C.c_void_p), ("X", C.c_int32), ("Y", C.c_int32), ("Z", C.c_int32),
                ("blocks", C.c_void_p), ("n_blocks", C.c_int32), ("t", C.c_void_p), ("face", C.c_void_p),
                ("block", C.c_void_p), ("hit", C.c_void_p), ("steps", C.c_void_p), ("shadow", C.c_void_p),
                ("gi_sh", C.c_void_p), ("gi_cocg", C.c_void_p), ("gi_luma", C.c_void_p), ("gi_aosky", C.c_void_p)]


class Tuning(C.Structure):
    _fields_ = [("refill_threshold", C.c_int32), ("trace_blocks", C.c_int32), ("fused_trace", C.c_int32),
                ("fused_prefilter", C.c_int32), ("overlap_shadow", C.c_int32), ("split_temporal", C.c_int32),
                ("reserved", C.c_int32 * 2)]


class BatchConfig(C.Structure):
    _fields_ = [("device", C.c_int32), ("max_worlds", C.c_int32), ("primary_max_steps", C.c_int32),
                ("shadow_max_steps", C.c_int32), ("diffuse_max_steps", C.c_int32),
                ("bounce_shadow_max_steps", C.c_int32), ("bounces", C.c_int32), ("spp", C.c_int32),
                ("reserved", C.c_int32 * 4)]


class BatchTuning(C.Structure):
    _fields_ = [("block_threads", C.c_int32), ("tiles_per_grab", C.c_int32), ("df_brick", C.c_int32),
                ("blocks", C.c_int32), ("rays_per_lane", C.c_int32), ("phased", C.c_int32),
                ("reserved", C.c_int32 * 2)]

    def as_dict(self) -> dict:
        return {"block_threads": self.block_threads, "tiles_per_grab": self.tiles_per_grab,
                "rays_per_lane": self.rays_per_lane, "rays_per_warp": 32 * self.rays_per_lane,
                "df_brick": self.df_brick, "blocks": self.blocks, "phased": self.phased}


class BatchTuneRecord(C.Structure):
    _fields_ = [("tuning", BatchTuning), ("ms", C.c_float), ("pad", C.c_float)]


BATCH_GRAPH, BATCH_PERSISTENT, BATCH_PER_WORLD = 0, 1, 2
BATCH_PLANES = ["T", "FACE", "BLOCK", "HIT", "STEPS", "SHADOW", "GI_SH", "GI_COCG", "GI_LUMA", "GI_AOSKY"]


BLOCK_DTYPE = np.dtype([("albedo", np.uint8, 3), ("roughness", np.uint8), ("metalness", np.uint8),
                        ("emissive", np.uint8)])


class VPTError(RuntimeError):
    def __init__(self, status: int, what: str):
        super().__init__(f"{what}: status {status}")
        self.status = status


def _load() -> C.CDLL:
    if not LIB_PATH.exists():
        raise ImportError(f"libvpt is not built ({LIB_PATH} missing); run __graft_entry__.build() or "
                          "python -m voxelpathtracer_gb300._build")
    lib = C.CDLL(str(LIB_PATH))
    P = C.c_void_p
    i32, u64, f32, sz = C.c_int32, C.c_uint64, C.c_float, C.c_size_t
    sigs = {
        "vpt_status_string": ([C.c_int], C.c_char_p),
        "vpt_abi_version": ([], C.c_int),
        "vpt_default_config": ([C.POINTER(Config)], C.c_int),
        "vpt_default_frame": ([C.POINTER(Frame)], C.c_int),
        "vpt_create": ([C.POINTER(P), C.POINTER(Config)], C.c_int),
        "vpt_destroy": ([P], C.c_int),
        "vpt_last_error": ([P], C.c_char_p),
        "vpt_upload_world": ([P, P, i32, i32, i32], C.c_int),
        "vpt_set_block_table": ([P, P, i32], C.c_int),
        "vpt_set_block_textures": ([P, C.POINTER(BlockTextures)], C.c_int),
        "vpt_generate_gbuffer": ([P], C.c_int),
        "vpt_build_df": ([P], C.c_int),
        "vpt_read_df": ([P, P, sz], C.c_int),
        "vpt_df_build_device": ([P, P, i32, i32, i32, P], C.c_int),
        "vpt_measure_l2_read": ([i32, C.c_uint64, i32, C.POINTER(C.c_float)], C.c_int),
        "vpt_trace_primary": ([P, C.POINTER(Camera)], C.c_int),
        "vpt_trace_shadow": ([P, C.POINTER(Frame)], C.c_int),
        "vpt_trace_diffuse": ([P, C.POINTER(Frame)], C.c_int),
        "vpt_svgf": ([P, C.POINTER(Camera), C.POINTER(Frame)], C.c_int),
        "vpt_trace_reflections": ([P, C.POINTER(Frame)], C.c_int),
        "vpt_shade": ([P, C.POINTER(Frame)], C.c_int),
        "vpt_trace_frame": ([P, C.POINTER(Camera), C.POINTER(Frame)], C.c_int),
        "vpt_trace_frame_noalloc": ([C.POINTER(TraceBuffers), C.POINTER(Config), C.POINTER(Camera),
                                     C.POINTER(Frame), P], C.c_int),
        "vpt_set_tuning": ([P, C.POINTER(Tuning)], C.c_int),
        "vpt_ground_truth": ([P, C.POINTER(Frame), i32, i32, i32, i32, i32, i32, C.c_uint32, P, P], C.c_int),
        "vpt_get_tuning": ([P, C.POINTER(Tuning)], C.c_int),
        "vpt_end_frame": ([P], C.c_int),
        "vpt_reset_history": ([P], C.c_int),
        "vpt_render_frame": ([P, C.POINTER(Camera), C.POINTER(Frame), P], C.c_int),
        "vpt_render_frame_async": ([P, C.POINTER(Camera), C.POINTER(Frame), P], C.c_int),
        "vpt_readback_wait": ([P], C.c_int),
        "vpt_plane_info": ([P, i32, C.POINTER(sz), C.POINTER(i32), C.POINTER(i32)], C.c_int),
        "vpt_plane_dims": ([P, i32, C.POINTER(i32), C.POINTER(i32)], C.c_int),
        "vpt_read_plane": ([P, i32, P, sz], C.c_int),
        "vpt_write_plane": ([P, i32, P, sz], C.c_int),
        "vpt_plane_device_ptr": ([P, i32, C.POINTER(P)], C.c_int),
        "vpt_synchronize": ([P], C.c_int),
        "vpt_set_stats": ([P, i32], C.c_int),
        "vpt_read_stats": ([P, C.POINTER(Stats)], C.c_int),
        "vpt_set_profiling": ([P, i32], C.c_int),
        "vpt_read_pass_times": ([P, C.POINTER(f32), i32], C.c_int),
        "vpt_launch_count": ([P, C.POINTER(u64)], C.c_int),
        "vpt_get_stream": ([P, C.POINTER(P)], C.c_int),
        "vpt_detmath": ([i32, P, P, P, i32, i32], C.c_int),
        "vpt_batch_default_config": ([C.POINTER(BatchConfig)], C.c_int),
        "vpt_batch_create": ([C.POINTER(P), C.POINTER(BatchConfig)], C.c_int),
        "vpt_batch_destroy": ([P], C.c_int),
        "vpt_batch_last_error": ([P], C.c_char_p),
        "vpt_batch_add_world": ([P, P, i32, i32, i32, P, i32, i32, i32, C.POINTER(i32)], C.c_int),
        "vpt_batch_set_camera": ([P, i32, C.POINTER(Camera)], C.c_int),
        "vpt_batch_build_df": ([P], C.c_int),
        "vpt_batch_read_df": ([P, i32, P, sz], C.c_int),
        "vpt_batch_set_tuning": ([P, C.POINTER(BatchTuning)], C.c_int),
        "vpt_batch_get_tuning": ([P, C.POINTER(BatchTuning)], C.c_int),
        "vpt_batch_trace": ([P, C.POINTER(Frame), i32], C.c_int),
        "vpt_batch_autotune": ([P, C.POINTER(Frame), i32, C.POINTER(BatchTuneRecord), i32, C.POINTER(i32)],
                               C.c_int),
        "vpt_batch_read_plane": ([P, i32, i32, P, sz], C.c_int),
        "vpt_batch_world_info": ([P, i32, C.POINTER(i32), C.POINTER(i32)], C.c_int),
        "vpt_batch_count": ([P, C.POINTER(i32)], C.c_int),
        "vpt_batch_synchronize": ([P], C.c_int),
        "vpt_batch_set_stats": ([P, i32], C.c_int),
        "vpt_batch_read_stats": ([P, C.POINTER(Stats)], C.c_int),
        "vpt_batch_launch_count": ([P, C.POINTER(u64)], C.c_int),
        "vpt_batch_get_stream": ([P, C.POINTER(P)], C.c_int),
        "vpt_shade_from": ([P, C.POINTER(Frame), i32], C.c_int),
        "vpt_edit_world": ([P, P, i32, i32, i32, i32, i32, i32], C.c_int),
        "vpt_save_world": ([C.c_char_p, P, i32, i32, i32, u64, i32], C.c_int),
        "vpt_import_mca_world": ([C.c_char_p, P, P, P, sz, C.POINTER(i32)], C.c_int),
        "vpt_load_world": ([C.c_char_p, P, sz, C.POINTER(i32), C.POINTER(u64)], C.c_int),
        "vpt_emissive_voxels": ([P, i32, i32, i32, P, i32, P, C.c_int64, C.POINTER(C.c_int64)], C.c_int),
        "vpt_learned_input": ([P, C.POINTER(Camera), C.POINTER(Frame)], C.c_int),
        "vpt_learned_features": ([P, i32, i32, i32, i32, P], C.c_int),
        "vpt_render_frame_learned": ([P, P, C.POINTER(Camera), C.POINTER(Frame), P, C.POINTER(i32)], C.c_int),
        "vpt_nn_conv3x3": ([P, i32, i32, P, i32, i32, i32, i32, P, P, i32, i32, P, P, P, P], C.c_int),
        "vpt_nn_conv3x3_dw": ([P, i32, i32, P, i32, i32, i32, i32, P, i32, P, P], C.c_int),
        "vpt_nn_status": ([P], C.c_int),
        "vpt_unet_layer_info": ([i32, C.POINTER(i32), C.POINTER(i32), C.POINTER(i32), C.POINTER(i32),
                                 C.POINTER(C.c_int64)], C.c_int),
        "vpt_unet_create": ([C.POINTER(P), i32, i32, i32, i32], C.c_int),
        "vpt_unet_destroy": ([P], C.c_int),
        "vpt_unet_last_error": ([P], C.c_char_p),
        "vpt_unet_param_count": ([P, C.POINTER(C.c_int64)], C.c_int),
        "vpt_unet_set_params": ([P, P, C.c_int64], C.c_int),
        "vpt_unet_get_params": ([P, P, C.c_int64], C.c_int),
        "vpt_unet_get_grads": ([P, P, C.c_int64], C.c_int),
        "vpt_unet_forward": ([P, P, i32, i32, i32, P], C.c_int),
        "vpt_unet_output": ([P, C.POINTER(P)], C.c_int),
        "vpt_unet_backward": ([P, P, P, i32, i32, i32, C.POINTER(C.c_double)], C.c_int),
        "vpt_unet_adam": ([P, f32, f32, f32, f32], C.c_int),
        "vpt_unet_synchronize": ([P], C.c_int),
        "vpt_unet_get_stream": ([P, C.POINTER(P)], C.c_int),
        "vpt_generate_world": ([P, i32, i32, i32, u64, i32], C.c_int),
        "vpt_generate_block_table": ([P, i32, u64], C.c_int),
        "vpt_camera_from_pose": ([C.POINTER(Camera), C.POINTER(f32), f32, f32, f32, f32, f32, f32], C.c_int),
    }
    for name, (argtypes, restype) in sigs.items():
        fn = getattr(lib, name)
        fn.argtypes = argtypes
        fn.restype = restype
    return lib


lib = _load()
EXPORTED = None  # filled lazily by tests


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def _check(status: int, what: str, ctx=None):
    if status != OK:
        msg = lib.vpt_status_string(status).decode()
        if ctx is not None:
            detail = lib.vpt_last_error(ctx)
            if detail:
                msg += f" ({detail.decode()})"
        raise VPTError(status, f"{what} failed: {msg}")


# ------------------------------------------------------------ host helpers --
def default_config(**kw) -> Config:
    cfg = Config()
    _check(lib.vpt_default_config(C.byref(cfg)), "vpt_default_config")
    for k, v in kw.items():
        if not hasattr(cfg, k):
            raise AttributeError(f"unknown config field {k}")
        setattr(cfg, k, v)
    return cfg


def default_frame(**kw) -> Frame:
    f = Frame()
    _check(lib.vpt_default_frame(C.byref(f)), "vpt_default_frame")
    for k, v in kw.items():
        if k in ("sun_dir", "sun_radiance", "moon_radiance"):
            getattr(f, k)[:] = [float(x) for x in v]
        else:
            setattr(f, k, v)
    return f


def generate_world(X: int, Y: int, Z: int, seed: int = 0, n_blocks: int = 100) -> np.ndarray:
    """Seeded value-noise terrain, shape (Z, Y, X) uint8 (vpt_generate_world)."""
    out = np.empty((Z, Y, X), dtype=np.uint8)
    _check(lib.vpt_generate_world(_ptr(out), X, Y, Z, seed, n_blocks), "vpt_generate_world")
    return out


def generate_block_table(n: int = 100, seed: int = 0) -> np.ndarray:
    """Seeded flat block table as a structured array (vpt_generate_block_table)."""
    out = np.zeros(n, dtype=BLOCK_DTYPE)
    _check(lib.vpt_generate_block_table(_ptr(out), n, seed), "vpt_generate_block_table")
    return out


def generate_block_textures(size: int = 32, layers: int = 12, n_blocks: int = 100, seed: int = 0,
                            emissive: bool = True, grass_block: int = 1) -> dict:
    """Seeded synthetic block texture arrays standing in for the reference's
    block PNGs: per layer a base colour with a two-scale noise pattern
    (albedo, sRGB-encoded), a normal map tilted around (0.5, 0.5, 1), PBR maps
    (roughness, metalness, displacement, AO) and sparse emissive masks; every
    block gets a layer in each array (emissive for about one block in five)
    and block `grass_block` (-1: none) gets separate top / side / bottom layers."""
    if size < 1 or size & (size - 1):
        raise ValueError("size must be a power of two")
    rng = np.random.default_rng(seed)
    yy, xx = np.meshgrid(np.arange(size), np.arange(size), indexing="ij")

    def pattern(k):
        f1, f2 = rng.integers(1, 4, size=2)
        ph = rng.uniform(0, 2 * np.pi, size=2)
        coarse = np.sin(2 * np.pi * f1 * xx / size + ph[0]) * np.cos(2 * np.pi * f2 * yy / size + ph[1])
        return 0.5 + 0.25 * coarse + 0.25 * (rng.random((size, size)) - 0.5)

    def u8(a):
        return np.clip(np.round(a * 255.0), 0, 255).astype(np.uint8)

    alb = np.empty((layers, size, size, 4), np.uint8)
    nrm = np.empty((layers, size, size, 4), np.uint8)
    pbr = np.empty((layers, size, size, 4), np.uint8)
    for l in range(layers):
        base = rng.uniform(0.15, 0.9, size=3)
        p = pattern(l)
        alb[l, ..., :3] = u8(base[None, None, :] * (0.6 + 0.8 * p[..., None] * 0.5))
        alb[l, ..., 3] = 255
        tilt = 0.35 * (pattern(l) - 0.5)
        tilt2 = 0.35 * (pattern(l) - 0.5)
        n = np.stack([tilt, tilt2, np.ones_like(tilt)], axis=-1)
        n /= np.linalg.norm(n, axis=-1, keepdims=True)
        nrm[l, ..., :3] = u8(n * 0.5 + 0.5)
        nrm[l, ..., 3] = 255
        pbr[l, ..., 0] = u8(np.clip(rng.uniform(0.2, 0.9) + 0.3 * (pattern(l) - 0.5), 0, 1))
        pbr[l, ..., 1] = u8(np.full((size, size), 1.0 if rng.random() < 0.15 else 0.0))
        pbr[l, ..., 2] = u8(pattern(l))
        pbr[l, ..., 3] = u8(np.clip(0.75 + 0.5 * (pattern(l) - 0.5), 0, 1))
    emi = None
    if emissive:
        emi = u8((rng.random((layers, size, size)) < 0.3) * rng.uniform(0.3, 1.0, size=(layers, 1, 1)))
    ids = rng.integers(0, layers, size=(4, 128)).astype(np.int32)
    if emissive:
        ids[3] = np.where(rng.random(128) < 0.2, ids[3], -1)
    else:
        ids[3] = -1
    grass = np.full(10, -1, np.int32)
    if grass_block >= 0:
        grass[0] = grass_block
        grass[1:] = rng.integers(0, layers, size=9)
    # cut-out alpha (about a third of the texels see-through) and one block in
    # six transparent to the alpha test
    for l in range(layers):
        alb[l, ..., 3] = np.where(pattern(l) < 0.4, 0, 255).astype(np.uint8)
    transparent = (rng.random(128) < 1 / 6).astype(np.int32)
    return {"size": size, "albedo": alb, "normal": nrm, "pbr": pbr, "emissive": emi, "albedo_id": ids[0],
            "normal_id": ids[1], "pbr_id": ids[2], "emissive_id": ids[3], "grass": grass,
            "transparent": transparent}


def block_textures_struct(t: dict):
    """(vpt_block_textures, the arrays it points into) for a texture dict."""
    keep = {k: np.ascontiguousarray(t[k], np.uint8) for k in ("albedo", "normal", "pbr")}
    if t.get("emissive") is not None:
        keep["emissive"] = np.ascontiguousarray(t["emissive"], np.uint8)
    bt = BlockTextures()
    bt.size = int(t["size"])
    for k in ("albedo", "normal", "pbr", "emissive"):
        if k in keep:
            setattr(bt, k, keep[k].ctypes.data)
            setattr(bt, f"{k}_layers", int(keep[k].shape[0]))
    for k in ("albedo_id", "normal_id", "pbr_id", "emissive_id"):
        getattr(bt, k)[:] = [int(v) for v in np.asarray(t[k], np.int64)[:128]]
    bt.grass[:] = [int(v) for v in np.asarray(t["grass"], np.int64)[:10]]
    if t.get("transparent") is not None:
        bt.transparent[:] = [int(v) for v in np.asarray(t["transparent"], np.int64)[:128]]
    return bt, keep


def camera_from_pose(position, yaw_deg: float, pitch_deg: float, fov_deg: float = 90.0, aspect: float = 16 / 9,
                     znear: float = 0.1, zfar: float = 1000.0) -> Camera:
    cam = Camera()
    pos = (C.c_float * 3)(*[float(p) for p in position])
    _check(lib.vpt_camera_from_pose(C.byref(cam), pos, yaw_deg, pitch_deg, fov_deg, aspect, znear, zfar),
           "vpt_camera_from_pose")
    return cam


def save_world(path, voxels: np.ndarray, seed: int = 0, header: bool = True):
    """Writes a world file (vpt_save_world): header=False is the reference's raw .sav layout."""
    v = np.ascontiguousarray(voxels, dtype=np.uint8)
    Z, Y, X = v.shape
    _check(lib.vpt_save_world(str(path).encode(), _ptr(v), X, Y, Z, seed, 1 if header else 0), "vpt_save_world")


def load_world(path, dims=None):
    """Reads a world file; `dims` (X, Y, Z) is required for a raw .sav. Returns (voxels (Z, Y, X), seed)."""
    d = (C.c_int32 * 3)(*(dims if dims is not None else (0, 0, 0)))
    seed = C.c_uint64()
    _check(lib.vpt_load_world(str(path).encode(), None, 0, d, C.byref(seed)), "vpt_load_world")
    out = np.empty((d[2], d[1], d[0]), np.uint8)
    _check(lib.vpt_load_world(str(path).encode(), _ptr(out), out.nbytes, d, C.byref(seed)), "vpt_load_world")
    return out, int(seed.value)


MCA_WORLD = (384, 128, 384)   # X, Y, Z of the reference's imported world (Core/Macros.h)


def import_mca_world(directory, mcid_to_block=None, origin=(0.0, 0.0, 0.0)):
    """Imports every .mca region file of `directory` (vpt_import_mca_world) into
    the reference's 384 x 128 x 384 world; mcid_to_block maps Minecraft ids to
    block ids (identity when None). Returns (voxels (Z, Y, X), chunks read)."""
    lut = np.arange(256, dtype=np.uint8) if mcid_to_block is None else np.ascontiguousarray(mcid_to_block, np.uint8)
    if lut.shape != (256,):
        raise ValueError("mcid_to_block must have 256 entries")
    org = (C.c_float * 3)(*[float(v) for v in origin])
    X, Y, Z = MCA_WORLD
    out = np.empty((Z, Y, X), np.uint8)
    n = C.c_int32()
    _check(lib.vpt_import_mca_world(str(directory).encode(), _ptr(lut), org, _ptr(out), out.nbytes, C.byref(n)),
           "vpt_import_mca_world")
    return out, int(n.value)


def emissive_voxels(voxels: np.ndarray, table: np.ndarray) -> np.ndarray:
    """(n, 3) int32 x, y, z of the emissive voxels (the reference's light list)."""
    v = np.ascontiguousarray(voxels, dtype=np.uint8)
    t = np.ascontiguousarray(table, dtype=BLOCK_DTYPE)
    Z, Y, X = v.shape
    cnt = C.c_int64()
    _check(lib.vpt_emissive_voxels(_ptr(v), X, Y, Z, _ptr(t), t.size, None, 0, C.byref(cnt)), "vpt_emissive_voxels")
    out = np.zeros((cnt.value, 3), np.int32)
    if cnt.value:
        _check(lib.vpt_emissive_voxels(_ptr(v), X, Y, Z, _ptr(t), t.size, _ptr(out), cnt.value, C.byref(cnt)),
               "vpt_emissive_voxels")
    return out


def seeded_pose(seed: int, yaw_range=(0.0, 360.0), pitch_range=(-40.0, -10.0)):
    """Yaw and pitch drawn uniformly from the seed (the bench's camera rule)."""
    rng = np.random.default_rng(seed)
    return float(rng.uniform(*yaw_range)), float(rng.uniform(*pitch_range))


def detmath(op: int, x: np.ndarray, y: np.ndarray | None = None, on_device: bool = False) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.float32)
    yy = np.ascontiguousarray(y if y is not None else np.zeros_like(x), dtype=np.float32)
    out = np.empty_like(x)
    _check(lib.vpt_detmath(op, _ptr(x), _ptr(yy), _ptr(out), x.size, 1 if on_device else 0), "vpt_detmath")
    return out


# ---------------------------------------------------------------- context --
class Context:
    """One libvpt context: device buffers for a world and a W x H frame.

    Method names follow the steps of the reference's frame loop:
      upload_world     World::Buffer            (Core/World.h:167-171)
      set_block_table  BlockDataSSBO::CreateBuffers (Core/BlockDataSSBO.cpp:5-37)
      build_df         World::GenerateDistanceField (Core/World.cpp:69-113)
      trace_primary    initial trace pass       (Core/Pipeline.cpp:1959-2016)
      trace_shadow     shadow trace pass        (Core/Pipeline.cpp:2790-2850)
      trace_diffuse    diffuse GI trace pass    (Core/Pipeline.cpp:2169-2281)
      svgf             SVGF denoiser            (Core/Pipeline.cpp:2284-2615)
      shade            colour pass              (Core/Pipeline.cpp:3603-3821)
      end_frame        history ping-pong        (Core/Pipeline.cpp:1775-1788)
    """

    def __init__(self, config: Config | None = None, **overrides):
        cfg = config if config is not None else default_config()
        for k, v in overrides.items():
            setattr(cfg, k, v)
        self.config = cfg
        self._h = C.c_void_p()
        _check(lib.vpt_create(C.byref(self._h), C.byref(cfg)), "vpt_create")
        self.width, self.height = cfg.width, cfg.height
        self.world_shape = None

    # lifetime
    def close(self):
        if self._h:
            lib.vpt_destroy(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ck(self, status, what):
        _check(status, what, self._h)

    # world
    def upload_world(self, voxels: np.ndarray):
        v = np.ascontiguousarray(voxels, dtype=np.uint8)
        if v.ndim != 3:
            raise ValueError("voxels must have shape (Z, Y, X)")
        Z, Y, X = v.shape
        self._ck(lib.vpt_upload_world(self._h, _ptr(v), X, Y, Z), "vpt_upload_world")
        self.world_shape = (Z, Y, X)

    def set_block_table(self, table: np.ndarray):
        t = np.ascontiguousarray(table, dtype=BLOCK_DTYPE)
        self._ck(lib.vpt_set_block_table(self._h, _ptr(t), t.size), "vpt_set_block_table")

    def build_df(self):
        self._ck(lib.vpt_build_df(self._h), "vpt_build_df")

    def set_block_textures(self, textures):
        """Uploads block texture arrays (a dict as generate_block_textures makes; None removes them)."""
        if textures is None:
            self._ck(lib.vpt_set_block_textures(self._h, None), "vpt_set_block_textures")
            self._textures = None
            return
        bt, keep = block_textures_struct(textures)
        self._ck(lib.vpt_set_block_textures(self._h, C.byref(bt)), "vpt_set_block_textures")
        self._textures = keep

    def generate_gbuffer(self):
        """GenerateGBuffer: the GB_ALBEDO / GB_NORMAL / GB_PBR / GB_AO planes of this frame."""
        self._ck(lib.vpt_generate_gbuffer(self._h), "vpt_generate_gbuffer")

    def edit_world(self, origin, voxels: np.ndarray):
        """Writes the (d, h, w) block of voxels at origin (x0, y0, z0) and updates the distance field locally."""
        v = np.ascontiguousarray(voxels, dtype=np.uint8)
        d, h, w = v.shape
        x0, y0, z0 = origin
        self._ck(lib.vpt_edit_world(self._h, _ptr(v), x0, y0, z0, w, h, d), "vpt_edit_world")

    def read_df(self) -> np.ndarray:
        out = np.empty(self.world_shape, dtype=np.uint8)
        self._ck(lib.vpt_read_df(self._h, _ptr(out), out.nbytes), "vpt_read_df")
        return out

    # passes
    def trace_primary(self, cam: Camera):
        self._ck(lib.vpt_trace_primary(self._h, C.byref(cam)), "vpt_trace_primary")

    def trace_shadow(self, frame: Frame):
        self._ck(lib.vpt_trace_shadow(self._h, C.byref(frame)), "vpt_trace_shadow")

    def trace_diffuse(self, frame: Frame):
        self._ck(lib.vpt_trace_diffuse(self._h, C.byref(frame)), "vpt_trace_diffuse")

    def svgf(self, prev_cam: Camera | None, frame: Frame):
        self._ck(lib.vpt_svgf(self._h, C.byref(prev_cam) if prev_cam is not None else None, C.byref(frame)),
                 "vpt_svgf")

    def trace_reflections(self, frame: Frame):
        self._ck(lib.vpt_trace_reflections(self._h, C.byref(frame)), "vpt_trace_reflections")

    def shade(self, frame: Frame):
        self._ck(lib.vpt_shade(self._h, C.byref(frame)), "vpt_shade")

    def trace_frame(self, cam: Camera, frame: Frame):
        """Primary, sun-shadow and diffuse traces in one persistent kernel."""
        self._ck(lib.vpt_trace_frame(self._h, C.byref(cam), C.byref(frame)), "vpt_trace_frame")

    def set_tuning(self, refill_threshold: int | None = None, trace_blocks: int | None = None,
                   fused_trace: bool | None = None, fused_prefilter: bool | None = None,
                   overlap_shadow: bool | None = None, split_temporal: bool | None = None):
        t = self.tuning()
        if refill_threshold is not None:
            t.refill_threshold = refill_threshold
        if trace_blocks is not None:
            t.trace_blocks = trace_blocks
        if fused_trace is not None:
            t.fused_trace = 1 if fused_trace else 0
        if fused_prefilter is not None:
            t.fused_prefilter = 1 if fused_prefilter else 0
        if overlap_shadow is not None:
            t.overlap_shadow = 1 if overlap_shadow else 0
        if split_temporal is not None:
            t.split_temporal = 1 if split_temporal else 0
        self._ck(lib.vpt_set_tuning(self._h, C.byref(t)), "vpt_set_tuning")

    def tuning(self) -> Tuning:
        t = Tuning()
        self._ck(lib.vpt_get_tuning(self._h, C.byref(t)), "vpt_get_tuning")
        return t

    def ground_truth(self, frame: Frame, crop, spp: int = 4096, chunk: int = 256, seed: int = 0x5eed):
        """FP64 Welford mean and M2 of the diffuse GI (SH 4, CoCg 2, AO) over
        crop = (x0, y0, w, h) of the frame whose primary rays were traced last.
        Returns two (h, w, 7) float64 arrays."""
        x0, y0, w, h = crop
        mean = np.empty((h, w, 7), np.float64)
        m2 = np.empty((h, w, 7), np.float64)
        self._ck(lib.vpt_ground_truth(self._h, C.byref(frame), x0, y0, w, h, spp, chunk, seed, _ptr(mean),
                                      _ptr(m2)), "vpt_ground_truth")
        return mean, m2

    def end_frame(self):
        self._ck(lib.vpt_end_frame(self._h), "vpt_end_frame")

    def reset_history(self):
        self._ck(lib.vpt_reset_history(self._h), "vpt_reset_history")

    def render_frame(self, cam: Camera, frame: Frame, out: np.ndarray | None = None, readback: bool = True):
        if readback and out is None:
            out = np.empty((self.height, self.width, 3), dtype=np.float32)
        ptr = _ptr(out) if readback else None
        self._ck(lib.vpt_render_frame(self._h, C.byref(cam), C.byref(frame), ptr), "vpt_render_frame")
        return out

    def render_frame_async(self, cam: Camera, frame: Frame, out: np.ndarray):
        """vpt_render_frame_async: the image lands in `out` (float32 H x W x 3,
        ideally page-locked) while the next frame computes; returns once the
        previous call's image is complete. readback_wait() finishes the last."""
        if out.dtype != np.float32 or out.shape != (self.height, self.width, 3) or not out.flags.c_contiguous:
            raise ValueError("out must be a C-contiguous float32 (H, W, 3) array")
        self._ck(lib.vpt_render_frame_async(self._h, C.byref(cam), C.byref(frame), _ptr(out)),
                 "vpt_render_frame_async")
        self._async_out = getattr(self, "_async_out", [])[-1:] + [out]   # keep the in-flight buffers alive

    def readback_wait(self):
        self._ck(lib.vpt_readback_wait(self._h), "vpt_readback_wait")
        self._async_out = []

    # planes
    def plane_info(self, plane):
        pid = PLANE[plane] if isinstance(plane, str) else int(plane)
        nbytes, ch, dt = C.c_size_t(), C.c_int32(), C.c_int32()
        self._ck(lib.vpt_plane_info(self._h, pid, C.byref(nbytes), C.byref(ch), C.byref(dt)), "vpt_plane_info")
        return pid, nbytes.value, ch.value, _NP_DTYPE[dt.value]

    def shade_from(self, frame: Frame, source: int):
        """Colour pass from the denoised GI (0) or the temporal GI before spatial filtering (1)."""
        self._ck(lib.vpt_shade_from(self._h, C.byref(frame), source), "vpt_shade_from")

    def learned_input(self, cam: Camera, frame: Frame):
        self._ck(lib.vpt_learned_input(self._h, C.byref(cam), C.byref(frame)), "vpt_learned_input")

    def learned_features(self, crop, out):
        """16-channel BF16 features of crop (x0, y0, w, h) into the torch tensor `out` [h, w, 16]."""
        x0, y0, w, h = crop
        if tuple(out.shape[-3:]) != (h, w, 16) or not out.is_contiguous():
            raise ValueError("out must be a contiguous [h, w, 16] bfloat16 tensor")
        self._ck(lib.vpt_learned_features(self._h, x0, y0, w, h, out.data_ptr()), "vpt_learned_features")

    def render_frame_learned(self, cam: Camera, frame: Frame, net=None, out: np.ndarray | None = None,
                             readback: bool = True):
        """A frame with the U-Net as spatial denoiser (SVGF fallback when net is None); returns (rgb, used_net)."""
        if readback and out is None:
            out = np.empty((self.height, self.width, 3), dtype=np.float32)
        used = C.c_int32()
        self._ck(lib.vpt_render_frame_learned(self._h, net._h if net is not None else None, C.byref(cam),
                                              C.byref(frame), _ptr(out) if readback else None, C.byref(used)),
                 "vpt_render_frame_learned")
        return out, bool(used.value)

    def plane_dims(self, plane) -> tuple:
        """(height, width) of a plane: the GI grid's for the GI-side planes."""
        pid = PLANE[plane] if isinstance(plane, str) else int(plane)
        w, h = C.c_int32(), C.c_int32()
        self._ck(lib.vpt_plane_dims(self._h, pid, C.byref(w), C.byref(h)), "vpt_plane_dims")
        return h.value, w.value

    def read_plane(self, plane) -> np.ndarray:
        pid, nbytes, ch, dt = self.plane_info(plane)
        out = np.empty((*self.plane_dims(pid), ch), dtype=dt)
        self._ck(lib.vpt_read_plane(self._h, pid, _ptr(out), out.nbytes), "vpt_read_plane")
        return out

    def write_plane(self, plane, data: np.ndarray):
        pid, nbytes, ch, dt = self.plane_info(plane)
        a = np.ascontiguousarray(np.asarray(data).reshape(*self.plane_dims(pid), ch), dtype=dt)
        self._ck(lib.vpt_write_plane(self._h, pid, _ptr(a), a.nbytes), "vpt_write_plane")

    # instrumentation
    def synchronize(self):
        self._ck(lib.vpt_synchronize(self._h), "vpt_synchronize")

    def set_stats(self, enabled: bool):
        self._ck(lib.vpt_set_stats(self._h, 1 if enabled else 0), "vpt_set_stats")

    def read_stats(self) -> dict:
        s = Stats()
        self._ck(lib.vpt_read_stats(self._h, C.byref(s)), "vpt_read_stats")
        kinds = RAY_KINDS
        return {"rays": dict(zip(kinds, list(s.rays))), "steps": dict(zip(kinds, list(s.steps)))}

    def set_profiling(self, enabled: bool):
        self._ck(lib.vpt_set_profiling(self._h, 1 if enabled else 0), "vpt_set_profiling")

    def pass_times(self) -> dict:
        arr = (C.c_float * len(PASSES))()
        self._ck(lib.vpt_read_pass_times(self._h, arr, len(PASSES)), "vpt_read_pass_times")
        return dict(zip(PASSES, list(arr)))

    def launch_count(self) -> int:
        v = C.c_uint64()
        self._ck(lib.vpt_launch_count(self._h, C.byref(v)), "vpt_launch_count")
        return int(v.value)

    def stream(self) -> int:
        p = C.c_void_p()
        self._ck(lib.vpt_get_stream(self._h, C.byref(p)), "vpt_get_stream")
        return p.value or 0


class Batch:
    """Many worlds traced together (vpt_batch_*): each world has its own
    volume, block table, camera and ray tile; `trace` runs the primary,
    sun-shadow and diffuse passes of every world in one persistent launch
    (replayed from a CUDA graph by default) or, for comparison, as three pass
    kernels per world."""

    def __init__(self, max_worlds: int = 64, device: int = 0, **overrides):
        cfg = BatchConfig()
        _check(lib.vpt_batch_default_config(C.byref(cfg)), "vpt_batch_default_config")
        cfg.max_worlds = max_worlds
        cfg.device = device
        for k, v in overrides.items():
            if not hasattr(cfg, k):
                raise AttributeError(f"unknown batch config field {k}")
            setattr(cfg, k, v)
        self.config = cfg
        self._h = C.c_void_p()
        _check(lib.vpt_batch_create(C.byref(self._h), C.byref(cfg)), "vpt_batch_create")
        self.tiles = []

    def close(self):
        if self._h:
            lib.vpt_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ck(self, status, what):
        if status != OK:
            msg = lib.vpt_status_string(status).decode()
            detail = lib.vpt_batch_last_error(self._h) if self._h else b""
            if detail:
                msg += f" ({detail.decode()})"
            raise VPTError(status, f"{what} failed: {msg}")

    def add_world(self, voxels: np.ndarray, table: np.ndarray, width: int, height: int) -> int:
        v = np.ascontiguousarray(voxels, dtype=np.uint8)
        if v.ndim != 3:
            raise ValueError("voxels must have shape (Z, Y, X)")
        t = np.ascontiguousarray(table, dtype=BLOCK_DTYPE)
        Z, Y, X = v.shape
        wid = C.c_int32()
        self._ck(lib.vpt_batch_add_world(self._h, _ptr(v), X, Y, Z, _ptr(t), t.size, width, height, C.byref(wid)),
                 "vpt_batch_add_world")
        self.tiles.append((height, width))
        return int(wid.value)

    def set_camera(self, world: int, cam: Camera):
        self._ck(lib.vpt_batch_set_camera(self._h, world, C.byref(cam)), "vpt_batch_set_camera")

    def build_df(self):
        self._ck(lib.vpt_batch_build_df(self._h), "vpt_batch_build_df")

    def read_df(self, world: int) -> np.ndarray:
        dims = (C.c_int32 * 3)()
        self._ck(lib.vpt_batch_world_info(self._h, world, dims, None), "vpt_batch_world_info")
        out = np.empty((dims[2], dims[1], dims[0]), np.uint8)
        self._ck(lib.vpt_batch_read_df(self._h, world, _ptr(out), out.nbytes), "vpt_batch_read_df")
        return out

    def set_tuning(self, block_threads=None, tiles_per_grab=None, df_brick=None, blocks=None, rays_per_lane=None,
                   phased=None):
        t = self.tuning()
        for k, v in (("block_threads", block_threads), ("tiles_per_grab", tiles_per_grab), ("df_brick", df_brick),
                     ("blocks", blocks), ("rays_per_lane", rays_per_lane), ("phased", phased)):
            if v is not None:
                setattr(t, k, int(v))
        self._ck(lib.vpt_batch_set_tuning(self._h, C.byref(t)), "vpt_batch_set_tuning")

    def tuning(self) -> BatchTuning:
        t = BatchTuning()
        self._ck(lib.vpt_batch_get_tuning(self._h, C.byref(t)), "vpt_batch_get_tuning")
        return t

    def trace(self, frame: Frame, mode: int = BATCH_GRAPH):
        self._ck(lib.vpt_batch_trace(self._h, C.byref(frame), mode), "vpt_batch_trace")

    def autotune(self, frame: Frame, reps: int = 3) -> list:
        recs = (BatchTuneRecord * 128)()
        n = C.c_int32()
        self._ck(lib.vpt_batch_autotune(self._h, C.byref(frame), reps, recs, 128, C.byref(n)), "vpt_batch_autotune")
        return [dict(recs[k].tuning.as_dict(), ms=float(recs[k].ms)) for k in range(n.value)]

    def read_plane(self, world: int, plane) -> np.ndarray:
        pid = PLANE[plane] if isinstance(plane, str) else int(plane)
        name = PLANES[pid]
        H, W = self.tiles[world]
        ch = {"HIT": 3, "GI_SH": 4, "GI_COCG": 2, "GI_AOSKY": 2}.get(name, 1)
        dt = {"FACE": np.uint8, "BLOCK": np.uint8, "SHADOW": np.uint8, "HIT": np.int32, "STEPS": np.uint16}.get(
            name, np.float32)
        out = np.empty((H, W, ch) if ch > 1 else (H, W), dt)
        self._ck(lib.vpt_batch_read_plane(self._h, world, pid, _ptr(out), out.nbytes), "vpt_batch_read_plane")
        return out

    def count(self) -> int:
        n = C.c_int32()
        self._ck(lib.vpt_batch_count(self._h, C.byref(n)), "vpt_batch_count")
        return int(n.value)

    def synchronize(self):
        self._ck(lib.vpt_batch_synchronize(self._h), "vpt_batch_synchronize")

    def set_stats(self, enabled: bool):
        self._ck(lib.vpt_batch_set_stats(self._h, 1 if enabled else 0), "vpt_batch_set_stats")

    def read_stats(self) -> dict:
        s = Stats()
        self._ck(lib.vpt_batch_read_stats(self._h, C.byref(s)), "vpt_batch_read_stats")
        kinds = RAY_KINDS
        return {"rays": dict(zip(kinds, list(s.rays))), "steps": dict(zip(kinds, list(s.steps)))}

    def launch_count(self) -> int:
        v = C.c_uint64()
        self._ck(lib.vpt_batch_launch_count(self._h, C.byref(v)), "vpt_batch_launch_count")
        return int(v.value)

    def stream(self) -> int:
        p = C.c_void_p()
        self._ck(lib.vpt_batch_get_stream(self._h, C.byref(p)), "vpt_batch_get_stream")
        return p.value or 0


# --------------------------------------------------------- learned denoiser --
UNET_LAYERS = 11


def unet_layers() -> list:
    """(cin, cout, cin_real, cout_real, param offset) of each layer (vpt_unet_layer_info)."""
    out = []
    for l in range(UNET_LAYERS):
        a, b, c, d = C.c_int32(), C.c_int32(), C.c_int32(), C.c_int32()
        o = C.c_int64()
        _check(lib.vpt_unet_layer_info(l, C.byref(a), C.byref(b), C.byref(c), C.byref(d), C.byref(o)),
               "vpt_unet_layer_info")
        out.append((a.value, b.value, c.value, d.value, o.value))
    return out


def _dptr(t) -> int | None:
    """Device address of a torch tensor (None passes NULL)."""
    return None if t is None else int(t.data_ptr())


def nn_conv3x3(in0, c0, in1, c1, n, h, w, weight, bias, cout, relu=False, mask=None, out=None, out_f32=None,
               up0=False, stream=0):
    """vpt_nn_conv3x3 over torch device tensors (BF16 NHWC; see include/vpt.h)."""
    _check(lib.vpt_nn_conv3x3(_dptr(in0), c0, 1 if up0 else 0, _dptr(in1), c1, n, h, w, _dptr(weight), _dptr(bias),
                              cout, 1 if relu else 0, _dptr(mask), _dptr(out), _dptr(out_f32), stream or None),
           "vpt_nn_conv3x3")


def nn_conv3x3_dw(in0, c0, in1, c1, n, h, w, dy, cout, dw, up0=False, stream=0):
    _check(lib.vpt_nn_conv3x3_dw(_dptr(in0), c0, 1 if up0 else 0, _dptr(in1), c1, n, h, w, _dptr(dy), cout,
                                 _dptr(dw), stream or None), "vpt_nn_conv3x3_dw")


def nn_status(stream=0):
    _check(lib.vpt_nn_status(stream or None), "vpt_nn_status")


class UNet:
    """The learned denoiser (vpt_unet_*). Inputs and targets are torch CUDA
    tensors: input [n, h, w, 16] bfloat16, target [n, h, w, 3] float32."""

    def __init__(self, max_images: int, max_height: int, max_width: int, device: int = 0):
        self._h = C.c_void_p()
        _check(lib.vpt_unet_create(C.byref(self._h), device, max_images, max_height, max_width), "vpt_unet_create")
        n = C.c_int64()
        self._ck(lib.vpt_unet_param_count(self._h, C.byref(n)), "vpt_unet_param_count")
        self.n_params = int(n.value)
        self.device = device

    def close(self):
        if self._h:
            lib.vpt_unet_destroy(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ck(self, status, what):
        if status != OK:
            msg = lib.vpt_status_string(status).decode()
            detail = lib.vpt_unet_last_error(self._h) if self._h else b""
            if detail:
                msg += f" ({detail.decode()})"
            raise VPTError(status, f"{what} failed: {msg}")

    def set_params(self, p: np.ndarray):
        p = np.ascontiguousarray(p, dtype=np.float32)
        self._ck(lib.vpt_unet_set_params(self._h, _ptr(p), p.size), "vpt_unet_set_params")

    def params(self) -> np.ndarray:
        out = np.empty(self.n_params, np.float32)
        self._ck(lib.vpt_unet_get_params(self._h, _ptr(out), out.size), "vpt_unet_get_params")
        return out

    def grads(self) -> np.ndarray:
        out = np.empty(self.n_params, np.float32)
        self._ck(lib.vpt_unet_get_grads(self._h, _ptr(out), out.size), "vpt_unet_get_grads")
        return out

    def forward(self, x, out=None):
        n, h, w, _ = x.shape
        self._ck(lib.vpt_unet_forward(self._h, _dptr(x), n, h, w, _dptr(out)), "vpt_unet_forward")
        return out

    def backward(self, x, target) -> float:
        n, h, w, _ = x.shape
        loss = C.c_double()
        self._ck(lib.vpt_unet_backward(self._h, _dptr(x), _dptr(target), n, h, w, C.byref(loss)),
                 "vpt_unet_backward")
        return float(loss.value)

    def adam(self, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8):
        self._ck(lib.vpt_unet_adam(self._h, lr, beta1, beta2, eps), "vpt_unet_adam")

    def synchronize(self):
        self._ck(lib.vpt_unet_synchronize(self._h), "vpt_unet_synchronize")

    def stream(self) -> int:
        p = C.c_void_p()
        self._ck(lib.vpt_unet_get_stream(self._h, C.byref(p)), "vpt_unet_get_stream")
        return p.value or 0


def device_available() -> bool:
    """True when a CUDA device can be opened by libvpt."""
    h = C.c_void_p()
    cfg = default_config(width=8, height=8)
    st = lib.vpt_create(C.byref(h), C.byref(cfg))
    if st == OK:
        lib.vpt_destroy(h)
        return True
    return False
