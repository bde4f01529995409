"""The C ABI library without a GPU: it loads, exports every entry point the
header declares, validates arguments, reports a missing device, and its host
helpers (world generator, block table, camera) behave as documented."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

HEADER = Path(__file__).resolve().parent.parent / "include" / "vpt.h"


def declared_functions():
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    return sorted(set(re.findall(r"\b(vpt_[a-z0-9_]+)\s*\(", text)))


def test_every_declared_symbol_is_exported(vpt):
    names = declared_functions()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(vpt.lib, n)]
    assert not missing, missing


def test_abi_version_and_status_strings(vpt):
    assert vpt.lib.vpt_abi_version() == 3
    for s in range(7):
        assert vpt.lib.vpt_status_string(s)


def test_struct_sizes_match_header(vpt, oracle):
    assert C.sizeof(vpt.Camera) == 4 * (16 * 4 + 4)
    assert C.sizeof(vpt.Block) == 6
    assert C.sizeof(vpt.Frame) == C.sizeof(oracle.OFrame) == 4 * 16
    assert C.sizeof(vpt.Config) == C.sizeof(oracle.OParams)


def test_defaults(vpt):
    cfg = vpt.default_config()
    assert (cfg.width, cfg.height, cfg.spp, cfg.bounces, cfg.atrous_iterations) == (1920, 1080, 1, 1, 5)
    assert cfg.diffuse_max_steps == 48 and cfg.bounce_shadow_max_steps == 128 and cfg.shadow_max_steps == 350
    assert cfg.gi_divisor == 1 and cfg.reflection_spp == 0
    assert (cfg.reflection_max_steps, cfg.reflection_shadow_max_steps) == (64, 150)
    assert C.sizeof(vpt.Stats) == 12 * 8
    f = vpt.default_frame()
    assert abs(np.linalg.norm(list(f.sun_dir)) - 1) < 1e-6 and f.temporal == 1


def test_invalid_arguments_are_rejected(vpt):
    h = C.c_void_p()
    bad = vpt.default_config(width=0)
    assert vpt.lib.vpt_create(C.byref(h), C.byref(bad)) == vpt.ERR_INVALID_ARG
    bad = vpt.default_config(spp=0)
    assert vpt.lib.vpt_create(C.byref(h), C.byref(bad)) == vpt.ERR_INVALID_ARG
    bad = vpt.default_config(storage=7)
    assert vpt.lib.vpt_create(C.byref(h), C.byref(bad)) == vpt.ERR_INVALID_ARG
    for field, value in (("reflection_spp", 17), ("reflection_spp", -1), ("reflection_max_steps", -1)):
        bad = vpt.default_config(**{field: value})
        assert vpt.lib.vpt_create(C.byref(h), C.byref(bad)) == vpt.ERR_INVALID_ARG, field
    assert vpt.lib.vpt_create(None, None) == vpt.ERR_INVALID_ARG
    assert vpt.lib.vpt_destroy(None) == vpt.ERR_INVALID_ARG
    assert vpt.lib.vpt_upload_world(None, None, 1, 1, 1) == vpt.ERR_INVALID_ARG
    assert vpt.lib.vpt_df_build_device(None, None, 4, 4, 4, None) == vpt.ERR_INVALID_ARG
    assert vpt.lib.vpt_generate_world(None, 4, 4, 4, 0, 100) == vpt.ERR_INVALID_ARG
    with pytest.raises(vpt.VPTError):
        vpt.generate_world(0, 4, 4)


def test_no_device_fails_loudly(vpt):
    """Without a GPU the context cannot be created: there is no CPU fallback."""
    if vpt.device_available():
        pytest.skip("a CUDA device is present")
    with pytest.raises(vpt.VPTError) as e:
        vpt.Context(width=8, height=8)
    assert e.value.status == vpt.ERR_NO_DEVICE


def test_world_generator(vpt):
    a = vpt.generate_world(96, 64, 80, seed=3)
    b = vpt.generate_world(96, 64, 80, seed=3)
    assert a.shape == (80, 64, 96) and np.array_equal(a, b)
    assert not np.array_equal(a, vpt.generate_world(96, 64, 80, seed=4))
    solid = a > 0
    heights = solid.sum(axis=1)                    # (Z, X) column heights
    assert 24 <= heights.min() and heights.max() <= 57    # 40 + 16 * fbm, fbm in [-1, 1]
    # columns are solid from the bottom up: stone, three dirt layers, a top block
    for z, x in [(0, 0), (40, 50), (79, 95)]:
        col = a[z, :, x]
        h = heights[z, x]
        assert (col[:h] > 0).all() and (col[h:] == 0).all()
        assert (col[: h - 4] == 3).all() and (col[h - 4: h - 1] == 2).all() and col[h - 1] in [1] + list(range(4, 100))
    tops = a[np.arange(80)[:, None], heights - 1, np.arange(96)[None, :]]
    assert 0.03 < (tops >= 4).mean() < 0.10        # one column in 16 gets a scattered block


def test_block_table(vpt):
    t = vpt.generate_block_table(100, seed=9)
    assert t.shape == (100,) and t[0]["emissive"] == 0 and (t[0]["albedo"] == 0).all()
    assert t["emissive"].sum() == 5                # round(5% of 99)
    assert (t["emissive"][:4] == 0).all()          # terrain layers are never emissive
    assert np.array_equal(t, vpt.generate_block_table(100, seed=9))


def test_camera_matrices(vpt):
    cam = vpt.camera_from_pose((10.0, 20.0, 30.0), 40.0, -20.0, 90.0, 16 / 9)
    view = np.array(cam.view, np.float64).reshape(4, 4).T
    proj = np.array(cam.proj, np.float64).reshape(4, 4).T
    iv = np.array(cam.inv_view, np.float64).reshape(4, 4).T
    ip = np.array(cam.inv_proj, np.float64).reshape(4, 4).T
    assert np.allclose(view @ iv, np.eye(4), atol=1e-5) and np.allclose(proj @ ip, np.eye(4), atol=1e-5)
    assert np.allclose(iv[:3, 3], [10, 20, 30], atol=1e-4)
    front = -iv[:3, 2]
    yaw, pitch = np.radians(40.0), np.radians(-20.0)
    assert np.allclose(front, [np.cos(yaw) * np.cos(pitch), np.sin(pitch), np.sin(yaw) * np.cos(pitch)], atol=1e-6)
    assert abs(proj[1, 1] - 1.0) < 1e-6            # 90 degree vertical field of view
    with pytest.raises(vpt.VPTError):
        vpt.camera_from_pose((0, 0, 0), 0.0, 90.0)  # straight up: lookAt is degenerate
