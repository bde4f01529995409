"""The committed golden fixtures (tests/golden/*.npz, written by
tests/golden/make_golden.py from the CPU oracle) against the oracle on the CPU
and against libvpt on the GPU.

The CPU half pins the world generator, the distance field, the primary
traversal and a whole two-frame render of the oracle to the committed bits;
the GPU half holds the CUDA path to the same bits through the C ABI.
"""
import hashlib
import pathlib

import numpy as np
import pytest

GOLDEN = pathlib.Path(__file__).resolve().parent / "golden"


def digest(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def load(name):
    return dict(np.load(GOLDEN / name))


def bits_equal(a, b):
    a = np.ascontiguousarray(np.asarray(a).reshape(np.asarray(b).shape))
    b = np.ascontiguousarray(b)
    if a.dtype != b.dtype:
        return False
    return a.tobytes() == b.tobytes()


# ------------------------------------------------------- 128^3 primary --
def primary_scene(vpt):
    vox = vpt.generate_world(128, 128, 128, seed=0)
    blocks = vpt.generate_block_table(100, seed=0)
    yaw, pitch = vpt.seeded_pose(0)
    cam = vpt.camera_from_pose((64.0, 90.0, 64.0), yaw, pitch, 90.0, 640 / 360)
    cfg = vpt.default_config(width=640, height=360, primary_max_steps=256)
    return vox, blocks, cam, cfg


def check_primary(gold, g):
    for k in ("t", "face", "block", "hit", "steps"):
        v = np.asarray(g[k])
        assert bits_equal(v[::8, ::8], gold[f"{k}_sub"]), f"{k}: sub-sampled plane differs from the golden"
        assert digest(v) == str(gold[f"{k}_sha256"]), f"{k}: SHA-256 differs from the golden"


def test_golden_world_and_df_oracle(vpt, oracle):
    gold = load("primary_128.npz")
    vox, _, _, _ = primary_scene(vpt)
    assert digest(vox) == str(gold["world_sha256"])
    assert np.array_equal(np.bincount(vox.ravel(), minlength=256), gold["world_hist"])
    df = oracle.build_df(vox)
    assert digest(df) == str(gold["df_sha256"])
    assert np.array_equal(np.bincount(df.ravel(), minlength=256), gold["df_hist"])


def test_golden_primary_oracle(vpt, oracle):
    gold = load("primary_128.npz")
    vox, blocks, cam, cfg = primary_scene(vpt)
    assert np.array_equal(np.array(vpt.seeded_pose(0)), gold["pose"])
    g = oracle.trace_primary(oracle.World(vox, oracle.build_df(vox), blocks), cam, cfg)
    hits = float((g["t"] > 0).mean())
    assert 0.1 < hits < 0.9, f"golden view should mix terrain and sky, hit fraction {hits}"
    check_primary(gold, g)


@pytest.mark.gpu
def test_golden_primary_gpu(vpt, gpu):
    gold = load("primary_128.npz")
    vox, blocks, cam, _ = primary_scene(vpt)
    with vpt.Context(width=640, height=360, primary_max_steps=256) as ctx:
        ctx.upload_world(vox)
        ctx.set_block_table(blocks)
        ctx.build_df()
        assert digest(ctx.read_df()) == str(gold["df_sha256"])
        ctx.trace_primary(cam)
        g = {k: ctx.read_plane(k.upper()) for k in ("t", "face", "block", "hit", "steps")}
    g = {k: (v[..., 0] if v.shape[-1] == 1 else v) for k, v in g.items()}
    check_primary(gold, g)


# ------------------------------------------------------- 64^3 two frames --
W, H = 64, 40


def frame_scene(vpt, denoiser):
    vox = vpt.generate_world(64, 64, 64, seed=2)
    blocks = vpt.generate_block_table(100, seed=2)
    cfg = vpt.default_config(width=W, height=H, primary_max_steps=256, denoiser=denoiser)
    cams = [vpt.camera_from_pose((32.0, 60.0, 32.0), 40.0, -35.0, 90.0, W / H),
            vpt.camera_from_pose((32.5, 60.0, 32.25), 41.5, -35.0, 90.0, W / H)]
    frames = [vpt.default_frame(seed=5, frame_index=f, time=0.016 * f) for f in range(2)]
    return vox, blocks, cfg, cams, frames


@pytest.mark.parametrize("name,denoiser", [("frame_64_svgf.npz", 0), ("frame_64_atrous.npz", 1)],
                         ids=["svgf", "atrous"])
def test_golden_frames_oracle(vpt, oracle, name, denoiser):
    gold = load(name)
    vox, blocks, cfg, cams, frames = frame_scene(vpt, denoiser)
    world = oracle.World(vox, oracle.build_df(vox), blocks)
    prev_g, hist = oracle.empty_history(H, W)
    prev_cam = cams[0]
    for f, (cam, frame) in enumerate(zip(cams, frames)):
        r = oracle.render_frame(world, cam, prev_cam, cfg, frame, prev_g, hist)
        for k, v in r["g"].items():
            assert bits_equal(v, gold[f"f{f}_g_{k}"]), f"frame {f} {k}"
        assert bits_equal(r["shadow"], gold[f"f{f}_shadow"]), f"frame {f} shadow"
        for k, v in r["gi"].items():
            assert bits_equal(v, gold[f"f{f}_gi_{k}"]), f"frame {f} gi {k}"
        assert bits_equal(r["rgb"], gold[f"f{f}_rgb"]), f"frame {f} colour"
        prev_g = {k: r["g"][k] for k in ("t", "face", "block")}
        hist = r["svgf"]["temporal"]
        prev_cam = cam


@pytest.mark.gpu
@pytest.mark.parametrize("name,denoiser", [("frame_64_svgf.npz", 0), ("frame_64_atrous.npz", 1)],
                         ids=["svgf", "atrous"])
def test_golden_frames_gpu(vpt, gpu, name, denoiser):
    gold = load(name)
    vox, blocks, cfg, cams, frames = frame_scene(vpt, denoiser)
    with vpt.Context(width=W, height=H, primary_max_steps=256, denoiser=denoiser) as ctx:
        ctx.upload_world(vox)
        ctx.set_block_table(blocks)
        ctx.build_df()
        for f, (cam, frame) in enumerate(zip(cams, frames)):
            rgb = ctx.render_frame(cam, frame)
            assert bits_equal(rgb, gold[f"f{f}_rgb"]), f"frame {f} colour"
            # end_frame moved this frame's G-buffer to the PREV_* planes
            for k in ("t", "face", "block"):
                assert bits_equal(ctx.read_plane("PREV_" + k.upper()), gold[f"f{f}_g_{k}"]), f"frame {f} {k}"
            assert bits_equal(ctx.read_plane("SHADOW"), gold[f"f{f}_shadow"]), f"frame {f} shadow"
            for k in ("sh", "cocg", "luma", "aosky"):
                assert bits_equal(ctx.read_plane("GI_" + k.upper()), gold[f"f{f}_gi_{k}"]), f"frame {f} gi {k}"
