"""Writes the golden fixtures of this directory from the CPU oracle.

    python tests/golden/make_golden.py

Two cases, both seeded and small enough to commit:

  primary_128.npz   The 128^3 terrain world of seed 0 and its distance field
                    (as SHA-256 digests and value histograms), and 640x360
                    primary rays from a pinhole at (64, 90, 64) with yaw/pitch
                    drawn from seed 0, 90 degree FOV, 256-step cap: SHA-256 of
                    the full t / face / block / hit / steps planes plus every
                    8th row and column of them as arrays.
  frame_64_*.npz    Two consecutive frames (the second with a moved camera, so
                    temporal reprojection runs) of a 64x40 image of the 64^3
                    world of seed 2 with the 100-entry block table of seed 2
                    (about half the pixels hit terrain):
                    every G-buffer plane, the shadow plane, the raw GI planes and
                    the shaded colour, for the SVGF denoiser and for the plain
                    a-trous denoiser.

The reference ships no numeric fixtures for this path; these pin the oracle
(and through it the CUDA path) against silent drift. Regenerate only on a
deliberate change of the restated algorithm, and say which in the commit.
"""
import hashlib
import importlib.util
import json
import pathlib
import sys

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
REPO = HERE.parents[1]
sys.path.insert(0, str(REPO))


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def primary_case(vpt, oracle):
    X = Y = Z = 128
    W, H = 640, 360
    vox = vpt.generate_world(X, Y, Z, seed=0)
    df = oracle.build_df(vox)
    blocks = vpt.generate_block_table(100, seed=0)
    yaw, pitch = vpt.seeded_pose(0)
    cam = vpt.camera_from_pose((64.0, 90.0, 64.0), yaw, pitch, 90.0, W / H)
    cfg = vpt.default_config(width=W, height=H, primary_max_steps=256)
    g = oracle.trace_primary(oracle.World(vox, df, blocks), cam, cfg)
    out = {
        "world_sha256": digest(vox), "df_sha256": digest(df),
        "world_hist": np.bincount(vox.ravel(), minlength=256).astype(np.int64),
        "df_hist": np.bincount(df.ravel(), minlength=256).astype(np.int64),
        "pose": np.array([yaw, pitch], np.float64),
    }
    for k, v in g.items():
        out[f"{k}_sha256"] = digest(v)
        out[f"{k}_sub"] = np.ascontiguousarray(v[::8, ::8])
    return out


def frame_case(vpt, oracle, denoiser: int):
    X = Y = Z = 64
    W, H = 64, 40
    vox = vpt.generate_world(X, Y, Z, seed=2)
    blocks = vpt.generate_block_table(100, seed=2)
    df = oracle.build_df(vox)
    world = oracle.World(vox, df, blocks)
    cfg = vpt.default_config(width=W, height=H, primary_max_steps=256, denoiser=denoiser)
    cams = [vpt.camera_from_pose((32.0, 60.0, 32.0), 40.0, -35.0, 90.0, W / H),
            vpt.camera_from_pose((32.5, 60.0, 32.25), 41.5, -35.0, 90.0, W / H)]
    prev_g, hist = oracle.empty_history(H, W)
    prev_cam = cams[0]
    out = {}
    for f, cam in enumerate(cams):
        frame = vpt.default_frame(seed=5, frame_index=f, time=0.016 * f)
        r = oracle.render_frame(world, cam, prev_cam, cfg, frame, prev_g, hist)
        for k, v in r["g"].items():
            out[f"f{f}_g_{k}"] = v
        out[f"f{f}_shadow"] = r["shadow"]
        for k, v in r["gi"].items():
            out[f"f{f}_gi_{k}"] = v
        out[f"f{f}_rgb"] = r["rgb"]
        prev_g = {k: r["g"][k] for k in ("t", "face", "block")}
        hist = r["svgf"]["temporal"]
        prev_cam = cam
    return out


def load():
    spec = importlib.util.spec_from_file_location("_vpt_build", REPO / "voxelpathtracer_gb300" / "_build.py")
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    b.build_all()
    import oracle
    import voxelpathtracer_gb300 as vpt
    return vpt, oracle


def main():
    vpt, oracle = load()
    np.savez_compressed(HERE / "primary_128.npz", **primary_case(vpt, oracle))
    for name, den in (("frame_64_svgf.npz", 0), ("frame_64_atrous.npz", 1)):
        np.savez_compressed(HERE / name, **frame_case(vpt, oracle, den))
    sizes = {p.name: p.stat().st_size for p in sorted(HERE.glob("*.npz"))}
    print(json.dumps(sizes))


if __name__ == "__main__":
    main()
