"""The oracle's own input generators (oracle/inputs.py) against libvpt's.

The CPU reference arm of the benchmark builds its world, block table, cameras
and frame constants with oracle.inputs so that it never loads libvpt; the GPU
arm uses libvpt's host generators. Both follow the benchmark's description of
the seeded workload independently, so they must agree value for value: the
same voxels, the same table, the same fp32 matrices. Host code only (no GPU).
"""
import ctypes as C

import numpy as np
import pytest

from oracle import inputs


@pytest.mark.parametrize("dims,seed", [((64, 64, 64), 0), ((128, 128, 128), 0), ((37, 80, 19), 5),
                                       ((256, 48, 8), 123456789), ((1, 1, 1), 2)])
def test_world_generator_matches_libvpt(vpt, dims, seed):
    X, Y, Z = dims
    assert np.array_equal(inputs.generate_world(X, Y, Z, seed=seed), vpt.generate_world(X, Y, Z, seed=seed))


def test_world_generator_block_counts(vpt):
    for n in (4, 5, 17, 256):
        assert np.array_equal(inputs.generate_world(48, 64, 40, seed=9, n_blocks=n),
                              vpt.generate_world(48, 64, 40, seed=9, n_blocks=n))


@pytest.mark.parametrize("n,seed", [(100, 0), (100, 1), (256, 7), (5, 3), (1, 0), (21, 2 ** 63 + 5)])
def test_block_table_matches_libvpt(vpt, n, seed):
    a = inputs.generate_block_table(n, seed=seed)
    b = vpt.generate_block_table(n, seed=seed)
    assert a.tobytes() == b.tobytes()
    if n > 4:
        assert int(a["emissive"].sum()) == min(max(int(np.floor(0.05 * (n - 1) + 0.5)), 1), n - 4)


def test_cameras_match_libvpt(vpt):
    rng = np.random.default_rng(3)
    poses = [((128.0, 90.0, 128.0), *inputs.seeded_pose(0), 90.0, 1920 / 1080)]
    for _ in range(200):
        pos = tuple(float(v) for v in rng.uniform(-50, 600, 3))
        poses.append((pos, float(rng.uniform(-720, 720)), float(rng.uniform(-89, 89)), float(rng.uniform(1, 170)),
                      float(rng.uniform(0.1, 5000))))
    for pos, yaw, pitch, fov, aspect in poses:
        a = inputs.camera_from_pose(pos, yaw, pitch, fov, aspect)
        b = vpt.camera_from_pose(pos, yaw, pitch, fov, aspect)
        assert bytes(memoryview(a)) == bytes(memoryview(b)), (pos, yaw, pitch, fov, aspect)


def test_defaults_match_libvpt(vpt):
    assert C.sizeof(inputs.default_config()) == C.sizeof(vpt.default_config())
    assert bytes(memoryview(inputs.default_config())) == bytes(memoryview(vpt.default_config()))
    assert bytes(memoryview(inputs.default_config(width=640, height=360, primary_max_steps=256))) == \
        bytes(memoryview(vpt.default_config(width=640, height=360, primary_max_steps=256)))
    kw = dict(frame_index=7, seed=3, time=1.25)
    assert bytes(memoryview(inputs.default_frame(**kw))) == bytes(memoryview(vpt.default_frame(**kw)))
    assert inputs.seeded_pose(4) == vpt.seeded_pose(4)
