"""The oracle's math conventions and the benchmark's camera against the
reference's own glm (its vendored glm 0.9.8.5, built from the reference tree
by oracle/build_ref.py into oracle/_ref/libglm_ref.so; skipped where that tree
is absent, e.g. on the GPU machines).

The reference's hot path is GLSL, whose builtins the GPU driver evaluates; the
oracle (and every kernel, bit for bit) fixes one evaluation of each. This file
states where that equals glm's and where it deliberately does not:

* dot, cross, length and normalize (x * (1 / sqrt(dot(x, x)))) equal glm's
  bit for bit;
* mix is the GLSL specification's x * (1 - a) + y * a; glm evaluates
  x + a * (y - x), so the two differ in the last bits where they round
  differently;
* a matrix times a vector sums its four products left to right; glm sums them
  pairwise, (m0 x + m1 y) + (m2 z + m3 w);
* the benchmark's cameras are built in float64 and rounded once
  (vpt_camera_from_pose); the reference's FPSCamera (Core/FpsCamera.cpp) builds
  them in float32 with glm, from a front vector added to and subtracted from
  the position, which moves its view matrix by up to ~5e-4. Tracing the
  128^3 / 640x360 frame with either camera changes the hit voxel of about 1 in
  20,000 rays.
"""
import ctypes as C

import numpy as np
import pytest

from oracle import build_ref

LIB = build_ref.OUT_GLM


@pytest.fixture(scope="module")
def glm():
    if build_ref.build_glm() is None or not LIB.exists():
        pytest.skip("the reference tree (its vendored glm) is not present")
    L = C.CDLL(str(LIB))
    P = C.c_void_p
    L.glmref_vecmath.argtypes = [C.c_int, P, P, P, P, C.c_int]
    L.glmref_fps_camera.argtypes = [P] + [C.c_float] * 6 + [P] * 4
    return L


def glm_vecmath(L, op, a, b, c):
    a, b, c = (np.ascontiguousarray(x, np.float32) for x in (a, b, c))
    out = np.zeros((a.shape[0], 4 if op == 5 else 3), np.float32)
    L.glmref_vecmath(op, a.ctypes.data, b.ctypes.data, c.ctypes.data, out.ctypes.data, a.shape[0])
    return out


def glm_camera(L, pos, yaw, pitch, fov, aspect, vpt):
    mats = [np.zeros(16, np.float32) for _ in range(4)]
    p = np.asarray(pos, np.float32)
    L.glmref_fps_camera(p.ctypes.data, yaw, pitch, fov, aspect, 0.1, 1000.0, *[m.ctypes.data for m in mats])
    cam = vpt.Camera()
    for name, m in zip(("view", "proj", "inv_view", "inv_proj"), mats):
        getattr(cam, name)[:] = m.tolist()
    cam.position[:] = [float(v) for v in p]
    return cam


@pytest.fixture(scope="module")
def inputs():
    rng = np.random.default_rng(0)
    n = 100000
    return (rng.uniform(-100, 100, (n, 3)), rng.uniform(-100, 100, (n, 3)), rng.uniform(0, 1, (n, 3)),
            rng.uniform(-2, 2, (n, 16)), rng.uniform(-100, 100, (n, 4)))


@pytest.mark.parametrize("op", [0, 1, 2, 3], ids=["dot", "cross", "length", "normalize"])
def test_vector_builtins_equal_glm(oracle, glm, inputs, op):
    a, b, c, _, _ = inputs
    mine, theirs = oracle.vecmath(op, a, b, c), glm_vecmath(glm, op, a, b, c)
    assert np.array_equal(mine.view(np.uint32), theirs.view(np.uint32))


def test_mix_is_the_glsl_formula(oracle, glm, inputs):
    a, b, c, _, _ = inputs
    mine, theirs = oracle.vecmath(4, a, b, c)[:, 0], glm_vecmath(glm, 4, a, b, c)[:, 0]
    x, y, t = a[:, 0].astype(np.float32), b[:, 0].astype(np.float32), c[:, 0].astype(np.float32)
    spec = (x * (np.float32(1) - t) + y * t).astype(np.float32)     # x (1 - a) + y a, each step rounded
    assert np.array_equal(mine.view(np.uint32), spec.view(np.uint32))
    scale = np.abs(x) + np.abs(y)
    assert (np.abs(mine.astype(np.float64) - theirs) <= 4 * np.finfo(np.float32).eps * scale).all()
    assert 0.3 < float((mine == theirs).mean()) < 0.9   # the two evaluations do differ


def test_matrix_vector_sums_left_to_right(oracle, glm, inputs):
    _, _, c, m, v = inputs
    mine, theirs = oracle.vecmath(5, m, v, c), glm_vecmath(glm, 5, m, v, c)
    M = m.astype(np.float32).reshape(-1, 4, 4)   # [item][column][row]
    V = v.astype(np.float32)
    seq = M[:, 0, :] * V[:, 0:1]
    for k in (1, 2, 3):
        seq = (seq + M[:, k, :] * V[:, k:k + 1]).astype(np.float32)
    assert np.array_equal(mine.view(np.uint32), seq.view(np.uint32))
    terms = np.abs(M * V[:, :, None]).sum(axis=1)
    assert (np.abs(mine.astype(np.float64) - theirs) <= 4 * np.finfo(np.float32).eps * terms).all()


def test_benchmark_camera_against_fps_camera(vpt, oracle, glm):
    """vpt_camera_from_pose against the reference's FPSCamera construction, and
    what the difference does to a traced frame (128^3 world, 640x360)."""
    W, H = 640, 360
    yaw, pitch = vpt.seeded_pose(0)
    mine = vpt.camera_from_pose((64.0, 90.0, 64.0), yaw, pitch, 90.0, W / H)
    ref = glm_camera(glm, (64.0, 90.0, 64.0), yaw, pitch, 90.0, W / H, vpt)
    d = {k: np.abs(np.array(getattr(mine, k), np.float64) - np.array(getattr(ref, k), np.float64)).max()
         for k in ("view", "proj", "inv_view", "inv_proj")}
    assert d["view"] < 2e-3 and d["inv_view"] < 2e-3 and d["proj"] < 1e-6 and d["inv_proj"] < 1e-5, d
    vox = vpt.generate_world(128, 128, 128, seed=0)
    world = oracle.World(vox, oracle.build_df(vox), vpt.generate_block_table(100, seed=0))
    cfg = vpt.default_config(width=W, height=H, primary_max_steps=256)
    g1, g2 = oracle.trace_primary(world, mine, cfg), oracle.trace_primary(world, ref, cfg)
    differ = float((g1["hit"] != g2["hit"]).any(-1).mean())
    assert differ < 1e-3, differ
