"""The SVGF temporal pass's reprojection against an analytic projection.

SVGF/TemporalFilter.glsl rebuilds each texel's world position from the hit
distance (GetPositionAt, :82-86) and projects it through the previous frame's
view-projection (ProjectPositionPrevious / Reprojection, :61-73). libvpt's
k_temporal equals the oracle's temporal pass bit for bit on every plane
(tests/test_gpu_parity.py, tests/test_parity_configs.py), so pinning the
oracle's geometry pins the kernel's. Here the oracle's positions and
reprojected coordinates are checked against an independent float64
construction: the primary ray intersected with the plane of the face the
traversal reported, projected through float64 glm::lookAt / glm::perspective
matrices of the previous pose. Host code only.
"""
import numpy as np
import pytest

W, H = 96, 64


def glm_camera64(pos, yaw_deg, pitch_deg, fov_deg=90.0, aspect=W / H, znear=0.1, zfar=1000.0):
    """float64 view and projection matrices (row-major numpy, column vectors)."""
    yaw, pitch = np.radians(yaw_deg), np.radians(pitch_deg)
    f = np.array([np.cos(yaw) * np.cos(pitch), np.sin(pitch), np.sin(yaw) * np.cos(pitch)])
    f /= np.linalg.norm(f)
    s = np.cross(f, [0.0, 1.0, 0.0])
    s /= np.linalg.norm(s)
    u = np.cross(s, f)
    eye = np.asarray(pos, np.float64)
    view = np.eye(4)
    view[0, :3], view[1, :3], view[2, :3] = s, u, -f
    view[:3, 3] = [-s @ eye, -u @ eye, f @ eye]
    th = np.tan(np.radians(fov_deg) / 2.0)
    proj = np.zeros((4, 4))
    proj[0, 0] = 1.0 / (aspect * th)
    proj[1, 1] = 1.0 / th
    proj[2, 2] = -(zfar + znear) / (zfar - znear)
    proj[3, 2] = -1.0
    proj[2, 3] = -(2.0 * zfar * znear) / (zfar - znear)
    return view, proj, eye


NORMALS = np.array([[0, 0, 1], [0, 0, -1], [0, 1, 0], [0, -1, 0], [-1, 0, 0], [1, 0, 0]], np.float64)


@pytest.mark.parametrize("move", ["pan", "translate", "static"])
def test_reprojection_matches_analytic_projection(vpt, oracle, move):
    X = Y = Z = 64
    vox = vpt.generate_world(X, Y, Z, seed=1)
    blocks = vpt.generate_block_table(100, seed=1)
    world = oracle.World(vox, oracle.build_df(vox), blocks)
    yaw, pitch = vpt.seeded_pose(1)
    prev_pose = ((X / 2, 58.0, Z / 2), yaw, pitch)
    cur_pose = {"pan": ((X / 2 + 0.7, 58.2, Z / 2 - 0.4), yaw + 2.0, pitch + 1.0),
                "translate": ((X / 2 + 1.5, 57.0, Z / 2 + 0.5), yaw, pitch),
                "static": prev_pose}[move]
    cam = vpt.camera_from_pose(cur_pose[0], cur_pose[1], cur_pose[2], 90.0, W / H)
    prev_cam = vpt.camera_from_pose(prev_pose[0], prev_pose[1], prev_pose[2], 90.0, W / H)
    cfg = vpt.default_config(width=W, height=H, primary_max_steps=256)
    g = oracle.trace_primary(world, cam, cfg)
    pos, uv_prev = oracle.reproject(cam, prev_cam, g["t"])

    view, proj, eye = glm_camera64(*cur_pose)
    pview, pproj, _ = glm_camera64(*prev_pose)
    inv_vp = np.linalg.inv(proj @ view)
    hit = g["t"] > 0
    assert 0.2 < hit.mean() < 0.98
    checked = 0
    for j, i in zip(*np.nonzero(hit)):
        # the primary ray through the texel centre, float64
        ndc = np.array([(i + 0.5) / W * 2 - 1, (j + 0.5) / H * 2 - 1, -1.0, 1.0])
        p = inv_vp @ ndc
        d = p[:3] / p[3] - eye
        d /= np.linalg.norm(d)
        # the plane of the face the traversal reports: the hit voxel's face
        # whose outward normal points back along the ray
        n = NORMALS[g["face"][j, i]]
        if abs(d @ n) < 0.1:
            continue   # grazing rays: the plane intersection is ill-conditioned
        vx = g["hit"][j, i].astype(np.float64)
        plane = vx + (n > 0)   # +x face at x + 1, -x face at x, ...
        axis = int(np.argmax(np.abs(n)))
        P = eye + d * ((plane[axis] - eye[axis]) / d[axis])
        # GetPositionAt's position, from the fp32 hit distance (the traversal
        # stops within its 1e-4 nudge of the face)
        assert np.abs(pos[j, i] - P).max() < 2e-3, (i, j, pos[j, i], P)
        # Reprojection: previous view-projection, perspective divide, to [0, 1]
        c = pproj @ pview @ np.append(P, 1.0)
        uv = c[:2] / c[3] * 0.5 + 0.5
        assert np.abs(uv_prev[j, i] - uv).max() < 1e-5, (i, j, uv_prev[j, i], uv)
        if move == "static":   # the previous coordinate of an unmoved camera is the texel centre
            assert np.abs(uv - [(i + 0.5) / W, (j + 0.5) / H]).max() < 1e-9
        checked += 1
    assert checked > 0.5 * hit.sum()
