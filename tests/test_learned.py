"""The learned denoiser inside the frame path: its SVGF fallback, its input
features, and what a network trained on this tracer's pairs gains."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DIMS = (128, 128, 128)
W, H = 320, 192


@pytest.fixture(scope="module")
def world(vpt):
    vox = vpt.generate_world(*DIMS, seed=21)
    blocks = vpt.generate_block_table(100, seed=21)
    return vox, blocks


def make_ctx(vpt, world, **kw):
    c = vpt.Context(width=W, height=H, **kw)
    c.upload_world(world[0])
    c.set_block_table(world[1])
    c.build_df()
    return c


def pan(vpt, k):
    yaw, pitch = 40.0 + 0.5 * k, -30.0
    return vpt.camera_from_pose((64.0 + 0.1 * k, 90.0, 64.0), yaw, pitch, 90.0, W / H)


def test_fallback_is_the_svgf_frame(vpt, world, gpu):
    """Without a network the learned frame path renders the SVGF frame, bit for bit."""
    with make_ctx(vpt, world) as a, make_ctx(vpt, world) as b:
        for k in range(3):
            fr = vpt.default_frame(frame_index=k, seed=2)
            ref = a.render_frame(pan(vpt, k), fr)
            got, used = b.render_frame_learned(pan(vpt, k), fr, None)
            assert not used
            assert np.array_equal(ref.view(np.uint32), got.view(np.uint32))


def test_features_follow_the_planes(vpt, world, gpu):
    import torch
    with make_ctx(vpt, world) as c:
        for k in range(2):
            c.render_frame(pan(vpt, k), vpt.default_frame(frame_index=k, seed=3), readback=False)
        fr = vpt.default_frame(frame_index=2, seed=3)
        c.learned_input(pan(vpt, 2), fr)
        crop = (40, 24, 64, 48)
        x0, y0, cw, ch = crop
        out = torch.empty((ch, cw, 16), dtype=torch.bfloat16, device="cuda")
        c.learned_features(crop, out)
        got = out.float().cpu().numpy()
        sl = (slice(y0, y0 + ch), slice(x0, x0 + cw))
        color = c.read_plane("COLOR")[sl].astype(np.float64)
        t = c.read_plane("T")[sl][..., 0].astype(np.float64)
        face = c.read_plane("FACE")[sl][..., 0]
        block = c.read_plane("BLOCK")[sl][..., 0]
        var = c.read_plane("VAR_VARIANCE")[sl][..., 0].astype(np.float64)
        c.shade_from(fr, 2)
        raw = c.read_plane("COLOR")[sl].astype(np.float64)
    blocks = world[1]
    ref = np.zeros((ch, cw, 16))
    ref[..., 0:3] = np.log1p(np.maximum(color, 0))
    alb = blocks["albedo"][block] / 255.0
    ref[..., 3:6] = np.where((block > 0)[..., None], alb, 0.0)
    normals = np.array([[0, 0, 1], [0, 0, -1], [0, 1, 0], [0, -1, 0], [-1, 0, 0], [1, 0, 0]], np.float64)
    ref[..., 6:9] = np.where((face <= 5)[..., None], normals[np.minimum(face, 5)], 0.0)
    ref[..., 9] = np.where(t > 0, np.minimum(t, 512) / 128, 0.0)
    ref[..., 10] = np.log1p(np.maximum(var, 0))
    ref[..., 11:14] = np.log1p(np.maximum(raw, 0))
    assert (face <= 5).any() and (face > 5).any()
    assert not np.allclose(ref[..., 0:3], ref[..., 11:14])     # accumulated and raw colour differ
    assert np.allclose(got, ref, rtol=1e-2, atol=1e-2), np.abs(got - ref).max()
    assert np.all(got[..., 14:] == 0)


def test_trained_network_gains_over_its_input(vpt, gpu):
    """Train briefly on tracer-generated 1-spp / high-spp pairs; on held-out
    crops the network's error is well below that of its noisy input (the
    frame without a spatial denoiser)."""
    from voxelpathtracer_gb300 import learned
    X, T = learned.generate_pairs(160, crop=(64, 64), spp=256, n_worlds=2, dims=DIMS, frame_size=(W, H),
                                  history=(1, 24), seed=5)
    with vpt.UNet(8, 64, 64) as net:
        net.set_params(learned.he_init(1))
        losses = learned.train(net, X[:128], T[:128], steps=800, batch=8, lr=2e-3)
        pred = learned.predict_crops(net, X[128:])
    noisy = learned.crop_rmse(X[128:, ..., :3].float(), T[128:])
    net_err = learned.crop_rmse(pred, T[128:])
    print(f"holdout RMSE: noisy input {noisy:.4f}, network {net_err:.4f}; loss {losses[0]:.5f} -> {losses[-1]:.5f}")
    assert np.isfinite(net_err)
    assert net_err < 0.85 * noisy


def test_learned_frame_with_a_network(vpt, world, gpu):
    from voxelpathtracer_gb300 import learned
    with make_ctx(vpt, world) as c, vpt.UNet(1, H, W) as net:
        net.set_params(learned.he_init(0))
        c.set_profiling(True)
        for k in range(2):
            rgb, used = c.render_frame_learned(pan(vpt, k), vpt.default_frame(frame_index=k, seed=4), net)
            assert used
            assert np.isfinite(rgb).all() and (rgb >= 0).all()
        assert c.pass_times()["learned"] > 0


def test_pair_generation_fp16_two_bounces(vpt, gpu):
    """Pairs for the large configuration: FP16 input planes, 2 bounces, the
    ground truth from a second (FP32) context."""
    from voxelpathtracer_gb300 import learned
    X, T = learned.generate_pairs(6, crop=(32, 32), spp=64, n_worlds=1, dims=(64, 64, 64), frame_size=(128, 64),
                                  history=(1, 6), seed=2, bounces=2, storage=1)
    x, t = X.float().cpu().numpy(), T.cpu().numpy()
    assert np.isfinite(x).all() and np.isfinite(t).all()
    assert (x[..., :3] > 0).any() and (t > 0).any()
    assert np.all(x[..., 14:] == 0)
