"""vpt_render_frame_async: the double-buffered readback delivers the same
images as vpt_render_frame, each complete once the next call returns (the
last one after vpt_readback_wait), in FP32 and FP16 storage."""
import numpy as np
import pytest

W, H = 96, 64


@pytest.mark.gpu
@pytest.mark.parametrize("storage", [0, 1], ids=["f32", "f16"])
def test_async_readback_matches_render_frame(vpt, storage, gpu):
    vox = vpt.generate_world(64, 64, 64, seed=4)
    blocks = vpt.generate_block_table(100, seed=4)
    yaw, pitch = vpt.seeded_pose(4)
    cams = [vpt.camera_from_pose((32.0 + 0.5 * k, 58.0, 32.0), yaw + 2.0 * k, pitch, 90.0, W / H) for k in range(5)]
    frames = [vpt.default_frame(frame_index=k, seed=2, time=0.1 * k) for k in range(5)]
    ctxs = []
    for _ in range(2):
        c = vpt.Context(width=W, height=H, primary_max_steps=256, storage=storage)
        c.upload_world(vox)
        c.set_block_table(blocks)
        c.build_df()
        ctxs.append(c)
    sync, asyn = ctxs
    want = [sync.render_frame(cam, fr) for cam, fr in zip(cams, frames)]
    outs = [np.full((H, W, 3), np.nan, np.float32) for _ in range(2)]
    for k, (cam, fr) in enumerate(zip(cams, frames)):
        asyn.render_frame_async(cam, fr, outs[k % 2])
        if k > 0:
            assert np.array_equal(outs[(k - 1) % 2], want[k - 1]), f"frame {k - 1}"
    asyn.readback_wait()
    assert np.array_equal(outs[(len(cams) - 1) % 2], want[-1])
    # the colour plane is this context's too, after the last frame
    for c in ctxs:
        c.close()
