"""vpt_trace_frame_noalloc, the frame trace that allocates nothing.

Some callers cannot allocate GPU memory while they render: engines that hand
out every byte of device memory from a budget fixed at start-up, and frame
loops that cannot absorb cudaMalloc's implicit device synchronisation. For
them libvpt has a variant of vpt_trace_frame that takes every input and
output buffer from the caller and keeps its only scratch (the work queue's
counter) in a small static device array. This test owns all device buffers
(allocated here, by the caller), calls the variant through the C ABI twice in
a row, and checks each result bit for bit against vpt_trace_frame on a
libvpt context. The file sorts last so that a run stopping at the first
failure has run every other test before it.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

W, H = 80, 48
PLANES = ["T", "FACE", "BLOCK", "HIT", "STEPS", "SHADOW", "GI_SH", "GI_COCG", "GI_LUMA", "GI_AOSKY"]


def test_noalloc_trace_matches_context_trace_twice(vpt, gpu):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda", 0)
    X, Y, Z = 56, 56, 56
    vox = vpt.generate_world(X, Y, Z, seed=7)
    blocks = vpt.generate_block_table(100, seed=7)
    cams = [vpt.camera_from_pose((28.0, 52.0, 28.0), 33.0, -28.0, 90.0, W / H),
            vpt.camera_from_pose((29.5, 51.0, 26.0), 140.0, -35.0, 90.0, W / H)]
    cfg = vpt.default_config(width=W, height=H, primary_max_steps=256)

    # caller-owned device buffers
    d_vox = torch.from_numpy(vox.reshape(-1)).to(dev)
    d_df = torch.empty_like(d_vox)
    d_blocks = torch.from_numpy(blocks.view(np.uint8).copy()).to(dev)
    assert vpt.lib.vpt_df_build_device(C.c_void_p(d_vox.data_ptr()), C.c_void_p(d_df.data_ptr()), X, Y, Z,
                                       None) == vpt.OK
    out = {
        "T": torch.empty(H * W, dtype=torch.float32, device=dev),
        "FACE": torch.empty(H * W, dtype=torch.uint8, device=dev),
        "BLOCK": torch.empty(H * W, dtype=torch.uint8, device=dev),
        "HIT": torch.empty(H * W * 3, dtype=torch.int32, device=dev),
        "STEPS": torch.empty(H * W, dtype=torch.int16, device=dev),
        "SHADOW": torch.empty(H * W, dtype=torch.uint8, device=dev),
        "GI_SH": torch.empty(H * W * 4, dtype=torch.float32, device=dev),
        "GI_COCG": torch.empty(H * W * 2, dtype=torch.float32, device=dev),
        "GI_LUMA": torch.empty(H * W, dtype=torch.float32, device=dev),
        "GI_AOSKY": torch.empty(H * W * 2, dtype=torch.float32, device=dev),
    }
    p = lambda t: t.data_ptr()  # noqa: E731
    bufs = vpt.TraceBuffers(p(d_vox), p(d_df), X, Y, Z, p(d_blocks), len(blocks), p(out["T"]), p(out["FACE"]),
                            p(out["BLOCK"]), p(out["HIT"]), p(out["STEPS"]), p(out["SHADOW"]), p(out["GI_SH"]),
                            p(out["GI_COCG"]), p(out["GI_LUMA"]), p(out["GI_AOSKY"]))

    with vpt.Context(cfg) as ctx:
        ctx.upload_world(vox)
        ctx.set_block_table(blocks)
        ctx.build_df()
        for call, cam in enumerate(cams):
            frame = vpt.default_frame(frame_index=call, seed=4)
            ctx.trace_frame(cam, frame)
            torch.cuda.synchronize()
            st = vpt.lib.vpt_trace_frame_noalloc(C.byref(bufs), C.byref(cfg), C.byref(cam), C.byref(frame), None)
            assert st == vpt.OK, vpt.lib.vpt_status_string(st)
            torch.cuda.synchronize()
            for name in PLANES:
                want = ctx.read_plane(name).reshape(-1)
                got = out[name].cpu().numpy().view(want.dtype)
                if want.dtype.kind == "f":
                    same = (got.view(np.uint32) == want.view(np.uint32)) | ((got == 0) & (want == 0))
                else:
                    same = got == want
                assert same.all(), f"call {call}: {name} differs in {int((~same).sum())} of {same.size} values"
            ctx.end_frame()


def _caller_buffers(vpt, torch, dev, vox, blocks, W, H):
    """Device buffers a caller would own for a W x H trace of world vox."""
    Z, Y, X = vox.shape
    d_vox = torch.from_numpy(vox.reshape(-1)).to(dev)
    d_df = torch.empty_like(d_vox)
    d_blocks = torch.from_numpy(blocks.view(np.uint8).copy()).to(dev)
    assert vpt.lib.vpt_df_build_device(C.c_void_p(d_vox.data_ptr()), C.c_void_p(d_df.data_ptr()), X, Y, Z,
                                       None) == vpt.OK
    n = W * H
    out = {"T": torch.empty(n, dtype=torch.float32, device=dev), "FACE": torch.empty(n, dtype=torch.uint8, device=dev),
           "BLOCK": torch.empty(n, dtype=torch.uint8, device=dev),
           "HIT": torch.empty(n * 3, dtype=torch.int32, device=dev),
           "STEPS": torch.empty(n, dtype=torch.int16, device=dev),
           "SHADOW": torch.empty(n, dtype=torch.uint8, device=dev),
           "GI_SH": torch.empty(n * 4, dtype=torch.float32, device=dev),
           "GI_COCG": torch.empty(n * 2, dtype=torch.float32, device=dev),
           "GI_LUMA": torch.empty(n, dtype=torch.float32, device=dev),
           "GI_AOSKY": torch.empty(n * 2, dtype=torch.float32, device=dev)}
    p = lambda t: t.data_ptr()  # noqa: E731
    bufs = vpt.TraceBuffers(p(d_vox), p(d_df), X, Y, Z, p(d_blocks), len(blocks), p(out["T"]), p(out["FACE"]),
                            p(out["BLOCK"]), p(out["HIT"]), p(out["STEPS"]), p(out["SHADOW"]), p(out["GI_SH"]),
                            p(out["GI_COCG"]), p(out["GI_LUMA"]), p(out["GI_AOSKY"]))
    return bufs, out, (d_vox, d_df, d_blocks)


def test_noalloc_rejects_oversized_and_missing_buffers(vpt, gpu):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda", 0)
    cam = vpt.camera_from_pose((32.0, 60.0, 32.0), 30.0, -50.0)
    frame = vpt.default_frame()
    call = lambda b, c: vpt.lib.vpt_trace_frame_noalloc(C.byref(b), C.byref(c), C.byref(cam),  # noqa: E731
                                                         C.byref(frame), None)
    # missing buffers
    assert call(vpt.TraceBuffers(), vpt.default_config(width=64, height=64)) == vpt.ERR_INVALID_ARG

    # valid caller buffers for the largest accepted width, so the size checks
    # themselves are what reject the oversized calls below
    Wmax, Hs = 16384, 4
    vox = vpt.generate_world(64, 64, 64, seed=3)
    blocks = vpt.generate_block_table(100, seed=3)
    bufs, out, keep = _caller_buffers(vpt, torch, dev, vox, blocks, Wmax, Hs)
    for w, h in ((Wmax + 1, Hs), (20000, Hs), (Hs, 20000), (64, 16385)):
        assert call(bufs, vpt.default_config(width=w, height=h)) == vpt.ERR_INVALID_ARG, (w, h)
    # every plane is width x height: a coarser GI grid is refused, not written past its end
    assert call(bufs, vpt.default_config(width=64, height=64, gi_divisor=2)) == vpt.ERR_INVALID_ARG
    torch.cuda.synchronize()

    # the largest width passes and traces what a context traces
    cfg = vpt.default_config(width=Wmax, height=Hs, primary_max_steps=64)
    # a 0.05 degree vertical field of view keeps the 16384 x 4 strip's
    # horizontal one near 120 degrees, so most rays reach the terrain
    cam = vpt.camera_from_pose((32.0, 60.0, 32.0), 30.0, -50.0, 0.05, Wmax / Hs)
    assert call(bufs, cfg) == vpt.OK
    torch.cuda.synchronize()
    with vpt.Context(cfg) as ctx:
        ctx.upload_world(vox)
        ctx.set_block_table(blocks)
        ctx.build_df()
        ctx.trace_frame(cam, frame)
        want = ctx.read_plane("T").reshape(-1)
        want_steps = ctx.read_plane("STEPS").reshape(-1)
    got = out["T"].cpu().numpy()
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    assert np.array_equal(out["STEPS"].cpu().numpy().view(np.uint16), want_steps)
    assert (got > 0).mean() > 0.5
    del keep
