"""World files (the reference's raw .sav layout and the headed form), the
emissive light list, and block edits with the incremental distance-field
update, which must equal a full rebuild of the edited world bit for bit."""
import numpy as np
import pytest


# ------------------------------------------------------------ world files --
def test_world_file_round_trip_raw_and_headed(vpt, tmp_path):
    vox = vpt.generate_world(40, 64, 24, seed=3)
    raw = tmp_path / "w.sav"
    vpt.save_world(raw, vox, header=False)
    assert raw.stat().st_size == vox.size                       # exactly the reference's raw dump
    assert np.array_equal(np.fromfile(raw, np.uint8).reshape(vox.shape), vox)
    got, seed = vpt.load_world(raw, dims=(40, 64, 24))
    assert np.array_equal(got, vox) and seed == 0
    headed = tmp_path / "w.vptw"
    vpt.save_world(headed, vox, seed=0x1234_5678_9ABC, header=True)
    got, seed = vpt.load_world(headed)
    assert np.array_equal(got, vox) and seed == 0x1234_5678_9ABC


def test_world_file_rejects_truncated_and_oversized(vpt, tmp_path):
    vox = vpt.generate_world(16, 16, 16, seed=1)
    p = tmp_path / "t.sav"
    vpt.save_world(p, vox, header=False)
    data = p.read_bytes()
    p.write_bytes(data[:-1])
    with pytest.raises(vpt.VPTError):
        vpt.load_world(p, dims=(16, 16, 16))
    p.write_bytes(data + b"\0")
    with pytest.raises(vpt.VPTError):
        vpt.load_world(p, dims=(16, 16, 16))
    with pytest.raises(vpt.VPTError):              # raw file without dimensions
        vpt.load_world(p)
    h = tmp_path / "t.vptw"
    vpt.save_world(h, vox, header=True)
    hb = h.read_bytes()
    h.write_bytes(hb[:40])
    with pytest.raises(vpt.VPTError):
        vpt.load_world(h)
    with pytest.raises(vpt.VPTError):
        vpt.load_world(tmp_path / "missing.sav", dims=(16, 16, 16))


def test_emissive_voxels_match_numpy(vpt):
    vox = vpt.generate_world(48, 64, 40, seed=9)
    table = vpt.generate_block_table(100, seed=9)
    got = vpt.emissive_voxels(vox, table)
    em = table["emissive"][vox] > 0
    z, y, x = np.nonzero(em)
    ref = np.stack([x, y, z], axis=1).astype(np.int32)
    order = np.lexsort((ref[:, 0], ref[:, 1], ref[:, 2]))      # x fastest
    assert len(got) > 0 and np.array_equal(got, ref[order])


# ------------------------------------------------------------ block edits --
def edit_sequence(rng, shape, n):
    Z, Y, X = shape
    for _ in range(n):
        w, h, d = (int(rng.integers(1, 9)) for _ in range(3))
        x0, y0, z0 = int(rng.integers(0, X - w + 1)), int(rng.integers(0, Y - h + 1)), int(rng.integers(0, Z - d + 1))
        kind = rng.integers(0, 3)
        if kind == 0:
            blk = np.zeros((d, h, w), np.uint8)                           # dig
        elif kind == 1:
            blk = rng.integers(1, 100, (d, h, w)).astype(np.uint8)        # build
        else:
            blk = ((rng.random((d, h, w)) < 0.5) * rng.integers(1, 100, (d, h, w))).astype(np.uint8)
        yield (x0, y0, z0), blk


@pytest.mark.gpu
@pytest.mark.parametrize("dims", [(64, 48, 80), (600, 8, 12), (12, 300, 20)])
def test_incremental_df_equals_rebuild(vpt, oracle, gpu, dims):
    """Successive digs, builds and mixed edits; worlds longer than twice the
    254 cap along one axis exercise the partial update box and its ring."""
    X, Y, Z = dims
    rng = np.random.default_rng(X + Y + Z)
    vox = vpt.generate_world(X, Y, Z, seed=4) if Y >= 48 else \
        ((rng.random((Z, Y, X)) < 0.02) * rng.integers(1, 100, (Z, Y, X))).astype(np.uint8)
    with vpt.Context(width=8, height=8) as ctx:
        ctx.upload_world(vox)
        ctx.set_block_table(vpt.generate_block_table(100, seed=4))
        ctx.build_df()
        for origin, blk in edit_sequence(rng, vox.shape, 6):
            x0, y0, z0 = origin
            d, h, w = blk.shape
            vox[z0:z0 + d, y0:y0 + h, x0:x0 + w] = blk
            ctx.edit_world(origin, blk)
            assert np.array_equal(ctx.read_df(), oracle.build_df(vox)), f"after edit at {origin} of {blk.shape}"


@pytest.mark.gpu
def test_edit_then_trace_matches_oracle(vpt, oracle, gpu):
    """A traced frame after an edit sees the edited world and its updated field."""
    X, Y, Z = 64, 64, 64
    W, H = 64, 40
    vox = vpt.generate_world(X, Y, Z, seed=2)
    blocks = vpt.generate_block_table(100, seed=2)
    cam = vpt.camera_from_pose((32.0, 60.0, 32.0), 40.0, -35.0, 90.0, W / H)
    with vpt.Context(width=W, height=H, primary_max_steps=256) as ctx:
        ctx.upload_world(vox)
        ctx.set_block_table(blocks)
        ctx.build_df()
        tower = np.full((12, 20, 6), 7, np.uint8)                 # a pillar in the view
        ctx.edit_world((40, 40, 40), tower)
        vox[40:52, 40:60, 40:46] = tower
        ctx.trace_primary(cam)
        t = ctx.read_plane("T")[..., 0]
        ref = oracle.trace_primary(oracle.World(vox, oracle.build_df(vox), blocks), cam,
                                   vpt.default_config(width=W, height=H, primary_max_steps=256))
    assert np.array_equal(t.view(np.uint32), ref["t"].view(np.uint32))


def test_edit_rejects_out_of_range(vpt):
    import ctypes as C
    assert vpt.lib.vpt_edit_world(None, None, 0, 0, 0, 1, 1, 1) == vpt.ERR_INVALID_ARG
