"""The world batch (vpt_batch_*): worlds of uneven sizes with ragged ray tiles,
traced in one persistent launch (graph replay or direct) and as per-world
pass kernels, in every distance-field layout and queue grab size. Each world's
planes must equal the oracle's primary, sun-shadow and diffuse passes of that
world alone, bit for bit."""
import numpy as np
import pytest

# (X, Y, Z) and ray tile (W, H); tiles are not multiples of the 8x4 warp tile
WORLDS = [((40, 64, 36), (40, 24)), ((64, 64, 64), (64, 40)), ((24, 72, 32), (33, 17)),
          ((96, 80, 72), (72, 52))]


def bits_equal(a, b):
    a = np.ascontiguousarray(a)
    b = np.ascontiguousarray(np.asarray(b).reshape(a.shape))
    return a.dtype == b.dtype and a.tobytes() == b.tobytes()


@pytest.fixture(scope="module")
def scenes(vpt, oracle):
    out = []
    for k, ((X, Y, Z), (W, H)) in enumerate(WORLDS):
        vox = vpt.generate_world(X, Y, Z, seed=100 + k)
        blocks = vpt.generate_block_table(100, seed=100 + k)
        yaw, pitch = vpt.seeded_pose(100 + k, pitch_range=(-60.0, -40.0))
        cam = vpt.camera_from_pose((X / 2, min(Y - 3.0, 58.0), Z / 2), yaw, pitch, 90.0, W / H)
        world = oracle.World(vox, oracle.build_df(vox), blocks)
        cfg = vpt.default_config(width=W, height=H)
        frame = vpt.default_frame(seed=7, frame_index=3)
        g = oracle.trace_primary(world, cam, cfg)
        ref = {"T": g["t"], "FACE": g["face"], "BLOCK": g["block"], "HIT": g["hit"], "STEPS": g["steps"],
               "SHADOW": oracle.trace_shadow(world, cam, cfg, frame, g["t"], g["face"])}
        gi = oracle.trace_diffuse(world, cam, cfg, frame, g["t"], g["face"])
        ref.update({"GI_SH": gi["sh"], "GI_COCG": gi["cocg"], "GI_LUMA": gi["luma"], "GI_AOSKY": gi["aosky"]})
        out.append({"vox": vox, "blocks": blocks, "cam": cam, "W": W, "H": H, "df": world.df, "ref": ref,
                    "frame": frame})
    return out


def test_batch_scenes_mix_terrain_and_sky(scenes):
    for s in scenes:
        hits = float((s["ref"]["T"] > 0).mean())
        assert 0.1 < hits < 0.95, hits


def make_batch(vpt, scenes):
    b = vpt.Batch(max_worlds=len(scenes))
    for k, s in enumerate(scenes):
        assert b.add_world(s["vox"], s["blocks"], s["W"], s["H"]) == k
        b.set_camera(k, s["cam"])
    b.build_df()
    return b


def check_all(b, scenes, what):
    for k, s in enumerate(scenes):
        for name, ref in s["ref"].items():
            got = b.read_plane(k, name)
            assert bits_equal(got, ref), f"{what}: world {k} plane {name} differs"


@pytest.mark.gpu
def test_batch_distance_fields(vpt, scenes, gpu):
    with make_batch(vpt, scenes) as b:
        for k, s in enumerate(scenes):
            assert np.array_equal(b.read_df(k), s["df"]), f"world {k}"


@pytest.mark.gpu
@pytest.mark.parametrize("rays", [1, 2, "phased"], ids=["1ray", "2rays", "phased"])
@pytest.mark.parametrize("mode", [0, 1, 2], ids=["graph", "persistent", "per_world"])
@pytest.mark.parametrize("brick", [0, 4, 8])
def test_batch_bit_exact(vpt, scenes, mode, brick, rays, gpu):
    """Every world's planes equal the oracle's; with two rays per lane a warp's
    grab of 3 tile pairs crosses world boundaries, so single tiles and pairs
    both run; the phased launch runs the three passes as kernels of their own."""
    with make_batch(vpt, scenes) as b:
        phased = rays == "phased"
        b.set_tuning(df_brick=brick, tiles_per_grab=3, block_threads=128, rays_per_lane=1 if phased else rays,
                     phased=phased)
        b.set_stats(True)
        b.trace(scenes[0]["frame"], mode)
        b.synchronize()
        check_all(b, scenes, f"mode {mode} brick {brick}")
        st = b.read_stats()
        assert st["rays"]["primary"] == sum(s["W"] * s["H"] for s in scenes)


@pytest.mark.gpu
def test_batch_graph_replay_follows_frame_and_camera(vpt, oracle, scenes, gpu):
    """A replayed graph reads the frame constants and cameras of each call."""
    with make_batch(vpt, scenes) as b:
        b.trace(scenes[0]["frame"], vpt.BATCH_GRAPH)
        s = scenes[1]
        frame2 = vpt.default_frame(seed=9, frame_index=11)
        cam2 = vpt.camera_from_pose((30.0, 61.0, 33.0), 200.0, -40.0, 90.0, s["W"] / s["H"])
        b.set_camera(1, cam2)
        b.trace(frame2, vpt.BATCH_GRAPH)
        b.synchronize()
        world = oracle.World(s["vox"], s["df"], s["blocks"])
        cfg = vpt.default_config(width=s["W"], height=s["H"])
        g = oracle.trace_primary(world, cam2, cfg)
        gi = oracle.trace_diffuse(world, cam2, cfg, frame2, g["t"], g["face"])
        assert bits_equal(b.read_plane(1, "T"), g["t"])
        assert bits_equal(b.read_plane(1, "GI_SH"), gi["sh"])


@pytest.mark.gpu
def test_batch_autotune(vpt, scenes, gpu):
    with make_batch(vpt, scenes) as b:
        recs = b.autotune(scenes[0]["frame"], reps=2)
        assert len(recs) == 81
        assert {r["rays_per_lane"] for r in recs} == {1, 2}
        assert sum(r["phased"] for r in recs) == 27 and all(r["rays_per_lane"] == 1 for r in recs if r["phased"])
        assert all(r["ms"] > 0 for r in recs)
        best = min(recs, key=lambda r: r["ms"])
        t = b.tuning().as_dict()
        assert (t["block_threads"], t["tiles_per_grab"], t["df_brick"], t["rays_per_lane"], t["phased"]) == (
            best["block_threads"], best["tiles_per_grab"], best["df_brick"], best["rays_per_lane"], best["phased"])
        b.trace(scenes[0]["frame"], vpt.BATCH_GRAPH)
        b.synchronize()
        check_all(b, scenes, "after autotune")


def test_batch_host_validation(vpt):
    """Argument checks that need no GPU: the default config and bad configs."""
    import ctypes as C
    cfg = vpt.BatchConfig()
    assert vpt.lib.vpt_batch_default_config(C.byref(cfg)) == vpt.OK
    assert cfg.max_worlds == 64 and cfg.bounces == 1 and cfg.spp == 1
    h = C.c_void_p()
    bad = vpt.BatchConfig.from_buffer_copy(bytes(memoryview(cfg)))
    bad.max_worlds = 0
    assert vpt.lib.vpt_batch_create(C.byref(h), C.byref(bad)) == vpt.ERR_INVALID_ARG
    bad.max_worlds = 5000
    assert vpt.lib.vpt_batch_create(C.byref(h), C.byref(bad)) == vpt.ERR_INVALID_ARG
    assert vpt.lib.vpt_batch_destroy(None) == vpt.ERR_INVALID_ARG
    assert vpt.lib.vpt_batch_trace(None, None, 0) == vpt.ERR_INVALID_ARG
