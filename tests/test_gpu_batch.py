"""Mixed-robot batches replayed as one CUDA graph, and the edge-schedule autotuner, through the
C ABI: verdicts must equal the single-check entry point's (and the CPU oracle's) bit for bit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROBOTS = ("ur5", "fetch", "baxter", "panda")


def _scene_with_cloud(robot, seed=1, n_points=4000):
    """The 60-primitive scene plus a surface pointcloud whose CAPT uses the robot's radii."""
    import vamp_gb300 as vg
    from vamp_gb300 import scenes

    rb = getattr(vg, robot)
    r_min, r_max = rb.min_max_radii()
    scene = dict(scenes.scene_config1(seed))
    scene["pointclouds"] = [{"points": scenes.surface_pointcloud(seed + 50, n_points=n_points), "r_min": r_min,
                             "r_max": r_max, "r_point": scenes.POINT_RADIUS}]
    return scene


def _single(torch, robot, env, da, db, res):
    from vamp_gb300._lib import lib

    n = len(da)
    out = torch.empty(n, dtype=torch.uint8, device="cuda")
    blocks = torch.empty(n, dtype=torch.int32, device="cuda")
    rc = lib.vg_validate_motions_device(robot.encode(), env.handle, da.data_ptr(), db.data_ptr(), n, res, out.data_ptr(),
                                        blocks.data_ptr(), torch.cuda.current_stream().cuda_stream)
    assert rc == 0, lib.vg_last_error()
    torch.cuda.synchronize()
    return out.cpu().numpy(), blocks.cpu().numpy()


def test_mixed_batch_graph_matches_single_checks_and_the_oracle():
    import torch

    import vamp_gb300 as vg
    from oracle.vgo import Port
    from vamp_gb300 import scenes
    from vamp_gb300._lib import lib

    port = Port()
    parts = []
    for i, r in enumerate(ROBOTS):
        rb = getattr(vg, r)
        scene = _scene_with_cloud(r)
        env = vg.Environment.from_scene(scene)
        a, b = scenes.edges(rb.s_m, rb.s_a, 1024 + 257 * i, 900 + i)  # uneven sizes
        parts.append((r, rb, scene, env, a, b, torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()))
    batch = lib.vg_batch_create()
    try:
        outs = []
        for r, rb, scene, env, a, b, da, db in parts:
            out = torch.full((len(a),), 7, dtype=torch.uint8, device="cuda")
            blocks = torch.full((len(a),), -1, dtype=torch.int32, device="cuda")
            rc = lib.vg_batch_add_motions(batch, r.encode(), env.handle, da.data_ptr(), db.data_ptr(), len(a), rb.resolution(),
                                          None, 0, out.data_ptr(), blocks.data_ptr())
            assert rc == 0, lib.vg_last_error()
            outs.append((out, blocks))
        s = torch.cuda.current_stream().cuda_stream
        for launch in range(2):  # capture, then replay
            for out, blocks in outs:
                out.fill_(7)
                blocks.fill_(-1)
            assert lib.vg_batch_launch(batch, s) == 0, lib.vg_last_error()
            torch.cuda.synchronize()
            for (r, rb, scene, env, a, b, da, db), (out, blocks) in zip(parts, outs):
                ref, ref_blocks = _single(torch, r, env, da, db, rb.resolution())
                assert np.array_equal(out.cpu().numpy(), ref), (r, launch)
                assert np.array_equal(blocks.cpu().numpy(), ref_blocks), (r, launch)
        # and the CPU oracle on a slice of every robot's edges
        for (r, rb, scene, env, a, b, da, db), (out, _) in zip(parts, outs):
            prb = port.robot(r)
            penv = port.env(scene)
            k = 192
            want = penv.validate_motions(prb, a[:k], b[:k], rb.resolution())[0]
            assert np.array_equal(out.cpu().numpy()[:k], want), r
            assert 0 < int(out.sum()) < len(a), r
    finally:
        lib.vg_batch_destroy(batch)


def test_batch_follows_an_environment_change():
    import torch

    import vamp_gb300 as vg
    from vamp_gb300 import scenes
    from vamp_gb300._lib import lib

    rb = vg.panda
    env = vg.Environment.from_scene(scenes.scene_config1(3))
    a, b = scenes.edges(rb.s_m, rb.s_a, 2048, 17)
    da, db = torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()
    out = torch.empty(len(a), dtype=torch.uint8, device="cuda")
    batch = lib.vg_batch_create()
    try:
        assert lib.vg_batch_add_motions(batch, b"panda", env.handle, da.data_ptr(), db.data_ptr(), len(a), 32, None, 0,
                                        out.data_ptr(), None) == 0
        s = torch.cuda.current_stream().cuda_stream
        assert lib.vg_batch_launch(batch, s) == 0, lib.vg_last_error()
        torch.cuda.synchronize()
        before = out.cpu().numpy().copy()
        env.add_sphere([0.45, 0.0, 0.45, 0.25])  # in front of the robot: more edges collide
        assert lib.vg_batch_launch(batch, s) == 0, lib.vg_last_error()
        torch.cuda.synchronize()
        after = out.cpu().numpy()
        ref, _ = _single(torch, "panda", env, da, db, 32)
        assert np.array_equal(after, ref)
        assert after.sum() < before.sum()
    finally:
        lib.vg_batch_destroy(batch)


def test_batch_with_a_learned_order_keeps_the_verdicts():
    import torch

    import vamp_gb300 as vg
    from vamp_gb300 import scenes
    from vamp_gb300._lib import lib

    rb = vg.fetch
    env = vg.Environment.from_scene(_scene_with_cloud("fetch"))
    a, b = scenes.edges(rb.s_m, rb.s_a, 3000, 23)
    da, db = torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()
    out = torch.empty(len(a), dtype=torch.uint8, device="cuda")
    blocks = torch.empty(len(a), dtype=torch.int32, device="cuda")
    m = lib.vg_mlp_create(rb.dimension(), 9)  # untrained: any order must keep the verdicts
    batch = lib.vg_batch_create()
    try:
        assert lib.vg_batch_add_motions(batch, b"fetch", env.handle, da.data_ptr(), db.data_ptr(), len(a), rb.resolution(),
                                        m, 8, out.data_ptr(), blocks.data_ptr()) == 0
        assert lib.vg_batch_launch(batch, torch.cuda.current_stream().cuda_stream) == 0, lib.vg_last_error()
        torch.cuda.synchronize()
        ref, ref_blocks = _single(torch, "fetch", env, da, db, rb.resolution())
        got = out.cpu().numpy()
        assert np.array_equal(got, ref)
        assert np.array_equal(blocks.cpu().numpy()[ref == 1], ref_blocks[ref == 1])
    finally:
        lib.vg_batch_destroy(batch)
        lib.vg_mlp_destroy(m)


@pytest.mark.parametrize("robot", ROBOTS)
def test_autotuner_picks_a_schedule_without_changing_verdicts(robot):
    import ctypes

    import torch

    import vamp_gb300 as vg
    from vamp_gb300 import scenes
    from vamp_gb300._lib import lib

    rb = getattr(vg, robot)
    env = vg.Environment.from_scene(scenes.scene_config1(4))
    a, b = scenes.edges(rb.s_m, rb.s_a, 4096, 71)
    da, db = torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()
    before, before_blocks = _single(torch, robot, env, da, db, rb.resolution())
    sched, bps, ms = ctypes.c_int(-1), ctypes.c_int(-1), ctypes.c_float(-1)
    rc = lib.vg_autotune_motions(robot.encode(), env.handle, da.data_ptr(), db.data_ptr(), len(a), rb.resolution(),
                                 ctypes.byref(sched), ctypes.byref(bps), ctypes.byref(ms),
                                 torch.cuda.current_stream().cuda_stream)
    assert rc == 0, lib.vg_last_error()
    assert sched.value in (0, 1, 2, 3) and bps.value >= 0 and ms.value > 0
    after, after_blocks = _single(torch, robot, env, da, db, rb.resolution())
    assert np.array_equal(after, before)
    assert np.array_equal(after_blocks, before_blocks)
