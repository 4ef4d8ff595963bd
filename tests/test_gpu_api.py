"""The Python wrappers of the autotuner, batches and the collision predictor (vamp_gb300.api)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_predictor_batch_and_autotune_through_the_python_api():
    import torch

    import vamp_gb300 as vg
    from vamp_gb300 import scenes

    env = vg.Environment.from_scene(scenes.scene_config1(5))
    a, b = scenes.edges(vg.panda.s_m, vg.panda.s_a, 8192, 55)
    da, db = torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()
    plain = vg.panda.validate_motion_batch(da, db, env).cpu().numpy()

    pick = vg.autotune(vg.panda, env, da, db)
    assert pick["schedule"] in vg.SCHEDULES and pick["ms"] > 0
    assert np.array_equal(vg.panda.validate_motion_batch(da, db, env).cpu().numpy(), plain)

    pred = vg.CollisionPredictor(vg.panda, seed=2)
    losses = pred.train_on_environment(env, n=1 << 17, epochs=2)
    assert losses.shape == (2,) and np.all(np.isfinite(losses)) and losses[1] <= losses[0]
    p = pred.predict(torch.from_numpy(scenes.configurations(vg.panda.s_m, vg.panda.s_a, 1000, 3)).cuda())
    assert p.shape == (1000,) and float(p.min()) >= 0.0 and float(p.max()) <= 1.0
    params = pred.parameters()
    pred.load_parameters(params)
    assert np.array_equal(pred.parameters(), params)
    learned = pred.validate_motion_batch(da, db, env).cpu().numpy()
    assert np.array_equal(learned, plain)

    env2 = vg.Environment.from_scene(scenes.scene_config1(6))
    a2, b2 = scenes.edges(vg.ur5.s_m, vg.ur5.s_a, 3000, 56)
    da2, db2 = torch.from_numpy(a2).cuda(), torch.from_numpy(b2).cuda()
    out1 = torch.empty(len(a), dtype=torch.uint8, device="cuda")
    out2 = torch.empty(len(a2), dtype=torch.uint8, device="cuda")
    batch = vg.Batch()
    batch.add(vg.panda, env, da, db, out1, predictor=pred)
    batch.add(vg.ur5, env2, da2, db2, out2)
    for _ in range(2):
        batch.launch()
        torch.cuda.synchronize()
        assert np.array_equal(out1.cpu().numpy(), plain)
        assert np.array_equal(out2.cpu().numpy(), vg.ur5.validate_motion_batch(a2, b2, env2))


@pytest.mark.parametrize("lanes,sqrt_mode", [(8, 0), (4, 1)])
def test_fkcc_blocks_are_the_oracles(port, lanes, sqrt_mode):
    """vg_fkcc_blocks (Robot::fkcc on caller-given blocks, block semantics) against the oracle's
    fkcc on the same blocks, host and device forms, with a pointcloud in the scene."""
    import torch

    import vamp_gb300 as vg
    from vamp_gb300 import scenes

    scene = scenes.scene_config1(4)
    scene["pointclouds"] = [{"points": scenes.surface_pointcloud(8, 3000), "r_min": 0.012, "r_max": 0.08,
                             "r_point": scenes.POINT_RADIUS}]
    rb = port.robot("panda")
    blocks = scenes.configurations(rb.s_m, rb.s_a, 600 * lanes, 19).reshape(600, lanes, 7)
    env = vg.Environment.from_scene(scene, lanes, sqrt_mode)
    host = vg.panda.fkcc_blocks(blocks, env)
    dev = vg.panda.fkcc_blocks(torch.from_numpy(blocks).cuda(), env).cpu().numpy()
    penv = port.env(scene, sqrt_mode)
    want = np.array([penv.fkcc_block(rb, np.ascontiguousarray(q)) for q in blocks], np.uint8)
    assert np.array_equal(host, want)
    assert np.array_equal(dev, want)
    assert 0 < want.sum() < len(want)


def test_imported_tree_checks_as_the_built_one(port):
    """A tree imported in the reference layout (vg_env_add_pointcloud_layout) gives the verdicts
    of the same tree built by vg_env_add_pointcloud."""
    import vamp_gb300 as vg
    from vamp_gb300 import scenes

    pts = scenes.surface_pointcloud(10, 5000)
    built = vg.Environment()
    built.add_pointcloud(pts, 0.012, 0.08, scenes.POINT_RADIUS)
    imported = vg.Environment()
    imported.add_pointcloud_layout(port.capt(pts, 0.012, 0.08, scenes.POINT_RADIUS))
    rb = port.robot("panda")
    a, b = scenes.edges(rb.s_m, rb.s_a, 2048, 20)
    assert np.array_equal(vg.panda.validate_motion_batch(a, b, built, 32), vg.panda.validate_motion_batch(a, b, imported, 32))
