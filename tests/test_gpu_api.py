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
