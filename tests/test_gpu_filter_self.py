"""filter_self_from_pointcloud on the GPU against the reference's fixture and the oracle."""
import numpy as np
import pytest

from conftest import golden, scene_of

pytestmark = pytest.mark.gpu


def test_filter_self_matches_reference_and_oracle(port):
    import torch

    import vamp_gb300 as vg
    from vamp_gb300 import scenes

    g = golden("filter_self_panda")
    env = vg.Environment.from_scene(scene_of(g))
    for i in range(len(g["q"])):
        kept = vg.panda.filter_self_from_pointcloud(g["points"], float(g["radius"]), g["q"][i], env)
        assert np.array_equal(kept, g[f"kept{i}"]), i
        dev = vg.panda.filter_self_from_pointcloud(torch.from_numpy(g["points"]).cuda(), float(g["radius"]), g["q"][i], env)
        assert np.array_equal(dev.cpu().numpy(), g[f"kept{i}"]), i
    # other robots and a pointcloud scene, against the oracle
    for name, seed in (("fetch", 3), ("baxter", 4)):
        prb = port.robot(name)
        scene = scenes.scene_config1(seed)
        q = scenes.configurations(prb.s_m, prb.s_a, 1, seed)[0]
        pts = np.random.default_rng(seed).uniform(-1.2, 1.2, (20000, 3)).astype(np.float32)
        want = port.env(scene).filter_self(prb, pts, 0.02, q)
        got = getattr(vg, name).filter_self_from_pointcloud(pts, 0.02, q, vg.Environment.from_scene(scene))
        assert np.array_equal(got, want), name
    assert vg.panda.filter_self_from_pointcloud(np.zeros((0, 3), np.float32), 0.01, g["q"][0]).shape == (0, 3)
