"""The batched roadmap on the GPU: its nodes are the samples the oracle finds valid and its edges
exactly the candidate neighbour edges whose motion the oracle validates."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
THREADS = max(1, min(16, os.cpu_count() or 1))


def test_roadmap_is_the_oracles(port):
    import torch

    import vamp_gb300 as vg
    from vamp_gb300 import scenes
    from vamp_gb300.roadmap import build_roadmap, neighbour_pairs

    rb, prb = vg.panda, port.robot("panda")
    scene = scenes.scene_config0(51)
    env, penv = vg.Environment.from_scene(scene), port.env(scene)
    samples = scenes.configurations(prb.s_m, prb.s_a, 3000, 52)
    rm = build_roadmap(rb, env, torch.from_numpy(samples).cuda())
    valid = penv.validate_states(prb, samples, threads=THREADS).astype(bool)
    nodes = samples[valid]
    assert np.array_equal(rm["nodes"].cpu().numpy(), nodes)
    pairs, _ = neighbour_pairs(rm["nodes"], float(np.prod(prb.s_m.astype(np.float64))))
    p = pairs.cpu().numpy()
    ok, _ = penv.validate_motions(prb, nodes[p[:, 0]], nodes[p[:, 1]], prb.resolution, threads=THREADS)
    assert np.array_equal(rm["edges"].cpu().numpy(), p[ok.astype(bool)])
    assert rm["candidates"] == len(p) and 0 < rm["valid_edges"] < len(p)
