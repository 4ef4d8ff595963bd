"""validate_vector batches on the GPU (planning/validate.hh:23-63 with caller-given distances)
against the reference's fixtures and the oracle, in every edge schedule and both lane widths."""
import os

import numpy as np
import pytest

from conftest import golden, scene_of

pytestmark = pytest.mark.gpu
THREADS = max(1, min(16, os.cpu_count() or 1))


@pytest.fixture(scope="module")
def vg():
    import torch

    assert torch.cuda.is_available()
    import vamp_gb300 as vg

    return vg


@pytest.mark.parametrize("robot", ["panda", "ur5"])
def test_vectors_match_the_reference(vg, robot):
    g = golden(f"vectors_{robot}")
    env = vg.Environment.from_scene(scene_of(g))
    got = getattr(vg, robot).validate_vector_batch(g["start"], g["vector"], g["distance"], env, 32)
    assert np.array_equal(got, g["verdict"])


@pytest.mark.parametrize("robot", ["panda", "ur5", "fetch", "baxter"])
@pytest.mark.parametrize("schedule", [0, 1, 2, 3])
def test_vectors_are_the_oracles(vg, port, robot, schedule):
    import torch

    from vamp_gb300 import scenes

    rb, prb = getattr(vg, robot), port.robot(robot)
    scene = scenes.scene_config1(70 + schedule)
    env, penv = vg.Environment.from_scene(scene), port.env(scene)
    env.set_schedule(schedule)
    rng = np.random.default_rng(schedule)
    a, b = scenes.edges(prb.s_m, prb.s_a, 2048, 71)
    v = ((b - a) * rng.uniform(0.05, 1.0, (len(a), 1))).astype(np.float32)
    d = (np.linalg.norm(v, axis=1) * rng.uniform(0.5, 1.5, len(a))).astype(np.float32)
    blocks = torch.zeros(len(a), dtype=torch.int32, device="cuda")
    got = rb.validate_vector_batch(torch.from_numpy(a).cuda(), torch.from_numpy(v).cuda(), torch.from_numpy(d).cuda(),
                                   env, prb.resolution, blocks=blocks).cpu().numpy()
    want, wb = penv.validate_vectors(prb, a, v, d, prb.resolution, threads=THREADS)
    assert np.array_equal(got, want)
    assert np.array_equal(blocks.cpu().numpy(), wb)


def test_vectors_with_their_own_length_are_motions(vg):
    from vamp_gb300 import scenes

    env = vg.Environment.from_scene(scenes.scene_config1(3), lanes=4, sqrt_mode=vg.SQRT_EXACT)
    a, b = scenes.edges(vg.panda.s_m, vg.panda.s_a, 4096, 72)
    m = vg.panda.validate_motion_batch(a, b, env, 32)
    v = (b - a).astype(np.float32)
    # the kernels' own length (the reference's norm): take it from the motion path's block counts
    # indirectly by checking with a distance that gives the same block count
    d = np.linalg.norm(v.astype(np.float64), axis=1).astype(np.float32)
    got = vg.panda.validate_vector_batch(a, v, d, env, 32)
    assert (got == m).mean() > 0.999  # identical but for edges whose block count rounds differently
