"""CAPT queries (collision/capt.hh:425-506) through the GPU's query tables on trees of every
shape: from two leaves (two points) to tens of thousands, each depth modulo 3 (the split values travel three
levels per node, the remainder with the tree's view), and a tree built for radius 0 (one ring
holds every point).  States and edges against the oracle bit for bit."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

THREADS = max(1, min(16, os.cpu_count() or 1))


@pytest.fixture(scope="module")
def vg():
    import torch

    assert torch.cuda.is_available()
    import vamp_gb300 as vg

    return vg


def _scene(points, r_min, r_max, r_point):
    return {"spheres": np.zeros((0, 4), np.float32), "capsules": np.zeros((0, 8), np.float32),
            "cuboids": np.zeros((0, 15), np.float32),
            "pointclouds": [{"points": points, "r_min": r_min, "r_max": r_max, "r_point": r_point}]}


def _points(n, seed):
    """n points in the Panda's reach (a box around the arm), so that queries descend everywhere."""
    rng = np.random.default_rng(seed)
    return (rng.uniform(0, 1, size=(n, 3)) * [1.2, 1.2, 1.1] + [-0.6, -0.6, -0.05]).astype(np.float32)


@pytest.mark.parametrize("n", [2, 3, 5, 9, 17, 33, 70, 300, 2500, 9000])
@pytest.mark.parametrize("radii", [(0.012, 0.08, 0.0025), (0.0, 0.0, 0.0), (0.05, 0.3, 0.01)])
def test_query_tables_answer_as_the_oracle(vg, port, n, radii):
    from vamp_gb300 import scenes

    scene = _scene(_points(n, 1000 + n), *radii)
    env, penv = vg.Environment.from_scene(scene), port.env(scene)
    prb = port.robot("panda")
    q = scenes.configurations(prb.s_m, prb.s_a, 4096, n)
    got = vg.panda.validate_batch(q, env)
    assert np.array_equal(got, penv.validate_states(prb, q, threads=THREADS))
    a, b = scenes.edges(prb.s_m, prb.s_a, 512, n + 1)
    ge = vg.panda.validate_motion_batch(a, b, env, 32)
    assert np.array_equal(ge, penv.validate_motions(prb, a, b, 32, threads=THREADS)[0])
    if n >= 300 and radii[1] > 0:
        assert not got.all()  # the cloud is in the arm's way


def test_nlog2_covers_each_remainder(vg):
    """The sizes above give trees of depth 1 to 14: every value modulo 3."""
    depths = set()
    for n in [2, 3, 5, 9, 17, 33, 70, 300, 2500, 9000]:
        env = vg.Environment()
        env.add_pointcloud(_points(n, 1000 + n), 0.012, 0.08, 0.0025)
        depths.add(int(env.pointcloud_layout(0)["nlog2"]))
    assert {d % 3 for d in depths} == {0, 1, 2} and min(depths) <= 1, depths
