"""Small host batches of edges (vg_validate_motions / vg_validate_vectors with at most 4,096
blocks in all, a planner's single extension among them) are checked block by block: every block
is built on the host with the edge kernels' arithmetic (planning/validate.hh:24-56) and all of
them go to the caller-given-blocks kernel at once.  Their verdicts equal the edge kernels' (which
CUDA tensors take) and the oracle's, in both lane widths and with an extended environment."""
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


def _device(rb, a, b, env, res):
    import torch

    return rb.validate_motion_batch(torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda(), env, res).cpu().numpy()


@pytest.mark.parametrize("robot", ["panda", "ur5", "fetch", "baxter"])
@pytest.mark.parametrize("lanes", [8, 4])
def test_small_batches_equal_the_edge_kernels_and_the_oracle(vg, port, robot, lanes):
    from vamp_gb300 import scenes

    rb, prb = getattr(vg, robot), port.robot(robot)
    scene = scenes.scene_config1(90 + lanes)
    sqrt_mode = vg.SQRT_X86 if lanes == 8 else vg.SQRT_EXACT
    env = vg.Environment.from_scene(scene, lanes=lanes, sqrt_mode=sqrt_mode)
    penv = port.env(scene, sqrt_mode)
    a, b = scenes.edges(prb.s_m, prb.s_a, 400, 91)
    want = penv.validate_motions(prb, a, b, prb.resolution, lanes=lanes, threads=THREADS)[0]
    for lo, hi in ((0, 1), (1, 3), (3, 10), (10, 74), (74, 400)):
        host = rb.validate_motion_batch(a[lo:hi], b[lo:hi], env, prb.resolution)
        assert np.array_equal(host, _device(rb, a[lo:hi], b[lo:hi], env, prb.resolution)), (lo, hi)
        assert np.array_equal(host, want[lo:hi]), (lo, hi)
    # one edge at a time, as the drop-in's validate_motion sends them
    for i in range(0, 400, 37):
        assert rb.validate_motion_batch(a[i:i + 1], b[i:i + 1], env, prb.resolution)[0] == want[i], i


def test_small_vector_batches_equal_the_edge_kernels_and_the_oracle(vg, port):
    import torch

    from vamp_gb300 import scenes

    rb, prb = vg.panda, port.robot("panda")
    scene = scenes.scene_config1(95)
    env, penv = vg.Environment.from_scene(scene), port.env(scene)
    rng = np.random.default_rng(96)
    a, b = scenes.edges(prb.s_m, prb.s_a, 200, 97)
    v = ((b - a) * rng.uniform(0.05, 1.0, (len(a), 1))).astype(np.float32)
    d = (np.linalg.norm(v, axis=1) * rng.uniform(0.5, 1.5, len(a))).astype(np.float32)
    want = penv.validate_vectors(prb, a, v, d, 32, threads=THREADS)[0]
    for lo, hi in ((0, 1), (1, 9), (9, 200)):
        host = rb.validate_vector_batch(a[lo:hi], v[lo:hi], d[lo:hi], env, 32)
        dev = rb.validate_vector_batch(torch.from_numpy(a[lo:hi]).cuda(), torch.from_numpy(v[lo:hi]).cuda(),
                                       torch.from_numpy(d[lo:hi]).cuda(), env, 32).cpu().numpy()
        assert np.array_equal(host, dev), (lo, hi)
        assert np.array_equal(host, want[lo:hi]), (lo, hi)


def test_edge_cases_of_the_block_path(vg, port):
    from vamp_gb300 import scenes

    rb, prb = vg.panda, port.robot("panda")
    scene = scenes.scene_config1(98)
    env, penv = vg.Environment.from_scene(scene), port.env(scene)
    a, b = scenes.edges(prb.s_m, prb.s_a, 64, 99)
    # zero-length edges: one block at the start configuration
    assert np.array_equal(rb.validate_motion_batch(a, a, env, 32), penv.validate_motions(prb, a, a.copy(), 32)[0])
    # an edge of more blocks than the block path takes goes to the edge kernels, alone or with others
    for n in (1, 5):
        big = rb.validate_motion_batch(a[:n], b[:n], env, 4096)
        assert np.array_equal(big, _device(rb, a[:n], b[:n], env, 4096))
        assert np.array_equal(big, penv.validate_motions(prb, a[:n], b[:n], 4096)[0])


def test_block_path_with_an_extended_environment(vg):
    from vamp_gb300 import scenes

    env = vg.Environment.from_scene(scenes.scene_config1(100))
    xs = np.linspace(-1.0, 1.0, 9, dtype=np.float32)
    h = (0.05 * np.sin(3.0 * xs)[:, None] * np.cos(2.0 * xs)[None, :]).astype(np.float32)
    env.add_heightfield(vg.make_heightfield((0.0, 0.0, 0.0), (0.25, 0.25, 1.0), (9, 9), h.reshape(-1)))
    a, b = scenes.edges(vg.panda.s_m, vg.panda.s_a, 50, 101)
    for lo, hi in ((0, 1), (1, 50)):
        host = vg.panda.validate_motion_batch(a[lo:hi], b[lo:hi], env, 32)
        assert np.array_equal(host, _device(vg.panda, a[lo:hi], b[lo:hi], env, 32))
