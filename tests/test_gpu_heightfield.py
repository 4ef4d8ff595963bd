"""Heightfields on the GPU (collision/sphere_heightfield.hh:9-30 inside every environment query):
Panda states against the reference's fixture, every robot's states and edges against the oracle
bit for bit (alone, with primitives, with a pointcloud and an attachment), and debug reports."""
import os

import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu

ROBOTS = ["panda", "ur5", "fetch", "baxter"]
THREADS = max(1, min(16, os.cpu_count() or 1))


@pytest.fixture(scope="module")
def vg():
    import torch

    assert torch.cuda.is_available()
    import vamp_gb300 as vg

    return vg


def _scene(hf, base=None):
    base = base or {"spheres": np.zeros((0, 4), np.float32), "capsules": np.zeros((0, 8), np.float32),
                    "cuboids": np.zeros((0, 15), np.float32)}
    return {**base, "heightfields": [hf]}


def test_heightfield_states_match_the_reference(vg):
    g = golden("heightfield")
    hf = {"centre": g["centre"], "scale": g["scale"], "xd": int(g["xd"]), "yd": int(g["yd"]), "data": g["data"]}
    env = vg.Environment.from_scene(_scene(hf))
    assert np.array_equal(vg.panda.validate_batch(g["q"], env), g["state_verdict"])


@pytest.mark.parametrize("robot", ROBOTS)
def test_heightfield_checks_are_the_oracles(vg, port, robot):
    import torch

    from vamp_gb300 import scenes

    rb, prb = getattr(vg, robot), port.robot(robot)
    scene = _scene(scenes.heightfield(40 + len(robot)), scenes.scene_config0(41))
    env, penv = vg.Environment.from_scene(scene), port.env(scene)
    q = scenes.configurations(prb.s_m, prb.s_a, 4096, 42)
    got = rb.validate_batch(q, env)
    assert np.array_equal(got, penv.validate_states(prb, q, threads=THREADS))
    a, b = scenes.edges(prb.s_m, prb.s_a, 2048, 43)
    blocks = torch.zeros(len(a), dtype=torch.int32, device="cuda")
    ge = rb.validate_motion_batch(torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda(), env, prb.resolution,
                                  blocks=blocks).cpu().numpy()
    ce, cb = penv.validate_motions(prb, a, b, prb.resolution, threads=THREADS)
    assert np.array_equal(ge, ce) and np.array_equal(blocks.cpu().numpy(), cb)
    plain = rb.validate_batch(q, vg.Environment.from_scene(scenes.scene_config0(41)))
    assert not (got & ~plain).any()  # the terrain only removes configurations


def test_heightfield_pointcloud_and_attachment_together(vg, port):
    from vamp_gb300 import scenes

    prb = port.robot("panda")
    scene = _scene(scenes.heightfield(7), scenes.pointcloud_scene(8, 0.012, 0.08, n_points=20000))
    tf = np.eye(4, dtype=np.float32)
    tf[2, 3] = 0.12
    scene["attachment"] = {"tf": tf, "spheres": np.array([[0, 0, 0, 0.06]], np.float32)}
    env, penv = vg.Environment.from_scene(scene), port.env(scene)
    a, b = scenes.edges(prb.s_m, prb.s_a, 2048, 9)
    assert np.array_equal(vg.panda.validate_motion_batch(a, b, env, 32),
                          penv.validate_motions(prb, a, b, 32, threads=THREADS)[0])


def test_heightfield_debug_reports(vg, port):
    from vamp_gb300 import scenes

    prb = port.robot("panda")
    scene = _scene(scenes.heightfield(11), scenes.scene_config0(12))
    env, penv = vg.Environment.from_scene(scene), port.env(scene)
    q = scenes.configurations(prb.s_m, prb.s_a, 512, 13)
    bits, pairs = vg.panda.debug_batch(q, env)
    pbits, ppairs = penv.debug(prb, q)
    assert np.array_equal(bits, pbits) and np.array_equal(pairs, ppairs)
    hf_id = len(scene["spheres"]) + len(scene["capsules"]) + len(scene["cuboids"])
    assert ((pbits[:, :, hf_id >> 5] >> (hf_id & 31)) & 1).any()  # the terrain shows up in the reports


def test_heightfield_api(vg):
    a = np.zeros((4, 6), np.uint8)
    a[0, :] = 255
    hf = vg.array_to_heightfield(a, (0, 0, 0), (0.1, 0.1, 1.0))
    assert hf.dimensions == (4, 6) and hf.data.reshape(4, 6)[-1].max() == 1.0  # flipped, scaled
    env = vg.Environment()
    env.add_heightfield(hf)
    with pytest.raises(ValueError):
        env.add_heightfield(vg.make_heightfield((0, 0, 0), (1, 1, 1), (3, 3), np.zeros(8)))


def test_batch_graph_with_extended_environments(vg, port):
    """A CUDA-graph batch mixing an environment with a heightfield and an attachment and a plain
    one: replays give the single checks' (and the oracle's) verdicts."""
    import torch

    from vamp_gb300 import scenes

    tf = np.eye(4, dtype=np.float32)
    tf[2, 3] = 0.1
    ext = _scene(scenes.heightfield(21), scenes.scene_config1(22))
    ext["attachment"] = {"tf": tf, "spheres": np.array([[0, 0, 0, 0.05]], np.float32)}
    plain = scenes.scene_config1(23)
    parts = [("panda", ext), ("ur5", plain)]
    b = vg.Batch()
    keep = []
    for name, scene in parts:
        prb = port.robot(name)
        a, bb = scenes.edges(prb.s_m, prb.s_a, 1024, 24)
        da, db = torch.from_numpy(a).cuda(), torch.from_numpy(bb).cuda()
        out = torch.zeros(len(a), dtype=torch.uint8, device="cuda")
        env = vg.Environment.from_scene(scene)
        b.add(getattr(vg, name), env, da, db, out)
        keep.append((name, scene, a, bb, out, env))
    for _ in range(2):  # capture, then replay
        b.launch()
        torch.cuda.synchronize()
        for name, scene, a, bb, out, env in keep:
            prb = port.robot(name)
            want, _ = port.env(scene).validate_motions(prb, a, bb, prb.resolution, threads=THREADS)
            assert np.array_equal(out.cpu().numpy(), want), name
