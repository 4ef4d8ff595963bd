"""Attachments on the GPU (Robot::fkcc_attach, robots/panda.hh:10265-15445; Environment.attach):
verdicts and per-edge block counts bit-identical to the oracle for every robot, with primitive
and pointcloud scenes; the end-effector transform against the oracle and the reference's eefk."""
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


def _attach(scene: dict, spheres, offset: float = 0.14) -> dict:
    tf = np.eye(4, dtype=np.float32)
    tf[2, 3] = offset
    return {**scene, "attachment": {"tf": tf, "spheres": np.asarray(spheres, np.float32).reshape(-1, 4)}}


@pytest.mark.parametrize("robot", ROBOTS)
def test_eefk_matches_oracle_and_reference(vg, port, robot):
    g = golden(f"eefk_{robot}")
    rb = getattr(vg, robot)
    T = rb.eefk(g["q"])
    prb = port.robot(robot)
    assert np.array_equal(T, np.stack([prb.ee_pose(q) for q in g["q"]]))
    assert np.abs(T - g["T"]).max() < 1e-5


@pytest.mark.parametrize("robot", ROBOTS)
def test_attachment_verdicts_are_the_oracles(vg, port, robot):
    import torch

    from vamp_gb300 import scenes

    rb, prb = getattr(vg, robot), port.robot(robot)
    scene = _attach(scenes.scene_config1(21), [[0, 0, 0, 0.07], [0.05, 0, 0.03, 0.03]])
    env, penv = vg.Environment.from_scene(scene), port.env(scene)
    q = scenes.configurations(prb.s_m, prb.s_a, 4096, 22)
    got = rb.validate_batch(q, env)
    assert np.array_equal(got, penv.validate_states(prb, q, threads=THREADS))
    plain = rb.validate_batch(q, vg.Environment.from_scene(scenes.scene_config1(21)))
    assert (plain & ~got).any() and not (got & ~plain).any()  # the attachment only adds failures
    a, b = scenes.edges(prb.s_m, prb.s_a, 2048, 23)
    blocks = torch.zeros(len(a), dtype=torch.int32, device="cuda")
    res = prb.resolution
    ge = rb.validate_motion_batch(torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda(), env, res,
                                  blocks=blocks).cpu().numpy()
    ce, cb = penv.validate_motions(prb, a, b, res, threads=THREADS)
    assert np.array_equal(ge, ce)
    assert np.array_equal(blocks.cpu().numpy(), cb)


def test_attachment_with_a_pointcloud_and_detach(vg, port):
    """Panda carrying a sphere through the 50,000-point surface cloud; detach restores the plain
    verdicts; a 4-lane environment (the reference's Arm build) gives the oracle's too."""
    import torch

    from vamp_gb300 import scenes

    rb, prb = vg.panda, port.robot("panda")
    scene = scenes.pointcloud_scene(4, 0.012, 0.08)
    att = _attach(scene, [[0, 0, 0, 0.05]], offset=0.1)
    env, penv = vg.Environment.from_scene(att), port.env(att)
    a, b = scenes.edges(prb.s_m, prb.s_a, 2048, 31)
    ge = rb.validate_motion_batch(torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda(), env, 32).cpu().numpy()
    ce, _ = penv.validate_motions(prb, a, b, 32, threads=THREADS)
    assert np.array_equal(ge, ce)
    env.detach()
    gd = rb.validate_motion_batch(torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda(), env, 32).cpu().numpy()
    cd, _ = port.env(scene).validate_motions(prb, a, b, 32, threads=THREADS)
    assert np.array_equal(gd, cd) and (gd & ~ge).any()
    env4 = vg.Environment.from_scene(att, lanes=4, sqrt_mode=vg.SQRT_EXACT)
    g4 = rb.validate_motion_batch(a, b, env4, 32)
    c4, _ = port.env(att, sqrt_mode=1).validate_motions(prb, a, b, 32, lanes=4, threads=THREADS)
    assert np.array_equal(g4, c4)


def test_attachment_object_mirrors_the_binding(vg):
    """vamp.Attachment: relative frame, spheres, set_ee_pose / posed_spheres."""
    from vamp_gb300 import scenes

    tf = np.eye(4, dtype=np.float32)
    tf[:3, 3] = [0.0, 0.0, 0.14]
    a = vg.Attachment(tf)
    a.add_sphere([0, 0, 0, 0.07])
    a.add_spheres([[0.1, 0, 0, 0.02]])
    q = scenes.configurations(vg.panda.s_m, vg.panda.s_a, 1, 3)[0]
    T = vg.panda.eefk(q)
    a.set_ee_pose(T)
    want = (T.astype(np.float64) @ tf.astype(np.float64) @ np.array([0.1, 0, 0, 1.0]))[:3]
    assert np.abs(a.posed_spheres[1, :3] - want).max() < 1e-6 and a.posed_spheres[0, 3] == np.float32(0.07)
    env = vg.Environment()
    env.attach(a)
    assert vg.panda.validate(q, env) in (True, False)
