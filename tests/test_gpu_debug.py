"""Debug reports (Robot::fkcc_debug) on the GPU against the reference's fixtures and the CPU
oracle: per fine sphere the objects it collides with, per fine self pair whether it collides."""
import numpy as np
import pytest

from conftest import golden, scene_of

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("robot", ["panda", "baxter"])
def test_debug_reports_match_the_reference_fixture(robot):
    import vamp_gb300 as vg

    g = golden(f"debug_{robot}")
    env = vg.Environment.from_scene(scene_of(g))
    bits, pairs = getattr(vg, robot).debug_batch(g["q"], env)
    assert np.array_equal(bits, g["env_bits"])
    assert np.array_equal(pairs, g["pairs"])


@pytest.mark.parametrize("robot", ["panda", "ur5", "fetch", "baxter"])
@pytest.mark.parametrize("sqrt_mode", [0, 1])
def test_debug_reports_match_the_oracle(port, robot, sqrt_mode):
    import torch

    import vamp_gb300 as vg
    from oracle.vgo import SQRT_EXACT, SQRT_X86
    from vamp_gb300 import scenes

    scene = scenes.scene_config0(5) if robot == "panda" else scenes.scene_config1(5)
    rb = port.robot(robot)
    q = scenes.configurations(rb.s_m, rb.s_a, 700, 31)
    want_bits, want_pairs = port.env(scene, sqrt_mode=SQRT_X86 if sqrt_mode == 0 else SQRT_EXACT).debug(rb, q)
    env = vg.Environment.from_scene(scene, lanes=8 if sqrt_mode == 0 else 4, sqrt_mode=sqrt_mode)
    bits, pairs = getattr(vg, robot).debug_batch(torch.from_numpy(q).cuda(), env)
    assert np.array_equal(bits.cpu().numpy().view(np.uint32), want_bits)
    assert np.array_equal(pairs.cpu().numpy(), want_pairs)
    assert want_bits.any() and want_pairs.any()
    # the single-configuration form
    objs, prs = getattr(vg, robot).debug(q[3], env)
    assert len(objs) == rb.fine
    for i, lst in enumerate(objs):
        assert all((want_bits[3, i, o // 32] >> (o % 32)) & 1 for o in lst)
