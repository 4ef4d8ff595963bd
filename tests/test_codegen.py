"""Generated robot code is in sync with the robot models and the generator."""
import json

import pytest

from conftest import ROOT


@pytest.mark.parametrize("robot", ["panda", "ur5", "fetch", "baxter"])
def test_generated_code_is_current(robot):
    from vamp_gb300.robotgen import codegen

    model = json.loads((ROOT / "vamp_gb300" / "robots" / f"{robot}.json").read_text())
    assert (ROOT / "vamp_gb300" / "csrc" / "robots" / f"{robot}.cuh").read_text() == codegen.gen_cuda(model)
    assert (ROOT / "oracle" / "port" / "robots" / f"{robot}.h").read_text() == codegen.gen_c(model)


@pytest.mark.parametrize("robot", ["panda", "ur5", "fetch", "baxter"])
def test_model_spheres_follow_urdf_kinematics(port, robot):
    """FP64 FK of the generated oracle against the URDF kinematics evaluated in numpy."""
    import numpy as np

    from vamp_gb300 import scenes
    from vamp_gb300.robotgen import urdf as U

    model = json.loads((ROOT / "vamp_gb300" / "robots" / f"{robot}.json").read_text())
    rb = port.robot(robot)
    joints = [U.Joint(j["name"], j["type"], j["parent"], j["child"], tuple(j["xyz"]), tuple(j["rpy"]), tuple(j["axis"]))
              for j in model["joints"]]
    links = {n: U.Link(n) for j in joints for n in (j.parent, j.child)}
    urdf = U.Urdf(robot, links, joints, {j.child: j for j in joints})
    for q in scenes.configurations(rb.s_m, rb.s_a, 4, 3):
        tf = U.link_transforms(urdf, dict(zip(model["joint_names"], q.astype(np.float64))))
        s64 = rb.spheres_f64(q.astype(np.float64))
        for i, f in enumerate(model["fine_spheres"]):
            R, t = tf[f["link"]]
            assert np.abs(t + R @ np.array(f["p"]) - s64[i, :3]).max() < 1e-9
