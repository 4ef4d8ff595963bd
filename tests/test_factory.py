"""Primitive constructors with the reference's parameterisation (collision/factory.hh)."""
import numpy as np
import pytest


def test_capsule_endpoints_follow_the_reference_arithmetic():
    from vamp_gb300 import scenes
    from vamp_gb300.factory import Capsule

    rng = np.random.default_rng(1)
    for _ in range(200):
        p1, p2 = rng.uniform(-1, 1, (2, 3)).astype(np.float32)
        c = Capsule.from_endpoints(p1, p2, 0.05)
        f = scenes.capsule_fields(p1, p2, 0.05)  # the same capsule with v . v summed in float64
        got = np.array([c.x1, c.y1, c.z1, c.xv, c.yv, c.zv, c.r, c.rdv], np.float32)
        assert np.array_equal(got[:7], f[:7])
        assert abs(int(got[7].view(np.int32)) - int(f[7].view(np.int32))) <= 2  # rdv within 2 ulp


def test_cuboid_and_centred_capsule_geometry():
    from vamp_gb300.factory import Capsule, Cuboid, euler_xyz_matrix

    R = euler_xyz_matrix((0.3, -0.2, 1.1))
    assert np.allclose(R @ R.T, np.eye(3))
    c = Cuboid((0.1, 0.2, 0.3), (0.3, -0.2, 1.1), (0.05, 0.1, 0.2))
    a1 = np.array([c.axis_1_x, c.axis_1_y, c.axis_1_z], np.float64)
    assert np.allclose(a1, R[:, 0], atol=1e-7) and c.axis_3_r == np.float32(0.2)
    k = Capsule((0, 0, 1), (0, 0, 0), 0.1, 0.4)  # upright: end points 0.2 above and below
    assert abs(k.x1) < 1e-7 and abs(k.y1) < 1e-7 and k.z1 == np.float32(1.2) and abs(k.zv + 0.4) < 1e-7


def test_environment_takes_factory_objects():
    vg = pytest.importorskip("vamp_gb300")
    from vamp_gb300.factory import Capsule, Cuboid, Sphere

    try:
        env = vg.Environment()
    except ImportError:
        pytest.skip("library not built")
    env.add_sphere(Sphere((0.5, 0, 0.4), 0.1))
    env.add_cuboid(Cuboid((0, 0.5, 0.2), (0, 0, 0.3), (0.1, 0.1, 0.1)))
    env.add_capsule(Capsule((0.3, 0.3, 0.3), (0.2, 0, 0), 0.05, 0.3))
    assert len(env.objects(0)) == 1 and len(env.objects(1)) == 1
    assert len(env.objects(3)) + len(env.objects(4)) == 1
