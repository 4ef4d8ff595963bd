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


def _euler_float32(euler_xyz, order):
    """Rz(phi) Ry(theta) Rx(rho) with float32 sines, cosines and products (each product and sum
    rounded to float32), multiplied in the given order: a stand-in for composing the rotation in
    float, as the reference does through Eigen (collision/factory.hh:26-61)."""
    f = np.float32
    rho, theta, phi = (f(v) for v in euler_xyz)
    cx, sx, cy, sy, cz, sz = (f(np.cos(rho)), f(np.sin(rho)), f(np.cos(theta)), f(np.sin(theta)), f(np.cos(phi)),
                              f(np.sin(phi)))
    rx = np.array([[1, 0, 0], [0, cx, -sx], [0, sx, cx]], np.float32)
    ry = np.array([[cy, 0, sy], [0, 1, 0], [-sy, 0, cy]], np.float32)
    rz = np.array([[cz, -sz, 0], [sz, cz, 0], [0, 0, 1]], np.float32)

    def mul(a, b):
        out = np.zeros((3, 3), np.float32)
        for i in range(3):
            for j in range(3):
                acc = f(a[i, 0] * b[0, j])
                acc = f(acc + f(a[i, 1] * b[1, j]))
                out[i, j] = f(acc + f(a[i, 2] * b[2, j]))
        return out

    return mul(mul(rz, ry), rx) if order == 0 else mul(rz, mul(ry, rx))


def test_euler_rotation_rounding_is_bounded():
    """The Euler constructors round Rz Ry Rx from float64, where the reference composes it in
    float through Eigen (its order of operations is not reproduced: Eigen is not available).  Over
    random angles the two differ by a few float32 ulps per axis component at most; an axis off by
    that much moves a cuboid test's distance by under 1e-6 m for half extents up to 1 m, inside the
    1e-5 m band where a verdict may differ from the reference's and is counted as explained."""
    from vamp_gb300.factory import euler_xyz_matrix

    rng = np.random.default_rng(4)
    worst, differ, n = 0.0, 0, 4000
    for _ in range(n):
        e = rng.uniform(-np.pi, np.pi, 3)
        r64 = euler_xyz_matrix(e).astype(np.float32).astype(np.float64)
        for order in (0, 1):
            d = float(np.abs(r64 - _euler_float32(e, order).astype(np.float64)).max())
            worst = max(worst, d)
            differ += d > 0.0
    assert worst <= 4e-7, worst  # 2.7e-7 on these angles
    assert differ > 0  # the two roundings do differ: the bound, not equality, is what holds
