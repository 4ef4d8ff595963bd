"""The GPU CAPT build (vg_env_add_pointcloud_device) against the host build, which follows the
reference's collision/capt.hh:294-365 bit for bit (pinned by the cloud fixtures in test_oracle.py).

The two builds must give the same tree: every split value, leaf box, block range and afforded
point, in the same order; and hence the same verdicts."""
import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def vg():
    import torch

    assert torch.cuda.is_available()
    import vamp_gb300 as vg

    return vg


def _layouts_equal(a: dict, b: dict):
    assert a["nlog2"] == b["nlog2"]
    for k in ("tests", "aabbs", "aff_starts", "aff", "top"):
        assert a[k].shape == b[k].shape, k
        # bitwise, so that NaN and -0.0 count too
        assert np.array_equal(a[k].view(np.uint32), b[k].view(np.uint32)), k


def _both(vg, points, r_min, r_max, r_point):
    import torch

    host = vg.Environment()
    host.add_pointcloud(points, r_min, r_max, r_point)
    dev = vg.Environment()
    dev.add_pointcloud_device(torch.from_numpy(np.ascontiguousarray(points, np.float32)).cuda(), r_min, r_max, r_point)
    return host, dev


def _clouds():
    from vamp_gb300 import scenes

    rng = np.random.default_rng(5)
    g = golden("cloud_panda")
    grid = (rng.integers(0, 6, size=(3000, 3)) * 0.05).astype(np.float32)  # many equal coordinates
    yield "golden", g["points"], float(g["r"][0]), float(g["r"][1])
    yield "surface-panda", scenes.surface_pointcloud(9, 50000), 0.012, 0.08
    yield "surface-fetch", scenes.surface_pointcloud(4, 30000), 0.01, 0.15
    yield "surface-baxter", scenes.surface_pointcloud(6, 12000), 0.02, 0.5
    yield "uniform-4097", rng.uniform(-1, 1, size=(4097, 3)).astype(np.float32), 0.01, 0.1
    yield "grid-ties", grid, 0.012, 0.08
    yield "two", np.array([[0, 0, 0], [0.1, 0.2, 0.3]], np.float32), 0.0, 0.05
    yield "three", rng.uniform(0, 0.1, size=(3, 3)).astype(np.float32), 0.01, 0.2


@pytest.mark.parametrize("case", list(range(8)))
def test_device_build_is_the_host_build(vg, case):
    from vamp_gb300 import scenes

    name, pts, r_min, r_max = list(_clouds())[case]
    host, dev = _both(vg, pts, r_min, r_max, scenes.POINT_RADIUS)
    _layouts_equal(host.pointcloud_layout(0), dev.pointcloud_layout(0))


def test_device_and_host_clouds_mix_in_order(vg):
    """Host, device, host: each tree stays at its index and the verdicts are the all-host ones."""
    import torch

    from vamp_gb300 import scenes

    clouds = [scenes.surface_pointcloud(s, 8000) for s in (11, 12, 13)]
    radii = (0.012, 0.08, scenes.POINT_RADIUS)
    ref = vg.Environment()
    for c in clouds:
        ref.add_pointcloud(c, *radii)
    mix = vg.Environment()
    mix.add_pointcloud(clouds[0], *radii)
    mix.add_pointcloud_device(torch.from_numpy(clouds[1]).cuda(), *radii)
    mix.add_pointcloud(clouds[2], *radii)
    for i in range(3):
        _layouts_equal(ref.pointcloud_layout(i), mix.pointcloud_layout(i))
    rb = vg.panda
    a, b = scenes.edges(rb.s_m, rb.s_a, 4096, 3)
    ga = rb.validate_motion_batch(torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda(), ref, 32).cpu().numpy()
    gb = rb.validate_motion_batch(torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda(), mix, 32).cpu().numpy()
    assert np.array_equal(ga, gb)
    q = scenes.configurations(rb.s_m, rb.s_a, 8192, 4)
    assert np.array_equal(rb.validate_batch(q, ref), rb.validate_batch(q, mix))


def test_device_build_rejects_bad_arguments(vg):
    import torch

    env = vg.Environment()
    one = torch.zeros((1, 3), device="cuda")
    with pytest.raises(vg.VampError):
        env.add_pointcloud_device(one, 0.01, 0.1, 0.0025)
    two = torch.zeros((2, 3), device="cuda")
    with pytest.raises(vg.VampError):
        env.add_pointcloud_device(two, 0.2, 0.1, 0.0025)
    with pytest.raises(ValueError):
        env.add_pointcloud_device(torch.zeros((4, 3)), 0.01, 0.1, 0.0025)
