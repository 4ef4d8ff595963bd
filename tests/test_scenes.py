"""The synthetic workloads have the shapes and collision rates they claim."""
import numpy as np

from vamp_gb300 import scenes


def test_scenes_are_seeded():
    a, b = scenes.scene_config1(3), scenes.scene_config1(3)
    for k in ("spheres", "capsules", "cuboids"):
        assert np.array_equal(a[k], b[k])
    assert a["spheres"].shape == (24, 4) and a["cuboids"].shape == (24, 15) and a["capsules"].shape == (12, 8)


def test_cuboid_axes_are_orthonormal():
    c = scenes.scene_config1(1)["cuboids"]
    for row in c:
        R = np.stack([row[3:6], row[6:9], row[9:12]], axis=1).astype(np.float64)
        assert np.abs(R.T @ R - np.eye(3)).max() < 1e-6


def test_workspace_scene_collides_30_to_50_percent_of_edges(port):
    rb = port.robot("panda")
    env = port.env(scenes.scene_config1(1))
    a, b = scenes.edges(rb.s_m, rb.s_a, 2048, 5)
    ok, _ = env.validate_motions(rb, a, b, 32, threads=4)
    assert 0.3 <= 1.0 - ok.mean() <= 0.5


def test_pointcloud_shape():
    p = scenes.surface_pointcloud(1, n_points=5000)
    assert p.shape == (5000, 3) and p.dtype == np.float32 and np.isfinite(p).all()
