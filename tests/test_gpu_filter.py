"""The GPU pointcloud filter (vg_filter_pointcloud[_device]) against the reference's fixtures and
the oracle (collision/filter.hh:176-320): the same kept points in the same order, bit for bit."""
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


def _case(g: dict, i: int):
    p = g[f"params{i}"]
    return g[f"points{i}"], float(p[0]), float(p[1]), p[2:5], p[5:8], p[8:11], bool(p[11])


def _same(a: np.ndarray, b: np.ndarray) -> bool:
    return a.shape == b.shape and np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_filter_matches_the_reference_fixtures(vg):
    import torch

    g = golden("filter")
    for i in range(6):
        pts, md, mr, o, lo, hi, cull = _case(g, i)
        kept, ns = vg.filter_pointcloud(pts, md, mr, o, lo, hi, cull)
        assert _same(kept, g[f"kept{i}"]), i
        assert ns > 0
        dev = vg.filter_pointcloud_device(torch.from_numpy(pts).cuda(), md, mr, o, lo, hi, cull).cpu().numpy()
        assert _same(dev, g[f"kept{i}"]), i


def _clouds():
    from vamp_gb300 import scenes

    rng = np.random.default_rng(17)
    org = np.array([0.0, 0.0, 0.333], np.float32)
    big = scenes.surface_pointcloud(5, 400_000)
    yield "surface 400k cull", big, 0.01, 1.19, org, org - 1.19, org + 1.19, True
    yield "surface 400k", big, 0.005, 1.19, org, org - 1.19, org + 1.19, False
    dense = np.concatenate([np.zeros((70_000, 3), np.float32),                       # a repeated point
                            rng.normal(0.3, 0.002, (50_000, 3)).astype(np.float32),  # a dense blob
                            scenes.surface_pointcloud(6, 30_000)])
    rng.shuffle(dense)
    yield "duplicates and a dense blob", dense, 0.01, 1.2, org, org - 1.2, org + 1.2, True
    yield "duplicates, no cull", dense, 0.02, 1.2, org, org - 1.2, org + 1.2, False
    yield "one point", np.array([[0.1, 0.2, 0.3]], np.float32), 0.01, 1.0, org, org - 1, org + 1, True
    yield "two close points", np.array([[0.1, 0.2, 0.3], [0.1, 0.2, 0.305]], np.float32), 0.01, 1.0, org, org - 1, \
        org + 1, False
    yield "zero min_dist", rng.uniform(-1, 1, (5000, 3)).astype(np.float32), 0.0, 1.0, org, org - 1, org + 1, True


@pytest.mark.parametrize("case", list(range(7)))
def test_filter_is_the_oracles(vg, port, case):
    import torch

    name, pts, md, mr, o, lo, hi, cull = list(_clouds())[case]
    want = port.filter_pointcloud(pts, md, mr, o, lo, hi, cull)
    kept, _ = vg.filter_pointcloud(pts, md, mr, o, lo, hi, cull)
    assert _same(kept, want), (name, kept.shape, want.shape)
    dev = vg.filter_pointcloud_device(torch.from_numpy(pts).cuda(), md, mr, o, lo, hi, cull).cpu().numpy()
    assert _same(dev, want), name


def test_filter_properties_at_a_million_points(vg):
    """Size-independent properties on 1,048,576 points: the kept points are input points, inside
    the cull region (copies of point 0 aside), and no two consecutive kept points lie within
    min_dist of each other in the last pass's order (the order they are returned in)."""
    import torch

    from vamp_gb300 import scenes

    org = np.array([0.0, 0.0, 0.333], np.float32)
    pts = scenes.surface_pointcloud(8, 1 << 20)
    kept = vg.filter_pointcloud_device(torch.from_numpy(pts).cuda(), 0.008, 1.19, org, org - 1.19, org + 1.19,
                                       True).cpu().numpy()
    assert 0 < len(kept) < len(pts)
    d = np.linalg.norm(kept[1:] - org, axis=1)
    inside = d < 1.19
    assert inside.mean() > 0.999  # only copies of point 0 may lie outside
    rows = {r.tobytes() for r in pts}
    assert all(r.tobytes() in rows for r in kept)
    gap = np.sum((kept[1:].astype(np.float64) - kept[:-1]) ** 2, axis=1)
    assert gap.min() > 0.008 ** 2 * (1 - 1e-5)


def test_filter_empty_and_bad_arguments(vg):
    kept, _ = vg.filter_pointcloud(np.zeros((0, 3), np.float32), 0.01, 1.0, [0, 0, 0], [-1] * 3, [1] * 3, True)
    assert kept.shape == (0, 3)
    with pytest.raises(ValueError):
        vg.filter_pointcloud_device(np.zeros((4, 3), np.float32), 0.01, 1.0, [0, 0, 0], [-1] * 3, [1] * 3, True)
