"""The batched roadmap's neighbour selection against the reference's incremental loop
(planning/prm.hh:104-150: each valid sample joined to its nearest earlier nodes, at most
max_neighbors(size) within neighbor_radius(size); PRM* parameters, planning/roadmap.hh:41-67),
restated here as a plain loop over numpy arrays."""
import math

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from vamp_gb300.roadmap import neighbour_pairs, prmstar_neighbors, prmstar_table  # noqa: E402


def _incremental(nodes: np.ndarray, space: float, k_max=None, radius=None):
    out = []
    for i in range(len(nodes)):
        k, r = prmstar_neighbors(nodes.shape[1], space, i)
        k = k_max if k_max is not None else k
        r = radius if radius is not None else r
        if i == 0 or k == 0:
            continue
        d = np.linalg.norm(nodes[:i].astype(np.float64) - nodes[i], axis=1)
        for j in np.argsort(d, kind="stable")[:k]:
            if d[j] <= r:
                out.append((int(j), i))
    return out


@pytest.mark.parametrize("dim", [6, 7, 14])
def test_prmstar_table_is_the_per_node_form(dim):
    ks, rs = prmstar_table(dim, 3.7, 0, 5000)
    for i in range(5000):
        assert (ks[i], rs[i]) == prmstar_neighbors(dim, 3.7, i), i


def test_prmstar_parameters():
    k, r = prmstar_neighbors(7, 1.0, 1000)
    assert k == math.ceil((math.e + math.e / 7) * math.log(1000))
    assert r > 0 and prmstar_neighbors(7, 1.0, 1) == (0, 0.0)
    assert prmstar_neighbors(7, 1.0, 4000)[1] < r  # the radius shrinks as the roadmap grows


@pytest.mark.parametrize("k_max,radius", [(None, None), (5, None), (None, 0.8), (7, 1.2)])
def test_neighbour_pairs_are_the_incremental_loops(k_max, radius):
    rng = np.random.default_rng(3)
    nodes = rng.uniform(-1, 1, (700, 7)).astype(np.float32)
    space = 2.0 ** 7
    got, dist = neighbour_pairs(torch.from_numpy(nodes), space, k_max, radius, chunk=256)
    want = _incremental(nodes, space, k_max, radius)
    assert [tuple(p) for p in got.tolist()] == want
    assert torch.all(dist >= 0)
