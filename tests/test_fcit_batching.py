"""Batched FCIT* checks (vamp_gb300.fcit): the sample loop (planning/fcit.hh:320-336) and the
lazy edge checks (fcit.hh:230-245) answered from batches give exactly the one-at-a-time answers.
The CPU tests run the batching logic on the CPU oracle's checkers; the GPU test runs it on the GPU
and compares with the oracle."""
import numpy as np
import pytest


def oracle_checkers(port, scene, resolution=32):
    penv = port.env(scene)
    rb = port.robot("panda")
    states = lambda q: penv.validate_states(rb, np.ascontiguousarray(q, np.float32))  # noqa: E731
    edges = lambda a, b: penv.validate_motions(rb, a, b, resolution)[0]  # noqa: E731
    return states, edges


def one_at_a_time(states, draws, batch_size):
    kept = []
    for i, q in enumerate(draws):
        if len(kept) == batch_size:
            break
        if states(q[None])[0]:
            kept.append(i)
    return kept


def lazy_queries(configs, rng, n_nodes=60, ahead=16):
    """A search-like query pattern: nodes in random order, each with its neighbours sorted by
    distance; the first few edges prefetched, queries mostly near the front of the list and some
    further out."""
    out = []
    for i in rng.permutation(len(configs))[:n_nodes]:
        d = np.linalg.norm(configs - configs[i], axis=1)
        nbrs = [int(j) for j in np.argsort(d) if j != i]
        picks = sorted(set(rng.integers(0, 24, 6).tolist() + rng.integers(0, len(nbrs), 3).tolist()))
        out.append((int(i), nbrs, [nbrs[k] for k in picks]))
    return out


def call_bound(pattern, ahead):
    """Calls the cache may make: one per node for its nearest neighbours, plus one per query for
    an edge outside that first batch."""
    return sum(1 + sum(1 for p in qs if nbrs.index(p) >= ahead) for _, nbrs, qs in pattern)


def run_cache(edges, configs, pattern, ahead=16):
    from vamp_gb300.fcit import EdgeCache

    cache = EdgeCache(edges, configs, ahead=ahead)
    got = []
    for node, nbrs, queries in pattern:
        cache.prefetch(node, nbrs)
        got += [cache.valid(p, node) for p in queries]
    return cache, got


def test_sample_batch_keeps_the_draws_the_sample_loop_keeps(port):
    from vamp_gb300 import scenes
    from vamp_gb300.fcit import sample_batch

    rb = port.robot("panda")
    states, _ = oracle_checkers(port, scenes.scene_config1(1))
    draws = scenes.configurations(rb.s_m, rb.s_a, 600, 31)
    for batch_size, chunk in ((40, 16), (100, 64), (5, 4096)):
        idx, used = sample_batch(states, draws, batch_size, chunk)
        want = one_at_a_time(states, draws, batch_size)
        assert idx.tolist() == want
        assert used == want[-1] + 1


def test_edge_cache_answers_as_per_edge_checks(port):
    from vamp_gb300 import scenes

    rb = port.robot("panda")
    scene = scenes.scene_config1(1)
    states, edges = oracle_checkers(port, scene)
    cand = scenes.configurations(rb.s_m, rb.s_a, 400, 32)
    configs = cand[states(cand) == 1][:150]
    pattern = lazy_queries(configs, np.random.default_rng(5))
    cache, got = run_cache(edges, configs, pattern)
    want = [bool(edges(configs[p][None], configs[i][None])[0]) for i, _, qs in pattern for p in qs]
    assert got == want
    assert cache.calls <= call_bound(pattern, 16) and cache.calls < cache.queries
    assert 0 < sum(want) < len(want)


@pytest.mark.gpu
def test_fcit_batching_on_the_gpu_gives_the_oracles_answers(port):
    import vamp_gb300 as vg
    from vamp_gb300 import scenes
    from vamp_gb300.fcit import gpu_checkers, sample_batch

    rb = port.robot("panda")
    scene = scenes.scene_config1(1)
    g_states, g_edges = gpu_checkers(vg.panda, vg.Environment.from_scene(scene))
    o_states, o_edges = oracle_checkers(port, scene)
    draws = scenes.configurations(rb.s_m, rb.s_a, 5000, 33)
    idx, used = sample_batch(g_states, draws, 1000, 2048)
    assert idx.tolist() == one_at_a_time(o_states, draws[:used + 1], 1000)
    configs = draws[idx[:300]]
    pattern = lazy_queries(configs, np.random.default_rng(6), n_nodes=120)
    cache, got = run_cache(g_edges, configs, pattern, ahead=64)
    want = [bool(o_edges(configs[p][None], configs[i][None])[0]) for i, _, qs in pattern for p in qs]
    assert got == want
    assert cache.calls <= call_bound(pattern, 64) and cache.calls < cache.queries
