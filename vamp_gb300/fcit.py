"""Batched checks for FCIT*-style planners (planning/fcit.hh).

The reference's FCIT* calls the hot path one item at a time in two places:
  * the sample loop (fcit.hh:320-336) draws configurations until `batch_size` of them are valid,
    checking each with Robot::fkcc on a block that broadcasts the one configuration;
  * the search (fcit.hh:230-245) checks an edge parent -> node with validate_motion when it pops
    it from its queue, lazily, and remembers invalid edges in each node's invalidList.
Here both go to the GPU in batches with the same outcomes:
  * sample_batch checks draws in chunks and keeps the first `batch_size` valid ones in draw order:
    exactly the draws the one-at-a-time loop keeps (a broadcast block is the single
    configuration's check, which Robot.validate_batch computes);
  * EdgeCache answers the search's edge queries from verdicts computed in batches: when a node's
    neighbour list is sorted, the edges to its nearest neighbours (the ones the search pops first)
    are checked together, and a query for an edge not yet known checks it with the next batch of
    that node's neighbours.  A verdict depends only on the edge's two configurations, so every
    answer is the one validate_motion gives, whatever was checked ahead.

Both take the batch checkers as functions, so that the same logic runs on the GPU
(gpu_checkers) or, in tests, on any other implementation of the reference's checks.
"""
from __future__ import annotations

from typing import Callable

import numpy as np

StatesFn = Callable[[np.ndarray], np.ndarray]            # [n, dim] -> uint8 [n], 1 = valid
EdgesFn = Callable[[np.ndarray, np.ndarray], np.ndarray]  # starts, goals [n, dim] -> uint8 [n]


def gpu_checkers(robot, environment, resolution: int | None = None):
    """(states, edges) batch checkers on the GPU for one robot and environment: the reference's
    validate(q) per configuration and validate_motion at the robot's resolution per edge."""
    res = robot.resolution() if resolution is None else int(resolution)

    def states(q: np.ndarray) -> np.ndarray:
        return robot.validate_batch(np.ascontiguousarray(q, np.float32), environment)

    def edges(a: np.ndarray, b: np.ndarray) -> np.ndarray:
        return robot.validate_motion_batch(np.ascontiguousarray(a, np.float32), np.ascontiguousarray(b, np.float32),
                                           environment, res)

    return states, edges


def sample_batch(states: StatesFn, draws: np.ndarray, batch_size: int, chunk: int = 4096):
    """Indices into `draws` (the sampler's configurations in draw order) of the first batch_size
    valid ones, and the number of draws consumed (up to and including the last one kept), as the
    sample loop (fcit.hh:320-336) keeps them.  Draws are checked `chunk` at a time."""
    draws = np.asarray(draws, np.float32)
    kept: list[int] = []
    pos = 0
    while len(kept) < batch_size and pos < len(draws):
        want = batch_size - len(kept)
        n = min(len(draws) - pos, max(chunk, 2 * want))
        valid = states(draws[pos:pos + n])
        for i in np.nonzero(valid)[0][:want]:
            kept.append(pos + int(i))
        pos += n
    used = kept[-1] + 1 if len(kept) == batch_size else len(draws)
    return np.array(kept, np.int64), used


class EdgeCache:
    """Validity of edges between roadmap nodes (configs[i]), computed in batches.

    prefetch(node, neighbours) checks the edges neighbours[k] -> node for the first `ahead`
    neighbours not yet known (a node's sorted neighbour list, nearest first, as FCIT* builds it,
    fcit.hh:270-311).  valid(parent, node) answers validate_motion(configs[parent], configs[node])
    (fcit.hh:238), checking it together with the node's next unchecked neighbours when it is not
    known yet.  Edges are directed as the search checks them: parent first."""

    def __init__(self, edges: EdgesFn, configs: np.ndarray, ahead: int = 256):
        self.edges = edges
        self.configs = np.asarray(configs, np.float32)
        self.ahead = int(ahead)
        self.known: dict[tuple[int, int], bool] = {}
        self.pending: dict[int, list[int]] = {}  # node -> its neighbours not yet checked, nearest first
        self.calls = 0
        self.checked = 0
        self.queries = 0

    def add_configs(self, configs: np.ndarray) -> None:
        """New roadmap nodes (a sample batch), appended after the existing ones."""
        self.configs = np.concatenate([self.configs, np.asarray(configs, np.float32)])

    def _check(self, pairs: list[tuple[int, int]]) -> None:
        if not pairs:
            return
        p = np.array(pairs, np.int64)
        v = self.edges(self.configs[p[:, 0]], self.configs[p[:, 1]])
        self.calls += 1
        self.checked += len(pairs)
        for (a, b), ok in zip(pairs, v):
            self.known[(a, b)] = bool(ok)

    def prefetch(self, node: int, neighbours) -> None:
        self.pending[node] = [int(j) for j in neighbours if (int(j), node) not in self.known]
        self._next_batch(node)

    def _next_batch(self, node: int) -> None:
        todo = self.pending.get(node, [])
        batch = [(j, node) for j in todo[: self.ahead]]
        self.pending[node] = todo[self.ahead:]
        self._check(batch)

    def valid(self, parent: int, node: int) -> bool:
        self.queries += 1
        key = (int(parent), int(node))
        if key not in self.known:
            if int(parent) in self.pending.get(int(node), []):
                # check it with the node's next neighbours in line
                rest = self.pending[int(node)]
                rest.remove(int(parent))
                self.pending[int(node)] = [int(parent)] + rest
                self._next_batch(int(node))
            else:
                self._check([key])
        return self.known[key]
