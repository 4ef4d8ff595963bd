"""Batched roadmap construction: the neighbour edges of a probabilistic roadmap checked as one
GPU batch.

The reference's PRM (planning/prm.hh:104-150) grows its roadmap one sample at a time: a valid
sample is connected to its nearest earlier nodes (at most max_neighbors, within
neighbor_radius, both functions of the roadmap's size; planning/roadmap.hh:41-67 for PRM*),
each edge checked by its own validate_motion call.  Here the same roadmap is built in three
batched steps: the samples are validated together (Robot.validate_batch), each valid sample's
neighbours among the earlier valid samples are found together (distances on the GPU), and all
candidate edges are checked in one call (Robot.validate_motion_batch at the robot's
resolution).  The nodes and edges are those the incremental loop would produce for the same
sample sequence; only the order of work changes.
"""
from __future__ import annotations

import math

import numpy as np


def unit_ball_measure(dim: int) -> float:
    """Volume of the unit ball in `dim` dimensions (planning/roadmap.hh:17-22)."""
    return math.pi ** (dim / 2.0) / math.gamma(dim / 2.0 + 1.0)


def prmstar_neighbors(dim: int, space_measure: float, num_states: int, gamma_scale: float = 2.0):
    """PRM* neighbour count and radius for a roadmap of num_states nodes
    (PRMStarNeighborParams, planning/roadmap.hh:41-67)."""
    if num_states < 2:
        return 0, 0.0
    k = int(math.ceil((math.e + math.e / dim) * math.log(num_states)))
    ratio = space_measure / unit_ball_measure(dim)
    c = 2.0 * (1.0 + 1.0 / dim) ** (1.0 / dim) * ratio ** (1.0 / dim)
    r = gamma_scale * c * (math.log(num_states) / num_states) ** (1.0 / dim)
    return k, r


def prmstar_table(dim: int, space_measure: float, i0: int, i1: int, gamma_scale: float = 2.0):
    """prmstar_neighbors(dim, space_measure, i) for i in [i0, i1), as two lists: the same float
    operations in the same order, with the terms that do not depend on i computed once."""
    f = math.e + math.e / dim
    ratio = space_measure / unit_ball_measure(dim)
    c = 2.0 * (1.0 + 1.0 / dim) ** (1.0 / dim) * ratio ** (1.0 / dim)
    inv = 1.0 / dim
    ks = [int(math.ceil(f * math.log(i))) if i >= 2 else 0 for i in range(i0, i1)]
    rs = [gamma_scale * c * (math.log(i) / i) ** inv if i >= 2 else 0.0 for i in range(i0, i1)]
    return ks, rs


def neighbour_pairs(nodes, space_measure: float, k_max: int | None = None, radius: float | None = None,
                    chunk: int = 4096):
    """Candidate edges (earlier node, node) of the incremental roadmap over `nodes` [n, dim] (a
    torch tensor, any device): node i is joined to its nearest earlier nodes, at most k(i), within
    r(i), where k(i), r(i) are the PRM* values for a roadmap of i nodes unless k_max / radius fix
    them.  Returns (pairs [m, 2] int64, distances [m]) on the nodes' device, in node order, each
    node's neighbours nearest first."""
    import torch

    n, dim = nodes.shape
    pairs, dists = [], []
    for i0 in range(1, n, chunk):
        i1 = min(n, i0 + chunk)
        rows = nodes[i0:i1]
        d = torch.cdist(rows, nodes[:i1])  # [rows, i1]
        idx = torch.arange(i0, i1, device=nodes.device)
        later = torch.arange(i1, device=nodes.device)[None, :] >= idx[:, None]  # self and later nodes
        d = d.masked_fill(later, float("inf"))
        ks, rs = prmstar_table(dim, space_measure, i0, i1)
        if k_max is not None:
            ks = [k_max] * (i1 - i0)
        if radius is not None:
            rs = [radius] * (i1 - i0)
        kmax = max(1, min(max(ks), i1))
        vals, order = torch.topk(d, kmax, dim=1, largest=False)
        kt = torch.tensor(ks, device=nodes.device)[:, None]
        rt = torch.tensor(rs, device=nodes.device, dtype=vals.dtype)[:, None]
        keep = (torch.arange(kmax, device=nodes.device)[None, :] < kt) & (vals <= rt) & torch.isfinite(vals)
        r_idx, c_idx = torch.nonzero(keep, as_tuple=True)
        pairs.append(torch.stack([order[r_idx, c_idx], idx[r_idx]], dim=1))
        dists.append(vals[r_idx, c_idx])
    if not pairs:
        return torch.zeros((0, 2), dtype=torch.int64, device=nodes.device), torch.zeros(0, device=nodes.device)
    return torch.cat(pairs), torch.cat(dists)


def build_roadmap(robot, environment, samples, k_max: int | None = None, radius: float | None = None,
                  resolution: int | None = None) -> dict:
    """The roadmap over `samples` [n, dim] (a CUDA tensor, in sampling order): the valid samples
    become nodes; each is joined to its PRM* neighbours among the earlier nodes by the edges
    whose straight-line motion is valid.  Returns nodes [v, dim], edges [e, 2] (node indices,
    earlier node first), their lengths, and the counts of candidates and valid edges."""
    import torch

    if not (isinstance(samples, torch.Tensor) and samples.is_cuda):
        raise ValueError("build_roadmap takes a CUDA tensor of samples")
    q = samples.to(torch.float32).contiguous()
    valid = robot.validate_batch(q, environment).bool()
    nodes = q[valid].contiguous()
    space = float(np.prod(robot.s_m.astype(np.float64)))
    pairs, dist = neighbour_pairs(nodes, space, k_max, radius)
    res = robot.resolution() if resolution is None else resolution
    if len(pairs):
        ok = robot.validate_motion_batch(nodes[pairs[:, 0]].contiguous(), nodes[pairs[:, 1]].contiguous(), environment,
                                         res).bool()
    else:
        ok = torch.zeros(0, dtype=torch.bool, device=q.device)
    return {"nodes": nodes, "edges": pairs[ok], "lengths": dist[ok], "candidates": int(len(pairs)),
            "valid_samples": int(valid.sum()), "valid_edges": int(ok.sum())}
