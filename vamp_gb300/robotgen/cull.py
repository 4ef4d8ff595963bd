"""Self-collision sphere pairs that cannot collide inside the joint limits.

The reference tests every fine sphere pair of a link pair whenever the two links' coarse spheres
overlap.  For links a few joints apart the coarse spheres may always overlap (Panda link5 and
its hand: 216 pairs on every configuration) although most fine pairs never get close.  This
module proves, offline and in float64, which pairs stay apart by more than a margin for every
configuration in the joint limits widened by a slack; the kernels skip those pairs whenever every
configuration of the warp lies inside the widened limits, and test every pair otherwise.  A
skipped pair could only have changed a verdict if its FP32 test value could turn negative, which
the margin excludes (FP32 centre errors are ~1e-6 m, the margin is 100x that).

Method: the relative pose of two links depends only on the joints on the kinematic path between
them.  For paths of at most MAX_JOINTS joints the pair distance is evaluated on a grid over those
joints; within a grid cell a centre moves by at most sum_k dist(centre, axis_k) * h_k / 2, so
    min over the box >= min over the grid - sum_k D_k * h_k / 2,
with D_k the largest distance of the moving sphere's centre from joint k's axis over the grid.
A pair is culled when that bound exceeds MARGIN.
"""
from __future__ import annotations

import numpy as np

from .urdf import axis_rotation, rpy_matrix

SLACK_RAD = 1e-3     # joint limits widened by this much on both sides
MARGIN = 1e-4        # metres of clearance a culled pair keeps at every configuration
MAX_JOINTS = 2       # grid analysis only for link pairs at most this many joints apart
STEP_RAD = 0.004     # grid step


def _parents(model):
    return {j["child"]: j for j in model["joints"]}


def _chain(model, link):
    """Joints from the root down to link."""
    par = _parents(model)
    out = []
    while link in par:
        out.append(par[link])
        link = par[link]["parent"]
    return out[::-1]


def _tf(j, q=0.0):
    T = np.eye(4)
    T[:3, :3] = rpy_matrix(j["rpy"])
    T[:3, 3] = j["xyz"]
    M = np.eye(4)
    if j["type"] in ("revolute", "continuous") and j["name"] is not None:
        M[:3, :3] = axis_rotation(j["axis"], q)
    elif j["type"] == "prismatic":
        a = np.asarray(j["axis"], float)
        M[:3, 3] = a / np.linalg.norm(a) * q
    return T @ M


def pair_path(model, a, b):
    """(joints on the path a -> common ancestor, joints on the path ancestor -> b)."""
    ca, cb = _chain(model, a), _chain(model, b)
    k = 0
    while k < min(len(ca), len(cb)) and ca[k]["name"] == cb[k]["name"]:
        k += 1
    return ca[k:], cb[k:]


def _rot_batch(axis, q):
    """Rotations about `axis` by every angle in q (Rodrigues), shape [n, 3, 3]."""
    a = np.asarray(axis, float)
    a = a / np.linalg.norm(a)
    K = np.array([[0, -a[2], a[1]], [a[2], 0, -a[0]], [-a[1], a[0], 0]])
    c, s = np.cos(q)[:, None, None], np.sin(q)[:, None, None]
    return c * np.eye(3) + s * K + (1 - c) * np.outer(a, a)


def _moving_frame(model, link, p):
    """(moving frame of link, offset of point p of link in that frame)."""
    par = _parents(model)
    cur, chain = link, []
    while cur in par and par[cur]["type"] == "fixed":
        chain.append(par[cur])
        cur = par[cur]["parent"]
    T = np.eye(4)
    for j in reversed(chain):
        T = T @ _tf(j)
    return cur, (T @ np.array([*p, 1.0]))[:3]


def _b_centres(model, down, qs, b_off) -> dict:
    """World (A-frame) centres of the B spheres for the joint values qs [n, joints]."""
    n = len(qs)
    T = np.broadcast_to(np.eye(4), (n, 4, 4)).copy()
    mi = 0
    for j in down:
        if j["type"] == "fixed":
            T = T @ _tf(j)
            continue
        pre = np.eye(4)
        pre[:3, :3] = rpy_matrix(j["rpy"])
        pre[:3, 3] = j["xyz"]
        T = T @ pre
        w = np.asarray(j["axis"], float)
        M = np.broadcast_to(np.eye(4), (n, 4, 4)).copy()
        M[:, :3, :3] = _rot_batch(w / np.linalg.norm(w), qs[:, mi])
        T = T @ M
        mi += 1
    return {sb: np.einsum("nij,j->ni", T, np.array([*off, 1.0]))[:, :3] for sb, off in b_off.items()}


def analyse(model: dict, boxes: list | None = None) -> list:
    """For each self check, the indices (into its fine pair list) of pairs that may collide
    inside the widened limits; None when the check was not analysed (all pairs kept).

    With `boxes` (a list), also appends per self check either None or, per live pair, its
    danger box: (joint indices, [lo, hi] per joint) containing every configuration inside the
    widened limits at which the pair may come within MARGIN.  Outside the box the pair keeps
    MARGIN clearance, by the same grid-plus-Lipschitz bound: a configuration with distance
    <= MARGIN has a grid point within half a step per joint whose distance is <= MARGIN plus the
    bound's slack, and the box covers every such grid point's cell."""
    names = model["joint_names"]
    lo = np.array(model["s_a"], float) - SLACK_RAD
    hi = np.array(model["s_a"], float) + np.array(model["s_m"], float) + SLACK_RAD
    fine = model["fine_spheres"]
    out = []
    for chk in model["self_checks"]:
        pairs = chk["fine"]
        fa = {_moving_frame(model, fine[sa]["link"], fine[sa]["p"])[0] for sa, _ in pairs}
        fb = {_moving_frame(model, fine[sb]["link"], fine[sb]["p"])[0] for _, sb in pairs}
        if len(fa) != 1 or len(fb) != 1:
            out.append(None)
            if boxes is not None:
                boxes.append(None)
            continue
        fa, fb = fa.pop(), fb.pop()
        ca, cb = _chain(model, fa), _chain(model, fb)
        if [j["name"] for j in cb[: len(ca)]] != [j["name"] for j in ca]:
            out.append(None)  # analysed only when A's frame is an ancestor of B's frame
            if boxes is not None:
                boxes.append(None)
            continue
        down = cb[len(ca):]
        moving = [j for j in down if j["type"] != "fixed"]
        if not moving or len(moving) > MAX_JOINTS or any(j["name"] not in names for j in moving):
            out.append(None)
            if boxes is not None:
                boxes.append(None)
            continue
        idx = [names.index(j["name"]) for j in moving]
        grids, steps = [], []
        for k in idx:
            n = int(np.ceil((hi[k] - lo[k]) / STEP_RAD)) + 1
            grids.append(np.linspace(lo[k], hi[k], n))
            steps.append((hi[k] - lo[k]) / (n - 1))
        mesh = np.stack(np.meshgrid(*grids, indexing="ij"), -1).reshape(-1, len(idx))
        a_pts = {sa: (_moving_frame(model, fine[sa]["link"], fine[sa]["p"])[1], fine[sa]["r"]) for sa, _ in pairs}
        b_ids = sorted({sb for _, sb in pairs})
        b_off = {sb: _moving_frame(model, fine[sb]["link"], fine[sb]["p"])[1] for sb in b_ids}
        mins = np.full(len(pairs), np.inf)
        dmax = np.zeros((len(b_ids), len(idx)))

        CH = 50000
        for s in range(0, len(mesh), CH):
            qs = mesh[s : s + CH]
            n = len(qs)
            T = np.broadcast_to(np.eye(4), (n, 4, 4)).copy()
            axes_o, axes_w = [], []
            mi = 0
            for j in down:
                if j["type"] == "fixed":
                    T = T @ _tf(j)
                    continue
                pre = np.eye(4)
                pre[:3, :3] = rpy_matrix(j["rpy"])
                pre[:3, 3] = j["xyz"]
                T = T @ pre
                w = np.asarray(j["axis"], float)
                w = w / np.linalg.norm(w)
                axes_o.append(T[:, :3, 3].copy())
                axes_w.append(np.einsum("nij,j->ni", T[:, :3, :3], w))
                M = np.broadcast_to(np.eye(4), (n, 4, 4)).copy()
                if j["type"] == "prismatic":
                    raise ValueError("prismatic joints are not analysed")
                M[:, :3, :3] = _rot_batch(w, qs[:, mi])
                T = T @ M
                mi += 1
            bc = {}
            for bi, sb in enumerate(b_ids):
                c = np.einsum("nij,j->ni", T, np.array([*b_off[sb], 1.0]))[:, :3]
                bc[sb] = c
                for k in range(len(idx)):
                    v = c - axes_o[k]
                    d = np.linalg.norm(v - np.einsum("ni,ni->n", v, axes_w[k])[:, None] * axes_w[k], axis=1)
                    dmax[bi, k] = max(dmax[bi, k], d.max())
            for pi, (sa, sb) in enumerate(pairs):
                pa, ra = a_pts[sa]
                d = np.linalg.norm(bc[sb] - pa, axis=1) - (ra + fine[sb]["r"])
                mins[pi] = min(mins[pi], d.min())
        live = []
        for pi, (sa, sb) in enumerate(pairs):
            bi = b_ids.index(sb)
            bound = mins[pi] - sum(dmax[bi, k] * 1.01 * steps[k] / 2 for k in range(len(idx)))
            if not (bound > MARGIN):
                live.append(pi)
        out.append(live)
        if boxes is not None:
            # second pass: the grid points near enough to matter, per live pair
            slack = {pi: sum(dmax[b_ids.index(pairs[pi][1]), k] * 1.01 * steps[k] / 2 for k in range(len(idx)))
                     for pi in live}
            blo = {pi: np.full(len(idx), np.inf) for pi in live}
            bhi = {pi: np.full(len(idx), -np.inf) for pi in live}
            for s0 in range(0, len(mesh), CH):
                qs = mesh[s0 : s0 + CH]
                bc = _b_centres(model, down, qs, b_off)
                for pi in live:
                    sa, sb = pairs[pi]
                    pa, ra = a_pts[sa]
                    d = np.linalg.norm(bc[sb] - pa, axis=1) - (ra + fine[sb]["r"])
                    near = qs[d - slack[pi] <= MARGIN]
                    if len(near):
                        blo[pi] = np.minimum(blo[pi], near.min(0))
                        bhi[pi] = np.maximum(bhi[pi], near.max(0))
            per = []
            for pi in live:
                # one whole grid step of padding on each side (half a step covers the cells)
                per.append({"joints": idx, "lo": [float(blo[pi][k] - steps[k]) for k in range(len(idx))],
                            "hi": [float(bhi[pi][k] + steps[k]) for k in range(len(idx))]})
            boxes.append(per)
    return out


def main():
    import argparse
    import json
    from pathlib import Path

    from ..robots import HERE, model

    ap = argparse.ArgumentParser(description="write vamp_gb300/robots/<robot>.cull.json")
    ap.add_argument("robots", nargs="*", default=["panda", "ur5", "fetch", "baxter"])
    a = ap.parse_args()
    for r in a.robots:
        boxes = []
        live = analyse(model(r), boxes)
        out = {"slack_rad": SLACK_RAD, "margin": MARGIN, "step_rad": STEP_RAD, "max_joints": MAX_JOINTS, "live": live,
               "boxes": boxes}
        Path(HERE / f"{r}.cull.json").write_text(json.dumps(out) + "\n")
        kept = sum(len(c["fine"]) if l is None else len(l) for c, l in zip(model(r)["self_checks"], live))
        total = sum(len(c["fine"]) for c in model(r)["self_checks"])
        print(f"{r}: {kept} of {total} fine self pairs may collide inside the limits")


if __name__ == "__main__":
    main()
