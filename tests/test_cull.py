"""The self-pair culling and danger boxes against sampled configurations (float64 FK of the oracle).

The kernels skip a fine self pair when it was proven offline (robotgen/cull.py) to keep MARGIN
clearance: everywhere inside the widened joint limits (culled pairs), or wherever the check's
joints lie outside the pair's danger box (live pairs).  Here every such claim is checked on
random configurations: a skipped pair must never come within MARGIN."""
import json

import numpy as np
import pytest

from vamp_gb300.robots import HERE, model

ROBOTS = ("panda", "ur5", "fetch", "baxter")


@pytest.mark.parametrize("robot", ROBOTS)
def test_skipped_pairs_keep_their_margin(port, robot):
    m = model(robot)
    cull = json.loads((HERE / f"{robot}.cull.json").read_text())
    margin, slack = cull["margin"], cull["slack_rad"]
    rb = port.robot(robot)
    rng = np.random.default_rng(7)
    lo = np.array(m["s_a"], np.float64) - slack
    hi = lo + np.array(m["s_m"], np.float64) + 2 * slack
    n = 6000
    qs = lo + rng.random((n, len(lo))) * (hi - lo)
    sph = np.stack([rb.spheres_f64(q) for q in qs])  # [n, slots, 4]
    checked = outside = 0
    for ci, chk in enumerate(m["self_checks"]):
        live = cull["live"][ci]
        if live is None:
            continue
        pairs = chk["fine"]
        boxes = (cull.get("boxes") or [None] * len(m["self_checks"]))[ci]
        for pi, (sa, sb) in enumerate(pairs):
            d = np.linalg.norm(sph[:, sa, :3] - sph[:, sb, :3], axis=1) - (sph[:, sa, 3] + sph[:, sb, 3])
            if pi not in live:
                assert d.min() > margin, (robot, chk["links"], pi, d.min())  # culled: never close
                checked += n
                continue
            if not boxes:
                continue
            b = boxes[live.index(pi)]
            inside = np.ones(n, bool)
            for k, j in enumerate(b["joints"]):
                inside &= (qs[:, j] >= b["lo"][k]) & (qs[:, j] <= b["hi"][k])
            out = ~inside
            if out.any():
                assert d[out].min() > margin, (robot, chk["links"], pi, d[out].min())
            outside += int(out.sum())
            checked += n
    if robot == "panda":
        assert outside > 0 and checked > 0  # the boxes do exclude configurations


def test_danger_boxes_hold_just_outside_their_edges(port):
    """Configurations a little outside each Panda danger box (where a too-tight box would fail)."""
    m = model("panda")
    cull = json.loads((HERE / "panda.cull.json").read_text())
    margin, slack = cull["margin"], cull["slack_rad"]
    rb = port.robot("panda")
    rng = np.random.default_rng(11)
    lo = np.array(m["s_a"], np.float64) - slack
    hi = lo + np.array(m["s_m"], np.float64) + 2 * slack
    tested = 0
    for ci, chk in enumerate(m["self_checks"]):
        boxes = cull["boxes"][ci]
        if not boxes:
            continue
        for b, pi in zip(boxes, cull["live"][ci]):
            sa, sb = chk["fine"][pi]
            n = 400
            qs = lo + rng.random((n, len(lo))) * (hi - lo)
            # one joint just outside the box (within 0.05 rad of an edge), the other anywhere
            k = rng.integers(0, len(b["joints"]), n)
            side = rng.random(n) < 0.5
            off = rng.random(n) * 0.05 + 1e-6
            for i in range(n):
                j = b["joints"][k[i]]
                qs[i, j] = b["lo"][k[i]] - off[i] if side[i] else b["hi"][k[i]] + off[i]
            keep = np.all((qs >= lo) & (qs <= hi), axis=1)
            for q in qs[keep]:
                s = rb.spheres_f64(q)
                d = np.linalg.norm(s[sa, :3] - s[sb, :3]) - (s[sa, 3] + s[sb, 3])
                assert d > margin, (chk["links"], pi, q, d)
                tested += 1
    assert tested > 1000


@pytest.mark.parametrize("robot", ROBOTS)
def test_containing_spheres_hold_every_fine_sphere(port, robot):
    """The self checks skip a row of fine pairs when A's sphere misses B's containing sphere: it
    must contain each of B's fine spheres with the margin, at any configuration."""
    from vamp_gb300.robotgen.codegen import CONTAIN_MARGIN, Kin, containing_radius, slot_table

    m = model(robot)
    kin = Kin(m)
    slots, cslot = slot_table(m)
    rb = port.robot(robot)
    rng = np.random.default_rng(3)
    for q in np.array(m["s_a"]) + rng.random((20, len(m["s_a"]))) * np.array(m["s_m"]):
        s = rb.spheres_f64(q)
        for e in m["env_checks"]:
            c = s[cslot[e["link"]], :3]
            R = containing_radius(m, kin, e) + CONTAIN_MARGIN
            for f in e["fine"]:
                assert np.linalg.norm(s[f, :3] - c) + s[f, 3] <= R - 0.9 * CONTAIN_MARGIN, (robot, e["link"], f)
