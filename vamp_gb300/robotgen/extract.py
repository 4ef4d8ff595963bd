"""Robot model extraction (developer tool; needs the reference checkout, not used at run time).

Builds the JSON robot model that this project's code generator consumes.  The kinematics and the
fine collision spheres come from the spherized URDF that ships with the reference
(resources/<robot>/<robot>_spherized.urdf).  Three facts live only in the reference's generated
robot header (src/impl/vamp/robots/<robot>.hh) and are read from it as data:

* the per-robot constants: joint order, joint scaling s_m/s_a (panda.hh:50-66), radius range
  and motion resolution (panda.hh:13-18);
* the coarse link-bounding spheres: one per link, whose centres the header only gives as FK
  expressions; they are evaluated here in float64 and mapped back into the link frame;
* the collision-check schedule of Robot::fkcc (panda.hh:5630-10259): which links are checked
  against the environment and in which order, and which link pairs are self-collision tested,
  each as a coarse test gating a list of fine tests.

Every extracted quantity is cross-checked numerically against the URDF kinematics before it is
written.  Usage:

    python -m vamp_gb300.robotgen.extract --reference /path/to/vamp --robot panda
"""
from __future__ import annotations

import argparse
import json
import math
import re
from pathlib import Path

import numpy as np

from . import urdf as U

HERE = Path(__file__).resolve().parent
MODELS = HERE.parent / "robots"


# --------------------------------------------------------------------------------------------
# generated-header reading


def _body(text: str, signature: str) -> str:
    i = text.index(signature)
    j = text.index("{", text.index(")", text.index("x) noexcept", i)))
    depth, k = 0, j
    while True:
        if text[k] == "{":
            depth += 1
        elif text[k] == "}":
            depth -= 1
            if depth == 0:
                return text[j + 1 : k]
        k += 1


def _const_array(text: str, name: str) -> list:
    m = re.search(r"std::array<float, dimension> " + name + r"\{([^}]*)\}", text)
    return [float(t) for t in m.group(1).replace("\n", " ").split(",") if t.strip()]


def header_constants(text: str) -> dict:
    g = lambda pat: re.search(pat, text).group(1)
    names = re.search(r"joint_names = \{([^}]*)\}", text).group(1)
    return {
        "name": g(r'static constexpr const char \*name = "([^"]+)"'),
        "dimension": int(g(r"dimension = (\d+);")),
        "n_spheres": int(g(r"n_spheres = (\d+);")),
        "min_radius": float(g(r"min_radius = ([-0-9.e]+);")),
        "max_radius": float(g(r"max_radius = ([-0-9.e]+);")),
        "resolution": int(g(r"resolution = (\d+);")),
        "joint_names": re.findall(r'"([^"]+)"', names),
        "end_effector": g(r'end_effector = "([^"]+)"'),
        "s_m": _const_array(text, "s_m"),
        "s_a": _const_array(text, "s_a"),
    }


_TOK = re.compile(
    r"\s*(//[^\n]*|if\b|return false;|return true;|\{|\}|[vy]\[\d+\]\s*=[^;]*;|std::array<[^;]*;)", re.S
)


def parse_fkcc(body: str):
    """Split the fkcc body into FK statements and a check tree.

    Returns (statements, checks) where statements are (target, expression) pairs and checks is a
    list of nodes {"kind": "env"|"self", "slots": [..], "label": str, "children": [...],
    "fails": bool}.
    """
    stmts = []
    pos = 0
    label = [""]

    def parse_if(p):
        # p points just after "if"; read the balanced condition
        i = body.index("(", p)
        depth, k = 0, i
        while True:
            if body[k] == "(":
                depth += 1
            elif body[k] == ")":
                depth -= 1
                if depth == 0:
                    break
            k += 1
        cond = body[i + 1 : k]
        slots = [int(s) for s in re.findall(r"y\[(\d+)\]", cond)]
        if "sphere_environment_in_collision" in cond:
            assert len(slots) == 4 and slots == list(range(slots[0], slots[0] + 4)), cond
            node = {"kind": "env", "slots": [slots[0] // 4]}
        elif "sphere_sphere_self_collision" in cond:
            assert len(slots) == 8, cond
            assert slots[:4] == list(range(slots[0], slots[0] + 4)) and slots[4:] == list(range(slots[4], slots[4] + 4))
            node = {"kind": "self", "slots": [slots[0] // 4, slots[4] // 4]}
        else:
            raise ValueError(cond)
        node["label"] = label[0]
        node["children"] = []
        node["fails"] = False
        m = re.compile(r"\s*\{").match(body, k + 1)
        assert m, body[k : k + 40]
        return node, m.end()

    def parse_block(p, into):
        while True:
            m = _TOK.match(body, p)
            if not m:
                rest = body[p:].strip()
                assert rest == "", rest[:200]
                return p, True
            tok = m.group(1)
            p = m.end()
            if tok.startswith("//"):
                t = tok[2:].strip()
                if t and "collisions" not in t and "dependent variables" not in t:
                    label[0] = t
            elif tok == "if":
                node, p = parse_if(p)
                p, _ = parse_block(p, node["children"])
                into.append(node)
            elif tok == "}":
                return p, False
            elif tok == "{":
                raise ValueError("unexpected {")
            elif tok == "return false;":
                return_false_owner = into
                return_false_owner.append({"kind": "fail"})
            elif tok == "return true;" or tok.startswith("std::array"):
                pass
            else:
                tgt, expr = tok.split("=", 1)
                stmts.append((tgt.strip(), " ".join(expr.strip().rstrip(";").split())))

    checks = []
    parse_block(0, checks)

    def fold(nodes):
        out = []
        for n in nodes:
            if n["kind"] == "fail":
                continue
            ch = n["children"]
            n["fails"] = any(c["kind"] == "fail" for c in ch)
            n["children"] = fold(ch)
            out.append(n)
        return out

    return stmts, fold(checks)


def evaluate(stmts, q) -> dict:
    """Evaluate the FK statements in float64; returns the y slots."""
    env = {"v": {}, "y": {}, "x": list(map(float, q)), "sin": math.sin, "cos": math.cos}
    for tgt, expr in stmts:
        m = re.match(r"([vy])\[(\d+)\]", tgt)
        val = eval(expr, {"__builtins__": {}}, _Lookup(env))
        env[m.group(1)][int(m.group(2))] = float(val)
    return env["y"]


class _Lookup(dict):
    def __init__(self, env):
        super().__init__()
        self.env = env

    def __getitem__(self, k):
        return self.env[k]


def parse_attach(text: str) -> dict:
    """The attachment checks of Robot::fkcc_attach (e.g. panda.hh:10265-15445): the frame the
    attachment is posed at (the y slots of its transform) and, per robot link checked against
    the attachment, its coarse slot and fine slots."""
    body = _body(text, "inline static bool fkcc_attach(")
    frame = re.search(r"//\s*attaching at (\S+)", body).group(1)
    pose = int(re.search(r"set_attachment_pose\(environment, to_isometry\(&y\[(\d+)\]\)\)", body).group(1))
    tail = body[body.index("attachment vs. robot collisions") :]
    checks = []
    for part in re.split(r"//\s*Attachment vs\. ", tail)[1:]:
        link = part.split()[0]
        slots = [int(m) // 4 for m in re.findall(r"attachment_sphere_collision<[^>]*>\(environment, y\[(\d+)\]", part)]
        checks.append({"link": link, "coarse_slot": slots[0], "fine": slots[1:]})
    return {"frame": frame, "pose_slot": pose, "checks": checks}


def eefk_statements(text: str):
    """FK statements of Robot::eefk (the end-effector transform, y[0..11])."""
    body = _body(text, "inline static auto eefk(")
    return [(t.strip(), " ".join(e.strip().rstrip(";").split()))
            for t, e in re.findall(r"^\s*([vy]\[\d+\])\s*=\s*([^;]*;)", body, re.M)]


# --------------------------------------------------------------------------------------------
# model assembly


def build_model(reference: Path, robot: str, seed: int = 0) -> dict:
    hdr = (reference / "src/impl/vamp/robots" / f"{robot}.hh").read_text()
    consts = header_constants(hdr)
    stmts, checks = parse_fkcc(_body(hdr, "inline static bool fkcc("))
    udir = reference / "resources" / robot
    urdf = U.parse(str(udir / f"{robot}_spherized.urdf"))

    dim = consts["dimension"]
    jnames = consts["joint_names"]
    rng = np.random.default_rng(seed)
    s_m, s_a = np.array(consts["s_m"]), np.array(consts["s_a"])

    samples = [rng.random(dim) * s_m + s_a for _ in range(8)]
    ys = [evaluate(stmts, q) for q in samples]
    tfs = [U.link_transforms(urdf, dict(zip(jnames, q))) for q in samples]

    # The link each slot is checked under, from the schedule labels.
    slot_label = {}
    for c in checks:
        for ch in c["children"]:
            if ch["kind"] == "env":
                slot_label.setdefault(ch["slots"][0], c["label"])
            else:
                a, b = c["label"].split(" vs. ")
                slot_label.setdefault(ch["slots"][0], a)
                slot_label.setdefault(ch["slots"][1], b)

    # Fine spheres: the header numbers them in its own link order, so each slot is matched to
    # the URDF sphere with the same world position (at every sample) and radius.
    candidates = [(n, s) for n in urdf.links for s in urdf.links[n].spheres]
    fine = []
    for i in range(consts["n_spheres"]):
        matches = []
        for n, s in candidates:
            err = 0.0
            for y, tf in zip(ys, tfs):
                R, t = tf[n]
                w = t + R @ np.array(s[:3])
                err = max(err, float(np.abs(w - np.array([y[4 * i], y[4 * i + 1], y[4 * i + 2]])).max()))
            if err < 1e-9 and abs(y[4 * i + 3] - s[3]) < 1e-6:
                matches.append((n, s))
        assert matches, f"slot {i} has no URDF sphere"
        pick = [m for m in matches if m[0] == slot_label.get(i)] or matches
        n, s = pick[0]
        fine.append({"link": n, "p": list(s[:3]), "r": s[3]})

    # coarse spheres: env check roots and self check roots that are not fine slots
    coarse_slots = {}
    for c in checks:
        if c["kind"] == "env":
            coarse_slots[c["slots"][0]] = c["label"]
    n_fine = len(fine)

    # map coarse slots to link-frame offsets
    coarse = {}
    for slot, link in coarse_slots.items():
        assert slot >= n_fine, (slot, link)
        assert link in urdf.links, link
        offs = []
        for y, tf in zip(ys, tfs):
            R, t = tf[link]
            w = np.array([y[4 * slot], y[4 * slot + 1], y[4 * slot + 2]])
            offs.append(R.T @ (w - t))
        offs = np.array(offs)
        assert np.abs(offs - offs[0]).max() < 1e-9, (link, np.abs(offs - offs[0]).max())
        coarse[link] = {"slot": slot, "p": [float(v) for v in offs[0]], "r": float(ys[0][4 * slot + 3])}

    def fine_slots(node):
        return [ch["slots"] if node["kind"] == "self" else ch["slots"][0] for ch in node["children"]]

    env_checks = []
    self_checks = []
    for c in checks:
        assert c["fails"] is False, "top-level checks only gate"
        for ch in c["children"]:
            assert ch["kind"] == c["kind"] and ch["fails"] and not ch["children"]
        if c["kind"] == "env":
            env_checks.append({"link": c["label"], "fine": fine_slots(c)})
        else:
            a, b = c["label"].split(" vs. ")
            sa, sb = c["slots"]
            assert coarse[a]["slot"] == sa and coarse[b]["slot"] == sb, c["label"]
            self_checks.append({"links": [a, b], "fine": fine_slots(c)})

    # the links of every fine slot must agree with the check labels
    for e in env_checks:
        for s in e["fine"]:
            assert fine[s]["link"] == e["link"], (s, e["link"])
    for e in self_checks:
        for sa, sb in e["fine"]:
            assert fine[sa]["link"] == e["links"][0] and fine[sb]["link"] == e["links"][1]

    # attachment checks (fkcc_attach): the pose frame is the end effector, whose transform the
    # header's eefk computes (translation, then the rotation column-major, vector/math.hh:39-51)
    att = parse_attach(hdr)
    assert att["frame"] == consts["end_effector"], att["frame"]
    ee_stmts = eefk_statements(hdr)
    for q, tf in zip(samples, tfs):
        y = evaluate(ee_stmts, q)
        R, t = tf[att["frame"]]
        assert np.abs(np.array([y[k] for k in range(3)]) - t).max() < 1e-9
        assert np.abs(np.array([y[3 + k] for k in range(9)]).reshape(3, 3).T - R).max() < 1e-9
    for c in att["checks"]:
        assert coarse[c["link"]]["slot"] == c["coarse_slot"], c["link"]
        for s_ in c["fine"]:
            assert fine[s_]["link"] == c["link"], (s_, c["link"])
    attach_checks = [{"link": c["link"], "fine": c["fine"]} for c in att["checks"]]

    joints = []
    for j in urdf.joints:
        joints.append(
            {
                "name": j.name,
                "type": j.kind,
                "parent": j.parent,
                "child": j.child,
                "xyz": list(j.xyz),
                "rpy": list(j.rpy),
                "axis": list(j.axis),
            }
        )

    return {
        "name": consts["name"],
        "dimension": dim,
        "joint_names": jnames,
        "end_effector": consts["end_effector"],
        "resolution": consts["resolution"],
        "min_radius": consts["min_radius"],
        "max_radius": consts["max_radius"],
        "s_m": consts["s_m"],
        "s_a": consts["s_a"],
        "root": urdf.root,
        "joints": joints,
        "fine_spheres": fine,
        "coarse_spheres": {k: {"p": v["p"], "r": v["r"]} for k, v in coarse.items()},
        "env_checks": env_checks,
        "self_checks": self_checks,
        "attach_checks": attach_checks,
        "source": {
            "urdf": f"resources/{robot}/{robot}_spherized.urdf",
            "header": f"src/impl/vamp/robots/{robot}.hh",
        },
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", required=True)
    ap.add_argument("--robot", action="append", required=True)
    a = ap.parse_args()
    MODELS.mkdir(parents=True, exist_ok=True)
    for r in a.robot:
        m = build_model(Path(a.reference), r)
        (MODELS / f"{r}.json").write_text(json.dumps(m, indent=1) + "\n")
        n_self = sum(len(s["fine"]) for s in m["self_checks"])
        print(
            f"{r}: dim {m['dimension']}, {len(m['fine_spheres'])} fine + {len(m['coarse_spheres'])} coarse spheres, "
            f"{len(m['env_checks'])} env links, {len(m['self_checks'])} self pairs ({n_self} fine pairs)"
        )


if __name__ == "__main__":
    main()
