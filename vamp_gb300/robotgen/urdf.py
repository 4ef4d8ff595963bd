"""Spherized URDF reader and double-precision forward kinematics.

A robot for collision checking is a tree of rigid links joined by revolute, prismatic or fixed
joints; every link carries a set of collision spheres in its own frame.  The spherized URDFs that
ship with the reference (resources/<robot>/<robot>_spherized.urdf) describe exactly that, and the
reference's generated kernels (src/impl/vamp/robots/<robot>.hh) are compiled from them.  This
module parses such a file and evaluates its kinematics in float64; it is the basis of both the
FP64 FK oracle and the FP32 code generator.
"""
from __future__ import annotations

import math
import xml.etree.ElementTree as ET
from dataclasses import dataclass, field

import numpy as np


@dataclass
class Joint:
    name: str
    kind: str  # "revolute" | "continuous" | "prismatic" | "fixed"
    parent: str
    child: str
    xyz: tuple
    rpy: tuple
    axis: tuple
    lower: float = 0.0
    upper: float = 0.0


@dataclass
class Link:
    name: str
    spheres: list = field(default_factory=list)  # [(x, y, z, r)] in the link frame


@dataclass
class Urdf:
    name: str
    links: dict
    joints: list  # in file order
    child_joint: dict  # child link name -> Joint

    @property
    def root(self) -> str:
        children = {j.child for j in self.joints}
        roots = [n for n in self.links if n not in children]
        assert len(roots) == 1, roots
        return roots[0]

    def chain(self, link: str) -> list:
        """Joints from the root down to `link`."""
        out = []
        while link in self.child_joint:
            j = self.child_joint[link]
            out.append(j)
            link = j.parent
        return out[::-1]


def _floats(s: str | None, n: int, default=0.0) -> tuple:
    if s is None:
        return tuple([default] * n)
    v = [float(t) for t in s.split()]
    assert len(v) == n, s
    return tuple(v)


def parse(path: str) -> Urdf:
    root = ET.parse(path).getroot()
    links = {}
    for l in root.findall("link"):
        link = Link(l.get("name"))
        for c in l.findall("collision"):
            g = c.find("geometry")
            s = g.find("sphere") if g is not None else None
            if s is None:
                continue
            o = c.find("origin")
            xyz = _floats(o.get("xyz") if o is not None else None, 3)
            link.spheres.append((*xyz, float(s.get("radius"))))
        links[link.name] = link
    joints = []
    for j in root.findall("joint"):
        o = j.find("origin")
        a = j.find("axis")
        lim = j.find("limit")
        joints.append(
            Joint(
                name=j.get("name"),
                kind=j.get("type"),
                parent=j.find("parent").get("link"),
                child=j.find("child").get("link"),
                xyz=_floats(o.get("xyz") if o is not None else None, 3),
                rpy=_floats(o.get("rpy") if o is not None else None, 3),
                axis=_floats(a.get("xyz") if a is not None else None, 3, 0.0) if a is not None else (1.0, 0.0, 0.0),
                lower=float(lim.get("lower", 0.0)) if lim is not None else 0.0,
                upper=float(lim.get("upper", 0.0)) if lim is not None else 0.0,
            )
        )
    return Urdf(root.get("name"), links, joints, {j.child: j for j in joints})


def rpy_matrix(rpy) -> np.ndarray:
    """URDF fixed-axis roll-pitch-yaw: R = Rz(yaw) @ Ry(pitch) @ Rx(roll)."""
    r, p, y = rpy
    cr, sr, cp, sp, cy, sy = math.cos(r), math.sin(r), math.cos(p), math.sin(p), math.cos(y), math.sin(y)
    rx = np.array([[1, 0, 0], [0, cr, -sr], [0, sr, cr]])
    ry = np.array([[cp, 0, sp], [0, 1, 0], [-sp, 0, cp]])
    rz = np.array([[cy, -sy, 0], [sy, cy, 0], [0, 0, 1]])
    return rz @ ry @ rx


def axis_rotation(axis, angle: float) -> np.ndarray:
    a = np.asarray(axis, dtype=np.float64)
    a = a / np.linalg.norm(a)
    c, s = math.cos(angle), math.sin(angle)
    k = np.array([[0, -a[2], a[1]], [a[2], 0, -a[0]], [-a[1], a[0], 0]])
    return c * np.eye(3) + s * k + (1 - c) * np.outer(a, a)


def link_transforms(urdf: Urdf, joint_values: dict) -> dict:
    """World transform (R, t) of every link for the given joint values (name -> value)."""
    out = {urdf.root: (np.eye(3), np.zeros(3))}
    pending = list(urdf.joints)
    while pending:
        rest = []
        for j in pending:
            if j.parent not in out:
                rest.append(j)
                continue
            R, t = out[j.parent]
            Ro = rpy_matrix(j.rpy)
            t2 = t + R @ np.asarray(j.xyz)
            R2 = R @ Ro
            if j.kind in ("revolute", "continuous"):
                R2 = R2 @ axis_rotation(j.axis, joint_values.get(j.name, 0.0))
            elif j.kind == "prismatic":
                a = np.asarray(j.axis, dtype=np.float64)
                t2 = t2 + R2 @ (a / np.linalg.norm(a) * joint_values.get(j.name, 0.0))
            out[j.child] = (R2, t2)
        assert len(rest) < len(pending), "disconnected joints"
        pending = rest
    return out
