"""Primitive constructors with the reference's parameterisation (collision/factory.hh), returning
objects whose fields Environment.add_sphere / add_cuboid / add_capsule take.

* Sphere(center, radius).
* Cuboid(center, euler_xyz, half_extents): axes are the columns of Rz(phi) Ry(theta) Rx(rho)
  (factory.hh:26-61; Euler XYZ = (rho, theta, phi)), computed in float64 and rounded to float32
  (the reference composes them with Eigen in float, so they may differ in the last bit).
* Capsule.from_endpoints(p1, p2, radius): the segment p1 -> p2 (factory.hh:234-244), with the
  reference's float arithmetic: v = p2 - p1, dot = v . v (fused as fma(vz, vz, fma(vx, vx,
  vy * vy))), rdv = (float)(1.0 / dot).
* Capsule(center, euler_xyz, radius, length) (alias Cylinder): end points length / 2 from the
  centre along the rotated z axis (factory.hh:280-300), then from_endpoints.
"""
from __future__ import annotations

import math

import numpy as np

_f32 = np.float32


def _fma32(a, b, c) -> np.float32:
    """a * b + c rounded once to float32 (inputs float32: the product is exact in float64)."""
    return _f32(np.float64(a) * np.float64(b) + np.float64(c))


def euler_xyz_matrix(euler_xyz) -> np.ndarray:
    """Rz(phi) @ Ry(theta) @ Rx(rho) for euler_xyz = (rho, theta, phi), float64."""
    rho, theta, phi = (float(v) for v in euler_xyz)
    cx, sx, cy, sy, cz, sz = math.cos(rho), math.sin(rho), math.cos(theta), math.sin(theta), math.cos(phi), math.sin(phi)
    rx = np.array([[1, 0, 0], [0, cx, -sx], [0, sx, cx]])
    ry = np.array([[cy, 0, sy], [0, 1, 0], [-sy, 0, cy]])
    rz = np.array([[cz, -sz, 0], [sz, cz, 0], [0, 0, 1]])
    return rz @ ry @ rx


class Sphere:
    def __init__(self, center, radius: float):
        self.x, self.y, self.z = (_f32(v) for v in center)
        self.r = _f32(radius)


class Cuboid:
    def __init__(self, center, euler_xyz, half_extents):
        self.x, self.y, self.z = (_f32(v) for v in center)
        R = euler_xyz_matrix(euler_xyz)
        (self.axis_1_x, self.axis_1_y, self.axis_1_z), (self.axis_2_x, self.axis_2_y, self.axis_2_z), \
            (self.axis_3_x, self.axis_3_y, self.axis_3_z) = ((_f32(v) for v in R[:, k]) for k in range(3))
        self.axis_1_r, self.axis_2_r, self.axis_3_r = (_f32(v) for v in half_extents)


class Capsule:
    def __init__(self, center, euler_xyz, radius: float, length: float):
        R = euler_xyz_matrix(euler_xyz)
        c = np.asarray(center, np.float64)
        half = np.float64(_f32(length) / _f32(2))
        p1 = (c + R @ np.array([0.0, 0.0, half])).astype(np.float32)
        p2 = (c + R @ np.array([0.0, 0.0, -half])).astype(np.float32)
        self._set(p1, p2, radius)

    @classmethod
    def from_endpoints(cls, p1, p2, radius: float) -> "Capsule":
        c = cls.__new__(cls)
        c._set(np.asarray(p1, np.float32), np.asarray(p2, np.float32), radius)
        return c

    def _set(self, p1, p2, radius):
        self.x1, self.y1, self.z1 = (_f32(v) for v in p1)
        self.xv, self.yv, self.zv = (_f32(_f32(p2[k]) - _f32(p1[k])) for k in range(3))
        dot = _fma32(self.zv, self.zv, _fma32(self.xv, self.xv, _f32(self.yv * self.yv)))
        self.r = _f32(radius)
        self.rdv = _f32(1.0 / np.float64(dot)) if dot != 0 else _f32(np.inf)


Cylinder = Capsule
