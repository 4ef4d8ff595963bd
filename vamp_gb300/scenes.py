"""Seeded synthetic workloads: scenes, configurations and edges.

The reference's own benchmarks run on the MotionBenchMaker problem sets; this module stands in for
them with seeded synthetic inputs of the shapes the benchmarks use.  Primitive fields are
generated directly in the layout of the reference's structs (collision/shapes.hh), so every
implementation that consumes a scene sees identical floats.

Scene dictionaries:
    spheres     float32 [n, 4]   x y z r
    capsules    float32 [n, 8]   x1 y1 z1 xv yv zv r rdv     (rdv = 1 / |v|^2)
    cuboids     float32 [n, 15]  centre, axis_1, axis_2, axis_3, half extents
    pointclouds list of {points float32 [n, 3], r_min, r_max, r_point}
"""
from __future__ import annotations

import numpy as np

# Point radius the reference uses for pointcloud collision checking (src/vamp/constants.py:23).
POINT_RADIUS = 0.0025


def random_rotation(rng: np.random.Generator) -> np.ndarray:
    """Uniform random rotation: a unit quaternion from a normalised 4-D Gaussian."""
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array(
        [
            [1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
            [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
            [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)],
        ]
    )


def _unit(rng: np.random.Generator) -> np.ndarray:
    v = rng.normal(size=3)
    return v / np.linalg.norm(v)


def cuboid_fields(centre, R, half) -> np.ndarray:
    return np.array([*centre, *R[:, 0], *R[:, 1], *R[:, 2], *half], np.float32)


def capsule_fields(p1, p2, radius) -> np.ndarray:
    """Capsule from two endpoints, as factory::cylinder::endpoints::flat builds it
    (collision/factory.hh:112-124): v = p2 - p1 in float, rdv = 1 / (v . v)."""
    p1 = np.asarray(p1, np.float32)
    p2 = np.asarray(p2, np.float32)
    v = (p2 - p1).astype(np.float32)
    dot = float(np.dot(v.astype(np.float64), v.astype(np.float64)))
    return np.array([*p1, *v, radius, np.float32(1.0 / dot)], np.float32)


def _place(rng, placement: str) -> np.ndarray:
    if placement == "cube":
        # a 1.2 m cube standing on the floor around the robot base, keeping a 0.4 m radial
        # clearance around the base column (without it every configuration collides with the
        # fixed base links)
        while True:
            c = rng.uniform([-0.6, -0.6, 0.0], [0.6, 0.6, 1.2])
            if np.hypot(c[0], c[1]) >= 0.4:
                return c
    if placement == "workspace":
        # a 4 m x 4 m x 4 m volume from z = -1 m to z = 3 m around the base, keeping a 0.6 m
        # radial clearance around the base column so that the fixed base links stay free
        while True:
            c = rng.uniform([-2.0, -2.0, -1.0], [2.0, 2.0, 3.0])
            if np.hypot(c[0], c[1]) >= 0.6:
                return c
    raise ValueError(placement)


def primitive_scene(seed: int, n_spheres: int, n_cuboids: int, n_capsules: int, placement: str = "cube") -> dict:
    """Spheres r ~ U[0.05, 0.2]; cuboids with half extents ~ U[0.02, 0.3] and a uniform random
    orientation; capsules r ~ U[0.03, 0.15], length ~ U[0.1, 0.5], random axis."""
    rng = np.random.default_rng(seed)
    spheres = np.array([[*_place(rng, placement), rng.uniform(0.05, 0.2)] for _ in range(n_spheres)], np.float32)
    cuboids = np.array(
        [cuboid_fields(_place(rng, placement), random_rotation(rng), rng.uniform(0.02, 0.3, size=3)) for _ in range(n_cuboids)],
        np.float32,
    )
    caps = []
    for _ in range(n_capsules):
        c = _place(rng, placement)
        r = rng.uniform(0.03, 0.15)
        half = 0.5 * rng.uniform(0.1, 0.5)
        a = _unit(rng)
        caps.append(capsule_fields(c - half * a, c + half * a, r))
    return {
        "spheres": spheres.reshape(-1, 4),
        "cuboids": cuboids.reshape(-1, 15),
        "capsules": np.array(caps, np.float32).reshape(-1, 8),
        "pointclouds": [],
    }


def surface_pointcloud(seed: int, n_points: int = 50_000, n_shapes: int = 30, noise: float = 0.02,
                       placement: str = "workspace") -> np.ndarray:
    """Points sampled on the surfaces of random cuboids and cylinders (area-weighted), plus a
    fraction `noise` of points uniform in the placement volume."""
    rng = np.random.default_rng(seed)
    shapes = []
    for i in range(n_shapes):
        c = _place(rng, placement)
        R = random_rotation(rng)
        if i % 2 == 0:
            h = rng.uniform(0.02, 0.3, size=3)
            areas = 8 * np.array([h[1] * h[2], h[0] * h[2], h[0] * h[1]])
            shapes.append(("box", c, R, h, areas.sum(), areas))
        else:
            r = rng.uniform(0.03, 0.15)
            L = rng.uniform(0.1, 0.5)
            areas = np.array([2 * np.pi * r * L, 2 * np.pi * r * r])
            shapes.append(("cyl", c, R, (r, L), areas.sum(), areas))
    total = np.array([s[4] for s in shapes])
    n_noise = int(round(noise * n_points))
    n_surf = n_points - n_noise
    counts = rng.multinomial(n_surf, total / total.sum())
    pts = []
    for (kind, c, R, h, _, areas), k in zip(shapes, counts):
        if k == 0:
            continue
        if kind == "box":
            face = rng.choice(3, size=k, p=areas / areas.sum())
            sign = rng.choice([-1.0, 1.0], size=k)
            local = rng.uniform(-1, 1, size=(k, 3)) * h
            local[np.arange(k), face] = sign * h[face]
        else:
            r, L = h
            side = rng.random(k) < areas[0] / areas.sum()
            th = rng.uniform(0, 2 * np.pi, size=k)
            rad = np.where(side, r, r * np.sqrt(rng.random(k)))
            z = np.where(side, rng.uniform(-L / 2, L / 2, size=k), rng.choice([-L / 2, L / 2], size=k))
            local = np.stack([rad * np.cos(th), rad * np.sin(th), z], axis=1)
        pts.append(local @ R.T + c)
    for _ in range(n_noise):
        pts.append(_place(rng, placement)[None, :])
    out = np.concatenate(pts, axis=0).astype(np.float32)
    rng.shuffle(out)
    return out


def pointcloud_scene(seed: int, r_min: float, r_max: float, n_points: int = 50_000) -> dict:
    return {
        "spheres": np.zeros((0, 4), np.float32),
        "cuboids": np.zeros((0, 15), np.float32),
        "capsules": np.zeros((0, 8), np.float32),
        "pointclouds": [
            {"points": surface_pointcloud(seed, n_points), "r_min": r_min, "r_max": r_max, "r_point": POINT_RADIUS}
        ],
    }


def heightfield(seed: int, xd: int = 96, yd: int = 80, centre=(0.2, 0.0, -0.15), scale=(0.025, 0.03, 3.0)) -> dict:
    """A terrain for the heightfield primitive: smooth random bumps in [0, 1] on an xd x yd grid
    (row-major as the reference's png_to_heightfield flattens an image), placed at `centre`.  As
    in the reference's factory, `scale` holds the cell sizes in x and y and the divisor of the
    heights in z (height = value / scale_z + centre_z)."""
    rng = np.random.default_rng(seed)
    gx, gy = np.meshgrid(np.arange(xd), np.arange(yd), indexing="ij")
    h = np.zeros((xd, yd))
    for _ in range(12):
        cx, cy = rng.uniform(0, xd), rng.uniform(0, yd)
        w = rng.uniform(4, 15)
        h += rng.uniform(0.2, 1.0) * np.exp(-((gx - cx) ** 2 + (gy - cy) ** 2) / (2 * w * w))
    h = (h / h.max()).astype(np.float32)
    return {"centre": np.asarray(centre, np.float32), "scale": np.asarray(scale, np.float32), "xd": xd, "yd": yd,
            "data": h.reshape(-1)}


def configurations(s_m, s_a, n: int, seed: int) -> np.ndarray:
    """n configurations uniform within the joint limits: q = u * s_m + s_a, u ~ U[0, 1)^dim
    (the reference's scale_configuration, robots/panda.hh:77-80)."""
    rng = np.random.default_rng(seed)
    u = rng.random((n, len(s_m)), dtype=np.float32)
    return (u * np.asarray(s_m, np.float32) + np.asarray(s_a, np.float32)).astype(np.float32)


def edges(s_m, s_a, n: int, seed: int):
    """n straight-line edges with both endpoints uniform within the joint limits."""
    a = configurations(s_m, s_a, n, seed)
    b = configurations(s_m, s_a, n, seed + 7919)
    return a, b


# Workloads of the benchmark configurations -------------------------------------------------------

def scene_config0(seed: int = 0) -> dict:
    """Config 0: 8 spheres, 8 cuboids, 4 capsules in a 1.2 m cube around the base (about 25-50%
    of uniform Panda configurations are valid)."""
    return primitive_scene(seed, 8, 8, 4, "cube")


def scene_config1(seed: int = 1) -> dict:
    """Config 1: 24 spheres, 24 cuboids, 12 capsules placed in the 4 m workspace volume."""
    return primitive_scene(seed, 24, 24, 12, "workspace")


# The seeded inputs of the benchmark configurations at full size (one definition, shared by the
# benchmark, the tests and the fixture generator).

def workload_config0(s_m, s_a):
    """Config 0: the config-0 scene and 4,096 configurations uniform within the joint limits."""
    return scene_config0(0), configurations(s_m, s_a, 4096, 4096)


def workload_config1(s_m, s_a):
    """Config 1: the config-1 scene (seed 1) and 65,536 edges with endpoints uniform within the
    joint limits (seed 2024); checked at resolution 32."""
    a, b = edges(s_m, s_a, 65536, 2024)
    return scene_config1(1), a, b


def workload_config2(s_m, s_a, r_min: float, r_max: float):
    """Config 2: 50,000 points on the surfaces of 30 cuboids and capsules plus 2 % noise (seed 1),
    whose tree is built with the robot's sphere radius range; 1,048,576 configurations (seed 77)
    and 16,384 edges (seed 78) at resolution 32."""
    pts = surface_pointcloud(1, 50_000)
    scene = {"pointclouds": [{"points": pts, "r_min": r_min, "r_max": r_max, "r_point": POINT_RADIUS}]}
    q = configurations(s_m, s_a, 1 << 20, 77)
    a, b = edges(s_m, s_a, 16384, 78)
    return scene, q, a, b


def input_digest(*arrays) -> str:
    """SHA-256 of the arrays' float32 bytes, in order: fixtures of the reference's verdicts on the
    workloads above record it, so that a change of the seeded generator is caught instead of
    comparing verdicts of different inputs."""
    import hashlib

    h = hashlib.sha256()
    for x in arrays:
        h.update(np.ascontiguousarray(x, np.float32).tobytes())
    return h.hexdigest()
