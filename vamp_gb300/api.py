"""The Python API of vamp_gb300 (loaded on first use by the package).

The Python surface mirrors the reference's bindings (src/impl/vamp/bindings/robot_helper.hh and
environment.cc): an `Environment` built from primitives, and one submodule per robot with
`validate`, `validate_motion`, `fk`, `min_max_radii`, `dimension`, `resolution`.  Batched
forms (`validate_batch`, `validate_motion_batch`) check many configurations or edges in one GPU
launch; they accept numpy arrays (host) or CUDA torch tensors (device, current stream).
"""
from __future__ import annotations

import ctypes

import numpy as np

from ._lib import SQRT_EXACT, SQRT_X86, VampError, check, lib

__all__ = [
    "Environment",
    "Robot",
    "VampError",
    "SQRT_X86",
    "SQRT_EXACT",
    "panda",
    "ur5",
    "fetch",
    "baxter",
    "ROBOTS",
]

_p = ctypes.c_void_p


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(_p)


class Environment:
    """collision::Environment<float> (src/impl/vamp/collision/environment.hh:15-85).

    Primitive fields follow the reference structs (collision/shapes.hh):
      sphere  x y z r
      capsule x1 y1 z1 xv yv zv r rdv   (rdv = 1 / (v . v))
      cuboid  centre, axis_1, axis_2, axis_3, half extents (15 floats)
    Objects are kept sorted by their distance to the origin, as the reference sorts them.
    """

    KINDS = ("spheres", "capsules", "z_aligned_capsules", "cuboids", "z_aligned_cuboids")

    def __init__(self, lanes: int = 8, sqrt_mode: int = SQRT_X86):
        self._h = lib.vg_env_create()
        if not self._h:
            raise VampError("vg_env_create failed")
        self.set_mode(lanes, sqrt_mode)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib.vg_env_destroy(h)
            self._h = None

    @property
    def handle(self):
        return self._h

    def set_mode(self, lanes: int, sqrt_mode: int) -> None:
        """Which reference build to reproduce: (8, SQRT_X86) for AVX2, (4, SQRT_EXACT) for NEON."""
        check(lib.vg_env_set_mode(self._h, lanes, sqrt_mode))
        self.lanes, self.sqrt_mode = lanes, sqrt_mode

    def set_schedule(self, schedule: int) -> None:
        """GPU edge schedule: 1 a warp per edge, 0 a lane-block per edge, 2 a warp per edge with
        the register-rich build, 3 as 2 with the segments an edge leaves free starting on the
        next edge, -1 (default) each robot's own (2 for the Panda, UR5 and Fetch, 1 for Baxter).
        Verdicts and block counts are the same in every schedule."""
        check(lib.vg_env_set_schedule(self._h, schedule))

    def add_sphere(self, sphere) -> None:
        f = np.ascontiguousarray(_fields(sphere, ("x", "y", "z", "r")), np.float32)
        check(lib.vg_env_add_sphere(self._h, _ptr(f)))

    def add_capsule(self, capsule) -> None:
        f = np.ascontiguousarray(_fields(capsule, ("x1", "y1", "z1", "xv", "yv", "zv", "r", "rdv")), np.float32)
        check(lib.vg_env_add_capsule(self._h, _ptr(f)))

    add_cylinder = add_capsule

    def add_cuboid(self, cuboid) -> None:
        names = ("x", "y", "z", "axis_1_x", "axis_1_y", "axis_1_z", "axis_2_x", "axis_2_y", "axis_2_z",
                 "axis_3_x", "axis_3_y", "axis_3_z", "axis_1_r", "axis_2_r", "axis_3_r")
        f = np.ascontiguousarray(_fields(cuboid, names), np.float32)
        check(lib.vg_env_add_cuboid(self._h, _ptr(f)))

    @classmethod
    def from_scene(cls, scene: dict, lanes: int = 8, sqrt_mode: int = SQRT_X86) -> "Environment":
        env = cls(lanes, sqrt_mode)
        for s in np.asarray(scene.get("spheres", np.zeros((0, 4))), np.float32):
            env.add_sphere(s)
        for c in np.asarray(scene.get("capsules", np.zeros((0, 8))), np.float32):
            env.add_capsule(c)
        for c in np.asarray(scene.get("cuboids", np.zeros((0, 15))), np.float32):
            env.add_cuboid(c)
        for pc in scene.get("pointclouds", []):
            env.add_pointcloud(pc["points"], pc["r_min"], pc["r_max"], pc["r_point"])
        for hf in scene.get("heightfields", []):
            env.add_heightfield(HeightField(hf["centre"], hf["scale"], (hf["xd"], hf["yd"]), hf["data"]))
        if scene.get("attachment") is not None:
            a = Attachment(scene["attachment"]["tf"])
            a.add_spheres(np.asarray(scene["attachment"]["spheres"], np.float32).reshape(-1, 4))
            env.attach(a)
        return env

    def add_pointcloud(self, points, r_min: float, r_max: float, r_point: float) -> int:
        """A pointcloud checked as a CAPT (collision/capt.hh), built on the host.  Returns the build
        time in nanoseconds, as the reference's binding does (bindings/environment.cc:150-161)."""
        import time

        pts = np.ascontiguousarray(points, np.float32).reshape(-1, 3)
        t0 = time.perf_counter_ns()
        check(lib.vg_env_add_pointcloud(self._h, _ptr(pts), len(pts), float(r_min), float(r_max), float(r_point)))
        return time.perf_counter_ns() - t0

    def add_pointcloud_device(self, points, r_min: float, r_max: float, r_point: float) -> None:
        """The same CAPT built on the GPU from a CUDA tensor of points [n, 3] (float32); the layout
        is bit-identical to add_pointcloud's."""
        import torch

        if not (isinstance(points, torch.Tensor) and points.is_cuda):
            raise ValueError("add_pointcloud_device takes a CUDA tensor")
        pts = points.detach().to(torch.float32).reshape(-1, 3).contiguous()
        with torch.cuda.device(pts.device):
            check(lib.vg_env_add_pointcloud_device(self._h, pts.data_ptr(), pts.shape[0], float(r_min), float(r_max),
                                                   float(r_point), _stream(pts)))

    def add_heightfield(self, heightfield: "HeightField") -> None:
        """Environment.add_heightfield (bindings/environment.cc:146-149)."""
        h = heightfield
        c, sc = (np.ascontiguousarray(v, np.float32).reshape(3) for v in (h.centre, h.scale))
        data = np.ascontiguousarray(h.data, np.float32).reshape(-1)
        xd, yd = (int(v) for v in h.dimensions)
        if data.size != xd * yd:
            raise ValueError("heightfield data must hold dimensions[0] * dimensions[1] samples")
        check(lib.vg_env_add_heightfield(self._h, _ptr(c), _ptr(sc), xd, yd, _ptr(data)))

    def attach(self, attachment: "Attachment") -> None:
        """Attach spheres to the end effector (Environment.attach, bindings/environment.cc:162-164):
        a copy of the attachment; every later check runs fkcc_attach."""
        tf = np.ascontiguousarray(attachment.relative_frame, np.float32).reshape(16)
        sph = np.ascontiguousarray(attachment.spheres, np.float32).reshape(-1, 4)
        check(lib.vg_env_attach(self._h, _ptr(tf), _ptr(sph), len(sph)))

    def detach(self) -> None:
        check(lib.vg_env_detach(self._h))

    def pointcloud_layout(self, index: int = 0) -> dict:
        sizes = np.zeros(4, np.uint64)
        nul = ctypes.c_void_p()
        check(lib.vg_env_pointcloud_layout(self._h, index, _ptr(sizes), nul, nul, nul, nul, nul))
        nlog2, nt, nl, nb = (int(v) for v in sizes)
        out = dict(nlog2=nlog2, tests=np.zeros(nt, np.float32), aabbs=np.zeros((nl, 6), np.float32),
                   aff_starts=np.zeros(nl + 1, np.uint32), aff=np.zeros((nb, 3, 8), np.float32), top=np.zeros(6, np.float32))
        check(lib.vg_env_pointcloud_layout(self._h, index, _ptr(sizes), _ptr(out["tests"]), _ptr(out["aabbs"]),
                                           _ptr(out["aff_starts"]), _ptr(out["aff"]), _ptr(out["top"])))
        out["aff"] = out["aff"].transpose(1, 0, 2).copy()  # [3][blocks][8], as the oracle dumps it
        return out

    def add_primitive(self, kind: int, fields, min_distance: float) -> None:
        """One object in an explicit kind list (0 spheres, 1 capsules, 2 z-aligned capsules,
        3 cuboids, 4 z-aligned cuboids) with the caller's min_distance: for environments converted
        from the reference's collision::Environment, whose objects already sit in their lists."""
        f = np.ascontiguousarray(fields, np.float32).reshape(-1)
        if f.size != [4, 8, 8, 15, 15][kind]:
            raise ValueError("wrong number of fields for this kind")
        check(lib.vg_env_add_primitive(self._h, int(kind), _ptr(f), float(min_distance)))

    def add_pointcloud_layout(self, layout: dict) -> None:
        """A pointcloud tree as the reference built it, in the layout pointcloud_layout returns
        (nlog2, tests, aabbs, aff_starts, aff [3][blocks][8], top, radii = r_min, r_max, r_point)."""
        aff = np.ascontiguousarray(np.asarray(layout["aff"], np.float32).transpose(1, 0, 2))  # [blocks][3][8]
        arr = {k: np.ascontiguousarray(layout[k], np.float32) for k in ("tests", "aabbs", "top")}
        starts = np.ascontiguousarray(layout["aff_starts"], np.uint32)
        r = [float(v) for v in layout["radii"]]
        check(lib.vg_env_add_pointcloud_layout(self._h, int(layout["nlog2"]), _ptr(arr["tests"]), _ptr(arr["aabbs"]),
                                               _ptr(starts), _ptr(aff), aff.shape[0], _ptr(arr["top"]), *r))

    def objects(self, kind: int) -> np.ndarray:
        """Fields of every object of a kind in checking order, min_distance last."""
        n = ctypes.c_size_t()
        check(lib.vg_env_count(self._h, kind, ctypes.byref(n)))
        width = [5, 9, 9, 16, 16][kind]
        out = np.zeros((n.value, width), np.float32)
        for i in range(n.value):
            check(lib.vg_env_get(self._h, kind, i, _ptr(out[i])))
        return out


def _fields(obj, names):
    if hasattr(obj, names[0]):
        return [getattr(obj, n) for n in names]
    a = np.asarray(obj, np.float32).reshape(-1)
    if a.size != len(names):
        raise ValueError(f"expected {len(names)} fields, got {a.size}")
    return a


def _is_cuda_tensor(x) -> bool:
    return type(x).__module__.startswith("torch") and getattr(x, "is_cuda", False)


class Robot:
    """One robot's entry points, mirroring the reference's per-robot Python submodule
    (bindings/robot_helper.hh:349-648)."""

    def __init__(self, name: str):
        self.name = name
        self._b = name.encode()
        d, n, rmin, rmax, res = ctypes.c_int(), ctypes.c_int(), ctypes.c_float(), ctypes.c_float(), ctypes.c_int()
        check(lib.vg_robot_info(self._b, ctypes.byref(d), ctypes.byref(n), ctypes.byref(rmin), ctypes.byref(rmax), ctypes.byref(res)))
        self._dim, self._n, self._rmin, self._rmax, self._res = d.value, n.value, rmin.value, rmax.value, res.value
        self.s_m = np.zeros(self._dim, np.float32)
        self.s_a = np.zeros(self._dim, np.float32)
        check(lib.vg_robot_limits(self._b, _ptr(self.s_m), _ptr(self.s_a)))

    # constants ---------------------------------------------------------------------------
    def dimension(self) -> int:
        return self._dim

    def n_spheres(self) -> int:
        return self._n

    def resolution(self) -> int:
        return self._res

    def min_max_radii(self) -> tuple:
        return self._rmin, self._rmax

    def scale_configuration(self, u):
        return (np.asarray(u, np.float32) * self.s_m + self.s_a).astype(np.float32)

    def descale_configuration(self, q):
        return ((np.asarray(q, np.float32) - self.s_a) / self.s_m).astype(np.float32)

    def _in_bounds(self, q) -> bool:
        u = self.descale_configuration(q)
        return bool(np.all(u <= 1.0) and np.all(u >= 0.0))

    # single checks (reference semantics) ---------------------------------------------------
    def validate(self, configuration, environment: Environment, check_bounds: bool = False) -> bool:
        """Robot validity of one configuration (bindings/robot_helper.hh:256-267)."""
        q = np.ascontiguousarray(configuration, np.float32).reshape(1, self._dim)
        if check_bounds and not self._in_bounds(q[0]):
            return False
        return bool(self.validate_batch(q, environment)[0])

    def validate_motion(self, configuration_in, configuration_out, environment: Environment,
                        check_bounds: bool = True, resolution: int = 1) -> bool:
        """Straight-line motion validity (bindings/robot_helper.hh:269-290).  The Python binding
        of the reference checks at resolution 1; planners use the robot's resolution()."""
        a = np.ascontiguousarray(configuration_in, np.float32).reshape(1, self._dim)
        b = np.ascontiguousarray(configuration_out, np.float32).reshape(1, self._dim)
        if check_bounds and not (self._in_bounds(a[0]) and self._in_bounds(b[0])):
            return False
        return bool(self.validate_motion_batch(a, b, environment, resolution)[0])

    def filter_self_from_pointcloud(self, pc, point_radius: float, configuration, environment: Environment | None = None):
        """The points of pc (spheres of point_radius) that collide neither with the robot at
        `configuration` nor with the environment, in order (bindings/robot_helper.hh:307-345).
        pc: host array [n, 3] (returns an array) or CUDA tensor (returns a tensor)."""
        env = environment if environment is not None else Environment()
        q = np.ascontiguousarray(configuration, np.float32).reshape(self._dim)
        m = ctypes.c_size_t()
        if _is_cuda_tensor(pc):
            import torch

            pts = pc.detach().to(torch.float32).reshape(-1, 3).contiguous()
            out = torch.empty_like(pts)
            with torch.cuda.device(pts.device):
                check(lib.vg_filter_self_from_pointcloud_device(self._b, env.handle, pts.data_ptr(), pts.shape[0],
                                                                float(point_radius), _ptr(q), out.data_ptr(),
                                                                ctypes.byref(m), _stream(pts)))
            return out[: m.value]
        pts = np.ascontiguousarray(pc, np.float32).reshape(-1, 3)
        out = np.zeros_like(pts)
        check(lib.vg_filter_self_from_pointcloud(self._b, env.handle, _ptr(pts), len(pts), float(point_radius), _ptr(q),
                                                 _ptr(out), ctypes.byref(m)))
        return out[: m.value].copy()

    def eefk(self, configuration) -> np.ndarray:
        """End-effector transform, a row-major 4x4 float32 matrix (Robot::eefk; binding
        robot_helper.hh:302-305)."""
        q = np.ascontiguousarray(configuration, np.float32).reshape(-1, self._dim)
        out = np.zeros((len(q), 4, 4), np.float32)
        check(lib.vg_eefk(self._b, _ptr(q), len(q), _ptr(out)))
        return out[0] if np.ndim(configuration) == 1 else out

    def fk(self, configuration) -> np.ndarray:
        """Fine sphere centres and radii [n_spheres, 4] (Robot::sphere_fk)."""
        return self.fk_slots(np.asarray(configuration, np.float32).reshape(1, self._dim))[0, : self._n]

    # batched checks -----------------------------------------------------------------------
    def validate_batch(self, configurations, environment: Environment, out=None):
        """Validity of every configuration; numpy in -> numpy uint8 out, CUDA tensor in -> CUDA
        uint8 tensor out (asynchronous on the current stream)."""
        if _is_cuda_tensor(configurations):
            import torch

            q = configurations.contiguous()
            n = q.shape[0]
            out = torch.empty(n, dtype=torch.uint8, device=q.device) if out is None else out
            check(lib.vg_validate_states_device(self._b, environment.handle, q.data_ptr(), n, out.data_ptr(),
                                                torch.cuda.current_stream(q.device).cuda_stream))
            return out
        q = np.ascontiguousarray(configurations, np.float32).reshape(-1, self._dim)
        out = np.zeros(len(q), np.uint8) if out is None else out
        check(lib.vg_validate_states(self._b, environment.handle, _ptr(q), len(q), _ptr(out)))
        return out

    def fkcc_blocks(self, blocks, environment: Environment):
        """Robot::fkcc (robots/panda.hh:5226-5229) on configuration blocks [n][lanes][dim] (lanes
        the environment's: 8 or 4) with the reference's block semantics: 1 = the block is valid.
        numpy in -> numpy out; CUDA tensor in -> CUDA tensor out (current stream)."""
        if _is_cuda_tensor(blocks):
            import torch

            q = blocks.contiguous()
            out = torch.empty(q.shape[0], dtype=torch.uint8, device=q.device)
            check(lib.vg_fkcc_blocks_device(self._b, environment.handle, q.data_ptr(), q.shape[0], out.data_ptr(),
                                            torch.cuda.current_stream(q.device).cuda_stream))
            return out
        q = np.ascontiguousarray(blocks, np.float32).reshape(-1, environment.lanes, self._dim)
        out = np.zeros(len(q), np.uint8)
        check(lib.vg_fkcc_blocks(self._b, environment.handle, _ptr(q), len(q), _ptr(out)))
        return out

    def validate_motion_batch(self, starts, goals, environment: Environment, resolution: int | None = None,
                              out=None, blocks=None):
        """Validity of every edge starts[i] -> goals[i] at `resolution` (default: the robot's)."""
        res = self._res if resolution is None else int(resolution)
        if _is_cuda_tensor(starts):
            import torch

            a, b = starts.contiguous(), goals.contiguous()
            n = a.shape[0]
            out = torch.empty(n, dtype=torch.uint8, device=a.device) if out is None else out
            bp = blocks.data_ptr() if blocks is not None else None
            check(lib.vg_validate_motions_device(self._b, environment.handle, a.data_ptr(), b.data_ptr(), n, res,
                                                 out.data_ptr(), bp, torch.cuda.current_stream(a.device).cuda_stream))
            return out
        a = np.ascontiguousarray(starts, np.float32).reshape(-1, self._dim)
        b = np.ascontiguousarray(goals, np.float32).reshape(-1, self._dim)
        out = np.zeros(len(a), np.uint8) if out is None else out
        check(lib.vg_validate_motions(self._b, environment.handle, _ptr(a), _ptr(b), len(a), res, _ptr(out)))
        return out

    def validate_vector_batch(self, starts, vectors, distances, environment: Environment, resolution: int | None = None,
                              out=None, blocks=None):
        """validate_vector (planning/validate.hh:23-63) for every edge: from starts[i] along
        vectors[i], checked in max(ceil(distances[i] / lanes * resolution), 1) blocks, distances[i]
        being the length the caller gives (the reference's planners pass their extension
        length)."""
        res = self._res if resolution is None else int(resolution)
        if _is_cuda_tensor(starts):
            import torch

            a, v, d = starts.contiguous(), vectors.contiguous(), distances.to(torch.float32).contiguous()
            n = a.shape[0]
            out = torch.empty(n, dtype=torch.uint8, device=a.device) if out is None else out
            bp = blocks.data_ptr() if blocks is not None else None
            check(lib.vg_validate_vectors_device(self._b, environment.handle, a.data_ptr(), v.data_ptr(), d.data_ptr(), n,
                                                 res, out.data_ptr(), bp, torch.cuda.current_stream(a.device).cuda_stream))
            return out
        a = np.ascontiguousarray(starts, np.float32).reshape(-1, self._dim)
        v = np.ascontiguousarray(vectors, np.float32).reshape(-1, self._dim)
        d = np.ascontiguousarray(distances, np.float32).reshape(-1)
        out = np.zeros(len(a), np.uint8) if out is None else out
        check(lib.vg_validate_vectors(self._b, environment.handle, _ptr(a), _ptr(v), _ptr(d), len(a), res, _ptr(out)))
        return out

    def debug(self, configuration, environment: Environment):
        """Which objects each fine sphere collides with and which fine self pairs collide, for one
        configuration (the reference binding's debug(), bindings/robot_helper.hh:249-253): a list
        per fine sphere of object insertion indices (the reference lists object names), and the
        colliding fine pairs (i, j)."""
        bits, pairs = self.debug_batch(np.asarray(configuration, np.float32).reshape(1, self._dim), environment)
        objs = [[w * 32 + b for w in range(bits.shape[2]) for b in range(32) if (int(bits[0, i, w]) >> b) & 1]
                for i in range(bits.shape[1])]
        from .robots import model

        order = [tuple(p) for e in model(self.name)["self_checks"] for p in e["fine"]]
        return objs, [order[k] for k in np.nonzero(pairs[0])[0]]

    def debug_batch(self, configurations, environment: Environment):
        """Debug reports of many configurations: (bits [n][fine][words] uint32 over object
        insertion indices, pair flags [n][self pairs] uint8 in the order of the self checks)."""
        fine, words, npairs = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        check(lib.vg_debug_sizes(self._b, environment.handle, ctypes.byref(fine), ctypes.byref(words), ctypes.byref(npairs)))
        if _is_cuda_tensor(configurations):
            import torch

            q = configurations.contiguous()
            n = q.shape[0]
            bits = torch.empty((n, fine.value, words.value), dtype=torch.int32, device=q.device)
            pairs = torch.empty((n, npairs.value), dtype=torch.uint8, device=q.device)
            check(lib.vg_debug_device(self._b, environment.handle, q.data_ptr(), n, bits.data_ptr(), pairs.data_ptr(),
                                      torch.cuda.current_stream(q.device).cuda_stream))
            return bits, pairs
        q = np.ascontiguousarray(configurations, np.float32).reshape(-1, self._dim)
        bits = np.zeros((len(q), fine.value, words.value), np.uint32)
        pairs = np.zeros((len(q), npairs.value), np.uint8)
        check(lib.vg_debug(self._b, environment.handle, _ptr(q), len(q), _ptr(bits), _ptr(pairs)))
        return bits, pairs

    def fk_slots(self, configurations) -> np.ndarray:
        """Every sphere slot (fine spheres, then each checked link's coarse sphere) [n, slots, 4]."""
        q = np.ascontiguousarray(configurations, np.float32).reshape(-1, self._dim)
        slots = self._slots()
        out = np.zeros((len(q), slots, 4), np.float32)
        check(lib.vg_sphere_fk(self._b, _ptr(q), len(q), _ptr(out)))
        return out

    def _slots(self) -> int:
        from .robots import slot_count

        return slot_count(self.name)


ROBOTS = ("panda", "ur5", "fetch", "baxter")
panda = Robot("panda")
ur5 = Robot("ur5")
fetch = Robot("fetch")
baxter = Robot("baxter")


# ------------------------------------------------------------------ autotuning, batches, learning
# None of these has a counterpart in the reference's bindings; they wrap the C ABI's batch,
# autotuner and learned-ordering entry points (include/vamp_gb300.h).  Device buffers are torch
# CUDA tensors; calls run on the current stream.

SCHEDULES = ("segment per edge", "warp per edge", "warp per edge, register-rich build",
             "warp per edge, register-rich build, free segments start the next edge")


def _stream(t):
    import torch

    return torch.cuda.current_stream(t.device).cuda_stream


class HeightField:
    """A heightfield (collision/shapes.hh:250-311): samples data[y * xd + x] for dimensions
    (xd, yd), placed at `centre`; scale holds the cell sizes in x and y and the divisor of the
    samples in z (as the reference's make_heightfield takes them)."""

    def __init__(self, centre, scale, dimensions, data):
        self.centre = np.asarray(centre, np.float32).reshape(3)
        self.scale = np.asarray(scale, np.float32).reshape(3)
        self.dimensions = (int(dimensions[0]), int(dimensions[1]))
        self.data = np.asarray(data, np.float32).reshape(-1)


def make_heightfield(center, scale, dimensions, data) -> HeightField:
    """make_heightfield (bindings/environment.cc:98; collision/factory.hh:406-422)."""
    return HeightField(center, scale, dimensions, data)


def array_to_heightfield(array, center, scaling) -> HeightField:
    """png_to_heightfield (src/vamp/__init__.py:54-66) after the image is decoded: a grey image
    [rows, cols] of 0..255, scaled to [0, 1] and flipped upside down."""
    a = np.flip(np.asarray(array, np.float64) * 1 / 255.0, axis=0)
    return make_heightfield(center, scaling, a.shape, a.reshape(-1))


class Attachment:
    """Spheres carried by the end effector (collision/attachments.hh:11-56; the binding
    vamp.Attachment, bindings/environment.cc:200-230): a relative frame (4x4 transform from the
    end effector) and spheres [x, y, z, r] in that frame.  Environment.attach copies it."""

    def __init__(self, tf):
        self.relative_frame = np.array(tf, np.float32).reshape(4, 4)
        self.spheres = np.zeros((0, 4), np.float32)
        self.posed_spheres = np.zeros((0, 4), np.float32)

    def add_sphere(self, sphere) -> None:
        self.add_spheres([sphere])

    def add_spheres(self, spheres) -> None:
        rows = [np.asarray(_fields(s, ("x", "y", "z", "r")), np.float32).reshape(4) for s in spheres]
        self.spheres = np.concatenate([self.spheres, np.array(rows, np.float32).reshape(-1, 4)])

    def set_ee_pose(self, tf) -> None:
        """posed_spheres at the end-effector transform tf (Attachment::pose; for display: the
        checks pose the spheres on the GPU)."""
        T = np.asarray(tf, np.float64).reshape(4, 4) @ self.relative_frame.astype(np.float64)
        c = self.spheres[:, :3].astype(np.float64) @ T[:3, :3].T + T[:3, 3]
        self.posed_spheres = np.concatenate([c, self.spheres[:, 3:4]], axis=1).astype(np.float32)


def filter_pointcloud(pc, min_dist: float, max_range: float, origin, workcell_min, workcell_max, cull: bool):
    """The reference's filter_pointcloud (collision/filter.hh:176-320; binding
    bindings/environment.cc:167-197), run on the GPU: returns (kept points [m, 3] float32, elapsed
    nanoseconds).  pc is an [n, 3] array or list of points in host memory."""
    pts = np.ascontiguousarray(pc, np.float32).reshape(-1, 3)
    out = np.zeros_like(pts)
    o, lo, hi = (np.ascontiguousarray(v, np.float32).reshape(3) for v in (origin, workcell_min, workcell_max))
    m = ctypes.c_size_t()
    ns = ctypes.c_uint64()
    check(lib.vg_filter_pointcloud(_ptr(pts), len(pts), float(min_dist), float(max_range), _ptr(o), _ptr(lo), _ptr(hi),
                                   int(bool(cull)), _ptr(out), ctypes.byref(m), ctypes.byref(ns)))
    return out[: m.value].copy(), ns.value


def filter_pointcloud_device(points, min_dist: float, max_range: float, origin, workcell_min, workcell_max,
                             cull: bool):
    """filter_pointcloud on a CUDA tensor of points [n, 3] (float32): the kept points as a CUDA
    tensor [m, 3], on the current stream."""
    import torch

    if not (isinstance(points, torch.Tensor) and points.is_cuda):
        raise ValueError("filter_pointcloud_device takes a CUDA tensor")
    pts = points.detach().to(torch.float32).reshape(-1, 3).contiguous()
    out = torch.empty_like(pts)
    o, lo, hi = (np.ascontiguousarray(v, np.float32).reshape(3) for v in (origin, workcell_min, workcell_max))
    m = ctypes.c_size_t()
    with torch.cuda.device(pts.device):
        check(lib.vg_filter_pointcloud_device(pts.data_ptr(), pts.shape[0], float(min_dist), float(max_range), _ptr(o),
                                              _ptr(lo), _ptr(hi), int(bool(cull)), out.data_ptr(), ctypes.byref(m),
                                              _stream(pts)))
    return out[: m.value]


def autotune(robot: Robot, environment: Environment, starts, goals, resolution: int | None = None) -> dict:
    """Times the edge-check schedules on these edges (CUDA tensors: a sample of the workload,
    best of the workload's own size) and keeps the fastest for this robot in `environment`."""
    res = robot.resolution() if resolution is None else int(resolution)
    a, b = starts.contiguous(), goals.contiguous()
    sched, bps, ms = ctypes.c_int(), ctypes.c_int(), ctypes.c_float()
    check(lib.vg_autotune_motions(robot.name.encode(), environment.handle, a.data_ptr(), b.data_ptr(), a.shape[0], res,
                                  ctypes.byref(sched), ctypes.byref(bps), ctypes.byref(ms), _stream(a)))
    return {"schedule": SCHEDULES[sched.value], "blocks_per_sm": bps.value or None, "ms": ms.value}


class CollisionPredictor:
    """The learned block ordering's network for one robot: sin/cos features -> 256 -> 256 -> 1,
    BF16 weights, FP32 accumulation, trained on the GPU (tcgen05 kernels) on exact verdicts."""

    def __init__(self, robot: Robot, seed: int = 0):
        self.robot = robot
        self._h = lib.vg_mlp_create(robot.dimension(), seed)
        if not self._h:
            check(-1)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib.vg_mlp_destroy(h)
            self._h = None

    @property
    def handle(self):
        return self._h

    def train(self, configurations, valid, epochs: int = 3, batch: int = 1024, lr: float = 1e-3) -> np.ndarray:
        """Adam on (configurations [n][dim] float32, valid [n] uint8: 1 = collision free) CUDA
        tensors; returns the mean loss of each epoch."""
        q, v = configurations.contiguous(), valid.contiguous()
        losses = np.zeros(epochs, np.float32)
        check(lib.vg_mlp_train_device(self._h, q.data_ptr(), v.data_ptr(), q.shape[0], epochs, batch, float(lr),
                                      _ptr(losses), _stream(q)))
        return losses

    def train_on_environment(self, environment: Environment, n: int = 1 << 21, epochs: int = 3, seed: int = 1):
        """Labels n uniform configurations with the exact checker in `environment`, then trains."""
        import torch

        from . import scenes

        q = torch.from_numpy(scenes.configurations(self.robot.s_m, self.robot.s_a, n, seed)).cuda()
        valid = self.robot.validate_batch(q, environment)
        return self.train(q, valid, epochs)

    def predict(self, configurations):
        """Collision probability per configuration (CUDA tensor in and out; fused inference)."""
        import torch

        q = configurations.contiguous()
        p = torch.empty(q.shape[0], dtype=torch.float32, device=q.device)
        check(lib.vg_mlp_infer_device(self._h, q.data_ptr(), q.shape[0], p.data_ptr(), _stream(q)))
        return p

    def parameters(self) -> np.ndarray:
        out = np.zeros(lib.vg_mlp_param_count(self.robot.dimension()), np.float32)
        check(lib.vg_mlp_get_params(self._h, _ptr(out)))
        return out

    def load_parameters(self, params) -> None:
        p = np.ascontiguousarray(params, np.float32)
        if p.size != lib.vg_mlp_param_count(self.robot.dimension()):
            raise ValueError("parameter count does not match this robot's network")
        check(lib.vg_mlp_set_params(self._h, _ptr(p)))

    def validate_motion_batch(self, starts, goals, environment: Environment, resolution: int | None = None,
                              probes: int = 8, out=None, blocks=None):
        """Edge verdicts (those of Robot.validate_motion_batch) with each edge's blocks checked
        in the order the network ranks them."""
        import torch

        res = self.robot.resolution() if resolution is None else int(resolution)
        a, b = starts.contiguous(), goals.contiguous()
        out = torch.empty(a.shape[0], dtype=torch.uint8, device=a.device) if out is None else out
        bp = blocks.data_ptr() if blocks is not None else None
        check(lib.vg_validate_motions_learned_device(self.robot.name.encode(), environment.handle, self._h, a.data_ptr(),
                                                     b.data_ptr(), a.shape[0], res, probes, out.data_ptr(), bp,
                                                     _stream(a)))
        return out


class Batch:
    """Edge checks of several robots / environments recorded once and replayed as one CUDA graph
    (vg_batch): refill the same tensors, then call launch()."""

    def __init__(self):
        self._h = lib.vg_batch_create()
        self._keep = []  # tensors, environments and predictors the graph refers to

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib.vg_batch_destroy(h)
            self._h = None

    def add(self, robot: Robot, environment: Environment, starts, goals, out, resolution: int | None = None,
            predictor: CollisionPredictor | None = None, probes: int = 8, blocks=None) -> None:
        res = robot.resolution() if resolution is None else int(resolution)
        a, b = starts.contiguous(), goals.contiguous()
        self._keep += [a, b, out, environment, predictor, blocks]
        check(lib.vg_batch_add_motions(self._h, robot.name.encode(), environment.handle, a.data_ptr(), b.data_ptr(),
                                       a.shape[0], res, predictor.handle if predictor else None,
                                       probes if predictor else 0, out.data_ptr(),
                                       blocks.data_ptr() if blocks is not None else None))

    def launch(self, stream=None) -> None:
        import torch

        s = torch.cuda.current_stream().cuda_stream if stream is None else stream
        check(lib.vg_batch_launch(self._h, s))
