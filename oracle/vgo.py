"""ctypes access to the CPU oracle (oracle/port, restated in C) and, where it has been built, to
the compiled reference (oracle/_ref).

Test infrastructure only: imported by tests/, __graft_entry__.smoke() and bench.py's CPU baseline.
The shipped library never imports this module.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
PORT_DIR = HERE / "port"
PORT_LIB = PORT_DIR / "_build" / "libvgo.so"
REF_LIB = HERE / "_ref" / "libvamp_ref.so"

_f = ctypes.c_float
_p = ctypes.c_void_p
_sz = ctypes.c_size_t

KIND_SPHERE, KIND_CAPSULE, KIND_ZCAPSULE, KIND_CUBOID, KIND_ZCUBOID = range(5)
SQRT_X86, SQRT_EXACT = 0, 1


def build_port(force: bool = False) -> Path:
    """Compile the C oracle with make (seconds)."""
    if force or not PORT_LIB.exists():
        subprocess.run(["make", "-s", "-C", str(PORT_DIR)], check=True)
    return PORT_LIB


def reference_checkout(reference: str | None = None) -> Path | None:
    """The reference checkout named by the argument or, failing that, by VG_REFERENCE (None if
    neither names a directory holding the reference's sources)."""
    name = reference or os.environ.get("VG_REFERENCE")
    if not name:
        return None
    ref = Path(name)
    return ref if (ref / "src" / "impl" / "vamp").is_dir() else None


def built_reference_headers() -> Path | None:
    """The reference's src/impl folder the reference oracle was last built from (None if it has
    not been built or the folder is gone)."""
    rec = HERE / "_ref" / "ref_src.txt"
    if not rec.exists():
        return None
    src = Path(rec.read_text().strip())
    return src if (src / "vamp").is_dir() else None


def build_reference(reference: str | None = None) -> Path | None:
    """Compile the reference oracle from the reference checkout (argument or VG_REFERENCE), if
    there is one: its AVX2 backend on x86-64 (8 lanes, the golden fixtures' build), its NEON
    backend on aarch64 (4 lanes)."""
    ref = reference_checkout(reference)
    if ref is None:
        return None
    subprocess.run(
        ["make", "-s", "-j4", "-C", str(HERE / "ref"), f"REF_SRC={ref / 'src' / 'impl'}"], check=True
    )
    return REF_LIB


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(_p)


class _Capt(ctypes.Structure):
    _fields_ = [
        ("nlog2", ctypes.c_int),
        ("n_tests", _sz),
        ("n_leaves", _sz),
        ("tests", ctypes.POINTER(ctypes.c_float)),
        ("aabbs", ctypes.POINTER(ctypes.c_float)),
        ("aff_starts", ctypes.POINTER(ctypes.c_uint32)),
        ("lanes", ctypes.c_int),
        ("n_blocks", _sz),
        ("cap_blocks", _sz),
        ("aff", ctypes.POINTER(ctypes.c_float) * 3),
        ("top", ctypes.c_float * 6),
        ("r_min", ctypes.c_float),
        ("r_max", ctypes.c_float),
        ("r_point", ctypes.c_float),
        ("points", ctypes.POINTER(ctypes.c_float)),
        ("n_points", _sz),
    ]


class Counters(ctypes.Structure):
    _fields_ = [
        ("tests", ctypes.c_uint64 * 5),
        ("capt_queries", ctypes.c_uint64),
        ("self_pairs", ctypes.c_uint64),
        ("sphere_queries", ctypes.c_uint64),
        ("blocks", ctypes.c_uint64),
        ("lanes", ctypes.c_uint64),
    ]


def capt_layout(c: _Capt) -> dict:
    L = c.lanes
    nb = c.n_blocks
    return dict(
        nlog2=c.nlog2,
        tests=np.ctypeslib.as_array(c.tests, (c.n_tests,)).copy(),
        aabbs=np.ctypeslib.as_array(c.aabbs, (c.n_leaves * 6,)).reshape(-1, 6).copy(),
        aff_starts=np.ctypeslib.as_array(c.aff_starts, (c.n_leaves + 1,)).copy(),
        aff=np.stack([np.ctypeslib.as_array(c.aff[k], (nb * L,)).reshape(nb, L).copy() for k in range(3)])
        if nb
        else np.zeros((3, 0, L), np.float32),
        top=np.array(c.top[:], np.float32),
        radii=np.array([c.r_min, c.r_max, c.r_point], np.float32),
    )


class Port:
    """The C oracle."""

    def __init__(self):
        lib = ctypes.CDLL(str(build_port()))
        lib.vgo_env_create.restype = _p
        lib.vgo_env_destroy.argtypes = [_p]
        for n in ("vgo_env_add_sphere", "vgo_env_add_capsule", "vgo_env_add_cuboid"):
            getattr(lib, n).argtypes = [_p, _p]
        lib.vgo_env_add_pointcloud.argtypes = [_p, _p, _sz, _f, _f, _f]
        lib.vgo_env_set_sqrt_mode.argtypes = [_p, ctypes.c_int]
        lib.vgo_env_count.argtypes = [_p, ctypes.c_int]
        lib.vgo_env_count.restype = _sz
        lib.vgo_env_get.argtypes = [_p, ctypes.c_int, _sz, _p]
        lib.vgo_robot_get.restype = _p
        lib.vgo_robot_get.argtypes = [ctypes.c_char_p]
        for n in ("vgo_robot_dim", "vgo_robot_slots", "vgo_robot_fine", "vgo_robot_resolution"):
            getattr(lib, n).argtypes = [_p]
        lib.vgo_robot_limits.argtypes = [_p, _p, _p]
        lib.vgo_robot_spheres_f32.argtypes = [_p, _p, _p]
        lib.vgo_robot_spheres_f64.argtypes = [_p, _p, _p]
        lib.vgo_sphere_env.argtypes = [_p, ctypes.c_int, _p, _p, _p, _p]
        lib.vgo_fkcc.argtypes = [_p, _p, ctypes.c_int, _p]
        lib.vgo_validate_motion.argtypes = [_p, _p, ctypes.c_int, _p, _p, ctypes.c_int, _p]
        lib.vgo_motion_blocks.argtypes = [_p, ctypes.c_int, _p, _p, ctypes.c_int, _p, _sz]
        lib.vgo_motion_blocks.restype = ctypes.c_long
        lib.vgo_motion_block_count.argtypes = [_p, ctypes.c_int, _p, _p, ctypes.c_int]
        lib.vgo_motion_block_count.restype = ctypes.c_long
        lib.vgo_validate_states.argtypes = [_p, _p, _p, _sz, _p, ctypes.c_int]
        lib.vgo_validate_motions.argtypes = [_p, _p, ctypes.c_int, _p, _p, _sz, ctypes.c_int, _p, _p, ctypes.c_int]
        lib.vgo_contact_distance_f64.argtypes = [_p, _p, _p]
        lib.vgo_contact_distance_f64.restype = ctypes.c_double
        lib.vgo_sqrt_x86.argtypes = [_f]
        lib.vgo_sqrt_x86.restype = _f
        lib.vgo_sincos.argtypes = [_f, _p, _p]
        lib.vgo_env_capt.argtypes = [_p, ctypes.c_int]
        lib.vgo_env_capt.restype = ctypes.POINTER(_Capt)
        lib.vgo_capt_build.argtypes = [_p, _sz, _f, _f, _f, ctypes.c_int]
        lib.vgo_capt_build.restype = ctypes.POINTER(_Capt)
        lib.vgo_capt_destroy.argtypes = [ctypes.POINTER(_Capt)]
        lib.vgo_validate_motions_counted.argtypes = [_p, _p, ctypes.c_int, _p, _p, _sz, ctypes.c_int, _p, _p]
        lib.vgo_env_total.argtypes = [_p]
        lib.vgo_robot_self_pairs.argtypes = [_p]
        lib.vgo_debug.argtypes = [_p, _p, _p, _p, ctypes.c_int, _p]
        lib.vgo_env_add_heightfield.argtypes = [_p, _p, _p, ctypes.c_int, ctypes.c_int, _p]
        lib.vgo_filter_self.argtypes = [_p, _p, _p, _sz, _f, _p, _p]
        lib.vgo_filter_self.restype = _sz
        lib.vgo_validate_vectors.argtypes = [_p, _p, ctypes.c_int, _p, _p, _p, _sz, ctypes.c_int, _p, _p, ctypes.c_int]
        lib.vgo_env_attach.argtypes = [_p, _p, _p, ctypes.c_int]
        lib.vgo_env_detach.argtypes = [_p]
        lib.vgo_robot_ee_pose.argtypes = [_p, _p, _p]
        lib.vgo_filter_pointcloud.argtypes = [_p, _sz, _f, _f, _p, _p, _p, ctypes.c_int, _p]
        lib.vgo_filter_pointcloud.restype = _sz
        lib.vgo_filter_remap.argtypes = [_f, _f, _f]
        lib.vgo_filter_remap.restype = ctypes.c_uint32
        lib.vgo_morton.argtypes = [ctypes.c_uint32] * 3
        lib.vgo_morton.restype = ctypes.c_uint32
        self.lib = lib

    def filter_pointcloud(self, points, min_dist, max_range, origin, workcell_min, workcell_max, cull) -> np.ndarray:
        """collision/filter.hh:176-278: the kept points, [m, 3]."""
        pts = np.ascontiguousarray(points, np.float32).reshape(-1, 3)
        out = np.zeros_like(pts)
        o, lo, hi = (np.ascontiguousarray(v, np.float32) for v in (origin, workcell_min, workcell_max))
        m = self.lib.vgo_filter_pointcloud(_ptr(pts), len(pts), min_dist, max_range, _ptr(o), _ptr(lo), _ptr(hi),
                                           int(bool(cull)), _ptr(out))
        return out[:m].copy()

    def sqrt_x86(self, v: np.ndarray) -> np.ndarray:
        return np.array([self.lib.vgo_sqrt_x86(float(x)) for x in np.asarray(v, np.float32)], np.float32)

    def sincos(self, x: np.ndarray):
        s = np.zeros(1, np.float32)
        c = np.zeros(1, np.float32)
        so, co = [], []
        for v in np.asarray(x, np.float32):
            self.lib.vgo_sincos(float(v), _ptr(s), _ptr(c))
            so.append(s[0])
            co.append(c[0])
        return np.array(so, np.float32), np.array(co, np.float32)

    def capt(self, points, r_min, r_max, r_point, lanes: int = 8) -> dict:
        pts = np.ascontiguousarray(points, np.float32)
        h = self.lib.vgo_capt_build(_ptr(pts), len(pts), r_min, r_max, r_point, lanes)
        if not h:
            raise RuntimeError("vgo_capt_build failed")
        try:
            return capt_layout(h.contents)
        finally:
            self.lib.vgo_capt_destroy(h)

    # environment -------------------------------------------------------------------------
    def env(self, scene, sqrt_mode: int = SQRT_X86):
        return PortEnv(self, scene, sqrt_mode)

    def robot(self, name: str):
        h = self.lib.vgo_robot_get(name.encode())
        if not h:
            raise KeyError(name)
        return PortRobot(self, h)


class PortRobot:
    def __init__(self, port: Port, h):
        self.port, self.h = port, h
        lib = port.lib
        self.dim = lib.vgo_robot_dim(h)
        self.slots = lib.vgo_robot_slots(h)
        self.fine = lib.vgo_robot_fine(h)
        self.resolution = lib.vgo_robot_resolution(h)
        self.s_m = np.zeros(self.dim, np.float32)
        self.s_a = np.zeros(self.dim, np.float32)
        lib.vgo_robot_limits(h, _ptr(self.s_m), _ptr(self.s_a))

    def spheres_f32(self, q: np.ndarray) -> np.ndarray:
        q = np.ascontiguousarray(q, np.float32)
        out = np.zeros((self.slots, 4), np.float32)
        self.port.lib.vgo_robot_spheres_f32(self.h, _ptr(q), _ptr(out))
        return out

    def ee_pose(self, q: np.ndarray) -> np.ndarray:
        """End-effector transform as a row-major 4x4 (R row-major and t, as the kernels compute it)."""
        q = np.ascontiguousarray(q, np.float32)
        T = np.zeros(12, np.float32)
        self.port.lib.vgo_robot_ee_pose(self.h, _ptr(q), _ptr(T))
        out = np.eye(4, dtype=np.float32)
        out[:3, :3] = T[:9].reshape(3, 3)
        out[:3, 3] = T[9:]
        return out

    def spheres_f64(self, q: np.ndarray) -> np.ndarray:
        q = np.ascontiguousarray(q, np.float64)
        out = np.zeros((self.slots, 4), np.float64)
        self.port.lib.vgo_robot_spheres_f64(self.h, _ptr(q), _ptr(out))
        return out


class PortEnv:
    def __init__(self, port: Port, scene, sqrt_mode: int):
        self.port = port
        lib = port.lib
        self.h = lib.vgo_env_create()
        lib.vgo_env_set_sqrt_mode(self.h, sqrt_mode)
        for s in np.asarray(scene.get("spheres", np.zeros((0, 4))), np.float32):
            lib.vgo_env_add_sphere(self.h, _ptr(np.ascontiguousarray(s)))
        for c in np.asarray(scene.get("capsules", np.zeros((0, 8))), np.float32):
            lib.vgo_env_add_capsule(self.h, _ptr(np.ascontiguousarray(c)))
        for c in np.asarray(scene.get("cuboids", np.zeros((0, 15))), np.float32):
            lib.vgo_env_add_cuboid(self.h, _ptr(np.ascontiguousarray(c)))
        for pc in scene.get("pointclouds", []):
            pts = np.ascontiguousarray(pc["points"], np.float32)
            rc = lib.vgo_env_add_pointcloud(self.h, _ptr(pts), len(pts), pc["r_min"], pc["r_max"], pc["r_point"])
            if rc:
                raise RuntimeError("pointcloud rejected")
        for hf in scene.get("heightfields", []):
            c, sc = (np.ascontiguousarray(hf[k], np.float32) for k in ("centre", "scale"))
            data = np.ascontiguousarray(hf["data"], np.float32)
            if lib.vgo_env_add_heightfield(self.h, _ptr(c), _ptr(sc), int(hf["xd"]), int(hf["yd"]), _ptr(data)):
                raise RuntimeError("heightfield rejected")
        if scene.get("attachment") is not None:
            tf = np.ascontiguousarray(scene["attachment"]["tf"], np.float32).reshape(16)
            sph = np.ascontiguousarray(scene["attachment"]["spheres"], np.float32).reshape(-1, 4)
            if lib.vgo_env_attach(self.h, _ptr(tf), _ptr(sph), len(sph)):
                raise RuntimeError("attachment rejected")

    def __del__(self):
        try:
            self.port.lib.vgo_env_destroy(self.h)
        except Exception:
            pass

    def objects(self, kind: int) -> np.ndarray:
        lib = self.port.lib
        n = lib.vgo_env_count(self.h, kind)
        width = [5, 9, 9, 16, 16][kind]
        out = np.zeros((n, width), np.float32)
        for i in range(n):
            lib.vgo_env_get(self.h, kind, i, _ptr(out[i]))
        return out

    def sphere_env(self, spheres: np.ndarray, lanes: int = 8) -> np.ndarray:
        """sphere_environment_in_collision per block of `lanes` spheres [n, 4] (1 = collides)."""
        s = np.ascontiguousarray(spheres, np.float32).reshape(-1, lanes, 4)
        out = np.zeros(len(s), np.uint8)
        for i, b in enumerate(s):
            cols = [np.ascontiguousarray(b[:, k]) for k in range(4)]
            out[i] = self.port.lib.vgo_sphere_env(self.h, lanes, *(_ptr(c) for c in cols))
        return out

    def validate_states(self, robot: PortRobot, q: np.ndarray, threads: int = 1) -> np.ndarray:
        q = np.ascontiguousarray(q, np.float32)
        out = np.zeros(len(q), np.uint8)
        self.port.lib.vgo_validate_states(robot.h, self.h, _ptr(q), len(q), _ptr(out), threads)
        return out

    def validate_motions(self, robot: PortRobot, a, b, resolution: int, lanes: int = 8, threads: int = 1):
        a = np.ascontiguousarray(a, np.float32)
        b = np.ascontiguousarray(b, np.float32)
        out = np.zeros(len(a), np.uint8)
        blocks = np.zeros(len(a), np.int32)
        self.port.lib.vgo_validate_motions(
            robot.h, self.h, lanes, _ptr(a), _ptr(b), len(a), resolution, _ptr(out), _ptr(blocks), threads
        )
        return out, blocks

    def fkcc_block(self, robot: PortRobot, q: np.ndarray) -> int:
        q = np.ascontiguousarray(q, np.float32)
        return self.port.lib.vgo_fkcc(robot.h, self.h, q.shape[0], _ptr(q))

    def filter_self(self, robot: PortRobot, points, point_radius: float, q) -> np.ndarray:
        """filter_self_from_pointcloud (bindings/robot_helper.hh:307-345): the kept points."""
        pts = np.ascontiguousarray(points, np.float32).reshape(-1, 3)
        out = np.zeros_like(pts)
        qq = np.ascontiguousarray(q, np.float32)
        m = self.port.lib.vgo_filter_self(robot.h, self.h, _ptr(pts), len(pts), point_radius, _ptr(qq), _ptr(out))
        return out[:m].copy()

    def validate_vectors(self, robot: PortRobot, start, vector, distance, resolution: int, lanes: int = 8,
                         threads: int = 1):
        """validate_vector (planning/validate.hh:23-63) per edge: (verdicts, blocks checked)."""
        s = np.ascontiguousarray(start, np.float32)
        v = np.ascontiguousarray(vector, np.float32)
        d = np.ascontiguousarray(distance, np.float32)
        out = np.zeros(len(s), np.uint8)
        blocks = np.zeros(len(s), np.int32)
        self.port.lib.vgo_validate_vectors(robot.h, self.h, lanes, _ptr(s), _ptr(v), _ptr(d), len(s), resolution,
                                           _ptr(out), _ptr(blocks), threads)
        return out, blocks

    def validate_motions_counted(self, robot: PortRobot, a, b, resolution: int, lanes: int = 8):
        a = np.ascontiguousarray(a, np.float32)
        b = np.ascontiguousarray(b, np.float32)
        out = np.zeros(len(a), np.uint8)
        cnt = Counters()
        self.port.lib.vgo_validate_motions_counted(
            robot.h, self.h, lanes, _ptr(a), _ptr(b), len(a), resolution, _ptr(out), ctypes.byref(cnt)
        )
        return out, cnt

    def capt(self, idx: int = 0) -> dict:
        h = self.port.lib.vgo_env_capt(self.h, idx)
        if not h:
            raise IndexError(idx)
        return capt_layout(h.contents)

    def debug(self, robot: PortRobot, q: np.ndarray):
        """Robot::fkcc_debug per configuration: (env bits [n][fine][words] uint32 over insertion
        ids, self pair flags [n][pairs] uint8)."""
        q = np.ascontiguousarray(q, np.float32).reshape(-1, robot.dim)
        words = max(1, (self.port.lib.vgo_env_total(self.h) + 31) // 32)
        np_ = self.port.lib.vgo_robot_self_pairs(robot.h)
        env_bits = np.zeros((len(q), robot.fine, words), np.uint32)
        pairs = np.zeros((len(q), np_), np.uint8)
        for i in range(len(q)):
            self.port.lib.vgo_debug(robot.h, self.h, _ptr(q[i]), _ptr(env_bits[i]), words, _ptr(pairs[i]))
        return env_bits, pairs

    def contact_distance(self, robot: PortRobot, q) -> float:
        q = np.ascontiguousarray(q, np.float64)
        return self.port.lib.vgo_contact_distance_f64(robot.h, self.h, _ptr(q))


class Reference:
    """The reference's own compiled code (x86-64 build of the reference sources)."""

    def __init__(self, path: Path = REF_LIB):
        if not Path(path).exists():
            raise FileNotFoundError(path)
        lib = ctypes.CDLL(str(path))
        lib.vgref_env_create.restype = _p
        lib.vgref_env_destroy.argtypes = [_p]
        lib.vgref_env_add_sphere.argtypes = [_p, _p]
        lib.vgref_env_add_capsule.argtypes = [_p, _p, ctypes.c_int]
        lib.vgref_env_add_cuboid.argtypes = [_p, _p, ctypes.c_int]
        lib.vgref_env_add_pointcloud.argtypes = [_p, _p, _sz, _f, _f, _f]
        lib.vgref_env_finalize.argtypes = [_p]
        lib.vgref_env_count.argtypes = [_p, ctypes.c_int]
        lib.vgref_env_count.restype = _sz
        lib.vgref_env_get.argtypes = [_p, ctypes.c_int, _sz, _p]
        lib.vgref_capt_build.argtypes = [_p, _sz, _f, _f, _f]
        lib.vgref_capt_build.restype = _p
        lib.vgref_capt_destroy.argtypes = [_p]
        lib.vgref_capt_sizes.argtypes = [_p, _p]
        lib.vgref_capt_dump.argtypes = [_p, _p, _p, _p, _p, _p, _p]
        lib.vgref_capt_collides_simd.argtypes = [_p, _p, _p, _p, _p]
        lib.vgref_vec_sqrt8.argtypes = [_p, _p]
        lib.vgref_vec_sincos8.argtypes = [_p, _p, _p]
        lib.vgref_sphere_env8.argtypes = [_p, _p, _p, _p, _p]
        lib.vgref_env_add_heightfield.argtypes = [_p, _p, _p, _sz, _sz, _p]
        for r in ("panda", "ur5", "fetch", "baxter"):
            getattr(lib, f"vgref_{r}_info").argtypes = [_p, _p, _p, _p, _p]
            getattr(lib, f"vgref_{r}_limits").argtypes = [_p, _p]
            getattr(lib, f"vgref_{r}_fkcc_block").argtypes = [_p, _p]
            getattr(lib, f"vgref_{r}_validate_states").argtypes = [_p, _p, _sz, _p, ctypes.c_int]
            getattr(lib, f"vgref_{r}_validate_motions").argtypes = [_p, _p, _p, _sz, ctypes.c_int, _p, ctypes.c_int]
            getattr(lib, f"vgref_{r}_validate_motions_counted").argtypes = [_p, _p, _p, _sz, ctypes.c_int, _p, _p,
                                                                             ctypes.c_int]
            getattr(lib, f"vgref_{r}_filter_self").argtypes = [_p, _p, _sz, _f, _p, _p]
            getattr(lib, f"vgref_{r}_filter_self").restype = _sz
            getattr(lib, f"vgref_{r}_validate_vectors").argtypes = [_p, _p, _p, _p, _sz, ctypes.c_int, _p, ctypes.c_int]
            getattr(lib, f"vgref_{r}_motion_blocks").argtypes = [_p, _p, ctypes.c_int, _p, _sz, ctypes.c_long]
            getattr(lib, f"vgref_{r}_motion_blocks").restype = ctypes.c_long
            getattr(lib, f"vgref_{r}_sphere_fk").argtypes = [_p, _p]
            getattr(lib, f"vgref_{r}_debug").argtypes = [_p, _p, _p, ctypes.c_int, _p, ctypes.c_int, _p]
        lib.vgref_filter_pointcloud.argtypes = [_p, _sz, _f, _f, _p, _p, _p, ctypes.c_int, _p, _p]
        lib.vgref_filter_remap.argtypes = [_f, _f, _f]
        lib.vgref_filter_remap.restype = ctypes.c_uint
        self.lib = lib

    def env(self, scene):
        return RefEnv(self, scene)

    def filter_pointcloud(self, points, min_dist, max_range, origin, workcell_min, workcell_max, cull) -> np.ndarray:
        """The reference's filter_pointcloud (collision/filter.hh:176-320): the kept points, [m, 3]."""
        pts = np.ascontiguousarray(points, np.float32).reshape(-1, 3)
        out = np.zeros_like(pts)
        m = _sz()
        o, lo, hi = (np.ascontiguousarray(v, np.float32) for v in (origin, workcell_min, workcell_max))
        self.lib.vgref_filter_pointcloud(_ptr(pts), len(pts), min_dist, max_range, _ptr(o), _ptr(lo), _ptr(hi),
                                         int(bool(cull)), _ptr(out), ctypes.byref(m))
        return out[: m.value].copy()

    def sphere_fk(self, robot: str, q: np.ndarray, n_spheres: int) -> np.ndarray:
        q = np.ascontiguousarray(q, np.float32)
        out = np.zeros((n_spheres, 4), np.float32)
        getattr(self.lib, f"vgref_{robot}_sphere_fk")(_ptr(q), _ptr(out))
        return out

    def motion_blocks(self, robot: str, a, b, resolution: int, cap: int = 4096, dim: int = 7, fail_at: int = -1):
        a = np.ascontiguousarray(a, np.float32)
        b = np.ascontiguousarray(b, np.float32)
        out = np.zeros((cap, dim, 8), np.float32)
        n = getattr(self.lib, f"vgref_{robot}_motion_blocks")(_ptr(a), _ptr(b), resolution, _ptr(out), cap, fail_at)
        return n, out[: min(n, cap)]

    def capt(self, points, r_min, r_max, r_point) -> dict:
        pts = np.ascontiguousarray(points, np.float32)
        h = self.lib.vgref_capt_build(_ptr(pts), len(pts), r_min, r_max, r_point)
        sizes = np.zeros(5, np.uint64)
        self.lib.vgref_capt_sizes(h, _ptr(sizes))
        nlog2, nt, nl, nb, L = (int(s) for s in sizes)
        tests = np.zeros(nt, np.float32)
        aabbs = np.zeros((nl, 6), np.float32)
        starts = np.zeros(nl + 1, np.uint32)
        aff = np.zeros((3, nb, L), np.float32)
        top = np.zeros(6, np.float32)
        radii = np.zeros(3, np.float32)
        self.lib.vgref_capt_dump(h, _ptr(tests), _ptr(aabbs), _ptr(starts), _ptr(aff), _ptr(top), _ptr(radii))
        self.lib.vgref_capt_destroy(h)
        return dict(nlog2=nlog2, tests=tests, aabbs=aabbs, aff_starts=starts, aff=aff, top=top, radii=radii)


class RefEnv:
    def __init__(self, ref: Reference, scene):
        self.ref = ref
        lib = ref.lib
        self.h = lib.vgref_env_create()
        for s in np.asarray(scene.get("spheres", np.zeros((0, 4))), np.float32):
            lib.vgref_env_add_sphere(self.h, _ptr(np.ascontiguousarray(s)))
        for c in np.asarray(scene.get("capsules", np.zeros((0, 8))), np.float32):
            lib.vgref_env_add_capsule(self.h, _ptr(np.ascontiguousarray(c)), int(c[3] == 0 and c[4] == 0))
        for c in np.asarray(scene.get("cuboids", np.zeros((0, 15))), np.float32):
            lib.vgref_env_add_cuboid(self.h, _ptr(np.ascontiguousarray(c)), int(c[11] == 1.0))
        for pc in scene.get("pointclouds", []):
            pts = np.ascontiguousarray(pc["points"], np.float32)
            lib.vgref_env_add_pointcloud(self.h, _ptr(pts), len(pts), pc["r_min"], pc["r_max"], pc["r_point"])
        for hf in scene.get("heightfields", []):
            c, sc = (np.ascontiguousarray(hf[k], np.float32) for k in ("centre", "scale"))
            data = np.ascontiguousarray(hf["data"], np.float32)
            lib.vgref_env_add_heightfield(self.h, _ptr(c), _ptr(sc), int(hf["xd"]), int(hf["yd"]), _ptr(data))
        lib.vgref_env_finalize(self.h)

    def sphere_env(self, spheres: np.ndarray) -> np.ndarray:
        """The reference's sphere_environment_in_collision per 8-lane block of spheres [n, 4]."""
        s = np.ascontiguousarray(spheres, np.float32).reshape(-1, 8, 4)
        out = np.zeros(len(s), np.uint8)
        for i, b in enumerate(s):
            cols = [np.ascontiguousarray(b[:, k]) for k in range(4)]
            out[i] = self.ref.lib.vgref_sphere_env8(self.h, *(_ptr(c) for c in cols))
        return out

    def __del__(self):
        try:
            self.ref.lib.vgref_env_destroy(self.h)
        except Exception:
            pass

    def objects(self, kind: int) -> np.ndarray:
        lib = self.ref.lib
        n = lib.vgref_env_count(self.h, kind)
        width = [5, 9, 9, 16, 16][kind]
        out = np.zeros((n, width), np.float32)
        for i in range(n):
            lib.vgref_env_get(self.h, kind, i, _ptr(out[i]))
        return out

    def debug(self, robot: str, q: np.ndarray, n_fine: int, n_objects: int):
        """Robot::fkcc_debug per configuration: (env bits [n][fine][words] over insertion ids,
        list per configuration of the colliding fine pairs (i, j) in the reference's order)."""
        q = np.ascontiguousarray(q, np.float32).reshape(len(q), -1)
        words = max(1, (n_objects + 31) // 32)
        bits = np.zeros((len(q), n_fine, words), np.uint32)
        out_pairs = []
        cap = 8192
        buf = np.zeros(2 * cap, np.int32)
        cnt = ctypes.c_int()
        fn = getattr(self.ref.lib, f"vgref_{robot}_debug")
        for i in range(len(q)):
            fn(self.h, _ptr(q[i]), _ptr(bits[i]), words, _ptr(buf), cap, ctypes.byref(cnt))
            out_pairs.append([(int(buf[2 * k]), int(buf[2 * k + 1])) for k in range(min(cnt.value, cap))])
        return bits, out_pairs

    def filter_self(self, robot: str, points, point_radius: float, q) -> np.ndarray:
        pts = np.ascontiguousarray(points, np.float32).reshape(-1, 3)
        out = np.zeros_like(pts)
        qq = np.ascontiguousarray(q, np.float32)
        m = getattr(self.ref.lib, f"vgref_{robot}_filter_self")(self.h, _ptr(pts), len(pts), point_radius, _ptr(qq),
                                                                _ptr(out))
        return out[:m].copy()

    def validate_vectors(self, robot: str, start, vector, distance, resolution: int, threads: int = 1):
        s = np.ascontiguousarray(start, np.float32)
        v = np.ascontiguousarray(vector, np.float32)
        d = np.ascontiguousarray(distance, np.float32)
        out = np.zeros(len(s), np.uint8)
        getattr(self.ref.lib, f"vgref_{robot}_validate_vectors")(self.h, _ptr(s), _ptr(v), _ptr(d), len(s), resolution,
                                                                _ptr(out), threads)
        return out

    def validate_states(self, robot: str, q, threads: int = 1):
        q = np.ascontiguousarray(q, np.float32)
        out = np.zeros(len(q), np.uint8)
        getattr(self.ref.lib, f"vgref_{robot}_validate_states")(self.h, _ptr(q), len(q), _ptr(out), threads)
        return out

    def validate_motions(self, robot: str, a, b, resolution: int, threads: int = 1):
        a = np.ascontiguousarray(a, np.float32)
        b = np.ascontiguousarray(b, np.float32)
        out = np.zeros(len(a), np.uint8)
        getattr(self.ref.lib, f"vgref_{robot}_validate_motions")(
            self.h, _ptr(a), _ptr(b), len(a), resolution, _ptr(out), threads
        )
        return out

    def validate_motions_counted(self, robot: str, a, b, resolution: int, threads: int = 1):
        """validate_motion per edge with the blocks the reference checked: (verdicts, blocks)."""
        a = np.ascontiguousarray(a, np.float32)
        b = np.ascontiguousarray(b, np.float32)
        out = np.zeros(len(a), np.uint8)
        blocks = np.zeros(len(a), np.int32)
        getattr(self.ref.lib, f"vgref_{robot}_validate_motions_counted")(
            self.h, _ptr(a), _ptr(b), len(a), resolution, _ptr(out), _ptr(blocks), threads
        )
        return out, blocks

    def fkcc_block(self, robot: str, q_lanes_dim: np.ndarray) -> int:
        """q is [8][dim]; the reference takes [dim][8]."""
        q = np.ascontiguousarray(np.asarray(q_lanes_dim, np.float32).T)
        return getattr(self.ref.lib, f"vgref_{robot}_fkcc_block")(self.h, _ptr(q))
