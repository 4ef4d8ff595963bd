"""The C ABI library: loads, exports what include/vamp_gb300.h declares, and its host-side
environment logic matches the CPU oracle (no GPU needed for any of this)."""
import ctypes
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT, golden, scene_of

HEADER = ROOT / "include" / "vamp_gb300.h"


def declared():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(vg_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    from vamp_gb300 import _lib

    names = declared()
    assert names, "no declarations found"
    out = subprocess.run(["nm", "-D", "--defined-only", str(_lib.LIB_PATH)], capture_output=True, text=True, check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if line.strip()}
    missing = [n for n in names if n not in exported]
    assert not missing, missing
    assert sorted(_lib.EXPORTED) == names


def test_robot_constants_match_the_oracle(port):
    import vamp_gb300 as vg

    for name in ("panda", "ur5", "fetch", "baxter"):
        r = getattr(vg, name)
        o = port.robot(name)
        assert r.dimension() == o.dim
        assert r.resolution() == o.resolution
        assert np.array_equal(r.s_m, o.s_m) and np.array_equal(r.s_a, o.s_a)


def test_environment_is_the_oracles_bit_for_bit(port):
    import vamp_gb300 as vg

    for name in ("states_panda_scene0", "states_panda_scene1", "states_baxter_scene1"):
        g = golden(name)
        mine = vg.Environment.from_scene(scene_of(g))
        ref = port.env(scene_of(g))
        for k in range(5):
            assert np.array_equal(mine.objects(k).view(np.uint32), ref.objects(k).view(np.uint32)), (name, k)


def test_z_aligned_routing_matches_the_reference_binding():
    import vamp_gb300 as vg

    env = vg.Environment()
    env.add_capsule([0, 0, 1, 0, 0, 0.5, 0.1, 4.0])  # xv == yv == 0
    env.add_cuboid([1, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0, 1, 0.1, 0.1, 0.1])  # axis_3_z == 1
    env.add_cuboid([1, 0, 0, 0, 1, 0, 0, 0, 1, 1, 0, 0, 0.1, 0.1, 0.1])
    counts = [len(env.objects(k)) for k in range(5)]
    assert counts == [0, 0, 1, 1, 1]


def test_errors_are_reported_not_raised_through_the_abi():
    import vamp_gb300 as vg
    from vamp_gb300._lib import lib

    assert lib.vg_robot_info(b"no_such_robot", None, None, None, None, None) == -1
    assert b"unknown robot" in lib.vg_last_error()
    env = vg.Environment()
    with pytest.raises(vg.VampError):
        env.set_mode(5, 0)
    assert lib.vg_env_add_sphere(None, None) == -1


def test_explicit_kind_and_caller_min_distance_are_kept():
    """vg_env_add_primitive: the object goes to the kind list named, with the caller's
    min_distance (a converted reference environment's objects already sit in their lists)."""
    import vamp_gb300 as vg

    env = vg.Environment()
    cub = [1, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0, 1, 0.1, 0.1, 0.1]  # z-aligned axes, put in the general list
    env.add_primitive(3, cub, 0.75)
    env.add_primitive(3, cub, 0.25)
    env.add_primitive(2, [0, 0, 1, 0.5, 0, 0.5, 0.1, 2.0], 0.5)  # not z-aligned, put in the z list
    assert [len(env.objects(k)) for k in range(5)] == [0, 0, 1, 2, 0]
    assert list(env.objects(3)[:, -1]) == [0.25, 0.75]  # kept sorted by min_distance
    with pytest.raises(ValueError):
        env.add_primitive(0, cub, 0.0)
    from vamp_gb300._lib import lib

    f = np.zeros(15, np.float32)
    assert lib.vg_env_add_primitive(env.handle, 5, f.ctypes.data, 0.0) == -1


def test_pointcloud_layout_import_round_trips(port):
    """vg_env_add_pointcloud_layout takes the reference's tree as built: importing the oracle's
    tree and reading it back gives the same arrays; inconsistent block ranges are refused."""
    import vamp_gb300 as vg
    from vamp_gb300 import scenes

    pts = scenes.surface_pointcloud(9, 1500)
    lay = port.capt(pts, 0.012, 0.08, scenes.POINT_RADIUS)
    env = vg.Environment()
    env.add_pointcloud_layout(lay)
    back = env.pointcloud_layout(0)
    for k in ("tests", "aabbs", "aff_starts", "aff", "top"):
        assert np.array_equal(np.asarray(back[k]), np.asarray(lay[k])), k
    bad = dict(lay)
    bad["aff_starts"] = lay["aff_starts"].copy()
    bad["aff_starts"][3], bad["aff_starts"][4] = bad["aff_starts"][4] + 1, bad["aff_starts"][3]
    with pytest.raises(vg.VampError):
        vg.Environment().add_pointcloud_layout(bad)
    short = dict(lay)
    short["aff_starts"] = lay["aff_starts"].copy()
    short["aff_starts"][-1] += 1  # more blocks than given
    with pytest.raises(vg.VampError):
        vg.Environment().add_pointcloud_layout(short)
