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
