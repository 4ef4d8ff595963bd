"""The CPU oracle (oracle/port) against the reference's own outputs (tests/golden)."""
import numpy as np
import pytest

from conftest import golden, scene_of
from flips import classify_edges, classify_states

ROBOTS = ["panda", "ur5", "fetch", "baxter"]


def test_lane_sqrt_is_the_reference_bit_for_bit(port):
    g = golden("lane_math")
    mine = port.sqrt_x86(g["sqrt_in"])
    ref = g["sqrt_out"]
    assert np.array_equal(np.isnan(mine), np.isnan(ref))
    ok = ~np.isnan(ref)
    assert np.array_equal(mine[ok].view(np.uint32), ref[ok].view(np.uint32))


def test_lane_sincos_close_to_reference(port):
    g = golden("lane_math")
    s, c = port.sincos(g["angle"])
    assert np.abs(s - g["sin"]).max() <= 3e-7
    assert np.abs(c - g["cos"]).max() <= 3e-7


@pytest.mark.parametrize("robot", ROBOTS)
def test_fk_matches_reference(port, robot):
    g = golden(f"fk_{robot}")
    rb = port.robot(robot)
    for q, ref in zip(g["q"], g["spheres"]):
        s32 = rb.spheres_f32(q)[: rb.fine]
        s64 = rb.spheres_f64(q.astype(np.float64))[: rb.fine]
        assert np.abs(s32 - ref).max() <= 1e-6
        # sphere centres within 1e-5 m of the FP64 kinematics
        assert np.abs(s64[:, :3] - ref[:, :3]).max() <= 1e-5
        assert np.array_equal(s32[:, 3], ref[:, 3])


@pytest.mark.parametrize(
    "name,robot",
    [("states_panda_scene0", "panda"), ("states_panda_scene1", "panda"), ("states_ur5_scene1", "ur5"),
     ("states_fetch_scene1", "fetch"), ("states_baxter_scene1", "baxter")],
)
def test_state_verdicts_match_reference(port, name, robot):
    g = golden(name)
    env = port.env(scene_of(g))
    rb = port.robot(robot)
    mine = env.validate_states(rb, g["q"])
    rep = classify_states(env, rb, g["q"], mine, g["verdict"])
    assert rep["unexplained"] == [], rep
    assert rep["flips"] <= max(1, len(g["q"]) // 1000)


def test_environment_order_matches_reference(port):
    g = golden("states_panda_scene1")
    env = port.env(scene_of(g))
    for k in range(5):
        mine, ref = env.objects(k), g[f"kind{k}"]
        assert mine.shape == ref.shape
        assert np.array_equal(mine[:, :-1], ref[:, :-1])  # same objects in the same order
        if len(ref):
            assert np.abs(mine[:, -1] - ref[:, -1]).max() <= 5e-7  # min_distance


@pytest.mark.parametrize(
    "name,robot",
    [("edges_panda_scene1_res32", "panda"), ("edges_panda_scene0_res1", "panda"), ("edges_panda_scene1_res8", "panda"),
     ("edges_ur5_scene1_res32", "ur5"), ("edges_fetch_scene1_res32", "fetch"), ("edges_baxter_scene1_res64", "baxter")],
)
def test_edge_verdicts_match_reference(port, name, robot):
    g = golden(name)
    env = port.env(scene_of(g))
    rb = port.robot(robot)
    res = int(g["resolution"])
    mine, _ = env.validate_motions(rb, g["a"], g["b"], res)
    rep = classify_edges(env, rb, g["a"], g["b"], res, mine, g["verdict"])
    assert rep["unexplained"] == [], rep
    assert rep["flips"] <= max(1, len(g["a"]) // 500)


def test_motion_states_are_the_reference_bit_for_bit(port):
    from flips import motion_states

    g = golden("motion_blocks_panda")
    rb = port.robot("panda")
    off = 0
    for a, b, n in zip(g["a"], g["b"], g["counts"]):
        ref = g["blocks"][off : off + n]
        off += n
        mine = motion_states(rb, a, b, 32).reshape(n, 8, 7)
        assert np.array_equal(mine.view(np.uint32), ref.view(np.uint32))


def test_capt_layout_is_the_reference_bit_for_bit(port):
    g = golden("capt_layout")
    lay = port.capt(g["points"], *map(float, g["r"]))
    assert lay["nlog2"] == int(g["nlog2"])
    for k in ("tests", "aabbs", "aff_starts", "aff", "top"):
        assert np.array_equal(lay[k], g[k], equal_nan=True), k


def test_threads_do_not_change_verdicts(port):
    g = golden("edges_panda_scene1_res32")
    env = port.env(scene_of(g))
    rb = port.robot("panda")
    one, b1 = env.validate_motions(rb, g["a"], g["b"], 32, threads=1)
    many, b4 = env.validate_motions(rb, g["a"], g["b"], 32, threads=4)
    assert np.array_equal(one, many) and np.array_equal(b1, b4)


def _cloud_scene(g):
    return {"spheres": np.zeros((0, 4), np.float32), "capsules": np.zeros((0, 8), np.float32),
            "cuboids": np.zeros((0, 15), np.float32),
            "pointclouds": [{"points": g["points"], "r_min": float(g["r"][0]), "r_max": float(g["r"][1]),
                             "r_point": float(g["r"][2])}]}


def test_pointcloud_verdicts_match_reference(port):
    g = golden("cloud_panda")
    env = port.env(_cloud_scene(g))
    rb = port.robot("panda")
    assert np.array_equal(env.validate_states(rb, g["q"]), g["state_verdict"])
    ev, _ = env.validate_motions(rb, g["a"], g["b"], 32)
    assert np.array_equal(ev, g["edge_verdict"])


def test_library_capt_layout_is_the_reference_bit_for_bit(port):
    """The shipped library's host-side CAPT builder against the reference's layout and the
    oracle's (no GPU needed)."""
    import vamp_gb300 as vg
    from vamp_gb300 import scenes

    g = golden("capt_layout")
    env = vg.Environment()
    env.add_pointcloud(g["points"], *map(float, g["r"]))
    lay = env.pointcloud_layout(0)
    for k in ("tests", "aabbs", "aff_starts", "aff", "top"):
        assert np.array_equal(lay[k], g[k], equal_nan=True), k
    pts = scenes.surface_pointcloud(7, 20000)
    env = vg.Environment()
    env.add_pointcloud(pts, 0.012, 0.08, scenes.POINT_RADIUS)
    mine, ref = env.pointcloud_layout(0), port.capt(pts, 0.012, 0.08, scenes.POINT_RADIUS)
    for k in ("tests", "aabbs", "aff_starts", "aff", "top"):
        assert np.array_equal(mine[k], ref[k], equal_nan=True), k


@pytest.mark.parametrize("robot", ["panda", "baxter"])
def test_debug_reports_match_the_reference(port, robot):
    """Robot::fkcc_debug: per fine sphere the objects it collides with, per fine self pair
    whether it collides (golden fixture from the compiled reference)."""
    g = golden(f"debug_{robot}")
    env = port.env(scene_of(g))
    bits, pairs = env.debug(port.robot(robot), g["q"])
    assert np.array_equal(bits, g["env_bits"])
    assert np.array_equal(pairs, g["pairs"])
    assert g["env_bits"].any() and g["pairs"].any()


def _filter_case(g: dict, i: int):
    p = g[f"params{i}"]
    return g[f"points{i}"], float(p[0]), float(p[1]), p[2:5], p[5:8], p[8:11], bool(p[11])


def test_filter_matches_the_reference(port):
    """filter_pointcloud (collision/filter.hh:176-320): the restated filter keeps exactly the
    reference's points, in its order (golden fixture from the compiled reference)."""
    g = golden("filter")
    for i in range(6):
        pts, md, mr, o, lo, hi, cull = _filter_case(g, i)
        kept = port.filter_pointcloud(pts, md, mr, o, lo, hi, cull)
        assert kept.shape == g[f"kept{i}"].shape and np.array_equal(kept, g[f"kept{i}"]), i
    assert len(g["kept4"]) == 1 and np.array_equal(g["kept4"][0], g["points4"][0])  # all culled: point 0 stays


def test_filter_conversion_and_morton(port):
    """remap_point's float -> uint32_t conversion and the Morton interleave (filter.hh:142-171)."""
    lib = port.lib
    assert lib.vgo_filter_remap(0.5, 0.0, 1.0) == 500
    assert lib.vgo_filter_remap(-0.0005, 0.0, 1.0) == 0        # (-1, 0) truncates to 0
    assert lib.vgo_filter_remap(-0.002, 0.0, 1.0) == 0xFFFFFFFF  # <= -1
    assert lib.vgo_filter_remap(5e6, 0.0, 1.0) == 0xFFFFFFFF     # >= 2^32
    assert lib.vgo_filter_remap(float("nan"), 0.0, 1.0) == 0xFFFFFFFF
    assert lib.vgo_morton(1, 0, 0) == 1 and lib.vgo_morton(0, 1, 0) == 2 and lib.vgo_morton(0, 0, 1) == 4
    assert lib.vgo_morton(0x7FF, 0, 0) == 0x49249249 and lib.vgo_morton(0, 0x7FF, 0) == 0x92492492
    assert lib.vgo_morton(0, 0, 0x7FF) == 0x24924924  # z keeps 10 bits


@pytest.mark.parametrize("robot", ["panda", "ur5", "fetch", "baxter"])
def test_ee_pose_matches_the_reference_eefk(port, robot):
    """The end-effector transform the attachment is posed at, against the reference's own eefk
    expressions (robots/<robot>.hh, Robot::eefk) evaluated in float64: FP32 rounding only."""
    g = golden(f"eefk_{robot}")
    rb = port.robot(robot)
    err = max(np.abs(rb.ee_pose(q) - T).max() for q, T in zip(g["q"], g["T"]))
    assert err < 1e-5, err


def _attach_scene(scene: dict, spheres, offset: float = 0.14) -> dict:
    tf = np.eye(4, dtype=np.float32)
    tf[2, 3] = offset
    return {**scene, "attachment": {"tf": tf, "spheres": np.asarray(spheres, np.float32).reshape(-1, 4)}}


def test_attachment_checks_in_the_oracle(port):
    """fkcc_attach in the oracle: an attachment far from everything changes no verdict; one that
    engulfs the workspace fails every configuration; a sphere at the hand only adds failures."""
    from vamp_gb300 import scenes

    rb = port.robot("panda")
    base = scenes.scene_config1(5)
    q = scenes.configurations(rb.s_m, rb.s_a, 600, 9)
    plain = port.env(base).validate_states(rb, q)
    far = port.env(_attach_scene(base, [[0, 0, 0, 0.001]], offset=50.0)).validate_states(rb, q)
    assert np.array_equal(plain, far)
    huge = port.env(_attach_scene(base, [[0, 0, 0, 3.0]])).validate_states(rb, q)
    assert not huge.any()
    hand = port.env(_attach_scene(base, [[0, 0, 0, 0.07]])).validate_states(rb, q)
    assert not (hand & ~plain).any() and (plain & ~hand).any()
    # the attachment against the robot itself: empty scene, a large sphere near the hand
    empty = {"spheres": np.zeros((0, 4), np.float32), "capsules": np.zeros((0, 8), np.float32),
             "cuboids": np.zeros((0, 15), np.float32)}
    self_only = port.env(_attach_scene(empty, [[0, 0, 0, 0.25]], offset=0.0)).validate_states(rb, q)
    plain_empty = port.env(empty).validate_states(rb, q)
    assert (plain_empty & ~self_only).any()


def _hf_scene(g: dict) -> dict:
    hf = {"centre": g["centre"], "scale": g["scale"], "xd": int(g["xd"]), "yd": int(g["yd"]), "data": g["data"]}
    return {"spheres": np.zeros((0, 4), np.float32), "capsules": np.zeros((0, 8), np.float32),
            "cuboids": np.zeros((0, 15), np.float32), "heightfields": [hf]}


def test_heightfield_matches_the_reference(port):
    """sphere_heightfield (collision/sphere_heightfield.hh:9-30) inside
    sphere_environment_in_collision, and Panda states above the terrain (golden fixture from the
    compiled reference)."""
    g = golden("heightfield")
    env = port.env(_hf_scene(g))
    assert np.array_equal(env.sphere_env(np.repeat(g["single"], 8, axis=0)), g["single_verdict"])
    assert np.array_equal(env.sphere_env(g["mixed"]), g["mixed_verdict"])
    assert np.array_equal(env.validate_states(port.robot("panda"), g["q"]), g["state_verdict"])
    assert 0.1 < g["single_verdict"].mean() < 0.9 and 0.1 < g["state_verdict"].mean() < 0.95


@pytest.mark.parametrize("robot", ["panda", "ur5"])
def test_validate_vector_matches_the_reference(port, robot):
    """validate_vector with caller-given distances (golden fixture from the compiled reference)."""
    g = golden(f"vectors_{robot}")
    env = port.env(scene_of(g))
    out, _ = env.validate_vectors(port.robot(robot), g["start"], g["vector"], g["distance"], 32)
    assert np.array_equal(out, g["verdict"])
    assert 0.1 < g["verdict"].mean() < 0.95


def test_filter_self_matches_the_reference(port):
    """filter_self_from_pointcloud (bindings/robot_helper.hh:307-345): uniform points and points
    around the robot's spheres (golden fixture from the compiled reference)."""
    g = golden("filter_self_panda")
    env = port.env(scene_of(g))
    for i in range(len(g["q"])):
        kept = env.filter_self(port.robot("panda"), g["points"], float(g["radius"]), g["q"][i])
        assert kept.shape == g[f"kept{i}"].shape and np.array_equal(kept, g[f"kept{i}"]), i
    assert len(g["kept0"]) < 0.8 * len(g["points"])  # the robot removes many of the near points
