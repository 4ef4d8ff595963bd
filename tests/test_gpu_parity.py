"""GPU kernels against the CPU oracle (bit-exact verdicts) and the reference (golden fixtures).

The oracle restates the reference's algorithm with the same FP32 operation sequence as the
kernels, so every verdict and every per-edge block count must match it exactly, at every size.
Against the reference's own outputs, verdicts may differ only for configurations within 1e-5 m
of contact (tests/flips.py)."""
import os

import numpy as np
import pytest

from conftest import golden, scene_of
from flips import classify_edges, classify_states

pytestmark = pytest.mark.gpu

ROBOTS = ["panda", "ur5", "fetch", "baxter"]
THREADS = max(1, min(16, os.cpu_count() or 1))


@pytest.fixture(scope="module")
def vg():
    import vamp_gb300 as vg

    return vg


@pytest.fixture(scope="module")
def torch():
    import torch

    assert torch.cuda.is_available()
    return torch


def test_fk_is_the_oracles_bit_for_bit(vg, port):
    from vamp_gb300 import scenes

    for name in ROBOTS:
        rb = port.robot(name)
        q = scenes.configurations(rb.s_m, rb.s_a, 256, 7)
        gpu = getattr(vg, name).fk_slots(q)
        cpu = np.stack([rb.spheres_f32(x) for x in q])
        assert np.array_equal(gpu.view(np.uint32), cpu.view(np.uint32)), name
        s64 = np.stack([rb.spheres_f64(x.astype(np.float64)) for x in q[:32]])
        assert np.abs(gpu[:32, :, :3] - s64[:, :, :3]).max() <= 1e-5


@pytest.mark.parametrize("robot", ROBOTS)
@pytest.mark.parametrize("scene_seed,placement", [(0, "cube"), (1, "workspace")])
def test_state_verdicts_are_the_oracles(vg, port, robot, scene_seed, placement):
    from vamp_gb300 import scenes

    scene = scenes.primitive_scene(scene_seed, 8 if placement == "cube" else 24, 8 if placement == "cube" else 24,
                                   4 if placement == "cube" else 12, placement)
    rb = port.robot(robot)
    q = scenes.configurations(rb.s_m, rb.s_a, 8192, 40 + scene_seed)
    gpu = getattr(vg, robot).validate_batch(q, vg.Environment.from_scene(scene))
    cpu = port.env(scene).validate_states(rb, q, threads=THREADS)
    assert np.array_equal(gpu, cpu)


@pytest.mark.parametrize(
    "name,robot",
    [("states_panda_scene0", "panda"), ("states_panda_scene1", "panda"), ("states_ur5_scene1", "ur5"),
     ("states_fetch_scene1", "fetch"), ("states_baxter_scene1", "baxter")],
)
def test_state_verdicts_match_reference(vg, port, name, robot):
    g = golden(name)
    gpu = getattr(vg, robot).validate_batch(g["q"], vg.Environment.from_scene(scene_of(g)))
    rep = classify_states(port.env(scene_of(g)), port.robot(robot), g["q"], gpu, g["verdict"])
    assert rep["unexplained"] == [], rep


@pytest.mark.parametrize(
    "name,robot",
    [("edges_panda_scene1_res32", "panda"), ("edges_panda_scene0_res1", "panda"), ("edges_panda_scene1_res8", "panda"),
     ("edges_ur5_scene1_res32", "ur5"), ("edges_fetch_scene1_res32", "fetch"), ("edges_baxter_scene1_res64", "baxter")],
)
def test_edge_verdicts_match_reference_and_oracle(vg, port, torch, name, robot):
    g = golden(name)
    res = int(g["resolution"])
    env = vg.Environment.from_scene(scene_of(g))
    r = getattr(vg, robot)
    a = torch.from_numpy(g["a"]).cuda()
    b = torch.from_numpy(g["b"]).cuda()
    blocks = torch.zeros(len(a), dtype=torch.int32, device="cuda")
    gpu = r.validate_motion_batch(a, b, env, res, blocks=blocks).cpu().numpy()
    penv = port.env(scene_of(g))
    cpu, cpu_blocks = penv.validate_motions(port.robot(robot), g["a"], g["b"], res, threads=THREADS)
    assert np.array_equal(gpu, cpu)
    assert np.array_equal(blocks.cpu().numpy(), cpu_blocks)
    rep = classify_edges(penv, port.robot(robot), g["a"], g["b"], res, gpu, g["verdict"])
    assert rep["unexplained"] == [], rep


def test_full_size_edge_batch_is_the_oracles(vg, port, torch):
    """The 65,536-edge Panda workload: every verdict and block count equals the oracle's."""
    from vamp_gb300 import scenes

    scene = scenes.scene_config1(1)
    rb = port.robot("panda")
    a, b = scenes.edges(rb.s_m, rb.s_a, 65536, 2024)
    env = vg.Environment.from_scene(scene)
    blocks = torch.zeros(len(a), dtype=torch.int32, device="cuda")
    gpu = vg.panda.validate_motion_batch(torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda(), env, 32,
                                         blocks=blocks).cpu().numpy()
    cpu, cpu_blocks = port.env(scene).validate_motions(rb, a, b, 32, threads=THREADS)
    assert np.array_equal(gpu, cpu)
    assert np.array_equal(blocks.cpu().numpy(), cpu_blocks)
    assert 0.3 <= 1 - gpu.mean() <= 0.5


@pytest.mark.parametrize("robot", ["panda", "baxter"])
def test_four_lane_exact_sqrt_mode_is_the_oracles(vg, port, robot):
    """The reference as built for Arm (NEON): 4-lane blocks and an exact square root."""
    from oracle.vgo import SQRT_EXACT
    from vamp_gb300 import scenes

    scene = scenes.scene_config1(6)
    rb = port.robot(robot)
    a, b = scenes.edges(rb.s_m, rb.s_a, 4096, 77)
    env = vg.Environment.from_scene(scene, lanes=4, sqrt_mode=vg.SQRT_EXACT)
    gpu = getattr(vg, robot).validate_motion_batch(a, b, env, rb.resolution)
    cpu, _ = port.env(scene, sqrt_mode=SQRT_EXACT).validate_motions(rb, a, b, rb.resolution, lanes=4, threads=THREADS)
    assert np.array_equal(gpu, cpu)
    q = scenes.configurations(rb.s_m, rb.s_a, 4096, 78)
    assert np.array_equal(getattr(vg, robot).validate_batch(q, env), port.env(scene, sqrt_mode=SQRT_EXACT).validate_states(rb, q))


def test_zero_length_edges_equal_state_checks(vg, port):
    """validate_motion(q, q) is one block of identical lanes: the state verdict."""
    from vamp_gb300 import scenes

    env = vg.Environment.from_scene(scenes.scene_config0(0))
    rb = port.robot("panda")
    q = scenes.configurations(rb.s_m, rb.s_a, 4096, 5)
    assert np.array_equal(vg.panda.validate_motion_batch(q, q, env, 32), vg.panda.validate_batch(q, env))


def test_edge_cases(vg, port):
    from vamp_gb300 import scenes

    env = vg.Environment.from_scene(scenes.scene_config1(1))
    rb = port.robot("panda")
    empty = np.zeros((0, 7), np.float32)
    assert vg.panda.validate_motion_batch(empty, empty, env).shape == (0,)
    assert vg.panda.validate_batch(empty, env).shape == (0,)
    # one edge; edges spanning the whole joint range (the longest possible)
    a = np.array([rb.s_a], np.float32)
    b = np.array([rb.s_a + rb.s_m], np.float32)
    for x, y in ((a, b), (b, a)):
        cpu, _ = port.env(scenes.scene_config1(1)).validate_motions(rb, x, y, 32)
        assert np.array_equal(vg.panda.validate_motion_batch(x, y, env, 32), cpu)
    # an empty environment: only self-collisions remain
    q = scenes.configurations(rb.s_m, rb.s_a, 2048, 9)
    none = {"spheres": np.zeros((0, 4), np.float32), "capsules": np.zeros((0, 8), np.float32),
            "cuboids": np.zeros((0, 15), np.float32), "pointclouds": []}
    assert np.array_equal(vg.panda.validate_batch(q, vg.Environment.from_scene(none)), port.env(none).validate_states(rb, q))


def test_large_environment(vg, port):
    """Hundreds of primitives (the environment image exceeds the default 48 KB of shared memory)."""
    from vamp_gb300 import scenes

    scene = scenes.primitive_scene(12, 300, 600, 150, "workspace")
    rb = port.robot("panda")
    a, b = scenes.edges(rb.s_m, rb.s_a, 2048, 13)
    gpu = vg.panda.validate_motion_batch(a, b, vg.Environment.from_scene(scene), 32)
    cpu, _ = port.env(scene).validate_motions(rb, a, b, 32, threads=THREADS)
    assert np.array_equal(gpu, cpu)


def test_bad_arguments_raise(vg):
    env = vg.Environment()
    q = np.zeros((4, 7), np.float32)
    with pytest.raises(vg.VampError):
        vg.panda.validate_motion_batch(q, q, env, resolution=0)


@pytest.mark.parametrize("lanes,sqrt_mode", [(8, 0), (4, 1)])
def test_both_edge_schedules_agree_with_the_oracle(vg, port, torch, lanes, sqrt_mode):
    """A warp per edge (consecutive blocks) and a lane-block per edge give the same verdicts
    and the same reference block counts."""
    from oracle.vgo import SQRT_EXACT, SQRT_X86
    from vamp_gb300 import scenes

    scene = scenes.scene_config1(8)
    rb = port.robot("panda")
    a, b = scenes.edges(rb.s_m, rb.s_a, 8192, 88)
    cpu, cpu_blocks = port.env(scene, sqrt_mode=SQRT_X86 if sqrt_mode == 0 else SQRT_EXACT).validate_motions(
        rb, a, b, 32, lanes=lanes, threads=THREADS)
    for schedule in (-1, 0, 1, 2, 3):
        env = vg.Environment.from_scene(scene, lanes=lanes, sqrt_mode=sqrt_mode)
        env.set_schedule(schedule)
        blocks = torch.zeros(len(a), dtype=torch.int32, device="cuda")
        gpu = vg.panda.validate_motion_batch(torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda(), env, 32,
                                             blocks=blocks).cpu().numpy()
        assert np.array_equal(gpu, cpu), schedule
        assert np.array_equal(blocks.cpu().numpy(), cpu_blocks), schedule


@pytest.mark.parametrize("lanes,sqrt_mode", [(8, 0), (4, 1)])
def test_packed_schedule_with_short_and_mixed_edges(vg, port, torch, lanes, sqrt_mode):
    """The packed schedule (free segments start the next edge) on edges of 1 to 12 blocks in
    random order, so that most warp iterations hold the end of one edge and the start of the
    next: the same verdicts and reference block counts as the oracle."""
    from oracle.vgo import SQRT_EXACT, SQRT_X86
    from vamp_gb300 import scenes

    scene = scenes.scene_config1(9)
    rb = port.robot("panda")
    a, b = scenes.edges(rb.s_m, rb.s_a, 6144, 89)
    rng = np.random.default_rng(90)
    # edge lengths 0 .. 3 rad (1 to 12 blocks at resolution 32, 8 lanes), zero-length edges included
    d = b - a
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    length = rng.uniform(0.0, 3.0, len(a)).astype(np.float32)
    length[::97] = 0.0
    b = (a + d * length[:, None]).astype(np.float32)
    cpu, cpu_blocks = port.env(scene, sqrt_mode=SQRT_X86 if sqrt_mode == 0 else SQRT_EXACT).validate_motions(
        rb, a, b, 32, lanes=lanes, threads=THREADS)
    assert 0.05 < 1.0 - cpu.mean() < 0.95
    env = vg.Environment.from_scene(scene, lanes=lanes, sqrt_mode=sqrt_mode)
    env.set_schedule(3)
    blocks = torch.zeros(len(a), dtype=torch.int32, device="cuda")
    gpu = vg.panda.validate_motion_batch(torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda(), env, 32,
                                         blocks=blocks).cpu().numpy()
    assert np.array_equal(gpu, cpu)
    assert np.array_equal(blocks.cpu().numpy(), cpu_blocks)


def _cloud(points, r_min=0.012, r_max=0.08):
    from vamp_gb300 import scenes

    return {"spheres": np.zeros((0, 4), np.float32), "capsules": np.zeros((0, 8), np.float32),
            "cuboids": np.zeros((0, 15), np.float32),
            "pointclouds": [{"points": points, "r_min": r_min, "r_max": r_max, "r_point": scenes.POINT_RADIUS}]}


def test_pointcloud_verdicts_match_reference_and_oracle(vg, port):
    g = golden("cloud_panda")
    scene = _cloud(g["points"], float(g["r"][0]), float(g["r"][1]))
    env = vg.Environment.from_scene(scene)
    penv = port.env(scene)
    rb = port.robot("panda")
    gs = vg.panda.validate_batch(g["q"], env)
    assert np.array_equal(gs, penv.validate_states(rb, g["q"]))
    assert np.array_equal(gs, g["state_verdict"])
    ge = vg.panda.validate_motion_batch(g["a"], g["b"], env, 32)
    cpu, _ = penv.validate_motions(rb, g["a"], g["b"], 32)
    assert np.array_equal(ge, cpu)
    assert np.array_equal(ge, g["edge_verdict"])


def test_pointcloud_with_primitives_is_the_oracles(vg, port, torch):
    """50,000 surface points plus the workspace primitives; states and edges."""
    from vamp_gb300 import scenes

    scene = scenes.scene_config1(3)
    scene["pointclouds"] = _cloud(scenes.surface_pointcloud(9, 50000))["pointclouds"]
    rb = port.robot("panda")
    env = vg.Environment.from_scene(scene)
    penv = port.env(scene)
    q = scenes.configurations(rb.s_m, rb.s_a, 8192, 91)
    assert np.array_equal(vg.panda.validate_batch(q, env), penv.validate_states(rb, q, threads=THREADS))
    a, b = scenes.edges(rb.s_m, rb.s_a, 4096, 92)
    blocks = torch.zeros(len(a), dtype=torch.int32, device="cuda")
    gpu = vg.panda.validate_motion_batch(torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda(), env, 32,
                                         blocks=blocks).cpu().numpy()
    cpu, cpu_blocks = penv.validate_motions(rb, a, b, 32, threads=THREADS)
    assert np.array_equal(gpu, cpu)
    assert np.array_equal(blocks.cpu().numpy(), cpu_blocks)
