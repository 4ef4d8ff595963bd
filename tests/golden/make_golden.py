"""Generates the golden fixtures in this folder from the reference's own compiled code.

The reference (CoMMALab/vamp) ships no tests and no golden vectors, so the fixtures are produced
by running the reference itself: its hot-path headers compiled from the reference checkout by
oracle/ref/Makefile (x86-64, AVX2 build, 8 lanes).  Run in a container that has the checkout:

    python tests/golden/make_golden.py --reference /path/to/vamp   (or VG_REFERENCE=/path/to/vamp)

Every fixture stores its inputs as well as the reference's outputs, so the tests need neither the
reference nor a particular random-number generator.
"""
from __future__ import annotations

import argparse
import os
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle.vgo import Port, Reference, build_reference  # noqa: E402
from vamp_gb300 import scenes  # noqa: E402

OUT = Path(__file__).resolve().parent
ROBOTS = ("panda", "ur5", "fetch", "baxter")


def scene_arrays(scene: dict) -> dict:
    return {"spheres": scene["spheres"], "capsules": scene["capsules"], "cuboids": scene["cuboids"]}


def env_dump(env) -> dict:
    return {f"kind{k}": env.objects(k) for k in range(5)}


def filter_cases() -> list:
    """Inputs of the pointcloud filter fixtures: (points, min_dist, max_range, origin, workcell
    min, workcell max, cull)."""
    rng = np.random.default_rng(81)
    org = np.array([0.0, 0.0, 0.333], np.float32)
    surf = scenes.surface_pointcloud(82, n_points=4000)
    uni = rng.uniform(-1.5, 1.5, (3000, 3)).astype(np.float32)
    grid = (rng.integers(0, 30, (4000, 3)) * 0.02 - 0.3).astype(np.float32)  # repeated points and ties
    far = (rng.uniform(-0.2, 0.2, (500, 3)) + 5.0).astype(np.float32)        # every point culled
    mixed = np.concatenate([far[:50], surf[:2000]]).astype(np.float32)       # point 0 culled
    box = lambda o, r: (o - r, o + r)  # noqa: E731
    return [
        (surf, 0.01, 1.19, org, *box(org, 1.19), True),
        (surf, 0.03, 0.9, org, *box(org, 0.9), False),
        (uni, 0.05, 0.6, org, *box(org, 0.6), False),  # points outside the mapping range
        (grid, 0.021, 1.0, org, *box(org, 1.0), True),
        (far, 0.01, 1.0, org, *box(org, 1.0), True),
        (mixed, 0.015, 1.2, org, org - np.float32(1.2), org + np.float32(0.5), True),
    ]


def filter_fixtures(ref: Reference) -> None:
    """The reference's filter_pointcloud (collision/filter.hh:176-320) on a few clouds."""
    out = {}
    for i, (pts, md, mr, o, lo, hi, cull) in enumerate(filter_cases()):
        kept = ref.filter_pointcloud(pts, md, mr, o, lo, hi, cull)
        out[f"points{i}"] = pts
        out[f"params{i}"] = np.concatenate([[md, mr], o, lo, hi, [float(cull)]]).astype(np.float32)
        out[f"kept{i}"] = kept
    np.savez_compressed(OUT / "filter.npz", **out)


def eefk_fixtures(reference: Path) -> None:
    """Robot::eefk (robots/<robot>.hh): the reference's own end-effector expressions evaluated in
    float64 on sampled configurations, as row-major 4x4 transforms."""
    from vamp_gb300.robotgen.extract import eefk_statements, evaluate

    for r in ROBOTS:
        text = (reference / "src/impl/vamp/robots" / f"{r}.hh").read_text()
        stmts = eefk_statements(text)
        rb = Port().robot(r)
        q = scenes.configurations(rb.s_m, rb.s_a, 64, 300 + len(r))
        T = np.zeros((len(q), 4, 4))
        for i, qi in enumerate(q):
            y = evaluate(stmts, qi.astype(np.float64))
            T[i, :3, 3] = [y[0], y[1], y[2]]
            T[i, :3, :3] = np.array([y[3 + k] for k in range(9)]).reshape(3, 3).T  # column-major
            T[i, 3, 3] = 1.0
        np.savez_compressed(OUT / f"eefk_{r}.npz", q=q, T=T)


def heightfield_fixtures(ref: Reference) -> None:
    """The heightfield primitive (collision/sphere_heightfield.hh:9-30) in the reference's
    sphere_environment_in_collision: blocks of one sphere repeated (single-sphere verdicts) and of
    8 different spheres, all over the grid's valid cells; and Panda configurations above the
    terrain (Robot::fkcc through validate)."""
    rng = np.random.default_rng(91)
    hf = scenes.heightfield(92)
    scene = {"spheres": np.zeros((0, 4), np.float32), "capsules": np.zeros((0, 8), np.float32),
             "cuboids": np.zeros((0, 15), np.float32), "heightfields": [hf]}
    n = 2000
    one = np.stack([rng.uniform(-0.9, 1.2, n), rng.uniform(-1.1, 1.2, n), rng.uniform(-0.2, 0.35, n),
                    rng.uniform(0.01, 0.1, n)], 1).astype(np.float32)
    mixed = np.stack([rng.uniform(-0.9, 1.2, 8 * 400), rng.uniform(-1.1, 1.2, 8 * 400),
                      rng.uniform(0.0, 0.35, 8 * 400), rng.uniform(0.01, 0.05, 8 * 400)], 1).astype(np.float32)
    renv = ref.env(scene)
    rb = Port().robot("panda")
    q = scenes.configurations(rb.s_m, rb.s_a, 1024, 93)
    np.savez_compressed(OUT / "heightfield.npz", centre=hf["centre"], scale=hf["scale"], xd=hf["xd"], yd=hf["yd"],
                        data=hf["data"], single=one, single_verdict=renv.sphere_env(np.repeat(one, 8, axis=0)),
                        mixed=mixed, mixed_verdict=renv.sphere_env(mixed), q=q,
                        state_verdict=renv.validate_states("panda", q))


def vector_fixtures(ref: Reference) -> None:
    """validate_vector (planning/validate.hh:23-63) as the planners call it: a start, a vector (an
    extension of at most 1.5 rad here) and the distance that sets the block count, half the time
    the vector's own length (float32 norm) and half the time another value."""
    for r, scene, seed in (("panda", scenes.scene_config1(5), 95), ("ur5", scenes.scene_config1(6), 96)):
        rb = Port().robot(r)
        rng = np.random.default_rng(seed)
        a, b = scenes.edges(rb.s_m, rb.s_a, 1024, seed)
        v = (b - a).astype(np.float32)
        norm = np.linalg.norm(v.astype(np.float64), axis=1)
        scale = np.minimum(1.0, 1.5 / np.maximum(norm, 1e-9))
        v = (v * scale[:, None]).astype(np.float32)
        d = np.linalg.norm(v.astype(np.float64), axis=1).astype(np.float32)
        other = rng.random(len(d)) < 0.5
        d[other] = (d[other] * rng.uniform(0.3, 2.0, other.sum())).astype(np.float32)
        verdict = ref.env(scene).validate_vectors(r, a, v, d, 32)
        np.savez_compressed(OUT / f"vectors_{r}.npz", start=a, vector=v, distance=d, verdict=verdict, **scene_arrays(scene))


def filter_self_fixtures(ref: Reference) -> None:
    """filter_self_from_pointcloud (bindings/robot_helper.hh:307-345) of a cloud around the Panda
    at a few configurations, in the 60-primitive scene."""
    rng = np.random.default_rng(97)
    scene = scenes.scene_config1(8)
    rb = Port().robot("panda")
    q = scenes.configurations(rb.s_m, rb.s_a, 4, 98)
    pts = rng.uniform([-0.8, -0.8, 0.0], [0.8, 0.8, 1.2], (6000, 3)).astype(np.float32)
    # and points around the robot's fine spheres at the first configuration, half inside reach
    sph = rb.spheres_f64(q[0].astype(np.float64))[: rb.fine]
    k = rng.integers(0, rb.fine, 3000)
    u = rng.normal(size=(3000, 3))
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    near = sph[k, :3] + u * (sph[k, 3] + 0.01 + rng.uniform(-0.01, 0.01, 3000))[:, None]
    pts = np.concatenate([pts, near.astype(np.float32)])
    renv = ref.env(scene)
    out = {"q": q, "points": pts, "radius": np.float32(0.01), **scene_arrays(scene)}
    for i, qi in enumerate(q):
        out[f"kept{i}"] = renv.filter_self("panda", pts, 0.01, qi)
    np.savez_compressed(OUT / "filter_self_panda.npz", **out)


def scene_inputs(scene: dict) -> list:
    """The arrays that define a scene, in a fixed order (for input_digest)."""
    out = [scene.get(k, np.zeros((0, 1), np.float32)) for k in ("spheres", "capsules", "cuboids")]
    out += [pc["points"] for pc in scene.get("pointclouds", [])]
    return out


def full_fixtures(ref: Reference) -> None:
    """The reference's verdicts (and blocks checked per edge) on the benchmark configurations at
    full size: config 0 (4,096 states), config 1 (65,536 edges at resolution 32) and config 2
    (1,048,576 states and 16,384 edges against a 50,000-point cloud).  Only the inputs' digest is
    stored; the tests regenerate the inputs from their seeds (vamp_gb300.scenes.workload_config*)."""
    rb = Port().robot("panda")
    threads = os.cpu_count() or 1
    scene, q = scenes.workload_config0(rb.s_m, rb.s_a)
    v = ref.env(scene).validate_states("panda", q, threads)
    np.savez_compressed(OUT / "full_config0.npz", digest=scenes.input_digest(*scene_inputs(scene), q),
                        verdict=np.packbits(v), n=len(q))
    scene, a, b = scenes.workload_config1(rb.s_m, rb.s_a)
    v, blocks = ref.env(scene).validate_motions_counted("panda", a, b, 32, threads)
    np.savez_compressed(OUT / "full_config1.npz", digest=scenes.input_digest(*scene_inputs(scene), a, b),
                        verdict=np.packbits(v), blocks=blocks.astype(np.uint16), n=len(a), resolution=32)
    from vamp_gb300.robots import model

    m = model("panda")
    scene, q, a, b = scenes.workload_config2(rb.s_m, rb.s_a, m["min_radius"], m["max_radius"])
    renv = ref.env(scene)
    sv = renv.validate_states("panda", q, threads)
    ev, blocks = renv.validate_motions_counted("panda", a, b, 32, threads)
    np.savez_compressed(OUT / "full_config2.npz", digest=scenes.input_digest(*scene_inputs(scene), q, a, b),
                        state_verdict=np.packbits(sv), n_states=len(q), edge_verdict=np.packbits(ev),
                        blocks=blocks.astype(np.uint16), n_edges=len(a), resolution=32)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("VG_REFERENCE"),
                    help="the reference checkout (default: $VG_REFERENCE)")
    ap.add_argument("--only", choices=["filter", "eefk", "heightfield", "vectors", "filter_self", "full"], default=None,
                    help="regenerate one group of fixtures")
    a = ap.parse_args()
    if not a.reference:
        raise SystemExit("name the reference checkout with --reference or VG_REFERENCE")
    if build_reference(a.reference) is None:
        raise SystemExit("reference checkout not found (or not x86-64): cannot generate golden fixtures")
    ref = Reference()
    port = Port()
    if a.only in (None, "filter"):
        filter_fixtures(ref)
    if a.only in (None, "eefk"):
        eefk_fixtures(Path(a.reference))
    if a.only in (None, "heightfield"):
        heightfield_fixtures(ref)
    if a.only in (None, "vectors"):
        vector_fixtures(ref)
    if a.only in (None, "filter_self"):
        filter_self_fixtures(ref)
    if a.only in (None, "full"):
        full_fixtures(ref)
    if a.only is not None:
        return

    # --- forward kinematics: fine sphere centres (Robot::sphere_fk)
    for r in ROBOTS:
        rb = port.robot(r)
        q = scenes.configurations(rb.s_m, rb.s_a, 32, 100 + len(r))
        sph = np.stack([ref.sphere_fk(r, qi, rb.fine) for qi in q])
        np.savez_compressed(OUT / f"fk_{r}.npz", q=q, spheres=sph)

    # --- per-configuration verdicts (validate(q): validate_motion(q, q) at resolution 1)
    cases = [
        ("states_panda_scene0", "panda", scenes.scene_config0(0), 2048, 11),
        ("states_panda_scene1", "panda", scenes.scene_config1(1), 2048, 12),
        ("states_ur5_scene1", "ur5", scenes.scene_config1(2), 1024, 13),
        ("states_fetch_scene1", "fetch", scenes.scene_config1(3), 1024, 14),
        ("states_baxter_scene1", "baxter", scenes.scene_config1(4), 1024, 15),
    ]
    for name, r, scene, n, seed in cases:
        rb = port.robot(r)
        q = scenes.configurations(rb.s_m, rb.s_a, n, seed)
        renv = ref.env(scene)
        verdict = renv.validate_states(r, q)
        np.savez_compressed(OUT / f"{name}.npz", q=q, verdict=verdict, **scene_arrays(scene), **env_dump(renv))

    # --- per-edge verdicts (validate_motion<Robot, 8, resolution>)
    cases = [
        ("edges_panda_scene1_res32", "panda", scenes.scene_config1(1), 2048, 21, 32),
        ("edges_panda_scene0_res1", "panda", scenes.scene_config0(0), 1024, 22, 1),
        ("edges_panda_scene1_res8", "panda", scenes.scene_config1(5), 1024, 23, 8),
        ("edges_ur5_scene1_res32", "ur5", scenes.scene_config1(2), 512, 24, 32),
        ("edges_fetch_scene1_res32", "fetch", scenes.scene_config1(3), 512, 25, 32),
        ("edges_baxter_scene1_res64", "baxter", scenes.scene_config1(4), 256, 26, 64),
    ]
    for name, r, scene, n, seed, res in cases:
        rb = port.robot(r)
        ea, eb = scenes.edges(rb.s_m, rb.s_a, n, seed)
        renv = ref.env(scene)
        verdict = renv.validate_motions(r, ea, eb, res)
        np.savez_compressed(OUT / f"{name}.npz", a=ea, b=eb, resolution=res, verdict=verdict, **scene_arrays(scene))

    # --- the exact states validate_motion visits, in order (planning/validate.hh:24-67)
    rb = port.robot("panda")
    ea, eb = scenes.edges(rb.s_m, rb.s_a, 16, 31)
    counts, blocks = [], []
    for i in range(len(ea)):
        n, blk = ref.motion_blocks("panda", ea[i], eb[i], 32, cap=512, dim=7)
        counts.append(n)
        blocks.append(blk.transpose(0, 2, 1))  # [block][lane][dim]
    np.savez_compressed(
        OUT / "motion_blocks_panda.npz", a=ea, b=eb, counts=np.array(counts), blocks=np.concatenate(blocks)
    )

    # --- the 8-lane sqrt of the early-exit bound, and the lane sin/cos
    rng = np.random.default_rng(41)
    v = np.concatenate(
        [rng.uniform(0, 4, 4096), rng.uniform(0, 1e-3, 1024), 10.0 ** rng.uniform(-30, 30, 1024), [0.0] * 8]
    ).astype(np.float32)
    v = v[: len(v) // 8 * 8]
    out = np.zeros_like(v)
    for i in range(0, len(v), 8):
        x = np.ascontiguousarray(v[i : i + 8])
        o = np.zeros(8, np.float32)
        ref.lib.vgref_vec_sqrt8(x.ctypes.data_as(__import__("ctypes").c_void_p), o.ctypes.data_as(__import__("ctypes").c_void_p))
        out[i : i + 8] = o
    ang = rng.uniform(-3.2, 3.9, 4096).astype(np.float32)
    s = np.zeros_like(ang)
    c = np.zeros_like(ang)
    import ctypes

    for i in range(0, len(ang), 8):
        x = np.ascontiguousarray(ang[i : i + 8])
        so = np.zeros(8, np.float32)
        co = np.zeros(8, np.float32)
        ref.lib.vgref_vec_sincos8(x.ctypes.data_as(ctypes.c_void_p), so.ctypes.data_as(ctypes.c_void_p), co.ctypes.data_as(ctypes.c_void_p))
        s[i : i + 8] = so
        c[i : i + 8] = co
    np.savez_compressed(OUT / "lane_math.npz", sqrt_in=v, sqrt_out=out, angle=ang, sin=s, cos=c)

    # --- CAPT layout of a small surface cloud (collision/capt.hh:294-365)
    pts = scenes.surface_pointcloud(51, n_points=3000)
    lay = ref.capt(pts, 0.012, 0.08, scenes.POINT_RADIUS)
    np.savez_compressed(OUT / "capt_layout.npz", points=pts, r=np.array([0.012, 0.08, scenes.POINT_RADIUS], np.float32), **lay)

    # --- pointcloud scenes: verdicts through the reference's CAPT (capt.hh:425-506)
    rb = port.robot("panda")
    cloud = scenes.surface_pointcloud(61, n_points=10000)
    scene = {"spheres": np.zeros((0, 4), np.float32), "capsules": np.zeros((0, 8), np.float32),
             "cuboids": np.zeros((0, 15), np.float32),
             "pointclouds": [{"points": cloud, "r_min": 0.012, "r_max": 0.08, "r_point": scenes.POINT_RADIUS}]}
    renv = ref.env(scene)
    q = scenes.configurations(rb.s_m, rb.s_a, 1024, 62)
    sv = renv.validate_states("panda", q)
    ea, eb = scenes.edges(rb.s_m, rb.s_a, 512, 63)
    ev = renv.validate_motions("panda", ea, eb, 32)
    np.savez_compressed(OUT / "cloud_panda.npz", points=cloud, r=np.array([0.012, 0.08, scenes.POINT_RADIUS], np.float32),
                        q=q, state_verdict=sv, a=ea, b=eb, edge_verdict=ev)

    # --- per-sphere collision reports (Robot::fkcc_debug, robots/panda.hh:468; the binding's debug())
    from vamp_gb300.robots import model as robot_model

    for r, scene, seed in (("panda", scenes.scene_config0(3), 71), ("baxter", scenes.scene_config1(3), 72)):
        rb = port.robot(r)
        q = scenes.configurations(rb.s_m, rb.s_a, 256, seed)
        renv = ref.env(scene)
        n_obj = len(scene["spheres"]) + len(scene["capsules"]) + len(scene["cuboids"])
        bits, pair_lists = renv.debug(r, q, rb.fine, n_obj)
        order = {tuple(p): i for i, p in enumerate(p for e in robot_model(r)["self_checks"] for p in e["fine"])}
        pairs = np.zeros((len(q), len(order)), np.uint8)
        for i, lst in enumerate(pair_lists):
            for pr in lst:
                pairs[i, order[pr]] = 1
        np.savez_compressed(OUT / f"debug_{r}.npz", q=q, env_bits=bits, pairs=pairs, **scene_arrays(scene))

    print("golden fixtures written to", OUT)


if __name__ == "__main__":
    main()
