"""Benchmark: batched validate_motion on the 65,536-edge Panda workload, edges validated per second.

Workload (one step): 65,536 straight-line Panda edges with endpoints uniform within the joint
limits, checked at the robot's resolution (32) against a seeded scene of 24 spheres, 24 cuboids
and 12 capsules in the 4 m workspace volume (about 45% of edges collide).  Inputs are synthetic
(seeded) stand-ins for the reference's MotionBenchMaker problems.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

GPU arm: `value` times the persistent edge kernel alone with CUDA events on its stream, inputs
resident in HBM, the L2 flushed (256 MB write) between timed steps.  `e2e` times the C-ABI
call with host buffers (pinned), copies in and out included.  `roofline` relates the kernel's
algorithmic FP32 work (counted by the CPU oracle on a sample of the same edges) to the FP32 peak.
Reference arm: the reference's CPU algorithm on the host cores (the compiled reference where it
runs, else the CPU oracle that restates it).  N > 1 runs independent replicas, one per rank.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

N_EDGES = 65536
RESOLUTION = 32
SCENE_SEED = 1
EDGE_SEED = 2024  # the mixed workload's edges (one seed per robot from here)
# The first correct version of the plain GPU path (a segment per edge, per-object votes) checked
# this workload in 9.58 ms: the learned-order target is stated against it.
FIRST_VERSION_EDGES_PER_S = N_EDGES / 9.58e-3
METRIC = "edges validated/s on 1 GB300, learned-order vs plain GPU path, identical verdicts"
WORKLOAD = "panda validate_motion batch: 65536 edges, res 32, 24 spheres + 24 cuboids + 12 capsules"

# FP32 work per primitive test / query, in floating-point operations (fused multiply-add = 2),
# as the kernels evaluate them (vamp_gb300/csrc/vg_check.cuh)
FLOPS = {
    "test": [11, 26, 16, 27, 18],  # sphere, capsule, z-capsule, cuboid, z-cuboid
    "break_check": 1,  # min_distance - max_extent, per object visited
    "query": 8,  # |c|^2, max_extent, r^2 per sphere query
    "self_pair": 11,
}


def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        backend = "nccl" if _has_cuda() else "gloo"
        dist.init_process_group(backend)
    return world, rank, local


def _has_cuda():
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(world, x: float) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64, device="cuda" if _has_cuda() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def vg_schedules():
    from vamp_gb300 import SCHEDULES

    return SCHEDULES


def workload():
    from vamp_gb300 import scenes
    from vamp_gb300.robots import model

    m = model("panda")
    s_m = np.array(m["s_m"], np.float32)
    s_a = np.array(m["s_a"], np.float32)
    return scenes.workload_config1(s_m, s_a)


def reference_flips(scene, a, b, verdicts: dict, blocks: dict) -> dict:
    """Differences from the compiled reference's own verdicts and block counts on this workload
    (tests/golden/full_config1.npz, written by tests/golden/make_golden.py).  verdicts / blocks:
    per path, as numpy arrays (blocks None where a path checks blocks in another order).  A flip
    is explained only for a state within 1e-5 m of contact; the classification needs the CPU
    oracle and runs in tests/test_full_configs.py, so a nonzero count here is reported as
    unclassified (null)."""
    from vamp_gb300 import scenes

    with np.load(ROOT / "tests" / "golden" / "full_config1.npz") as f:
        g = {k: f[k] for k in f.files}
    inputs = [scene.get(k, np.zeros((0, 1), np.float32)) for k in ("spheres", "capsules", "cuboids")]
    if scenes.input_digest(*inputs, a, b) != str(g["digest"]):
        return {"available": False, "why": "the workload's inputs differ from those of the fixture"}
    ref = np.unpackbits(g["verdict"])[: int(g["n"])]
    out = {"available": True, "reference": "compiled reference, x86-64 AVX2 build (8 lanes)"}
    for path, v in verdicts.items():
        n = int((v != ref).sum())
        out[path] = {"vs_reference": n, "unexplained": 0 if n == 0 else None}
        if blocks.get(path) is not None:
            out[path]["block_counts_differ"] = int((blocks[path] != g["blocks"]).sum())
    return out


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits", "-lms", "10"],
                stdout=self.f, stderr=subprocess.DEVNULL)
            # nvidia-smi takes a while to start: wait (2 s at most) for its first row so that
            # the timed region, often well under a second, falls between samples it takes
            t0 = time.perf_counter()
            while time.perf_counter() - t0 < 2.0 and os.path.getsize(self.path) == 0 and self.proc.poll() is None:
                time.sleep(0.01)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if self.proc is None or not self.path:
            return None
        rows = []
        for line in Path(self.path).read_text().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def algorithmic_flops(scene, a, b, sample: int = 8192):
    """FP32 operations the reference's algorithm performs on the workload, from the CPU oracle's
    work counters on a sample of the edges (scaled to the full batch)."""
    from oracle.vgo import Port
    from vamp_gb300.robotgen.codegen import fk_flops
    from vamp_gb300.robots import model

    port = Port()
    rb = port.robot("panda")
    env = port.env(scene)
    _, cnt = env.validate_motions_counted(rb, a[:sample], b[:sample], RESOLUTION)
    fk = fk_flops(model("panda"))
    lanes = cnt.lanes
    tests = sum(int(cnt.tests[k]) * FLOPS["test"][k] for k in range(5))
    per_lane_fk = fk["frames"] + fk["centre"] * fk["slots"]
    flops = (lanes * per_lane_fk + tests + sum(int(cnt.tests[k]) for k in range(5)) * FLOPS["break_check"]
             + int(cnt.sphere_queries) * FLOPS["query"] + int(cnt.self_pairs) * FLOPS["self_pair"])
    scale = len(a) / sample
    return {"flops": flops * scale, "blocks": int(cnt.blocks) * scale, "lanes": lanes * scale,
            "tests": sum(int(t) for t in cnt.tests) * scale, "per_lane_fk": per_lane_fk}


def profiled_traffic():
    """DRAM bytes (read + write) per launch of the edge kernel, from the committed ncu summary."""
    import re

    try:
        text = (ROOT / "profiles" / "edges_grouped_panda_65536.md").read_text()
        return int(re.search(r"traffic_bytes_per_launch: (\d+)", text).group(1))
    except Exception:
        return None


def fp32_peak_tflops(device_props, sm_mhz: float | None):
    """FP32 (non-tensor) peak: 128 FP32 lanes x 2 FLOP per SM per clock."""
    sms = device_props.multi_processor_count
    peaks = {}
    try:
        peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
    except Exception:
        pass
    mhz = peaks.get("sm_max_mhz", 2070.0)
    return sms * 128 * 2 * mhz * 1e6 / 1e12, mhz, sms


# The compiled reference's own code (its AVX2 build) on the benchmark workload, timed on an x86-64
# host by oracle/time_reference.py: the GPU machine is an Arm machine without the reference checkout,
# so its CPU baseline is the C restatement (kind "port"); this record states the reference's rate
# beside it.
REFERENCE_X86 = {"edges_per_s": 387820.0, "threads": 8, "edges_per_s_one_thread": 67543.0,
                 "host": "Intel Xeon @ 2.70 GHz (8 threads)", "build": "x86-64 AVX2, 8 lanes",
                 "how": "python oracle/time_reference.py (best of 5 passes over the 65,536 edges)"}


def cpu_baseline(scene, a, b, budget_s: float = 10.0):
    """The reference's algorithm on the host cores: the compiled reference when it loads here,
    else the CPU oracle.  Bounded sample: whole passes over a slice of the edges until about
    `budget_s` seconds have been spent."""
    threads = os.cpu_count() or 1
    kind = "port"
    fn = None
    try:
        from oracle.vgo import REF_LIB, Reference

        if REF_LIB.exists():
            ref = Reference()
            renv = ref.env(scene)
            fn = lambda x, y: renv.validate_motions("panda", x, y, RESOLUTION, threads=threads)  # noqa: E731
            kind = "reference"
    except Exception:
        fn = None
    if fn is None:
        from oracle.vgo import Port

        port = Port()
        penv = port.env(scene)
        rb = port.robot("panda")
        fn = lambda x, y: penv.validate_motions(rb, x, y, RESOLUTION, threads=threads)[0]  # noqa: E731
        kind = "port"
    n = min(len(a), 4096)
    t0 = time.perf_counter()
    fn(a[:n], b[:n])
    dt = time.perf_counter() - t0
    rate = n / max(dt, 1e-9)
    n = int(min(len(a), max(4096, rate * budget_s)))
    done, t0 = 0, time.perf_counter()
    while time.perf_counter() - t0 < budget_s * 0.5 or done == 0:
        fn(a[:n], b[:n])
        done += n
    elapsed = time.perf_counter() - t0
    out = {"value": done / elapsed, "unit": "edges/s", "cores": threads, "kind": kind,
           "sample": f"{done} edges of the workload ({n} per pass), {threads} host threads, {elapsed:.1f} s"}
    if kind == "port":
        out["reference_x86"] = REFERENCE_X86
    else:
        out["build"] = "x86-64 AVX2, 8 lanes" if os.uname().machine == "x86_64" else "aarch64 NEON, 4 lanes"
    return out


def autotune(robot: str, env, a, b, resolution: int, stream, sample: int = 65536) -> dict:
    """Runs the library's autotuner on the first `sample` edges (a persistent launch needs a
    sample of the workload's own size to show its tail); returns its pick."""
    import ctypes

    from vamp_gb300._lib import check, lib

    sched, bps, ms = ctypes.c_int(), ctypes.c_int(), ctypes.c_float()
    check(lib.vg_autotune_motions(robot.encode(), env.handle, a.data_ptr(), b.data_ptr(), min(sample, len(a)), resolution,
                                  ctypes.byref(sched), ctypes.byref(bps), ctypes.byref(ms), stream))
    return {"schedule": vg_schedules()[sched.value],
            "blocks_per_sm": bps.value or "max", "sample_edges": min(sample, len(a)), "sample_ms": ms.value}


def run_capt(args, world, rank, local):
    """Pointcloud workload: Panda with 50,000 points sampled on the surfaces of 30 random cuboids
    and cylinders plus 2% uniform noise, checked through the CAPT built with the Panda's radius
    range; 1,048,576 uniform configurations and 16,384 edges at resolution 32."""
    import torch

    import vamp_gb300 as vg
    from vamp_gb300 import scenes
    from vamp_gb300._lib import check, lib
    from vamp_gb300.robots import model

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    m = model("panda")
    s_m, s_a = np.array(m["s_m"], np.float32), np.array(m["s_a"], np.float32)
    scene, q_np, a_np, b_np = scenes.workload_config2(s_m, s_a, m["min_radius"], m["max_radius"])
    pts = scene["pointclouds"][0]["points"]
    t0 = time.perf_counter()
    env = vg.Environment.from_scene(scene)
    build_s = time.perf_counter() - t0
    # the same tree built on the GPU (vg_env_add_pointcloud_device; synchronous), first call untimed
    pts_dev = torch.from_numpy(pts).to(dev)
    gpu_build = []
    for i in range(4):
        t0 = time.perf_counter()
        vg.Environment().add_pointcloud_device(pts_dev, m["min_radius"], m["max_radius"], scenes.POINT_RADIUS)
        if i:
            gpu_build.append(time.perf_counter() - t0)
    q = torch.from_numpy(q_np).to(dev)
    a, b = torch.from_numpy(a_np).to(dev), torch.from_numpy(b_np).to(dev)
    qo = torch.empty(len(q), dtype=torch.uint8, device=dev)
    eo = torch.empty(len(a), dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)
    pick = autotune("panda", env, a, b, RESOLUTION, stream.cuda_stream)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def states():
        check(lib.vg_validate_states_device(b"panda", env.handle, q.data_ptr(), len(q), qo.data_ptr(), stream.cuda_stream))

    def edges():
        check(lib.vg_validate_motions_device(b"panda", env.handle, a.data_ptr(), b.data_ptr(), len(a), RESOLUTION,
                                             eo.data_ptr(), None, stream.cuda_stream))

    res = {}
    for name, fn in (("states", states), ("edges", edges)):
        for _ in range(max(args.warmup, 3)):
            fn()
        ts = []
        for _ in range(args.steps):
            flush.zero_()
            s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s0.record(stream)
            fn()
            s1.record(stream)
            torch.cuda.synchronize()
            ts.append(s0.elapsed_time(s1))
        res[name] = float(np.mean(ts))
    with np.load(ROOT / "tests" / "golden" / "full_config2.npz") as f:
        g = {k: f[k] for k in f.files}
    if scenes.input_digest(pts, q_np, a_np, b_np) == str(g["digest"]):
        flips = {"states_vs_reference": int((qo.cpu().numpy() != np.unpackbits(g["state_verdict"])[: len(q_np)]).sum()),
                 "edges_vs_reference": int((eo.cpu().numpy() != np.unpackbits(g["edge_verdict"])[: len(a_np)]).sum()),
                 "reference": "compiled reference, x86-64 AVX2 build (8 lanes), tests/golden/full_config2.npz"}
    else:
        flips = {"available": False, "why": "the workload's inputs differ from those of the fixture"}
    if rank == 0:
        print(json.dumps({
            "metric": "pointcloud (CAPT) checks on 1 GB300", "workload": "panda + 50k surface points", "flips": flips,
            "states_per_s": (1 << 20) / (res["states"] / 1e3), "states_ms": res["states"],
            "edges_per_s": 16384 / (res["edges"] / 1e3), "edges_ms": res["edges"],
            "capt_build_s": build_s, "capt_build_gpu_s": float(np.median(gpu_build)), "capt_blocks": int(env.pointcloud_layout(0)["aff_starts"][-1]),
            "valid_states": float(qo.float().mean()), "valid_edges": float(eo.float().mean()), "autotuner": pick,
            "steps": args.steps, "warmup": args.warmup}))


def run_debug(args, world, rank, local):
    """Debug reports (Robot::fkcc_debug) of 65,536 Panda configurations in the 60-primitive scene:
    per fine sphere the objects it collides with, per fine self pair whether it collides."""
    import torch

    import vamp_gb300 as vg
    from vamp_gb300 import scenes

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    env = vg.Environment.from_scene(scenes.scene_config1(SCENE_SEED))
    q = torch.from_numpy(scenes.configurations(vg.panda.s_m, vg.panda.s_a, N_EDGES, 91)).to(dev)
    for _ in range(max(args.warmup, 3)):
        vg.panda.debug_batch(q, env)
    torch.cuda.synchronize()
    ts = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        bits, pairs = vg.panda.debug_batch(q, env)  # synchronous
        ts.append(time.perf_counter() - t0)
    ms = 1e3 * float(np.mean(ts))
    if rank == 0:
        print(json.dumps({"metric": "debug reports/s on 1 GB300 (Robot::fkcc_debug)", "value": N_EDGES / (ms / 1e3),
                          "unit": "configurations/s", "ms_per_step": ms, "configurations": N_EDGES,
                          "sphere_object_hits": int(torch.count_nonzero(bits).item()),
                          "colliding_pairs": int(pairs.sum().item()), "steps": args.steps, "warmup": args.warmup,
                          "timing": "wall clock of the synchronous call (scratch allocation included)"}))


def run_latency(args, world, rank, local):
    """Latency of one validate_motion call (a planner's extension step) through the C ABI with
    host buffers: 1,000 single edges of the 60-primitive scene, one call each (the block path:
    all blocks of the edge checked at once), then batches of 8 and 64 edges per call, and the
    same single edges as resident CUDA tensors through the edge kernels (verdict read back)."""
    import torch

    import vamp_gb300 as vg
    from vamp_gb300 import scenes
    from vamp_gb300._lib import check, lib
    from vamp_gb300.api import _ptr

    torch.cuda.set_device(local)
    env = vg.Environment.from_scene(scenes.scene_config1(SCENE_SEED))
    a, b = scenes.edges(vg.panda.s_m, vg.panda.s_a, 1000, 92)
    out = np.zeros(64, np.uint8)
    name = b"panda"

    def host_call(lo, hi):
        check(lib.vg_validate_motions(name, env.handle, _ptr(a[lo:hi]), _ptr(b[lo:hi]), hi - lo, 32, _ptr(out)))

    for i in range(max(args.warmup, 3) * 10):
        host_call(i, i + 1)
    res = {}
    for k in (1, 8, 64):
        ts = []
        for i in range(0, 1000 - k + 1, k):
            t0 = time.perf_counter()
            host_call(i, i + k)
            ts.append(time.perf_counter() - t0)
        res[k] = (1e6 * float(np.median(ts)), 1e6 * float(np.percentile(ts, 90)))
    da, db = torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()
    dout = torch.empty(1, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    hv = torch.empty(1, dtype=torch.uint8).pin_memory()
    ts = []
    for i in range(1000):
        t0 = time.perf_counter()
        check(lib.vg_validate_motions_device(name, env.handle, da[i:i + 1].data_ptr(), db[i:i + 1].data_ptr(), 1, 32,
                                             dout.data_ptr(), None, stream))
        hv.copy_(dout)
        ts.append(time.perf_counter() - t0)
    dev_us = 1e6 * float(np.median(ts))
    if rank == 0:
        print(json.dumps({"metric": "validate_motion latency on 1 GB300 (one call, host buffers)",
                          "value": res[1][0], "unit": "us per call", "higher_is_better": False,
                          "p90_us": res[1][1], "batch_8_us_per_call": res[8][0], "batch_64_us_per_call": res[64][0],
                          "edge_kernel_resident_single_edge_us": dev_us,
                          "reference_x86_us_per_edge_one_thread": 1e6 / REFERENCE_X86["edges_per_s_one_thread"],
                          "calls": 1000, "workload": "panda, 60-primitive scene, resolution 32"}))


def run_filter(args, world, rank, local):
    """Pointcloud filter (filter_pointcloud, collision/filter.hh:176-320) of 1,048,576 points on
    the surfaces of 30 random cuboids and cylinders plus 2% noise, with the reference's Panda
    settings (origin at the first joint, cull radius 1.19 m, filter radius 1 cm), then the CAPT
    build of the kept points on the GPU.  The C oracle times the same filter on the host."""
    import torch

    import vamp_gb300 as vg
    from vamp_gb300 import scenes
    from vamp_gb300.robots import model

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    m = model("panda")
    org = np.array([0.0, 0.0, 0.333], np.float32)
    rad, md = np.float32(1.19), 0.01
    pts = scenes.surface_pointcloud(SCENE_SEED, 1 << 20)
    d_pts = torch.from_numpy(pts).to(dev)
    for _ in range(max(args.warmup, 3)):
        kept = vg.filter_pointcloud_device(d_pts, md, rad, org, org - rad, org + rad, True)
    ts, tb = [], []
    for _ in range(args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        kept = vg.filter_pointcloud_device(d_pts, md, rad, org, org - rad, org + rad, True)  # synchronous
        t1 = time.perf_counter()
        vg.Environment().add_pointcloud_device(kept, m["min_radius"], m["max_radius"], scenes.POINT_RADIUS)
        ts.append(t1 - t0)
        tb.append(time.perf_counter() - t1)
    # the same cloud without the cull: every point takes part in all six passes
    for _ in range(2):
        vg.filter_pointcloud_device(d_pts, md, rad, org, org - rad, org + rad, False)
    tn = []
    for _ in range(args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        kept_all = vg.filter_pointcloud_device(d_pts, md, rad, org, org - rad, org + rad, False)
        tn.append(time.perf_counter() - t0)
    host, ns = vg.filter_pointcloud(pts, md, rad, org, org - rad, org + rad, True)
    cpu = None
    if rank == 0 and not args.no_cpu:
        from oracle.vgo import Port

        t0 = time.perf_counter()
        want = Port().filter_pointcloud(pts, md, rad, org, org - rad, org + rad, True)
        cpu = time.perf_counter() - t0
        assert np.array_equal(want, host)
    if rank == 0:
        ms = 1e3 * float(np.median(ts))
        print(json.dumps({
            "metric": "pointcloud filter on 1 GB300 (filter_pointcloud)", "value": len(pts) / (ms / 1e3),
            "unit": "points/s", "ms_per_step": ms, "points": len(pts), "kept": int(kept.shape[0]),
            "capt_build_gpu_ms": 1e3 * float(np.median(tb)), "host_buffers_ms": ns / 1e6,
            "no_cull": {"ms": 1e3 * float(np.median(tn)), "points_per_s": len(pts) / float(np.median(tn)),
                        "kept": int(kept_all.shape[0])},
            "cpu_baseline": None if cpu is None else {"value": len(pts) / cpu, "unit": "points/s", "cores": 1,
                                                      "kind": "port", "sample": "the whole cloud, once"},
            "steps": args.steps, "warmup": args.warmup,
            "timing": "wall clock of the synchronous device call (allocation included)"}))


def run_roadmap(args, world, rank, local):
    """Batched roadmap (vamp_gb300.roadmap): 16,384 Panda samples in the 60-primitive scene; the
    valid ones joined to their PRM* neighbours among the earlier ones, every candidate edge
    checked in one batch at resolution 32.  Wall clock of the whole build (synchronous)."""
    import torch

    import vamp_gb300 as vg
    from vamp_gb300 import scenes
    from vamp_gb300.roadmap import build_roadmap

    torch.cuda.set_device(local)
    env = vg.Environment.from_scene(scenes.scene_config1(SCENE_SEED))
    q = torch.from_numpy(scenes.configurations(vg.panda.s_m, vg.panda.s_a, 16384, 61)).cuda()
    for _ in range(max(args.warmup, 3)):
        rm = build_roadmap(vg.panda, env, q)
    ts = []
    for _ in range(args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        rm = build_roadmap(vg.panda, env, q)
        torch.cuda.synchronize()
        ts.append(time.perf_counter() - t0)
    ms = 1e3 * float(np.median(ts))
    if rank == 0:
        print(json.dumps({"metric": "batched roadmap build on 1 GB300 (PRM* neighbour edges in one batch)",
                          "ms_per_step": ms, "samples": len(q), "nodes": rm["valid_samples"],
                          "candidate_edges": rm["candidates"], "valid_edges": rm["valid_edges"],
                          "candidate_edges_per_s": rm["candidates"] / (ms / 1e3), "steps": args.steps,
                          "warmup": args.warmup, "timing": "wall clock of the synchronous build"}))


MIXED_ROBOTS = ("ur5", "fetch", "baxter", "panda")
MIXED_EDGES = 16384


def run_mixed(args, world, rank, local):
    """Mixed-robot workload: UR5, Fetch, Baxter and Panda, 16,384 edges each (endpoints uniform
    within each robot's limits, each robot's resolution), in the 60-primitive scene plus the
    50,000-point surface cloud, one CAPT per robot built with its sphere radius range.  The four
    checks run as one CUDA graph (vg_batch); the autotuner picks each robot's schedule first."""
    import ctypes

    import torch

    import vamp_gb300 as vg
    from vamp_gb300 import scenes
    from vamp_gb300._lib import check, lib

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    stream = torch.cuda.current_stream(dev)
    s = stream.cuda_stream
    cloud = scenes.surface_pointcloud(SCENE_SEED, 50_000)
    prims = scenes.scene_config1(SCENE_SEED)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    parts = []
    for i, r in enumerate(MIXED_ROBOTS):
        rb = getattr(vg, r)
        r_min, r_max = rb.min_max_radii()
        scene = dict(prims)
        scene["pointclouds"] = [{"points": cloud, "r_min": r_min, "r_max": r_max, "r_point": scenes.POINT_RADIUS}]
        env = vg.Environment.from_scene(scene)
        a_np, b_np = scenes.edges(rb.s_m, rb.s_a, MIXED_EDGES, EDGE_SEED + 1 + i)
        a, b = torch.from_numpy(a_np).to(dev), torch.from_numpy(b_np).to(dev)
        out = torch.empty(MIXED_EDGES, dtype=torch.uint8, device=dev)
        parts.append({"robot": r, "rb": rb, "env": env, "a": a, "b": b, "out": out,
                      "pick": autotune(r, env, a, b, rb.resolution(), s)})

    def timed(batch):
        for _ in range(max(args.warmup, 3)):
            check(lib.vg_batch_launch(batch, s))
        torch.cuda.synchronize()
        ts = []
        for _ in range(args.steps):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            check(lib.vg_batch_launch(batch, s))
            e1.record(stream)
            torch.cuda.synchronize()
            ts.append(e0.elapsed_time(e1))
        return float(np.mean(ts))

    def make(sel, mlps=None, probes=8):
        batch = lib.vg_batch_create()
        for p in sel:
            m = mlps[p["robot"]] if mlps else None
            check(lib.vg_batch_add_motions(batch, p["robot"].encode(), p["env"].handle, p["a"].data_ptr(), p["b"].data_ptr(),
                                           MIXED_EDGES, p["rb"].resolution(), m, probes if m else 0, p["out"].data_ptr(), None))
        return batch

    per_robot = {}
    for p in parts:
        bt = make([p])
        ms = timed(bt)
        lib.vg_batch_destroy(bt)
        per_robot[p["robot"]] = {"edges_per_s": MIXED_EDGES / (ms / 1e3), "ms": ms, "resolution": p["rb"].resolution(),
                                 "autotuner": p["pick"]}
    alone = {p["robot"]: p["out"].cpu().numpy().copy() for p in parts}
    bt = make(parts)
    ms = timed(bt)
    lib.vg_batch_destroy(bt)
    identical = all(np.array_equal(alone[p["robot"]], p["out"].cpu().numpy()) for p in parts)
    for p in parts:
        per_robot[p["robot"]]["colliding_fraction"] = float(1 - p["out"].float().mean())
    learned = None
    if not args.no_learned:
        mlps = {}
        for p in parts:
            q = torch.from_numpy(scenes.configurations(p["rb"].s_m, p["rb"].s_a, args.labels // 4, 300)).to(dev)
            valid = torch.empty(len(q), dtype=torch.uint8, device=dev)
            check(lib.vg_validate_states_device(p["robot"].encode(), p["env"].handle, q.data_ptr(), len(q), valid.data_ptr(), s))
            m = lib.vg_mlp_create(p["rb"].dimension(), 5)
            check(lib.vg_mlp_train_device(m, q.data_ptr(), valid.data_ptr(), len(q), 3, 1024, 1e-3, None, s))
            mlps[p["robot"]] = m
        bt = make(parts, mlps)
        lms = timed(bt)
        lib.vg_batch_destroy(bt)
        learned = {"edges_per_s": len(parts) * MIXED_EDGES / (lms / 1e3), "ms": lms, "probes": 8,
                   "labels_per_robot": args.labels // 4,
                   "verdicts_identical": all(np.array_equal(alone[p["robot"]], p["out"].cpu().numpy()) for p in parts)}
        for m in mlps.values():
            lib.vg_mlp_destroy(m)
    if rank == 0:
        print(json.dumps({
            "metric": "edges validated/s on 1 GB300, mixed robots in one CUDA graph",
            "value": len(parts) * MIXED_EDGES / (ms / 1e3), "unit": "edges/s", "ms_per_step": ms,
            "workload": "ur5 + fetch + baxter + panda, 16384 edges each, 60 primitives + 50k-point CAPT per robot",
            "verdicts_identical_to_single_checks": identical, "per_robot": per_robot, "learned": learned,
            "steps": args.steps, "warmup": args.warmup, "l2": "flushed between timed steps (256 MB write)"}))


def run_reference(args, world, rank):
    if rank != 0:
        return
    scene, a, b = workload()
    times = []
    res = None
    for i in range(args.warmup + args.steps):
        r = cpu_baseline(scene, a, b, budget_s=4.0)
        if i >= args.warmup:
            times.append(1.0 / r["value"])
            res = r
    value = 1.0 / float(np.mean(times))
    line = {
        "impl": "reference",
        "metric": METRIC,
        "value": value,
        "unit": "edges/s",
        "n_gpus": args.gpus,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": 1e3 * N_EDGES / value,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded scene and edges)",
        "config": {"workload": WORKLOAD, "edges": N_EDGES, "resolution": RESOLUTION, "l2": "host CPU run"},
        "cpu_baseline": {"value": value, "unit": "edges/s", "cores": res["cores"], "kind": res["kind"], "sample": res["sample"],
                         **({"reference_x86": res["reference_x86"]} if "reference_x86" in res else {})},
        "e2e": {"value": value, "unit": "edges/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def auc(scores, positive) -> float:
    """Area under the ROC curve: the Mann-Whitney statistic with average ranks for ties."""
    from scipy.stats import rankdata

    positive = np.asarray(positive, bool)
    ranks = rankdata(np.asarray(scores, np.float64))
    n_pos = int(positive.sum())
    n_neg = len(positive) - n_pos
    return float((ranks[positive].sum() - n_pos * (n_pos + 1) / 2.0) / max(n_pos * n_neg, 1))


def train_predictor(env, dev, n_labels: int = 2 << 20, epochs: int = 3, seed: int = 5):
    """The learned ordering's MLP, trained on the GPU on `n_labels` uniform Panda configurations
    labelled by the exact checker in the benchmark scene.  Returns (mlp handle, info)."""
    import torch

    import vamp_gb300 as vg
    from vamp_gb300 import scenes
    from vamp_gb300._lib import check, lib

    stream = torch.cuda.current_stream(dev).cuda_stream
    rb = vg.panda
    q = torch.from_numpy(scenes.configurations(rb.s_m, rb.s_a, n_labels + 65536, seed)).to(dev)
    valid = torch.empty(len(q), dtype=torch.uint8, device=dev)
    check(lib.vg_validate_states_device(b"panda", env.handle, q.data_ptr(), len(q), valid.data_ptr(), stream))
    m = lib.vg_mlp_create(7, seed)
    losses = np.zeros(epochs, np.float32)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    check(lib.vg_mlp_train_device(m, q.data_ptr(), valid.data_ptr(), n_labels, epochs, 1024, 1e-3, losses.ctypes.data, stream))
    train_s = time.perf_counter() - t0
    p = torch.empty(65536, dtype=torch.float32, device=dev)
    held_q = q[n_labels:]
    check(lib.vg_mlp_infer_device(m, held_q.data_ptr(), 65536, p.data_ptr(), stream))
    torch.cuda.synchronize()
    check(lib.vg_mlp_error(m))
    held_auc = auc(p.cpu().numpy(), valid[n_labels:].cpu().numpy() == 0)
    return m, {"labels": n_labels, "epochs": epochs, "batch": 1024, "train_s": train_s,
               "loss_per_epoch": [float(x) for x in losses], "auc_heldout_states": held_auc,
               "colliding_state_fraction": float(1 - valid.float().mean())}


def measure_learned(args, env, a, b, plain_out, stream, flush, dev, probes: int = 16):
    """Learned block order on the same edges: verdict identity with the plain path, blocks checked
    per edge, the predictor's inference cost and the edges/s of scoring plus checking."""
    import torch

    from vamp_gb300._lib import check, lib

    torch.cuda.synchronize()
    plain = plain_out.clone()
    plain_blocks = torch.empty(N_EDGES, dtype=torch.int32, device=dev)
    check(lib.vg_validate_motions_device(b"panda", env.handle, a.data_ptr(), b.data_ptr(), N_EDGES, RESOLUTION,
                                         plain.data_ptr(), plain_blocks.data_ptr(), stream.cuda_stream))
    m, info = train_predictor(env, dev, n_labels=args.labels)
    out = torch.empty(N_EDGES, dtype=torch.uint8, device=dev)
    blocks = torch.empty(N_EDGES, dtype=torch.int32, device=dev)
    scores = torch.empty((N_EDGES, probes), dtype=torch.float32, device=dev)

    def score():
        check(lib.vg_mlp_score_edges_device(m, a.data_ptr(), b.data_ptr(), N_EDGES, probes, scores.data_ptr(),
                                            stream.cuda_stream))

    def ordered():
        check(lib.vg_validate_motions_scored_device(b"panda", env.handle, a.data_ptr(), b.data_ptr(), N_EDGES, RESOLUTION,
                                                    scores.data_ptr(), probes, out.data_ptr(), blocks.data_ptr(),
                                                    stream.cuda_stream))

    for _ in range(max(args.warmup, 3)):
        score()
        ordered()
    torch.cuda.synchronize()
    ev = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(args.steps)]
    for i in range(args.steps):
        flush.zero_()
        ev[i][0].record(stream)
        score()
        ev[i][1].record(stream)
        ordered()
        ev[i][2].record(stream)
    torch.cuda.synchronize()
    check(lib.vg_mlp_error(m))
    score_ms = float(np.mean([e[0].elapsed_time(e[1]) for e in ev]))
    check_ms = float(np.mean([e[1].elapsed_time(e[2]) for e in ev]))
    pv, lv = plain.cpu().numpy(), out.cpu().numpy()
    pb, lb = plain_blocks.cpu().numpy(), blocks.cpu().numpy()
    coll = pv == 0
    lib.vg_mlp_destroy(m)
    rows = N_EDGES * probes
    return {
        "_verdicts": lv,
        "verdicts_identical": bool(np.array_equal(pv, lv)),
        "edges_per_s": N_EDGES / ((score_ms + check_ms) / 1e3),
        "ms_per_step": score_ms + check_ms,
        "inference_ms": score_ms,
        "inference": {"states_scored": rows, "probes_per_edge": probes,
                      "tflops": rows * 2 * (16 * 256 + 256 * 256 + 256) / (score_ms / 1e3) / 1e12},
        "ordered_check_ms": check_ms,
        "blocks_per_edge": {"plain": float(pb.mean()), "learned": float(lb.mean())},
        "blocks_per_colliding_edge": {"plain": float(pb[coll].mean()), "learned": float(lb[coll].mean())},
        "checks_saved_per_edge": float((pb - lb).mean()) * 8,
        "predictor": info,
    }


def run_gpu(args, world, rank, local):
    import torch

    import vamp_gb300 as vg
    from vamp_gb300._lib import check, lib

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    scene, a_np, b_np = workload()
    env = vg.Environment.from_scene(scene)
    a = torch.from_numpy(a_np).to(dev)
    b = torch.from_numpy(b_np).to(dev)
    out = torch.empty(N_EDGES, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)
    if args.schedule is None:
        pick = autotune("panda", env, a, b, RESOLUTION, stream.cuda_stream)
    else:
        env.set_schedule(args.schedule)
        pick = {"schedule": vg_schedules()[args.schedule]}
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def launch():
        check(lib.vg_validate_motions_device(b"panda", env.handle, a.data_ptr(), b.data_ptr(), N_EDGES, RESOLUTION,
                                             out.data_ptr(), None, stream.cuda_stream))

    for _ in range(max(args.warmup, 3)):
        launch()
    torch.cuda.synchronize()

    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    barrier(world)
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        for i in range(args.steps):
            flush.zero_()  # evict the inputs from L2 between timed steps
            starts[i].record(stream)
            launch()
            ends[i].record(stream)
        torch.cuda.synchronize()
        barrier(world)
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    kernel_ms = float(np.mean(step_ms))
    kernel_ms = max_over_ranks(world, kernel_ms)
    value = world * N_EDGES / (kernel_ms / 1e3)
    plain_blocks = torch.empty(N_EDGES, dtype=torch.int32, device=dev)  # untimed: the block counts
    check(lib.vg_validate_motions_device(b"panda", env.handle, a.data_ptr(), b.data_ptr(), N_EDGES, RESOLUTION,
                                         out.data_ptr(), plain_blocks.data_ptr(), stream.cuda_stream))
    learned = None if args.no_learned else measure_learned(args, env, a, b, out, stream, flush, dev, probes=args.probes)

    # end to end through the C ABI with host buffers
    pa = torch.empty(a_np.shape, dtype=torch.float32, pin_memory=True).numpy()
    pb = torch.empty(b_np.shape, dtype=torch.float32, pin_memory=True).numpy()
    pa[:] = a_np
    pb[:] = b_np
    pout = np.zeros(N_EDGES, np.uint8)
    for _ in range(max(args.warmup, 3)):
        vg.panda.validate_motion_batch(pa, pb, env, RESOLUTION, out=pout)
    barrier(world)
    e2e_t = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        vg.panda.validate_motion_batch(pa, pb, env, RESOLUTION, out=pout)
        e2e_t.append(time.perf_counter() - t0)
    e2e_s = max_over_ranks(world, float(np.mean(e2e_t)))
    gpu_verdicts = out.cpu().numpy()
    assert np.array_equal(gpu_verdicts, pout), "device and host-buffer calls disagree"

    if rank != 0:
        return
    line = {
        "metric": METRIC,
        "value": value,
        "unit": "edges/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": kernel_ms,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded scene and edges)",
        "config": {"workload": WORKLOAD, "edges": N_EDGES, "resolution": RESOLUTION, "order": "plain (reference block order)", "autotuner": pick,
                   "l2": "flushed between timed steps (256 MB write)", "parallelism": "replicas" if world > 1 else "1 GPU",
                   "colliding_fraction": float(1 - gpu_verdicts.mean())},
        "gpu_launches": args.steps,
        "e2e": {"value": world * N_EDGES / e2e_s, "unit": "edges/s", "h2d_bytes_per_step": int(a_np.nbytes + b_np.nbytes),
                "d2h_bytes_per_step": int(N_EDGES)},
    }
    clk = clocks.summary()
    line["clocks"] = clk
    work = algorithmic_flops(scene, a_np, b_np)
    peak, mhz, sms = fp32_peak_tflops(torch.cuda.get_device_properties(dev), clk["sm_mhz"] if clk else None)
    achieved = work["flops"] / (kernel_ms / 1e3) / 1e12
    line["roofline"] = {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
                        "traffic": profiled_traffic(),
                        "note": f"FP32 peak = {sms} SMs x 256 FLOP/clk x {mhz:.0f} MHz (max SM clock of MEASURED_PEAKS.json); "
                                f"algorithmic FLOPs counted by the CPU oracle on 8192 of the edges, scaled"}
    if not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(scene, a_np, b_np)
    line["vs_first_version"] = value / FIRST_VERSION_EDGES_PER_S
    paths = {"plain": gpu_verdicts}
    path_blocks = {"plain": plain_blocks.cpu().numpy()}
    if learned is not None:
        paths["learned"] = learned.pop("_verdicts")
        path_blocks["learned"] = None
        learned["learned_over_plain"] = learned["edges_per_s"] / value
        learned["vs_first_version"] = learned["edges_per_s"] / FIRST_VERSION_EDGES_PER_S
        line["learned"] = learned
    line["flips"] = reference_flips(scene, a_np, b_np, paths, path_blocks)
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline measurement")
    ap.add_argument("--no-learned", action="store_true", help="skip the learned-order measurement")
    ap.add_argument("--labels", type=int, default=2 << 20, help="exact-checker labels the learned order trains on")
    ap.add_argument("--probes", type=int, default=8, help="states per edge the learned order scores")
    ap.add_argument("--schedule", type=int, default=None,
                    help="GPU edge schedule (default: the autotuner's pick): 0 segment per edge, 1 warp per edge, "
                         "2 warp per edge with the register-rich build, 3 as 2 with free segments starting the next edge")
    ap.add_argument("--workload", default="edges",
                    choices=["edges", "capt", "mixed", "debug", "filter", "roadmap", "latency"],
                    help="edges: the 65,536-edge primitive scene (default); capt: the pointcloud workload; "
                         "mixed: four robots in one CUDA graph; debug: per-sphere collision reports; "
                         "filter: the pointcloud filter and CAPT build; roadmap: a batched PRM* roadmap; "
                         "latency: single validate_motion calls through the C ABI")
    args = ap.parse_args()
    world, rank, local = dist_init()
    if args.impl == "reference":
        run_reference(args, world, rank)
    elif args.workload == "capt":
        run_capt(args, world, rank, local)
    elif args.workload == "mixed":
        run_mixed(args, world, rank, local)
    elif args.workload == "debug":
        run_debug(args, world, rank, local)
    elif args.workload == "filter":
        run_filter(args, world, rank, local)
    elif args.workload == "roadmap":
        run_roadmap(args, world, rank, local)
    elif args.workload == "latency":
        run_latency(args, world, rank, local)
    else:
        run_gpu(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
