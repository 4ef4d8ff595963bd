"""The C++ drop-in (include/vamp_gb300_dropin.hh): the reference's Robot::fkcc and
planning::validate_motion signatures answered on the GPU.

tests/dropin/dropin_check.cc calls the hot path the way the reference's planners do
(planning/rrtc.hh:136: validate_motion<Robot, rake, Robot::resolution>(a, b, env); and
Robot::template fkcc<rake>(env, block)).
  * CPU: built against the reference's own headers, it compiles with both the reference robot and
    the GPU robot (so a planner compiles unchanged), and its reference-robot run reproduces the
    compiled reference's verdicts - the input path is right.
  * GPU: built against tests/dropin/stand_in.hh (the GPU machine has no reference checkout), its
    GPU-robot run gives the C ABI's and the oracle's verdicts, and reports the latency of one
    validate_motion call (one edge per GPU call)."""
import os
import shutil
import struct
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
SRC = ROOT / "tests" / "dropin" / "dropin_check.cc"
LIB_DIR = ROOT / "vamp_gb300" / "_lib"
# the reference's release flags (cmake/CompilerSettings.cmake:5,19-22), for the reference build
REF_FLAGS = ["-O3", "-fno-math-errno", "-fno-signed-zeros", "-fno-trapping-math", "-fno-rounding-math",
             "-ffp-contract=fast", "-fassociative-math"]


def workload(port):
    """A config-1 style scene with a 2,000-point cloud, 256 Panda edges and 128 blocks of 8."""
    from vamp_gb300 import scenes

    scene = scenes.scene_config1(3)
    cloud = scenes.surface_pointcloud(7, 2000)
    scene["pointclouds"] = [{"points": cloud, "r_min": 0.012, "r_max": 0.08, "r_point": scenes.POINT_RADIUS}]
    rb = port.robot("panda")
    a, b = scenes.edges(rb.s_m, rb.s_a, 256, 17)
    blocks = scenes.configurations(rb.s_m, rb.s_a, 128 * 8, 18).reshape(128, 8, 7)
    return scene, a, b, blocks


def write_input(path: Path, port, scene, a, b, blocks) -> None:
    penv = port.env(scene)
    rows = [penv.objects(k) for k in range(5)]  # fields then min_distance, sorted
    out = bytearray(struct.pack("<8i", *[len(r) for r in rows], len(a), len(blocks), len(scene["pointclouds"])))
    for r in rows:
        out += np.ascontiguousarray(r, np.float32).tobytes()
    out += np.ascontiguousarray(a, np.float32).tobytes() + np.ascontiguousarray(b, np.float32).tobytes()
    out += np.ascontiguousarray(blocks, np.float32).tobytes()
    for pc in scene["pointclouds"]:
        lay = port.capt(pc["points"], pc["r_min"], pc["r_max"], pc["r_point"])
        nb = lay["aff"].shape[1]
        out += struct.pack("<3i", int(lay["nlog2"]), nb, len(pc["points"]))
        out += np.ascontiguousarray(pc["points"], np.float32).tobytes()
        out += lay["tests"].astype(np.float32).tobytes() + lay["aabbs"].astype(np.float32).tobytes()
        out += lay["aff_starts"].astype(np.uint32).tobytes()
        out += np.ascontiguousarray(lay["aff"].transpose(1, 0, 2), np.float32).tobytes()  # [blocks][3][8]
        out += lay["top"].astype(np.float32).tobytes() + lay["radii"].astype(np.float32).tobytes()
    path.write_bytes(bytes(out))


def read_output(path: Path, n_edges: int, n_blocks: int):
    raw = path.read_bytes()
    edges = np.frombuffer(raw[:n_edges], np.uint8).copy()
    blocks = np.frombuffer(raw[n_edges:n_edges + n_blocks], np.uint8).copy()
    per_call = struct.unpack("<d", raw[n_edges + n_blocks:n_edges + n_blocks + 8])[0]
    return edges, blocks, per_call


def compile_program(out: Path, extra: list) -> None:
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    cmd = [cxx, "-std=c++17", "-w", *extra, f"-I{ROOT / 'include'}", str(SRC), "-o", str(out), f"-L{LIB_DIR}",
           "-lvamp_gb300", f"-Wl,-rpath,{LIB_DIR}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]


def oracle_blocks(port, scene, blocks):
    penv = port.env(scene)
    rb = port.robot("panda")
    return np.array([penv.fkcc_block(rb, np.ascontiguousarray(q)) for q in blocks], np.uint8)


def test_dropin_compiles_against_the_reference_and_reproduces_it(port, tmp_path):
    """Needs the reference's headers (recorded when the reference oracle was built) and an x86-64
    host (the reference's AVX2 build)."""
    from oracle.vgo import Reference, built_reference_headers

    inc = built_reference_headers()
    if inc is None or os.uname().machine != "x86_64":
        pytest.skip("the reference's headers are not available here")
    if not (LIB_DIR / "libvamp_gb300.so").exists():
        pytest.skip("libvamp_gb300.so is not built")
    exe = tmp_path / "dropin_ref"
    compile_program(exe, ["-DVG_DROPIN_REFERENCE", "-march=native", "-mavx2", *REF_FLAGS,
                          f"-I{ROOT / 'oracle' / 'ref' / 'shim'}", f"-I{inc}"])
    scene, a, b, blocks = workload(port)
    write_input(tmp_path / "in.bin", port, scene, a, b, blocks)
    r = subprocess.run([str(exe), str(tmp_path / "in.bin"), str(tmp_path / "out.bin"), "--cpu"], capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    edges, blk, _ = read_output(tmp_path / "out.bin", len(a), len(blocks))
    ref = Reference().env(scene).validate_motions("panda", a, b, 32)
    assert np.array_equal(edges, ref)
    assert np.array_equal(blk, oracle_blocks(port, scene, blocks))
    assert 0 < edges.sum() < len(edges) and 0 < blk.sum() < len(blk)


@pytest.mark.gpu
def test_dropin_gpu_gives_the_c_abi_and_oracle_verdicts(port, tmp_path):
    import vamp_gb300 as vg

    exe = tmp_path / "dropin_gpu"
    compile_program(exe, ["-O2", "-ffp-contract=off", f"-I{ROOT / 'tests' / 'dropin'}"])
    scene, a, b, blocks = workload(port)
    write_input(tmp_path / "in.bin", port, scene, a, b, blocks)
    r = subprocess.run([str(exe), str(tmp_path / "in.bin"), str(tmp_path / "out.bin")], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr
    edges, blk, per_call = read_output(tmp_path / "out.bin", len(a), len(blocks))
    abi = vg.panda.validate_motion_batch(a, b, vg.Environment.from_scene(scene), 32)
    cpu, _ = port.env(scene).validate_motions(port.robot("panda"), a, b, 32)
    assert np.array_equal(edges, abi)
    assert np.array_equal(edges, cpu)
    assert np.array_equal(blk, oracle_blocks(port, scene, blocks))
    print(f"drop-in validate_motion: {per_call * 1e6:.1f} us per single-edge call")
